// batch.cu -- many images, uneven sizes, mixed operators, one CUDA-graph
// launch.
//
// The host groups the jobs into classes (operator x pixel type x radius) and
// cuts every job into strips (FIR: 128-column strips, box: ~1000-column
// strips; strip heights per operator chosen by the autotuner).  Each class
// runs as one specialised kernel with one CTA per strip, through the same
// strip routines the single-image kernels use, so every batched output is
// identical to the single-image call.  All class kernels are nodes of one
// CUDA graph without edges: they run concurrently, so compute-bound Gaussian
// strips and memory-bound box strips share the SMs.  (One kernel dispatching
// over all classes was tried first; the union of its register needs spilled
// heavily.)  Each image keeps its own TMA descriptor in global memory.
#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "batch_types.h"
#include "fir3_dispatch.h"
#include "fir_tc.h"
#include "box_kernels.h"
#include "box_ops.cuh"
#include "fir_v3.cuh"
#include "tucu_internal.h"

namespace
{

using namespace tucu;
using batch::BoxJobD;
using batch::FirJobD;
using batch::Item;

// Relative cost per pixel (FP32 operations bound the Gaussian, bytes the
// box); orders classes and items longest first.
double fir_cost(int r) { return 4.0 * r + 8.0; }
constexpr double kBoxCost = 10.0;

// A class: jobs that share one specialised kernel.
struct Class
{
    int kind;  // 0 = FIR, 1 = box, 2 = tensor-core FIR / box (any taps)
    int in_dtype;
    int out_dtype;
    int r;     // FIR radius; box: columns per lane of the strip (4 or 8)
    bool vec;  // box rows aligned for the copies of the strip's pixel groups
    bool win = false;  // box: the window-ring kernel
    const void* fn = nullptr;
    size_t smem = 0;
    double cost = 0.0;
    std::vector<Item> items;
    size_t offset = 0;  // first item in the device item array
};

const void* fir_class_kernel(int in_dt, int out_dt, int r, size_t* smem)
{
    fir::Batch3Fn fn = fir::batch3_fn(in_dt, out_dt);
    return fn ? fn(r, smem) : nullptr;
}

// Pads a lobe of length L (outermost first) on its outer side to radius R.
void pad_to(const float* lobe, int L, int R, float* out)
{
    const int r = L & ~1;
    for (int k = 0; k <= R; ++k)
        out[k] = 0.0f;
    for (int k = 0; k < L; ++k)
        out[R - r + k] = lobe[k];
}

const int kOpLobes[6][2] = {{0, 0}, {1, 0}, {0, 1}, {2, 0}, {1, 1}, {0, 2}};

}  // namespace

struct tucu_batch
{
    std::vector<tucu_batch_job> spec;
    std::vector<FirJobD> fjobs;
    std::vector<CUtensorMap> tmaps;
    std::vector<BoxJobD> bjobs;
    std::vector<tcf::TcJob> tjobs;
    std::vector<Class> classes;
    std::vector<Item> all_items;
    // device copies
    FirJobD* d_fjobs = nullptr;
    CUtensorMap* d_tmaps = nullptr;
    BoxJobD* d_bjobs = nullptr;
    tcf::TcJob* d_tjobs = nullptr;
    Item* d_items = nullptr;
    size_t cap_f = 0, cap_t = 0, cap_b = 0, cap_i = 0, cap_tj = 0;
    int tensor = 0;  // FIR and box jobs of f16 images on the tensor cores
    int device = -1;
    int planned = 0;
    size_t max_smem = 0;
    cudaGraphExec_t exec = nullptr;
    int graph_valid = 0;
    // pinned staging of the tables for stream-ordered uploads
    unsigned char* h_stage = nullptr;
    size_t h_stage_cap = 0;
};

static void free_device(tucu_batch* b)
{
    if (b->h_stage)
        cudaFreeHost(b->h_stage);
    b->h_stage = nullptr;
    b->h_stage_cap = 0;
    if (b->exec)
        cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    b->graph_valid = 0;
    cudaFree(b->d_fjobs);
    cudaFree(b->d_tmaps);
    cudaFree(b->d_bjobs);
    cudaFree(b->d_tjobs);
    cudaFree(b->d_items);
    b->d_tjobs = nullptr;
    b->cap_tj = 0;
    b->d_fjobs = nullptr;
    b->d_tmaps = nullptr;
    b->d_bjobs = nullptr;
    b->d_items = nullptr;
    b->cap_f = b->cap_t = b->cap_b = b->cap_i = 0;
}

template <class T>
static cudaError_t reserve(T** d, size_t* cap, size_t n)
{
    n = std::max<size_t>(1, n);
    if (n <= *cap)
        return cudaSuccess;
    cudaFree(*d);
    *d = nullptr;
    *cap = 0;
    cudaError_t e = cudaMalloc(d, n * sizeof(T));
    if (e == cudaSuccess)
        *cap = n;
    return e;
}

// Copies a table to the device: synchronously, or (stream != nullptr) from
// the batch's pinned staging area in stream order.
template <class T>
static cudaError_t upload(T** d, size_t* cap, const std::vector<T>& h, unsigned char* stage,
                          size_t* stage_off, cudaStream_t stream)
{
    cudaError_t e = reserve(d, cap, h.size());
    if (e != cudaSuccess || h.empty())
        return e;
    const size_t bytes = h.size() * sizeof(T);
    if (!stage)
        return cudaMemcpy(*d, h.data(), bytes, cudaMemcpyHostToDevice);
    std::memcpy(stage + *stage_off, h.data(), bytes);
    e = cudaMemcpyAsync(*d, stage + *stage_off, bytes, cudaMemcpyHostToDevice, stream);
    *stage_off += (bytes + 255) / 256 * 256;
    return e;
}

// Kernel arguments of one class (pointers into the device tables).
struct ClassArgs
{
    const void* jobs;
    const void* tmaps;
    const void* items;
    void* argv[3];
    int nargs;
};

// Grid of a class kernel: one CTA per item (FIR and tensor-core strips) or
// per eight warp items (box).
static dim3 class_grid(const Class& c)
{
    return dim3((unsigned)(c.kind == 1 ? c.items.size() / box::kWarps : c.items.size()));
}

static dim3 class_block(const Class& c) { return dim3(c.kind == 2 ? tcf::kThreads : 256); }

static ClassArgs class_args(const tucu_batch* b, const Class& c)
{
    ClassArgs a;
    a.items = b->d_items + c.offset;
    if (c.kind == 0) {
        a.jobs = b->d_fjobs;
        a.tmaps = b->d_tmaps;
        a.nargs = 3;
    } else if (c.kind == 2) {
        a.jobs = b->d_tjobs;
        a.tmaps = nullptr;
        a.nargs = 2;
    } else {
        a.jobs = b->d_bjobs;
        a.tmaps = nullptr;
        a.nargs = 2;
    }
    return a;
}

extern "C" {

int tucu_batch_create(tucu_batch** out)
{
    if (!out)
        return fail(TUCU_ERR_ARG, "null handle pointer");
    auto* b = new (std::nothrow) tucu_batch;
    if (!b)
        return fail(TUCU_ERR_NOMEM, "host allocation");
    *out = b;
    return TUCU_OK;
}

int tucu_batch_clear(tucu_batch* b)
{
    if (!b)
        return fail(TUCU_ERR_ARG, "null handle");
    b->spec.clear();
    b->planned = 0;
    b->graph_valid = 0;
    return TUCU_OK;
}

int tucu_batch_set_tensor_cores(tucu_batch* b, int on)
{
    if (!b)
        return fail(TUCU_ERR_ARG, "null handle");
    b->tensor = on ? 1 : 0;
    b->planned = 0;
    b->graph_valid = 0;
    return TUCU_OK;
}

int tucu_batch_add(tucu_batch* b, const tucu_batch_job* j)
{
    if (!b || !j)
        return fail(TUCU_ERR_ARG, "null argument");
    if (j->op != TUCU_BATCH_GAUSS && j->op != TUCU_BATCH_BOX)
        return fail(TUCU_ERR_ARG, "batched operators are Gaussian and box");
    if (!j->in || !j->out || j->rows <= 0 || j->cols <= 0)
        return fail(TUCU_ERR_ARG, "null image or empty size");
    if (j->in_dtype < TUCU_U8 || j->in_dtype > TUCU_I32 || j->out_dtype < TUCU_U8 ||
        j->out_dtype > TUCU_I32)
        return fail(TUCU_ERR_DTYPE, "unknown dtype");
    if (j->in_pitch < (size_t)j->cols * dtype_size(j->in_dtype) ||
        j->out_pitch < (size_t)j->cols * dtype_size(j->out_dtype))
        return fail(TUCU_ERR_ARG, "pitch smaller than a row");
    if (j->op == TUCU_BATCH_GAUSS) {
        if (j->in_dtype == TUCU_I32)
            return fail(TUCU_ERR_DTYPE, "Gaussian input must be u8, f16, bf16 or f32");
        if (j->gauss_op < 0 || j->gauss_op > 5 || !(j->sigma > 0.0f))
            return fail(TUCU_ERR_ARG, "bad Gaussian operator or sigma");
    } else if (j->winV < 1 || j->winH < 1 || j->winV > TUCU_WIN_LIMIT || j->winH > TUCU_WIN_LIMIT) {
        return fail(TUCU_ERR_WINDOW, "window size out of range");
    }
    b->spec.push_back(*j);
    b->planned = 0;
    b->graph_valid = 0;
    return (int)b->spec.size() - 1;
}

// Adds a job to the tensor-core class of its output type, cut into strips of
// 128 output columns x equal bands of at most fr rows; false when its input
// cannot be described by a TMA map (the job then takes the FP32-pipe path).
static bool add_tc_job(tucu_batch* b, const tucu_batch_job& s, const float* th, int nth,
                       const float* tv, int ntv, float post, int oy, int ox, int fr)
{
    tcf::TcJob J;
    if (!tcf::fill_job(&J, s.in, s.in_pitch, s.rows, s.cols, s.out, s.out_pitch, s.out_dtype, oy,
                       ox, th, nth, tv, ntv, post))
        return false;
    const int ji = (int)b->tjobs.size();
    b->tjobs.push_back(J);
    Class* cp = nullptr;
    for (Class& c : b->classes)
        if (c.kind == 2 && c.out_dtype == s.out_dtype)
            cp = &c;
    if (!cp) {
        Class c;
        c.kind = 2;
        c.in_dtype = s.in_dtype;
        c.out_dtype = s.out_dtype;
        c.r = 0;
        c.vec = false;
        b->classes.push_back(c);
        cp = &b->classes.back();
    }
    cp->cost += (double)s.rows * s.cols * 6.0;
    const int nb = (J.orows + fr - 1) / fr;
    const int band = ((J.orows + nb - 1) / nb + tcf::kCH - 1) / tcf::kCH * tcf::kCH;
    for (int y = 0; y < J.orows; y += band)
        for (int x = 0; x < J.ocols; x += tcf::kTW)
            cp->items.push_back({ji, x, y, std::min(band, J.orows - y)});
    return true;
}

static int plan_impl(tucu_batch* b, int fir_strip_rows, int box_strip_rows, bool on_stream,
                     cudaStream_t stream)
{
    if (!b)
        return fail(TUCU_ERR_ARG, "null handle");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    const int fr = fir_strip_rows > 0 ? (fir_strip_rows + fir3::kCH - 1) / fir3::kCH * fir3::kCH : 512;
    // Box bands in 16-row units (float sums restart on the absolute 64-row
    // grid whatever the band, so batched sums equal the single-image ones).
    const int br = box_strip_rows > 0 ? (box_strip_rows + 15) / 16 * 16 : 128;
    b->fjobs.clear();
    b->tmaps.clear();
    b->bjobs.clear();
    b->tjobs.clear();
    b->classes.clear();
    b->all_items.clear();
    auto class_of = [&](int kind, int dt, int odt, int r, bool vec, bool win = false) -> Class& {
        for (Class& c : b->classes)
            if (c.kind == kind && c.in_dtype == dt && c.out_dtype == odt && c.r == r && c.vec == vec &&
                c.win == win)
                return c;
        Class c;
        c.kind = kind;
        c.in_dtype = dt;
        c.out_dtype = odt;
        c.r = r;
        c.vec = vec;
        c.win = win;
        b->classes.push_back(c);
        return b->classes.back();
    };
    for (const tucu_batch_job& s : b->spec) {
        if (s.op == TUCU_BATCH_GAUSS) {
            float lb[3][TUCU_LOBE_MAX];
            int n[3];
            int rc = tucu_gauss_design(s.sigma, lb[0], &n[0], lb[1], &n[1], lb[2], &n[2]);
            if (rc)
                return rc;
            const int lh = kOpLobes[s.gauss_op][0], lv = kOpLobes[s.gauss_op][1];
            const int rh = n[lh] & ~1, rv = n[lv] & ~1;
            if (rh != rv)
                return fail(TUCU_ERR_ARG, "batched Gaussian operators need equal H/V radii");
            if (s.rows <= 2 * rv || s.cols <= 2 * rh)
                continue;  // nothing to write (TUCU_NOOP for the single call)
            if (b->tensor && tcf::eligible(s.in_dtype, s.out_dtype, 2 * rh + 1, 2 * rv + 1)) {
                float th[tcf::kMaxTaps], tv[tcf::kMaxTaps];
                const int nth = tcf::full_taps(lb[lh], n[lh], th), ntv = tcf::full_taps(lb[lv], n[lv], tv);
                if (add_tc_job(b, s, th, nth, tv, ntv, 1.0f, s.shift ? rv : 0, s.shift ? rh : 0, fr))
                    continue;
            }
            FirJobD J;
            std::memset(&J, 0, sizeof(J));
            const int R = rh;
            pad_to(lb[lh], n[lh], R, J.lobes.h[0]);
            pad_to(lb[lv], n[lv], R, J.lobes.v[0]);
            J.lobes.sym_h = n[lh] & 1;
            J.lobes.sym_v = n[lv] & 1;
            fir::FirJob& F = J.fir;
            F.src = s.in;
            F.src_pitch = s.in_pitch;
            F.rows = s.rows;
            F.cols = s.cols;
            F.orows = s.rows - 2 * rv;
            F.ocols = s.cols - 2 * rh;
            F.oy = s.shift ? rv : 0;
            F.ox = s.shift ? rh : 0;
            F.nh = 1;
            F.nout = 1;
            F.out_dtype = s.out_dtype;
            F.dst[0] = s.out;
            F.dst_pitch[0] = s.out_pitch;
            CUtensorMap tm;
            std::memset(&tm, 0, sizeof(tm));
            J.has_tmap = make_tmap_2d(&tm, s.in, s.in_dtype, s.cols, s.rows, s.in_pitch,
                                      fir::round_up(fir3::kTW + 2 * R, 16), fir3::kCH);
            const int ji = (int)b->fjobs.size();
            b->fjobs.push_back(J);
            b->tmaps.push_back(tm);
            Class& c = class_of(0, s.in_dtype, s.out_dtype, R, false);
            c.cost += (double)s.rows * s.cols * fir_cost(R);
            // Bands of equal height (at most fr rows) rather than fr-row
            // bands and a short remainder: every strip pays the 2R halo rows.
            const int nb = (F.orows + fr - 1) / fr;
            const int band = ((F.orows + nb - 1) / nb + fir3::kCH - 1) / fir3::kCH * fir3::kCH;
            for (int y = 0; y < F.orows; y += band)
                for (int x = 0; x < F.ocols; x += fir3::kTW)
                    c.items.push_back({ji, x, y, std::min(band, F.orows - y)});
        } else {
            if (s.rows < s.winV || s.cols < s.winH)
                continue;
            if (b->tensor && tcf::eligible(s.in_dtype, s.out_dtype, s.winH, s.winV)) {
                float ones[tcf::kMaxTaps];
                std::fill(ones, ones + tcf::kMaxTaps, 1.0f);
                const float post = s.normalize ? 1.0f / (float)(s.winV * s.winH) : 1.0f;
                if (add_tc_job(b, s, ones, s.winH, ones, s.winV, post, s.shift ? s.winV / 2 : 0,
                               s.shift ? s.winH / 2 : 0, fr))
                    continue;
            }
            BoxJobD J;
            std::memset(&J, 0, sizeof(J));
            J.src = s.in;
            J.src_pitch = s.in_pitch;
            J.rows = s.rows;
            J.cols = s.cols;
            J.wV = s.winV;
            J.wH = s.winH;
            J.orows = s.rows + 1 - s.winV;
            J.ocols = s.cols + 1 - s.winH;
            J.dst = s.out;
            J.dst_pitch = s.out_pitch;
            J.out_dtype = s.out_dtype;
            J.oy = s.shift ? s.winV / 2 : 0;
            J.ox = s.shift ? s.winH / 2 : 0;
            J.normalize = s.normalize ? 1 : 0;
            J.cls = box::store_class(s.out, s.out_pitch, J.ox, dtype_size(s.out_dtype));
            // The strip width rule of the single-image launch, so an image's
            // float sums are the same batched or alone.
            const int cpt = box::plain_cpt(s.winH);
            const bool vec = box::plain_vec(s.in, s.in_pitch, s.in_dtype, cpt);
            const int ji = (int)b->bjobs.size();
            b->bjobs.push_back(J);
            const bool win = box::plain_win(s.in_dtype, s.out_dtype, vec, cpt, s.winV);
            Class& c = class_of(1, s.in_dtype, s.out_dtype, cpt, vec, win);
            c.cost += (double)s.rows * s.cols * kBoxCost;
            // One item per warp (warp column x row band); a CTA takes eight
            // consecutive items, so narrow images leave no warp of a CTA idle.
            const int tw = box::out_cols_per_warp(J.wH, cpt);
            for (int y = 0; y < J.orows; y += br)
                for (int x = 0; x < J.ocols; x += tw)
                    c.items.push_back({ji, x, y, std::min(br, J.orows - y)});
        }
    }
    // FIR classes: tallest strips first, so the short ones fill the last
    // round.  Box classes: whole CTAs of warp items (the padding items do
    // nothing).
    for (Class& c : b->classes) {
        if (c.kind == 0 || c.kind == 2)
            std::stable_sort(c.items.begin(), c.items.end(),
                             [](const Item& x, const Item& y) { return x.nrows > y.nrows; });
        if (c.kind == 1)
            while (c.items.size() % box::kWarps)
                c.items.push_back({-1, 0, 0, 0});
    }
    // Most expensive class first (for the serial launch order); one item array.
    std::stable_sort(b->classes.begin(), b->classes.end(),
                     [](const Class& x, const Class& y) { return x.cost > y.cost; });
    b->max_smem = 0;
    for (Class& c : b->classes) {
        c.offset = b->all_items.size();
        b->all_items.insert(b->all_items.end(), c.items.begin(), c.items.end());
        if (c.kind == 0) {
            c.fn = fir_class_kernel(c.in_dtype, c.out_dtype, c.r, &c.smem);
            if (!c.fn)
                return fail(TUCU_ERR_ARG, "no batch kernel for this radius");
            if ((e = cudaFuncSetAttribute(c.fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)c.smem)) != cudaSuccess)
                return cuda_fail(e, "batch kernel shared memory");
        } else if (c.kind == 2) {
            c.fn = tcf::kernel_for(c.out_dtype);
            c.smem = tcf::smem_bytes();
            if (!c.fn)
                return fail(TUCU_ERR_DTYPE, "no tensor-core kernel for this type");
            if ((e = cudaFuncSetAttribute(c.fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)c.smem)) != cudaSuccess)
                return cuda_fail(e, "tensor-core kernel shared memory");
        } else {
            c.fn = box::batch_kernel(c.in_dtype, c.out_dtype, c.vec, c.r, c.win);
            c.smem = box::plain_smem_bytes(c.in_dtype, c.r, c.win);
            if (!c.fn)
                return fail(TUCU_ERR_DTYPE, "no box batch kernel for this type");
        }
        b->max_smem = std::max(b->max_smem, c.smem);
    }
    if (b->device != dev)
        free_device(b);
    b->device = dev;
    unsigned char* stage = nullptr;
    size_t soff = 0;
    if (on_stream) {
        const size_t need = b->fjobs.size() * sizeof(FirJobD) + b->tmaps.size() * sizeof(CUtensorMap) +
                            b->bjobs.size() * sizeof(BoxJobD) + b->tjobs.size() * sizeof(tcf::TcJob) +
                            b->all_items.size() * sizeof(Item) + 5 * 256;
        if (need > b->h_stage_cap) {
            // the previous uploads from the old area must be done before it goes
            if (b->h_stage) {
                cudaStreamSynchronize(stream);
                cudaFreeHost(b->h_stage);
            }
            b->h_stage = nullptr;
            b->h_stage_cap = 0;
            const size_t cap = std::max(need * 2, (size_t)1 << 20);
            if ((e = cudaHostAlloc(&b->h_stage, cap, cudaHostAllocDefault)) != cudaSuccess)
                return cuda_fail(e, "pinned batch staging");
            b->h_stage_cap = cap;
        }
        stage = b->h_stage;
    }
    if ((e = upload(&b->d_fjobs, &b->cap_f, b->fjobs, stage, &soff, stream)) != cudaSuccess ||
        (e = upload(&b->d_tmaps, &b->cap_t, b->tmaps, stage, &soff, stream)) != cudaSuccess)
        return cuda_fail(e, "batch FIR table");
    if ((e = upload(&b->d_bjobs, &b->cap_b, b->bjobs, stage, &soff, stream)) != cudaSuccess)
        return cuda_fail(e, "batch box table");
    if ((e = upload(&b->d_tjobs, &b->cap_tj, b->tjobs, stage, &soff, stream)) != cudaSuccess)
        return cuda_fail(e, "batch tensor-core table");
    if ((e = upload(&b->d_items, &b->cap_i, b->all_items, stage, &soff, stream)) != cudaSuccess)
        return cuda_fail(e, "batch work list");
    b->planned = 1;
    b->graph_valid = 0;
    return TUCU_OK;
}

}  // extern "C"

namespace tucu
{
// Plans with stream-ordered table uploads (the server's waves): the tables go
// through pinned staging owned by the batch, which the caller must not
// re-plan until the stream has passed this point.
int batch_plan_on_stream(tucu_batch* b, int fir_rows, int box_rows, cudaStream_t stream)
{
    return plan_impl(b, fir_rows, box_rows, true, stream);
}

// Grows the device tables ahead of time so that later plans do not allocate.
int batch_reserve(tucu_batch* b, size_t fir_jobs, size_t box_jobs, size_t items)
{
    if (!b)
        return fail(TUCU_ERR_ARG, "null handle");
    cudaError_t e;
    if ((e = reserve(&b->d_fjobs, &b->cap_f, fir_jobs)) != cudaSuccess ||
        (e = reserve(&b->d_tmaps, &b->cap_t, fir_jobs)) != cudaSuccess ||
        (e = reserve(&b->d_bjobs, &b->cap_b, box_jobs)) != cudaSuccess ||
        (e = reserve(&b->d_tjobs, &b->cap_tj, fir_jobs + box_jobs)) != cudaSuccess ||
        (e = reserve(&b->d_items, &b->cap_i, items)) != cudaSuccess)
        return cuda_fail(e, "batch tables");
    cudaGetDevice(&b->device);
    return TUCU_OK;
}
}  // namespace tucu

extern "C" {

int tucu_batch_plan(tucu_batch* b, int fir_strip_rows, int box_strip_rows)
{
    return plan_impl(b, fir_strip_rows, box_strip_rows, false, nullptr);
}

static cudaError_t launch_classes(tucu_batch* b, cudaStream_t st)
{
    for (const Class& c : b->classes) {
        if (c.items.empty())
            continue;
        ClassArgs a = class_args(b, c);
        void* argv[3] = {&a.jobs, c.kind == 0 ? (void*)&a.tmaps : (void*)&a.items, &a.items};
        cudaError_t e = cudaLaunchKernel(c.fn, class_grid(c), class_block(c), argv,
                                         c.smem, st);
        if (e != cudaSuccess)
            return e;
    }
    return cudaSuccess;
}

int tucu_batch_launch(tucu_batch* b, void* stream)
{
    if (!b)
        return fail(TUCU_ERR_ARG, "null handle");
    if (!b->planned)
        return fail(TUCU_ERR_STATE, "tucu_batch_plan must run after the last add");
    if (b->all_items.empty())
        return TUCU_NOOP;
    const cudaError_t e = launch_classes(b, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? TUCU_OK : cuda_fail(e, "batch launch");
}

int tucu_batch_graph_launch(tucu_batch* b, void* stream)
{
    if (!b)
        return fail(TUCU_ERR_ARG, "null handle");
    if (!b->planned)
        return fail(TUCU_ERR_STATE, "tucu_batch_plan must run after the last add");
    if (b->all_items.empty())
        return TUCU_NOOP;
    cudaError_t e;
    if (!b->graph_valid) {
        if (b->exec) {
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
        // One graph, one kernel node per class, no edges: the classes run
        // concurrently and their CTAs share the SMs.
        cudaGraph_t g = nullptr;
        if ((e = cudaGraphCreate(&g, 0)) != cudaSuccess)
            return cuda_fail(e, "graph create");
        for (const Class& c : b->classes) {
            if (c.items.empty())
                continue;
            ClassArgs a = class_args(b, c);
            void* argv[3] = {&a.jobs, c.kind == 0 ? (void*)&a.tmaps : (void*)&a.items, &a.items};
            cudaKernelNodeParams kp = {};
            kp.func = const_cast<void*>(c.fn);
            kp.gridDim = class_grid(c);
            kp.blockDim = class_block(c);
            kp.sharedMemBytes = (unsigned)c.smem;
            kp.kernelParams = argv;
            cudaGraphNode_t node;
            if ((e = cudaGraphAddKernelNode(&node, g, nullptr, 0, &kp)) != cudaSuccess) {
                cudaGraphDestroy(g);
                return cuda_fail(e, "graph kernel node");
            }
        }
        e = cudaGraphInstantiate(&b->exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess)
            return cuda_fail(e, "graph instantiate");
        b->graph_valid = 1;
    }
    e = cudaGraphLaunch(b->exec, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? TUCU_OK : cuda_fail(e, "graph launch");
}

int tucu_batch_info(const tucu_batch* b, int* njobs, int* nitems, int* nkernels, size_t* smem)
{
    if (!b)
        return fail(TUCU_ERR_ARG, "null handle");
    int nk = 0;
    for (const Class& c : b->classes)
        nk += c.items.empty() ? 0 : 1;
    if (njobs)
        *njobs = (int)(b->fjobs.size() + b->bjobs.size() + b->tjobs.size());
    if (nitems)
        *nitems = (int)b->all_items.size();
    if (nkernels)
        *nkernels = nk;
    if (smem)
        *smem = b->max_smem;
    return b->planned ? TUCU_OK : TUCU_NOOP;
}

void tucu_batch_destroy(tucu_batch* b)
{
    if (!b)
        return;
    free_device(b);
    delete b;
}

}  // extern "C"
