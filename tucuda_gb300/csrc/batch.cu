// batch.cu -- many images, uneven sizes, mixed operators, one persistent
// launch (captured once in a CUDA graph and replayed).
//
// The host plans a work list of strips (FIR: 64-column strips, box:
// ~1000-column strips; strip heights chosen per operator by the autotuner),
// ordered longest job first.  The persistent kernel runs one CTA per SM slot;
// each CTA pulls the next strip from an atomic queue counter and dispatches
// on (operator, pixel type, radius) to the same strip routines the
// single-image kernels use, so every batched output is identical to the
// single-image call.  Compute-bound Gaussian strips and memory-bound box
// strips share the SMs, which is what lets a mixed batch approach the HBM
// roofline.  Each image keeps its own TMA descriptor in global memory.
#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "box_kernels.h"
#include "box_ops.cuh"
#include "fir_strip.cuh"
#include "tucu_internal.h"

namespace tucu
{
namespace batch
{

enum Kind : int { kFir = 0, kBox = 1 };

// Device copy of one job.  Kept in global memory; strips read it through L1.
struct alignas(64) Job
{
    int kind;
    int in_dtype;
    int r;                 // FIR radius (both directions)
    int has_tmap;
    fir::FirJob fir;       // FIR geometry and outputs
    fir::LobeSet lobes;
    // box
    const void* src;
    size_t src_pitch;
    int rows, cols;
    int wV, wH, orows, ocols;
    void* dst;
    size_t dst_pitch;
    int out_dtype, oy, ox, normalize;
    int vec;               // rows 4-element aligned for vector loads
};

struct Item
{
    int job;
    int x0, y0, nrows;
};

constexpr int kBoxSmemOff = 1024;  // box scratch after the FIR barrier/coefficient area

// ---- device side ---------------------------------------------------------------

template <class TIn>
__device__ __noinline__ bool fir_item(const Job& J, const CUtensorMap* tmap, const Item& it,
                         unsigned char* smem, fir::Pipe& pipe)
{
    const int nsteps = (it.nrows + 31) / 32;
    switch (J.r) {
    case 2: return fir::run_strip<2, 2, 1, 32, TIn>(J.fir, J.lobes, tmap, it.x0, it.y0, nsteps, smem, pipe);
    case 4: return fir::run_strip<4, 4, 1, 32, TIn>(J.fir, J.lobes, tmap, it.x0, it.y0, nsteps, smem, pipe);
    case 8: return fir::run_strip<8, 8, 1, 32, TIn>(J.fir, J.lobes, tmap, it.x0, it.y0, nsteps, smem, pipe);
    default: return fir::run_strip<16, 16, 1, 32, TIn>(J.fir, J.lobes, tmap, it.x0, it.y0, nsteps, smem, pipe);
    }
}

template <class TIn, class Acc>
__device__ __noinline__ void box_item(const Job& J, const Item& it, unsigned char* smem)
{
    constexpr int U = box::BoxRows<TIn>::value;
    // The previous strip of this CTA may still read the shared buffers.
    __syncthreads();
    box::PlainEpi<Acc> epi{J.dst, J.dst_pitch, J.out_dtype, J.oy, J.ox, J.normalize,
                           (float)(J.wV * J.wH)};
    if (J.vec) {
        box::PlainProd<TIn, Acc, true> prod{J.src, J.src_pitch, J.rows, J.cols};
        box::run_strip<1, Acc, U>(prod, epi, J.wV, J.wH, it.x0, it.y0, it.nrows, J.ocols,
                                  J.ox & 3, smem + kBoxSmemOff);
    } else {
        box::PlainProd<TIn, Acc, false> prod{J.src, J.src_pitch, J.rows, J.cols};
        box::run_strip<1, Acc, U>(prod, epi, J.wV, J.wH, it.x0, it.y0, it.nrows, J.ocols,
                                  J.ox & 3, smem + kBoxSmemOff);
    }
}

__global__ void __launch_bounds__(fir::kThreads, 2)
    batch_kernel(const Job* __restrict__ jobs, const CUtensorMap* __restrict__ tmaps,
                 const Item* __restrict__ items, int nitems, unsigned* counter)
{
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
    int& s_item = *reinterpret_cast<int*>(smem + 8 * fir::kMaxStage);  // after the barriers
    if (threadIdx.x == 0) {
        for (int s = 0; s < fir::kMaxStage; ++s)
            mbar_init(&bars[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    fir::Pipe pipe{0};
    while (true) {
        if (threadIdx.x == 0)
            s_item = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int i = s_item;
        __syncthreads();  // everyone has read s_item before it is overwritten
        if (i >= nitems)
            break;
        const Item it = items[i];
        const Job& J = jobs[it.job];
        if (J.kind == kFir) {
            const CUtensorMap* tm = J.has_tmap ? &tmaps[it.job] : nullptr;
            bool ok = true;
            switch (J.in_dtype) {
            case U8: ok = fir_item<uint8_t>(J, tm, it, smem, pipe); break;
            case F16: ok = fir_item<__half>(J, tm, it, smem, pipe); break;
            case BF16: ok = fir_item<__nv_bfloat16>(J, tm, it, smem, pipe); break;
            default: ok = fir_item<float>(J, tm, it, smem, pipe); break;
            }
            if (!ok)
                return;  // a bounded wait ran out; the error word is set
        } else {
            switch (J.in_dtype) {
            case U8: box_item<uint8_t, int>(J, it, smem); break;
            case I32: box_item<int32_t, int>(J, it, smem); break;
            case F16: box_item<__half, float>(J, it, smem); break;
            case BF16: box_item<__nv_bfloat16, float>(J, it, smem); break;
            default: box_item<float, float>(J, it, smem); break;
            }
        }
    }
}

}  // namespace batch
}  // namespace tucu

TUCU_DEFINE_ERROR_ACCESSOR(tucu_batch_tu_error)

// ---- host side -------------------------------------------------------------------

using namespace tucu;

namespace
{

size_t fir_smem(int r, int dt)
{
    switch (dt) {
    case U8: return fir::smem_u8(r, r, 1);
    case F16: return fir::smem_f16(r, r, 1);
    case BF16: return fir::smem_bf16(r, r, 1);
    default: return fir::smem_f32(r, r, 1);
    }
}

size_t box_smem(int dt)
{
    switch (dt) {
    case U8: return sizeof(box::Smem<1, int, box::BoxRows<uint8_t>::value>);
    case I32: return sizeof(box::Smem<1, int, box::BoxRows<int32_t>::value>);
    case F16: return sizeof(box::Smem<1, float, box::BoxRows<__half>::value>);
    case BF16: return sizeof(box::Smem<1, float, box::BoxRows<__nv_bfloat16>::value>);
    default: return sizeof(box::Smem<1, float, box::BoxRows<float>::value>);
    }
}

// Relative cost of one pixel of a job (FP32 operations are the Gaussian's
// bound, bytes the box's); used only to order the queue longest first.
double job_cost(const batch::Job& j)
{
    const double px = (double)j.rows * j.cols;
    if (j.kind == batch::kFir)
        return px * (4.0 * j.r + 8.0);
    return px * 10.0;
}

}  // namespace

struct tucu_batch
{
    std::vector<tucu_batch_job> spec;
    std::vector<batch::Job> jobs;
    std::vector<CUtensorMap> tmaps;
    std::vector<batch::Item> items;
    // device copies
    batch::Job* d_jobs = nullptr;
    CUtensorMap* d_tmaps = nullptr;
    batch::Item* d_items = nullptr;
    unsigned* d_counter = nullptr;
    size_t cap_jobs = 0, cap_items = 0;
    int device = -1;
    int grid = 0;
    size_t smem = 0;
    int planned = 0;
    int fir_rows = 0, box_rows = 0;
    // graph
    cudaGraphExec_t exec = nullptr;
    cudaStream_t graph_stream = nullptr;
    int graph_valid = 0;
};

static void free_device(tucu_batch* b)
{
    if (b->exec)
        cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    b->graph_valid = 0;
    cudaFree(b->d_jobs);
    cudaFree(b->d_tmaps);
    cudaFree(b->d_items);
    cudaFree(b->d_counter);
    b->d_jobs = nullptr;
    b->d_tmaps = nullptr;
    b->d_items = nullptr;
    b->d_counter = nullptr;
    b->cap_jobs = b->cap_items = 0;
}

// Pads a lobe of length L (outermost first) on its outer side to radius R.
static void pad_to(const float* lobe, int L, int R, float* out)
{
    const int r = L & ~1;
    for (int k = 0; k <= R; ++k)
        out[k] = 0.0f;
    for (int k = 0; k < L; ++k)
        out[R - r + k] = lobe[k];
}

static const int kOpLobes[6][2] = {{0, 0}, {1, 0}, {0, 1}, {2, 0}, {1, 1}, {0, 2}};

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

int tucu_batch_plan(tucu_batch* b, int fir_strip_rows, int box_strip_rows)
{
    if (!b)
        return fail(TUCU_ERR_ARG, "null handle");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    const int fr = fir_strip_rows > 0 ? (fir_strip_rows + 31) / 32 * 32 : 256;
    // Box strips start on multiples of the float restart period, so batched
    // float sums equal the single-image ones.
    const int br = box_strip_rows > 0
                       ? (box_strip_rows + box::kRestart - 1) / box::kRestart * box::kRestart
                       : 128;
    b->jobs.clear();
    b->tmaps.clear();
    b->items.clear();
    size_t smem = 0;
    for (const tucu_batch_job& s : b->spec) {
        batch::Job J;
        std::memset(&J, 0, sizeof(J));
        J.in_dtype = s.in_dtype;
        J.rows = s.rows;
        J.cols = s.cols;
        J.src = s.in;
        J.src_pitch = s.in_pitch;
        J.dst = s.out;
        J.dst_pitch = s.out_pitch;
        J.out_dtype = s.out_dtype;
        CUtensorMap tm;
        std::memset(&tm, 0, sizeof(tm));
        if (s.op == TUCU_BATCH_GAUSS) {
            float lb[3][TUCU_LOBE_MAX];
            int n[3];
            int rc = tucu_gauss_design(s.sigma, lb[0], &n[0], lb[1], &n[1], lb[2], &n[2]);
            if (rc)
                return rc;
            const int lh = kOpLobes[s.gauss_op][0], lv = kOpLobes[s.gauss_op][1];
            const int R = std::max(n[lh] & ~1, n[lv] & ~1);
            // Each operator keeps its own valid region; with unequal radii the
            // strip radius is the larger one and the smaller lobe is padded.
            const int rh = n[lh] & ~1, rv = n[lv] & ~1;
            if (s.rows <= 2 * rv || s.cols <= 2 * rh)
                continue;  // nothing to write (TUCU_NOOP for the single call)
            J.kind = batch::kFir;
            J.r = R;
            pad_to(lb[lh], n[lh], R, J.lobes.h[0]);
            pad_to(lb[lv], n[lv], R, J.lobes.v[0]);
            J.lobes.sym_h = n[lh] & 1;
            J.lobes.sym_v = n[lv] & 1;
            fir::FirJob& F = J.fir;
            F.src = s.in;
            F.src_pitch = s.in_pitch;
            F.rows = s.rows;
            F.cols = s.cols;
            // With padding, the strip computes the R-valid region; shift the
            // source window so each output keeps its own operator geometry.
            F.orows = s.rows - 2 * rv;
            F.ocols = s.cols - 2 * rh;
            F.oy = s.shift ? rv : 0;
            F.ox = s.shift ? rh : 0;
            F.nh = 1;
            F.nout = 1;
            F.out_dtype = s.out_dtype;
            F.dst[0] = s.out;
            F.dst_pitch[0] = s.out_pitch;
            if (rh != R || rv != R) {
                // Unequal radii: run the operator as its own padded-geometry
                // job is not supported in the persistent kernel; reject.
                return fail(TUCU_ERR_ARG, "batched Gaussian operators need equal H/V radii");
            }
            J.has_tmap = make_tmap_2d(&tm, s.in, s.in_dtype, s.cols, s.rows, s.in_pitch,
                                      fir::round_up(fir::kTW + 2 * R, 16), 32);
            smem = std::max(smem, fir_smem(R, s.in_dtype));
        } else {
            if (s.rows < s.winV || s.cols < s.winH)
                continue;
            J.kind = batch::kBox;
            J.wV = s.winV;
            J.wH = s.winH;
            J.orows = s.rows + 1 - s.winV;
            J.ocols = s.cols + 1 - s.winH;
            J.oy = s.shift ? s.winV / 2 : 0;
            J.ox = s.shift ? s.winH / 2 : 0;
            J.normalize = s.normalize ? 1 : 0;
            const size_t a = 4 * (size_t)dtype_size(s.in_dtype);
            J.vec = (reinterpret_cast<uintptr_t>(s.in) % a) == 0 && (s.in_pitch % a) == 0;
            smem = std::max(smem, batch::kBoxSmemOff + box_smem(s.in_dtype));
        }
        b->jobs.push_back(J);
        b->tmaps.push_back(tm);
    }
    // Work list: jobs longest first, each cut into strips.
    std::vector<int> order(b->jobs.size());
    for (size_t i = 0; i < order.size(); ++i)
        order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
        return job_cost(b->jobs[a]) > job_cost(b->jobs[c]);
    });
    for (int ji : order) {
        const batch::Job& J = b->jobs[ji];
        if (J.kind == batch::kFir) {
            for (int y = 0; y < J.fir.orows; y += fr)
                for (int x = 0; x < J.fir.ocols; x += fir::kTW)
                    b->items.push_back({ji, x, y, std::min(fr, J.fir.orows - y)});
        } else {
            const int tw = box::out_cols_per_cta(J.wH);
            for (int y = 0; y < J.orows; y += br)
                for (int x = 0; x < J.ocols; x += tw)
                    b->items.push_back({ji, x, y, std::min(br, J.orows - y)});
        }
    }
    // Device buffers (grown on demand, reused across plans).
    if (b->device != dev)
        free_device(b);
    b->device = dev;
    const size_t nj = std::max<size_t>(1, b->jobs.size()), ni = std::max<size_t>(1, b->items.size());
    if (nj > b->cap_jobs) {
        cudaFree(b->d_jobs);
        cudaFree(b->d_tmaps);
        b->d_jobs = nullptr;
        b->d_tmaps = nullptr;
        if ((e = cudaMalloc(&b->d_jobs, nj * sizeof(batch::Job))) != cudaSuccess ||
            (e = cudaMalloc(&b->d_tmaps, nj * sizeof(CUtensorMap))) != cudaSuccess) {
            b->cap_jobs = 0;
            return cuda_fail(e, "batch job table");
        }
        b->cap_jobs = nj;
    }
    if (ni > b->cap_items) {
        cudaFree(b->d_items);
        b->d_items = nullptr;
        if ((e = cudaMalloc(&b->d_items, ni * sizeof(batch::Item))) != cudaSuccess) {
            b->cap_items = 0;
            return cuda_fail(e, "batch work list");
        }
        b->cap_items = ni;
    }
    if (!b->d_counter && (e = cudaMalloc(&b->d_counter, sizeof(unsigned))) != cudaSuccess)
        return cuda_fail(e, "batch queue counter");
    if (!b->jobs.empty()) {
        if ((e = cudaMemcpy(b->d_jobs, b->jobs.data(), b->jobs.size() * sizeof(batch::Job),
                            cudaMemcpyHostToDevice)) != cudaSuccess ||
            (e = cudaMemcpy(b->d_tmaps, b->tmaps.data(), b->tmaps.size() * sizeof(CUtensorMap),
                            cudaMemcpyHostToDevice)) != cudaSuccess ||
            (e = cudaMemcpy(b->d_items, b->items.data(), b->items.size() * sizeof(batch::Item),
                            cudaMemcpyHostToDevice)) != cudaSuccess)
            return cuda_fail(e, "batch upload");
    }
    smem = std::max<size_t>(smem, 2048);
    if ((e = cudaFuncSetAttribute(batch::batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem)) != cudaSuccess)
        return cuda_fail(e, "batch kernel shared memory");
    int per_sm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch::batch_kernel,
                                                           fir::kThreads, smem)) != cudaSuccess)
        return cuda_fail(e, "occupancy query");
    b->grid = std::max(1, per_sm) * sm_count();
    b->grid = std::min<int>(b->grid, std::max<size_t>(1, b->items.size()));
    b->smem = smem;
    b->fir_rows = fr;
    b->box_rows = br;
    b->planned = 1;
    b->graph_valid = 0;
    return TUCU_OK;
}

int tucu_batch_launch(tucu_batch* b, void* stream)
{
    if (!b)
        return fail(TUCU_ERR_ARG, "null handle");
    if (!b->planned)
        return fail(TUCU_ERR_STATE, "tucu_batch_plan must run after the last add");
    if (b->items.empty())
        return TUCU_NOOP;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemsetAsync(b->d_counter, 0, sizeof(unsigned), st);
    if (e != cudaSuccess)
        return cuda_fail(e, "queue reset");
    batch::batch_kernel<<<b->grid, fir::kThreads, b->smem, st>>>(
        b->d_jobs, b->d_tmaps, b->d_items, (int)b->items.size(), b->d_counter);
    e = cudaGetLastError();
    return e == cudaSuccess ? TUCU_OK : cuda_fail(e, "batch launch");
}

int tucu_batch_graph_launch(tucu_batch* b, void* stream)
{
    if (!b)
        return fail(TUCU_ERR_ARG, "null handle");
    if (!b->planned)
        return fail(TUCU_ERR_STATE, "tucu_batch_plan must run after the last add");
    if (b->items.empty())
        return TUCU_NOOP;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    if (!b->graph_valid) {
        if (b->exec) {
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
        // Capture on a private stream so the caller's stream (possibly the
        // legacy default stream, which cannot be captured) stays untouched.
        cudaStream_t cap;
        if ((e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking)) != cudaSuccess)
            return cuda_fail(e, "capture stream");
        cudaGraph_t g = nullptr;
        e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaMemsetAsync(b->d_counter, 0, sizeof(unsigned), cap);
            batch::batch_kernel<<<b->grid, fir::kThreads, b->smem, cap>>>(
                b->d_jobs, b->d_tmaps, b->d_items, (int)b->items.size(), b->d_counter);
            e = cudaStreamEndCapture(cap, &g);
        }
        if (e == cudaSuccess)
            e = cudaGraphInstantiate(&b->exec, g, 0);
        if (g)
            cudaGraphDestroy(g);
        cudaStreamDestroy(cap);
        if (e != cudaSuccess)
            return cuda_fail(e, "graph capture");
        b->graph_valid = 1;
    }
    e = cudaGraphLaunch(b->exec, st);
    return e == cudaSuccess ? TUCU_OK : cuda_fail(e, "graph launch");
}

int tucu_batch_info(const tucu_batch* b, int* njobs, int* nitems, int* grid, size_t* smem)
{
    if (!b)
        return fail(TUCU_ERR_ARG, "null handle");
    if (njobs)
        *njobs = (int)b->jobs.size();
    if (nitems)
        *nitems = (int)b->items.size();
    if (grid)
        *grid = b->grid;
    if (smem)
        *smem = b->smem;
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
