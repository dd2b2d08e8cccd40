// pipe.cu -- batches whose images live in host memory (tucu_pipe_*).
//
// The jobs are cut into `chunks` groups of consecutive jobs with about equal
// bytes; each group is its own planned batch (one CUDA graph).  A run issues,
// per group, the host -> device copies of its inputs on one stream, its graph
// on a second (after the copies), and the device -> host copies of its valid
// output regions on a third (after the graph), so the copies of one group
// overlap the filtering of the next and the two copy directions overlap each
// other.  The run is ordered after the caller's stream and the caller's
// stream after the run.  With TUCU_PIPE_SPANS, runs of consecutive jobs whose
// host and device images keep the same relative layout move as one byte
// range per direction and group (fewer, larger copies).
#include <algorithm>
#include <new>
#include <vector>

#include "tucu_common.cuh"
#include "tucu_internal.h"

namespace
{

struct HostJob
{
    tucu_batch_job job;
    const void* host_in;
    size_t host_in_pitch;
    void* host_out;
    size_t host_out_pitch;
    // valid output region (rows vr x cols vc at vy, vx); vr = 0: none
    int vy, vx, vr, vc;
};

// Valid region of a batch job, as the single-image calls write it.
int valid_region(HostJob& h)
{
    const tucu_batch_job& j = h.job;
    h.vr = h.vc = h.vy = h.vx = 0;
    int oy, ox, er, ec;
    if (j.op == TUCU_BATCH_GAUSS) {
        float l[3][TUCU_LOBE_MAX];
        int n[3];
        const int rc = tucu_gauss_design(j.sigma, l[0], &n[0], l[1], &n[1], l[2], &n[2]);
        if (rc < 0)
            return rc;
        // operator -> (H lobe, V lobe): smooth, diffH, diffV, diffHH, diffHV, diffVV
        static const int kH[6] = {0, 1, 0, 2, 1, 0}, kV[6] = {0, 0, 1, 0, 1, 2};
        const int RH = n[kH[j.gauss_op]] & ~1, RV = n[kV[j.gauss_op]] & ~1;
        er = j.rows - 2 * RV;
        ec = j.cols - 2 * RH;
        oy = RV;
        ox = RH;
    } else {
        er = j.rows + 1 - j.winV;
        ec = j.cols + 1 - j.winH;
        oy = j.winV / 2;
        ox = j.winH / 2;
    }
    if (er <= 0 || ec <= 0)
        return TUCU_OK;  // the filter writes nothing
    h.vr = er;
    h.vc = ec;
    h.vy = j.shift ? oy : 0;
    h.vx = j.shift ? ox : 0;
    return TUCU_OK;
}

// One host <-> device copy: `height` rows of `width` bytes (height 1: a
// contiguous range).
struct Copy
{
    void* dst;
    size_t dpitch;
    const void* src;
    size_t spitch;
    size_t width, height;
};

// Builds the copies of one group in one direction.  ext(i, &dev, &host,
// &bytes_first_row, &rows, &dev_pitch, &host_pitch) describes job i's region
// (false: nothing to copy).  Without spans each region is one pitched copy;
// with spans a region joins the open range when its host and device
// addresses differ by the range's offset, the pitches match and it starts
// at most kGap bytes past the range's end.
constexpr size_t kGap = 512 * 1024;

template <class Ext>
void build_copies(size_t first, size_t last, bool spans, bool to_device, Ext ext, std::vector<Copy>& out)
{
    out.clear();
    bool open = false;
    uintptr_t ds = 0, de = 0, delta = 0;
    auto close = [&] {
        if (!open)
            return;
        const char* d = reinterpret_cast<const char*>(ds);
        const char* h = reinterpret_cast<const char*>(ds + delta);
        const size_t n = de - ds;
        out.push_back(to_device ? Copy{const_cast<char*>(d), n, h, n, n, 1}
                                : Copy{const_cast<char*>(h), n, d, n, n, 1});
        open = false;
    };
    for (size_t i = first; i < last; ++i) {
        uintptr_t dv, hv;
        size_t w, rows, dp, hp;
        if (!ext(i, &dv, &hv, &w, &rows, &dp, &hp))
            continue;
        if (!spans || dp != hp) {
            close();
            void* d = reinterpret_cast<void*>(dv);
            void* h = reinterpret_cast<void*>(hv);
            out.push_back(to_device ? Copy{d, dp, h, hp, w, rows} : Copy{h, hp, d, dp, w, rows});
            continue;
        }
        const uintptr_t end = dv + (rows - 1) * dp + w;
        if (open && hv - dv == delta && dv >= ds && dv <= de + kGap) {
            de = std::max(de, end);
            continue;
        }
        close();
        open = true;
        ds = dv;
        de = end;
        delta = hv - dv;
    }
    close();
}

}  // namespace

struct tucu_pipe
{
    int chunks = 1;
    int flags = 0;
    std::vector<std::vector<Copy>> copies_in, copies_out;  // per group
    std::vector<HostJob> jobs;
    std::vector<tucu_batch*> parts;
    std::vector<size_t> first;  // first job of each part (+ end)
    cudaStream_t s_in = nullptr, s_run = nullptr, s_out = nullptr;
    std::vector<cudaEvent_t> ev_in, ev_run;
    cudaEvent_t ev_start = nullptr, ev_done = nullptr;
    int planned = 0;
    int device = -1;
};

namespace
{

void drop_parts(tucu_pipe* p)
{
    for (tucu_batch* b : p->parts)
        tucu_batch_destroy(b);
    p->parts.clear();
    p->first.clear();
    p->copies_in.clear();
    p->copies_out.clear();
    for (cudaEvent_t e : p->ev_in)
        cudaEventDestroy(e);
    for (cudaEvent_t e : p->ev_run)
        cudaEventDestroy(e);
    p->ev_in.clear();
    p->ev_run.clear();
}

cudaError_t issue(const Copy& c, cudaMemcpyKind kind, cudaStream_t s)
{
    if (c.height == 1)
        return cudaMemcpyAsync(c.dst, c.src, c.width, kind, s);
    return cudaMemcpy2DAsync(c.dst, c.dpitch, c.src, c.spitch, c.width, c.height, kind, s);
}

void drop_streams(tucu_pipe* p)
{
    for (cudaStream_t* s : {&p->s_in, &p->s_run, &p->s_out})
        if (*s) {
            cudaStreamDestroy(*s);
            *s = nullptr;
        }
    for (cudaEvent_t* e : {&p->ev_start, &p->ev_done})
        if (*e) {
            cudaEventDestroy(*e);
            *e = nullptr;
        }
}

}  // namespace

extern "C" {

int tucu_pipe_create(int chunks, tucu_pipe** out)
{
    using namespace tucu;
    if (!out)
        return fail(TUCU_ERR_ARG, "null handle pointer");
    if (chunks < 1 || chunks > 64)
        return fail(TUCU_ERR_ARG, "chunks must be 1..64");
    auto* p = new (std::nothrow) tucu_pipe;
    if (!p)
        return fail(TUCU_ERR_NOMEM, "host allocation");
    p->chunks = chunks;
    *out = p;
    return TUCU_OK;
}

int tucu_pipe_set_flags(tucu_pipe* p, int flags)
{
    using namespace tucu;
    if (!p)
        return fail(TUCU_ERR_ARG, "null handle");
    if (flags & ~(TUCU_PIPE_SPANS | TUCU_PIPE_TENSOR))
        return fail(TUCU_ERR_ARG, "unknown pipe flags");
    p->flags = flags;
    p->planned = 0;
    return TUCU_OK;
}

int tucu_pipe_add(tucu_pipe* p, const tucu_batch_job* job, const void* host_in, size_t host_in_pitch,
                  void* host_out, size_t host_out_pitch)
{
    using namespace tucu;
    if (!p || !job || !host_in || !host_out)
        return fail(TUCU_ERR_ARG, "null argument");
    if (job->in_dtype < TUCU_U8 || job->in_dtype > TUCU_I32 || job->out_dtype < TUCU_U8 ||
        job->out_dtype > TUCU_I32)
        return fail(TUCU_ERR_DTYPE, "unknown dtype");
    if (host_in_pitch < (size_t)job->cols * dtype_size(job->in_dtype) ||
        host_out_pitch < (size_t)job->cols * dtype_size(job->out_dtype))
        return fail(TUCU_ERR_ARG, "host pitch smaller than a row");
    if (job->op == TUCU_BATCH_GAUSS && (job->gauss_op < 0 || job->gauss_op > 5))
        return fail(TUCU_ERR_ARG, "bad Gaussian operator");
    HostJob h;
    h.job = *job;
    h.host_in = host_in;
    h.host_in_pitch = host_in_pitch;
    h.host_out = host_out;
    h.host_out_pitch = host_out_pitch;
    const int rc = valid_region(h);
    if (rc < 0)
        return rc;
    p->jobs.push_back(h);
    p->planned = 0;
    return (int)p->jobs.size() - 1;
}

int tucu_pipe_plan(tucu_pipe* p, int fir_strip_rows, int box_strip_rows)
{
    using namespace tucu;
    if (!p)
        return fail(TUCU_ERR_ARG, "null handle");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    drop_parts(p);
    if (p->device != dev)
        drop_streams(p);
    p->device = dev;
    p->planned = 0;
    if (!p->s_in) {
        for (cudaStream_t* s : {&p->s_in, &p->s_run, &p->s_out})
            if ((e = cudaStreamCreateWithFlags(s, cudaStreamNonBlocking)) != cudaSuccess)
                return cuda_fail(e, "pipe stream");
        if ((e = cudaEventCreateWithFlags(&p->ev_start, cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&p->ev_done, cudaEventDisableTiming)) != cudaSuccess)
            return cuda_fail(e, "pipe event");
    }
    // Consecutive jobs in groups of about equal bytes (input + output).
    size_t total = 0;
    std::vector<size_t> bytes(p->jobs.size());
    for (size_t i = 0; i < p->jobs.size(); ++i) {
        const tucu_batch_job& j = p->jobs[i].job;
        bytes[i] = (size_t)j.rows * j.cols * (dtype_size(j.in_dtype) + dtype_size(j.out_dtype));
        total += bytes[i];
    }
    const int k = std::max(1, std::min<int>(p->chunks, (int)p->jobs.size()));
    p->first.push_back(0);
    size_t acc = 0;
    for (size_t i = 0; i < p->jobs.size(); ++i) {
        acc += bytes[i];
        const int done = (int)p->first.size();  // groups closed so far + 1
        if (done < k && acc * k >= total * done && i + 1 < p->jobs.size())
            p->first.push_back(i + 1);
    }
    p->first.push_back(p->jobs.size());
    for (size_t g = 0; g + 1 < p->first.size(); ++g) {
        tucu_batch* b = nullptr;
        int rc = tucu_batch_create(&b);
        if (rc < 0)
            return rc;
        p->parts.push_back(b);
        if ((p->flags & TUCU_PIPE_TENSOR) && (rc = tucu_batch_set_tensor_cores(b, 1)) < 0)
            return rc;
        for (size_t i = p->first[g]; i < p->first[g + 1]; ++i)
            if ((rc = tucu_batch_add(b, &p->jobs[i].job)) < 0)
                return rc;
        if ((rc = tucu_batch_plan(b, fir_strip_rows, box_strip_rows)) < 0)
            return rc;
        const bool spans = (p->flags & TUCU_PIPE_SPANS) != 0;
        p->copies_in.emplace_back();
        p->copies_out.emplace_back();
        build_copies(p->first[g], p->first[g + 1], spans, true,
                     [&](size_t i, uintptr_t* dv, uintptr_t* hv, size_t* w, size_t* rows, size_t* dp,
                         size_t* hp) {
                         const HostJob& h = p->jobs[i];
                         *dv = reinterpret_cast<uintptr_t>(h.job.in);
                         *hv = reinterpret_cast<uintptr_t>(h.host_in);
                         *w = (size_t)h.job.cols * dtype_size(h.job.in_dtype);
                         *rows = (size_t)h.job.rows;
                         *dp = h.job.in_pitch;
                         *hp = h.host_in_pitch;
                         return true;
                     },
                     p->copies_in.back());
        build_copies(p->first[g], p->first[g + 1], spans, false,
                     [&](size_t i, uintptr_t* dv, uintptr_t* hv, size_t* w, size_t* rows, size_t* dp,
                         size_t* hp) {
                         const HostJob& h = p->jobs[i];
                         if (!h.vr)
                             return false;
                         const size_t eo = dtype_size(h.job.out_dtype);
                         *dv = reinterpret_cast<uintptr_t>(h.job.out) + (size_t)h.vy * h.job.out_pitch +
                               (size_t)h.vx * eo;
                         *hv = reinterpret_cast<uintptr_t>(h.host_out) + (size_t)h.vy * h.host_out_pitch +
                               (size_t)h.vx * eo;
                         *w = (size_t)h.vc * eo;
                         *rows = (size_t)h.vr;
                         *dp = h.job.out_pitch;
                         *hp = h.host_out_pitch;
                         return true;
                     },
                     p->copies_out.back());
        cudaEvent_t a, c;
        if ((e = cudaEventCreateWithFlags(&a, cudaEventDisableTiming)) != cudaSuccess)
            return cuda_fail(e, "pipe event");
        p->ev_in.push_back(a);
        if ((e = cudaEventCreateWithFlags(&c, cudaEventDisableTiming)) != cudaSuccess)
            return cuda_fail(e, "pipe event");
        p->ev_run.push_back(c);
    }
    p->planned = 1;
    return TUCU_OK;
}

int tucu_pipe_run(tucu_pipe* p, void* stream)
{
    using namespace tucu;
    if (!p)
        return fail(TUCU_ERR_ARG, "null handle");
    if (!p->planned)
        return fail(TUCU_ERR_STATE, "tucu_pipe_plan must run after the last add");
    cudaStream_t user = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    if ((e = cudaEventRecord(p->ev_start, user)) != cudaSuccess)
        return cuda_fail(e, "pipe start");
    for (cudaStream_t s : {p->s_in, p->s_run, p->s_out})
        if ((e = cudaStreamWaitEvent(s, p->ev_start, 0)) != cudaSuccess)
            return cuda_fail(e, "pipe start");
    for (size_t g = 0; g < p->parts.size(); ++g) {
        for (const Copy& c : p->copies_in[g])
            if ((e = issue(c, cudaMemcpyHostToDevice, p->s_in)) != cudaSuccess)
                return cuda_fail(e, "pipe copy in");
        if ((e = cudaEventRecord(p->ev_in[g], p->s_in)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(p->s_run, p->ev_in[g], 0)) != cudaSuccess)
            return cuda_fail(e, "pipe order");
        const int rc = tucu_batch_graph_launch(p->parts[g], p->s_run);
        if (rc < 0)
            return rc;
        if ((e = cudaEventRecord(p->ev_run[g], p->s_run)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(p->s_out, p->ev_run[g], 0)) != cudaSuccess)
            return cuda_fail(e, "pipe order");
        for (const Copy& c : p->copies_out[g])
            if ((e = issue(c, cudaMemcpyDeviceToHost, p->s_out)) != cudaSuccess)
                return cuda_fail(e, "pipe copy out");
    }
    // s_out waited for every group's graph, which waited for every copy in.
    if ((e = cudaEventRecord(p->ev_done, p->s_out)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(user, p->ev_done, 0)) != cudaSuccess)
        return cuda_fail(e, "pipe end");
    return TUCU_OK;
}

int tucu_pipe_info(const tucu_pipe* p, int* njobs, int* ngroups, int* nkernels, size_t* h2d_bytes,
                   size_t* d2h_bytes)
{
    using namespace tucu;
    if (!p)
        return fail(TUCU_ERR_ARG, "null handle");
    size_t in = 0, out = 0;
    if (p->planned) {
        for (const auto& v : p->copies_in)
            for (const Copy& c : v)
                in += c.width * c.height;
        for (const auto& v : p->copies_out)
            for (const Copy& c : v)
                out += c.width * c.height;
    } else {
        for (const HostJob& h : p->jobs) {
            in += (size_t)h.job.rows * h.job.cols * dtype_size(h.job.in_dtype);
            out += (size_t)h.vr * h.vc * dtype_size(h.job.out_dtype);
        }
    }
    int nk = 0;
    for (tucu_batch* b : p->parts) {
        int k = 0;
        tucu_batch_info(b, nullptr, nullptr, &k, nullptr);
        nk += k;
    }
    if (njobs)
        *njobs = (int)p->jobs.size();
    if (ngroups)
        *ngroups = (int)p->parts.size();
    if (nkernels)
        *nkernels = nk;
    if (h2d_bytes)
        *h2d_bytes = in;
    if (d2h_bytes)
        *d2h_bytes = out;
    return p->planned ? TUCU_OK : TUCU_NOOP;
}

void tucu_pipe_destroy(tucu_pipe* p)
{
    if (!p)
        return;
    drop_parts(p);
    drop_streams(p);
    delete p;
}

}  // extern "C"
