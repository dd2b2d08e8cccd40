// server.cu -- request loop with admission by HBM budget and continuous
// batching (tucu_server_* of the C ABI).
//
//   submit()  -> pending queue (FIFO)
//   scheduler -> whenever a stream slot is free: admits pending requests in
//                order while their device buffers fit in the arena, forms a
//                wave, and issues on the slot's stream: host->device copies,
//                one batched launch for the Gaussian and box requests, the
//                guided requests, device->host copies of the valid regions,
//                an event
//   reaper    -> waits for the oldest wave's event, completes its requests,
//                returns their buffers to the arena (which may admit more)
//
// Waves on different slots overlap (copies of one with kernels of another).
// The arena is one cudaMalloc at creation; requests never allocate.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "box_kernels.h"
#include "tucu_internal.h"

namespace
{

using namespace tucu;
using Clock = std::chrono::steady_clock;

double now_s()
{
    return std::chrono::duration<double>(Clock::now().time_since_epoch()).count();
}

size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// First-fit allocator over one device block (256-byte granules, coalescing).
class Arena
{
  public:
    bool init(size_t bytes)
    {
        size_ = round_up(bytes, 256);
        if (cudaMalloc(&base_, size_) != cudaSuccess) {
            base_ = nullptr;
            return false;
        }
        free_[0] = size_;
        return true;
    }
    void release()
    {
        if (base_)
            cudaFree(base_);
        base_ = nullptr;
    }
    size_t size() const { return size_; }
    size_t used() const { return used_; }
    bool alloc(size_t n, size_t* off)
    {
        n = round_up(n, 256);
        for (auto it = free_.begin(); it != free_.end(); ++it)
            if (it->second >= n) {
                *off = it->first;
                const size_t rest = it->second - n;
                const size_t at = it->first + n;
                free_.erase(it);
                if (rest)
                    free_[at] = rest;
                used_ += n;
                return true;
            }
        return false;
    }
    void free(size_t off, size_t n)
    {
        n = round_up(n, 256);
        used_ -= n;
        auto it = free_.emplace(off, n).first;
        auto next = std::next(it);
        if (next != free_.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_.erase(next);
        }
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_.erase(it);
            }
        }
    }
    char* ptr(size_t off) const { return static_cast<char*>(base_) + off; }

  private:
    void* base_ = nullptr;
    size_t size_ = 0, used_ = 0;
    std::map<size_t, size_t> free_;
};

struct Req
{
    uint64_t id;
    tucu_request r;
    double t_submit = 0.0, t_done = 0.0;
    int status = 1;  // TUCU_NOOP-like "open"; set to a final status on completion
    bool done = false, admitted = false, cancelled = false;
    // device layout inside the arena
    size_t off = 0, bytes = 0;
    size_t p_in = 0, p_guide = 0, p_out = 0, p_coef = 0;  // pitches
    size_t o_in = 0, o_guide = 0, o_out = 0, o_coef = 0;  // offsets from off
    // valid output region (rows, cols, origin); nothing if vr == 0
    int vy = 0, vx = 0, vr = 0, vc = 0;
};

struct Slot
{
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    tucu_batch* batch = nullptr;
    std::vector<Req*> reqs;
    bool busy = false;
};

int win_of(const tucu_request& r) { return 2 * r.radius + 1; }

}  // namespace

struct tucu_server
{
    Arena arena;
    int max_wave = 64;
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv_work, cv_reap, cv_done;
    std::deque<Req*> pending;
    std::deque<int> inflight;  // slot indices in issue order
    std::unordered_map<uint64_t, Req*> reqs;
    uint64_t next_id = 1;
    bool stop = false;
    std::thread sched, reaper;
    int device = 0;
    // stats
    uint64_t submitted = 0, completed = 0, rejected = 0, cancelled = 0, failed = 0, waves = 0;
    uint64_t wave_reqs = 0;
    std::vector<double> lat_ms;
    double t_first = 0.0, t_last = 0.0, pixels = 0.0;
    size_t peak = 0;
    // host-side fault injection: every n-th admission attempt fails as if the
    // arena were exhausted (TUCU_SERVER_FAIL_ADMIT_EVERY=n; 0 = off)
    uint64_t fail_every = 0, admit_attempts = 0;
};

namespace
{

// Device footprint and valid region of a request (shift = true geometry).
int layout(Req& q)
{
    const tucu_request& r = q.r;
    const int ei = dtype_size(r.in_dtype), eo = dtype_size(r.out_dtype);
    q.p_in = round_up((size_t)r.cols * ei, 256);
    q.p_out = round_up((size_t)r.cols * eo, 256);
    size_t o = 0;
    q.o_in = o;
    o += q.p_in * r.rows;
    if (r.op == TUCU_REQ_GUIDED && r.guide) {
        q.p_guide = q.p_in;
        q.o_guide = o;
        o += q.p_guide * r.rows;
    }
    q.o_out = o;
    o += q.p_out * r.rows;
    q.vr = 0;
    if (r.op == TUCU_REQ_GAUSS) {
        float l[3][TUCU_LOBE_MAX];
        int n[3];
        int rc = tucu_gauss_design(r.sigma, l[0], &n[0], l[1], &n[1], l[2], &n[2]);
        if (rc)
            return rc;
        const int R = n[0] & ~1;
        if (r.rows > 2 * R && r.cols > 2 * R) {
            q.vy = q.vx = R;
            q.vr = r.rows - 2 * R;
            q.vc = r.cols - 2 * R;
        }
    } else if (r.op == TUCU_REQ_BOX) {
        const int w = win_of(r);
        if (r.rows >= w && r.cols >= w) {
            q.vy = q.vx = w / 2;
            q.vr = r.rows + 1 - w;
            q.vc = r.cols + 1 - w;
        }
    } else {
        const int w = win_of(r);
        if (r.rows >= 2 * w - 1 && r.cols >= 2 * w - 1) {
            q.vy = q.vx = w - 1;
            q.vr = r.rows - 2 * (w - 1);
            q.vc = r.cols - 2 * (w - 1);
            const int cr = r.rows + 1 - w, cc = r.cols + 1 - w;
            q.p_coef = round_up((size_t)cc * 8, 256);
            q.o_coef = o;
            o += q.p_coef * cr;
        }
    }
    q.bytes = std::max<size_t>(o, 256);
    return TUCU_OK;
}

int check_request(const tucu_request& r)
{
    if (r.op < TUCU_REQ_GAUSS || r.op > TUCU_REQ_GUIDED)
        return fail(TUCU_ERR_ARG, "unknown request op");
    if (!r.in || !r.out || r.rows <= 0 || r.cols <= 0)
        return fail(TUCU_ERR_ARG, "null image or empty size");
    if (r.in_dtype < TUCU_U8 || r.in_dtype > TUCU_I32 || r.out_dtype < TUCU_U8 ||
        r.out_dtype > TUCU_I32)
        return fail(TUCU_ERR_DTYPE, "unknown dtype");
    if (r.in_pitch < (size_t)r.cols * dtype_size(r.in_dtype) ||
        r.out_pitch < (size_t)r.cols * dtype_size(r.out_dtype))
        return fail(TUCU_ERR_ARG, "pitch smaller than a row");
    if (r.op == TUCU_REQ_GAUSS) {
        if (!(r.sigma > 0.0f) || r.in_dtype == TUCU_I32)
            return fail(TUCU_ERR_ARG, "Gaussian request needs sigma > 0 and u8/f16/bf16/f32 input");
    } else {
        if (r.radius < 0 || win_of(r) > TUCU_WIN_LIMIT)
            return fail(TUCU_ERR_WINDOW, "window size out of range");
        if (r.op == TUCU_REQ_GUIDED) {
            if (r.in_dtype == TUCU_I32 || !std::isfinite(r.e))
                return fail(TUCU_ERR_ARG, "guided request needs u8/f16/bf16/f32 input, finite e");
            if (r.guide && r.guide_pitch < (size_t)r.cols * dtype_size(r.in_dtype))
                return fail(TUCU_ERR_ARG, "guide pitch smaller than a row");
        }
    }
    return TUCU_OK;
}

// Issues one wave on a slot (called without the server lock).
void issue_wave(tucu_server* s, Slot& sl)
{
    cudaStream_t st = sl.stream;
    tucu_batch_clear(sl.batch);
    int nbatch = 0;
    for (Req* q : sl.reqs) {
        const tucu_request& r = q->r;
        char* base = s->arena.ptr(q->off);
        const int ei = dtype_size(r.in_dtype);
        cudaMemcpy2DAsync(base + q->o_in, q->p_in, r.in, r.in_pitch, (size_t)r.cols * ei, r.rows,
                          cudaMemcpyHostToDevice, st);
        if (q->p_guide)
            cudaMemcpy2DAsync(base + q->o_guide, q->p_guide, r.guide, r.guide_pitch,
                              (size_t)r.cols * ei, r.rows, cudaMemcpyHostToDevice, st);
        if (!q->vr)
            continue;
        if (r.op == TUCU_REQ_GUIDED) {
            box::GuidedLaunch L;
            std::memset(&L, 0, sizeof(L));
            L.src = base + q->o_in;
            L.src_pitch = q->p_in;
            L.guide = q->p_guide ? base + q->o_guide : nullptr;
            L.guide_pitch = q->p_guide;
            L.rows = r.rows;
            L.cols = r.cols;
            L.in_dtype = r.in_dtype;
            L.wV = L.wH = win_of(r);
            L.e = r.e;
            L.coef = base + q->o_coef;
            L.coef_pitch = q->p_coef;
            L.dst = base + q->o_out;
            L.dst_pitch = q->p_out;
            L.out_dtype = r.out_dtype;
            L.oy = L.ox = win_of(r) - 1;
            box::launch_guided(L, st);
            continue;
        }
        tucu_batch_job j;
        std::memset(&j, 0, sizeof(j));
        j.in = base + q->o_in;
        j.in_pitch = q->p_in;
        j.in_dtype = r.in_dtype;
        j.out = base + q->o_out;
        j.out_pitch = q->p_out;
        j.out_dtype = r.out_dtype;
        j.rows = r.rows;
        j.cols = r.cols;
        j.shift = 1;
        if (r.op == TUCU_REQ_GAUSS) {
            j.op = TUCU_BATCH_GAUSS;
            j.gauss_op = TUCU_SMOOTH;
            j.sigma = r.sigma;
        } else {
            j.op = TUCU_BATCH_BOX;
            j.winV = j.winH = win_of(r);
            j.normalize = r.normalize;
        }
        tucu_batch_add(sl.batch, &j);
        ++nbatch;
    }
    if (nbatch && batch_plan_on_stream(sl.batch, 512, 128, st) == TUCU_OK)
        tucu_batch_launch(sl.batch, st);
    for (Req* q : sl.reqs) {
        if (!q->vr)
            continue;
        const tucu_request& r = q->r;
        const int eo = dtype_size(r.out_dtype);
        const char* src = s->arena.ptr(q->off) + q->o_out + (size_t)q->vy * q->p_out + (size_t)q->vx * eo;
        char* dst = static_cast<char*>(r.out) + (size_t)q->vy * r.out_pitch + (size_t)q->vx * eo;
        cudaMemcpy2DAsync(dst, r.out_pitch, src, q->p_out, (size_t)q->vc * eo, q->vr,
                          cudaMemcpyDeviceToHost, st);
    }
    cudaEventRecord(sl.done, st);
}

void scheduler_loop(tucu_server* s)
{
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        s->cv_work.wait(lk, [&] {
            if (s->stop && s->pending.empty())
                return true;
            if (s->pending.empty())
                return false;
            for (auto& sl : s->slots)
                if (!sl.busy)
                    return true;
            return false;
        });
        if (s->stop && s->pending.empty())
            break;
        int si = -1;
        for (size_t i = 0; i < s->slots.size(); ++i)
            if (!s->slots[i].busy) {
                si = (int)i;
                break;
            }
        Slot& sl = s->slots[si];
        sl.reqs.clear();
        while (!s->pending.empty() && (int)sl.reqs.size() < s->max_wave) {
            Req* q = s->pending.front();
            bool injected = false;
            if (s->fail_every && (++s->admit_attempts % s->fail_every) == 0)
                injected = true;
            size_t off = 0;
            if (injected || !s->arena.alloc(q->bytes, &off)) {
                bool idle = true;
                for (auto& o : s->slots)
                    if (o.busy)
                        idle = false;
                if (injected || (idle && sl.reqs.empty())) {
                    // Nothing in flight can free memory (or a failure was
                    // injected): the request fails instead of waiting.
                    s->pending.pop_front();
                    q->status = TUCU_ERR_NOMEM;
                    q->done = true;
                    q->t_done = now_s();
                    ++s->failed;
                    s->cv_done.notify_all();
                    continue;
                }
                break;  // wait for completions to free memory
            }
            s->pending.pop_front();
            q->off = off;
            q->admitted = true;
            sl.reqs.push_back(q);
        }
        if (sl.reqs.empty()) {
            // memory is full: wait for the reaper to free some
            s->cv_work.wait(lk);
            continue;
        }
        s->peak = std::max(s->peak, s->arena.used());
        sl.busy = true;
        ++s->waves;
        s->wave_reqs += sl.reqs.size();
        lk.unlock();
        issue_wave(s, sl);
        lk.lock();
        s->inflight.push_back(si);
        s->cv_reap.notify_one();
    }
}

void reaper_loop(tucu_server* s)
{
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        s->cv_reap.wait(lk, [&] { return !s->inflight.empty() || s->stop; });
        if (s->inflight.empty()) {
            if (s->stop)
                break;
            continue;
        }
        const int si = s->inflight.front();
        Slot& sl = s->slots[si];
        lk.unlock();
        const cudaError_t e = cudaEventSynchronize(sl.done);
        lk.lock();
        s->inflight.pop_front();
        const double t = now_s();
        for (Req* q : sl.reqs) {
            s->arena.free(q->off, q->bytes);
            q->t_done = t;
            q->done = true;
            if (e == cudaSuccess) {
                q->status = q->vr ? TUCU_OK : TUCU_NOOP;
                ++s->completed;
                s->lat_ms.push_back(1e3 * (t - q->t_submit));
                s->pixels += (double)q->r.rows * q->r.cols;
            } else {
                q->status = TUCU_ERR_CUDA;
                ++s->failed;
            }
        }
        s->t_last = t;
        sl.reqs.clear();
        sl.busy = false;
        s->cv_work.notify_all();
        s->cv_done.notify_all();
    }
}

}  // namespace

extern "C" {

int tucu_server_create(size_t budget_bytes, int streams, int max_wave, tucu_server** out)
{
    if (!out || budget_bytes < 4096 || streams < 1 || streams > 16 || max_wave < 1)
        return fail(TUCU_ERR_ARG, "bad server parameters");
    auto* s = new (std::nothrow) tucu_server;
    if (!s)
        return fail(TUCU_ERR_NOMEM, "host allocation");
    cudaGetDevice(&s->device);
    s->max_wave = max_wave;
    if (const char* f = std::getenv("TUCU_SERVER_FAIL_ADMIT_EVERY"))
        s->fail_every = (uint64_t)std::strtoull(f, nullptr, 10);
    if (!s->arena.init(budget_bytes)) {
        delete s;
        return fail(TUCU_ERR_NOMEM, "device arena of the budget size");
    }
    s->slots.resize(streams);
    for (auto& sl : s->slots) {
        cudaError_t e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
        int rc = e == cudaSuccess ? tucu_batch_create(&sl.batch) : TUCU_ERR_CUDA;
        if (rc == TUCU_OK)
            rc = batch_reserve(sl.batch, (size_t)max_wave, (size_t)max_wave, (size_t)max_wave * 256);
        if (rc != TUCU_OK) {
            for (auto& o : s->slots) {
                if (o.batch) tucu_batch_destroy(o.batch);
                if (o.done) cudaEventDestroy(o.done);
                if (o.stream) cudaStreamDestroy(o.stream);
            }
            s->arena.release();
            delete s;
            return e != cudaSuccess ? cuda_fail(e, "server streams") : rc;
        }
    }
    s->sched = std::thread(scheduler_loop, s);
    s->reaper = std::thread(reaper_loop, s);
    *out = s;
    return TUCU_OK;
}

int tucu_server_submit(tucu_server* s, const tucu_request* r, uint64_t* ticket)
{
    if (!s || !r || !ticket)
        return fail(TUCU_ERR_ARG, "null argument");
    int rc = check_request(*r);
    if (rc != TUCU_OK) {
        std::lock_guard<std::mutex> lk(s->mu);
        ++s->rejected;
        return rc;
    }
    auto* q = new (std::nothrow) Req;
    if (!q)
        return fail(TUCU_ERR_NOMEM, "host allocation");
    q->r = *r;
    rc = layout(*q);
    if (rc != TUCU_OK) {
        delete q;
        std::lock_guard<std::mutex> lk(s->mu);
        ++s->rejected;
        return rc;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (q->bytes > s->arena.size()) {
        ++s->rejected;
        delete q;
        return fail(TUCU_ERR_BUDGET, "request larger than the server's device budget");
    }
    q->id = s->next_id++;
    q->t_submit = now_s();
    if (!s->submitted)
        s->t_first = q->t_submit;
    ++s->submitted;
    s->reqs[q->id] = q;
    s->pending.push_back(q);
    *ticket = q->id;
    s->cv_work.notify_one();
    return TUCU_OK;
}

int tucu_server_wait(tucu_server* s, uint64_t ticket, double timeout_s, int* status)
{
    if (!s)
        return fail(TUCU_ERR_ARG, "null handle");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end())
        return fail(TUCU_ERR_ARG, "unknown ticket");
    Req* q = it->second;
    const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                        [&] { return q->done; });
    if (!ok)
        return TUCU_ERR_TIMEOUT;
    if (status)
        *status = q->status;
    s->reqs.erase(it);
    delete q;
    return TUCU_OK;
}

int tucu_server_cancel(tucu_server* s, uint64_t ticket)
{
    if (!s)
        return fail(TUCU_ERR_ARG, "null handle");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end())
        return fail(TUCU_ERR_ARG, "unknown ticket");
    Req* q = it->second;
    if (q->admitted || q->done)
        return fail(TUCU_ERR_STATE, "request already admitted");
    auto pit = std::find(s->pending.begin(), s->pending.end(), q);
    if (pit != s->pending.end())
        s->pending.erase(pit);
    q->cancelled = true;
    q->done = true;
    q->status = TUCU_ERR_CANCELLED;
    q->t_done = std::chrono::duration<double>(Clock::now().time_since_epoch()).count();
    ++s->cancelled;
    s->cv_done.notify_all();
    return TUCU_OK;
}

int tucu_server_drain(tucu_server* s, double timeout_s)
{
    if (!s)
        return fail(TUCU_ERR_ARG, "null handle");
    std::unique_lock<std::mutex> lk(s->mu);
    const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] {
        if (!s->pending.empty() || !s->inflight.empty())
            return false;
        for (auto& sl : s->slots)
            if (sl.busy)
                return false;
        return true;
    });
    return ok ? TUCU_OK : TUCU_ERR_TIMEOUT;
}

int tucu_server_set_tensor_cores(tucu_server* s, int on)
{
    if (!s)
        return fail(TUCU_ERR_ARG, "null handle");
    std::lock_guard<std::mutex> lk(s->mu);
    for (auto& sl : s->slots) {
        if (sl.busy || !s->pending.empty())
            return fail(TUCU_ERR_STATE, "set the arithmetic before the first request");
    }
    for (auto& sl : s->slots) {
        const int rc = tucu_batch_set_tensor_cores(sl.batch, on);
        if (rc < 0)
            return rc;
    }
    return TUCU_OK;
}

int tucu_server_get_stats(tucu_server* s, tucu_server_stats* o)
{
    if (!s || !o)
        return fail(TUCU_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(o, 0, sizeof(*o));
    o->submitted = s->submitted;
    o->completed = s->completed;
    o->rejected = s->rejected;
    o->cancelled = s->cancelled;
    o->failed = s->failed;
    std::vector<double> v = s->lat_ms;
    if (!v.empty()) {
        std::sort(v.begin(), v.end());
        auto pct = [&](double p) {
            const size_t i = std::min(v.size() - 1, (size_t)(p * (v.size() - 1) + 0.5));
            return v[i];
        };
        o->p50_ms = pct(0.50);
        o->p99_ms = pct(0.99);
        o->max_ms = v.back();
    }
    o->wall_s = s->t_last > s->t_first ? s->t_last - s->t_first : 0.0;
    o->gpix_per_s = o->wall_s > 0 ? s->pixels / o->wall_s / 1e9 : 0.0;
    o->waves = s->waves;
    o->mean_wave_requests = s->waves ? (double)s->wave_reqs / s->waves : 0.0;
    o->budget_bytes = s->arena.size();
    o->peak_bytes = s->peak;
    return TUCU_OK;
}

void tucu_server_destroy(tucu_server* s)
{
    if (!s)
        return;
    tucu_server_drain(s, 600.0);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    s->cv_reap.notify_all();
    s->sched.join();
    s->reaper.join();
    for (auto& sl : s->slots) {
        tucu_batch_destroy(sl.batch);
        cudaEventDestroy(sl.done);
        cudaStreamDestroy(sl.stream);
    }
    for (auto& kv : s->reqs)
        delete kv.second;
    s->arena.release();
    delete s;
}

}  // extern "C"
