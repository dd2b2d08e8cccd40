// tucu_internal.h -- host-side declarations shared by the library's
// translation units (not part of the C ABI).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <string>

#include "tucu_gb300.h"

namespace tucu
{

// Runs an idempotent per-device set-up step once per device.
class DeviceOnce
{
  public:
    template <class F>
    cudaError_t run(F&& f)
    {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess)
            return e;
        const uint64_t bit = 1ull << (dev & 63);
        if (done_.load(std::memory_order_acquire) & bit)
            return cudaSuccess;
        e = f();
        if (e == cudaSuccess)
            done_.fetch_or(bit, std::memory_order_acq_rel);
        return e;
    }

  private:
    std::atomic<uint64_t> done_{0};
};

// Thread-local last-error text behind tucu_last_error().
void set_last_error(const std::string& msg);
int fail(int status, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

// Fills a 2D tiled TMA descriptor for an image; returns false when the image
// cannot be described (base not 16-byte aligned, pitch not a multiple of 16,
// unsupported type) -- callers then use plain loads.  swizzle128: the box's
// 128-byte rows land in shared memory with the 128-byte swizzle (16-byte
// chunk c of row r at chunk c ^ (r % 8)), the layout the tensor cores read.
bool make_tmap_2d(CUtensorMap* map, const void* base, int dtype, int cols, int rows,
                  size_t pitch, int box_w, int box_h, bool swizzle128 = false);

// Number of SMs of the current device (cached per device).
int sm_count();

// Output rows per strip for the FIR kernels, which run one CTA per strip of
// `ncx` column blocks x a band of rows.  Picks the band height (a multiple
// of ch, at least max(ch, 4*rv), at most max_strip) that minimises
// rounds x strip cost, where rounds = ceil(strips / slots), slots = CTAs
// resident on the device at once, and a strip of s rows costs 2s + 2rv + ch
// (horizontal taps over s + 2rv rows, vertical taps over s rows, one chunk
// of pipeline fill).  Whole rounds matter: 360 strips on 304 slots take as
// long as 608.
int plan_strip_rows(int orows, int ncx, long slots, int ch, int rv, int max_strip);

// Resident CTAs per SM of `kernel` at `threads` threads and `smem` bytes of
// dynamic shared memory (at least 1).
int ctas_per_sm(const void* kernel, int threads, size_t smem);

// Batched launch helpers for the server (batch.cu).
int batch_plan_on_stream(tucu_batch* b, int fir_rows, int box_rows, cudaStream_t stream);
int batch_reserve(tucu_batch* b, size_t fir_jobs, size_t box_jobs, size_t items);

}  // namespace tucu
