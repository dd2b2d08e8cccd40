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
// unsupported type) -- callers then use plain loads.
bool make_tmap_2d(CUtensorMap* map, const void* base, int dtype, int cols, int rows,
                  size_t pitch, int box_w, int box_h);

// Number of SMs of the current device (cached per device).
int sm_count();

// Batched launch helpers for the server (batch.cu).
int batch_plan_on_stream(tucu_batch* b, int fir_rows, int box_rows, cudaStream_t stream);
int batch_reserve(tucu_batch* b, size_t fir_jobs, size_t box_jobs, size_t items);

}  // namespace tucu
