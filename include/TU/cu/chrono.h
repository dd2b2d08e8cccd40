/*
 * TU/cu/chrono.h -- TU::cu::clock, the GPU clock of the reference
 * (TU/cu/chrono.h:50-90, chrono.cc): a std::chrono-style clock whose now()
 * is the time of a CUDA event recorded on the legacy default stream, in
 * milliseconds since the first call.  now() waits for the event, so the
 * difference of two readings covers the GPU work issued between them.
 * Used as the CLOCK argument of the filter classes (whose print() then
 * reports the GPU time of their convolve calls) and by timing code.
 */
#ifndef TUCU_CXX_CHRONO_H
#define TUCU_CXX_CHRONO_H

#include <cuda_runtime.h>

#include <chrono>

namespace TU
{
namespace cu
{

class clock
{
  public:
    using rep = float;
    using period = std::milli;
    using duration = std::chrono::duration<rep, period>;
    using time_point = std::chrono::time_point<clock>;
    constexpr static bool is_steady = true;

    static time_point now()
    {
        static cudaEvent_t origin = record();
        cudaEvent_t e = record();
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, origin, e);
        cudaEventDestroy(e);
        return time_point(duration(ms));
    }

  private:
    static cudaEvent_t record()
    {
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        cudaEventRecord(e, 0);
        cudaEventSynchronize(e);
        return e;
    }
};

}  // namespace cu
}  // namespace TU

#endif
