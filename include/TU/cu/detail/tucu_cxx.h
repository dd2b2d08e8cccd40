/*
 * Shared plumbing of the C++ filter classes (TU/cu/FIRFilter.h,
 * FIRGaussianConvolver.h, BoxFilter.h, GuidedFilter.h): pixel types to
 * tucu_dtype, status codes to exceptions, row iterators to (pointer, pitch,
 * rows, cols).
 */
#ifndef TUCU_CXX_DETAIL_H
#define TUCU_CXX_DETAIL_H

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include <chrono>
#include <ostream>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "../../../tucu_gb300.h"
#include "../Array++.h"
#include "../algorithm.h"
#include "../chrono.h"
#include "../vec.h"

namespace TU
{
namespace cu
{
namespace detail
{

template <class T> struct Dtype;
template <> struct Dtype<unsigned char> { static constexpr int value = TUCU_U8; };
template <> struct Dtype<__half> { static constexpr int value = TUCU_F16; };
template <> struct Dtype<__nv_bfloat16> { static constexpr int value = TUCU_BF16; };
template <> struct Dtype<float> { static constexpr int value = TUCU_F32; };
template <> struct Dtype<int32_t> { static constexpr int value = TUCU_I32; };

template <class T>
constexpr int dtype_of() { return Dtype<typename std::remove_const<T>::type>::value; }

/* Negative status -> std::runtime_error (the reference throws for bad lobe
 * and window sizes and exits on CUDA errors); TUCU_NOOP (image smaller than
 * the support) is the reference's silent return. */
inline int check(int status, const char* what)
{
    if (status < 0) {
        const char* d = tucu_last_error();
        throw std::runtime_error(std::string(what) + ": " + tucu_status_string(status) +
                                 (d && *d ? std::string(" (") + d + ")" : std::string()));
    }
    return status;
}

/* The CLOCK template argument of the reference's filter classes (their
 * Profiler<CLOCK> base): with a clock (TU::cu::clock, a std::chrono clock)
 * every convolve call is timed with it and print() reports the count and the
 * mean; with void (the default) nothing is timed and print() writes nothing. */
template <class CLOCK>
class CallTimer
{
  public:
    void print(std::ostream& out) const
    {
        if (n_)
            out << n_ << " calls, " << total_ms_ / (double)n_ << " ms per call" << std::endl;
    }

  protected:
    class Scope
    {
      public:
        explicit Scope(const CallTimer* t) : t_(t), t0_(CLOCK::now()) {}
        ~Scope()
        {
            const auto d = CLOCK::now() - t0_;
            ++t_->n_;
            t_->total_ms_ += std::chrono::duration<double, std::milli>(d).count();
        }
        Scope(const Scope&) = delete;

      private:
        const CallTimer* t_;
        typename CLOCK::time_point t0_;
    };
    Scope timed() const { return Scope(this); }

  private:
    mutable size_t n_ = 0;
    mutable double total_ms_ = 0.0;
};

template <>
class CallTimer<void>
{
  public:
    void print(std::ostream&) const {}

  protected:
    struct Scope
    {
    };
    Scope timed() const { return Scope(); }
};

/* A row range [ib, ie) as the C ABI takes it. */
template <class IT>
struct Rows
{
    const void* ptr;
    size_t pitch;
    int rows, cols, dtype;
};

template <class T>
inline Rows<RowIterator<const T>> rows_of(RowIterator<const T> ib, RowIterator<const T> ie)
{
    return {ib.ptr(), ib.pitch(), (int)(ie - ib), ib.cols(), dtype_of<T>()};
}

}  // namespace detail
}  // namespace cu
}  // namespace TU

#endif
