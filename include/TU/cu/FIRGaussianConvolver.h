/*
 * TU/cu/FIRGaussianConvolver.h -- TU::cu::FIRGaussianConvolver2 over the GB300
 * C ABI.
 *
 * Same class name, members and argument meaning as the reference's
 * FIRGaussianConvolver2 (TU/cu/FIRGaussianConvolver.h:57-101, 123-242):
 * constructed with sigma; smooth / diffH / diffV / diffHH / diffHV / diffVV
 * (ib, ie, out, shift) filter rows [ib, ie) into out with the lobes the
 * reference designs for sigma (truncation rule of lobeSize,
 * FIRGaussianConvolver.cu:52-98); the valid region and the no-op on small
 * images follow FIRFilter2.  Runs on the current stream through
 * tucu_gauss_convolve.
 */
#ifndef TUCU_CXX_FIRGAUSSIANCONVOLVER_H
#define TUCU_CXX_FIRGAUSSIANCONVOLVER_H

#include "detail/tucu_cxx.h"

namespace TU
{
namespace cu
{

template <class T = float>
class FIRGaussianConvolver2
{
  public:
    explicit FIRGaussianConvolver2(float sigma = 1.0f)
    {
        detail::check(tucu_gauss_create(sigma, &h_), "FIRGaussianConvolver2");
    }
    ~FIRGaussianConvolver2() { tucu_gauss_destroy(h_); }
    FIRGaussianConvolver2(const FIRGaussianConvolver2&) = delete;
    FIRGaussianConvolver2& operator=(const FIRGaussianConvolver2&) = delete;

    float sigma() const { return tucu_gauss_sigma(h_); }

    /* Not in the reference: true designs the lobes in the reference's own
     * float arithmetic (bit-equal to its lobes) instead of FP64 rounded once
     * (tucu_gauss_set_reference_lobes). */
    FIRGaussianConvolver2& setReferenceLobes(bool on)
    {
        detail::check(tucu_gauss_set_reference_lobes(h_, on ? 1 : 0),
                      "FIRGaussianConvolver2::setReferenceLobes");
        return *this;
    }
    FIRGaussianConvolver2& initialize(float sigma)
    {
        detail::check(tucu_gauss_initialize(h_, sigma), "FIRGaussianConvolver2::initialize");
        return *this;
    }

    template <class S, class D>
    void smooth(RowIterator<S> ib, RowIterator<S> ie, RowIterator<D> out, bool shift = true) const
    {
        run(TUCU_SMOOTH, ib, ie, out, shift);
    }
    template <class S, class D>
    void diffH(RowIterator<S> ib, RowIterator<S> ie, RowIterator<D> out, bool shift = true) const
    {
        run(TUCU_DIFF_H, ib, ie, out, shift);
    }
    template <class S, class D>
    void diffV(RowIterator<S> ib, RowIterator<S> ie, RowIterator<D> out, bool shift = true) const
    {
        run(TUCU_DIFF_V, ib, ie, out, shift);
    }
    template <class S, class D>
    void diffHH(RowIterator<S> ib, RowIterator<S> ie, RowIterator<D> out, bool shift = true) const
    {
        run(TUCU_DIFF_HH, ib, ie, out, shift);
    }
    template <class S, class D>
    void diffHV(RowIterator<S> ib, RowIterator<S> ie, RowIterator<D> out, bool shift = true) const
    {
        run(TUCU_DIFF_HV, ib, ie, out, shift);
    }
    template <class S, class D>
    void diffVV(RowIterator<S> ib, RowIterator<S> ie, RowIterator<D> out, bool shift = true) const
    {
        run(TUCU_DIFF_VV, ib, ie, out, shift);
    }

    /* Not in the reference: true runs later calls with an f16 input (rows on
     * 16-byte boundaries), an f16 or f32 output and at most 33 taps per
     * direction on the tensor cores, FP32-accurate but not bit-equal to the
     * reference arithmetic. */
    FIRGaussianConvolver2& setTensorCores(bool on)
    {
        detail::check(tucu_gauss_set_tensor_cores(h_, on ? 1 : 0), "FIRGaussianConvolver2::setTensorCores");
        return *this;
    }

    void setStream(cudaStream_t s) { stream_ = s; }

  private:
    template <class S, class D>
    void run(int op, RowIterator<S> ib, RowIterator<S> ie, RowIterator<D> out, bool shift) const
    {
        detail::check(tucu_gauss_convolve(h_, op, ib.ptr(), ib.pitch(), (int)(ie - ib), ib.cols(),
                                          detail::dtype_of<S>(), out.ptr(), out.pitch(),
                                          detail::dtype_of<D>(), shift ? 1 : 0, stream_),
                      "FIRGaussianConvolver2");
    }

    tucu_gauss* h_ = nullptr;
    cudaStream_t stream_ = nullptr;
};

}  // namespace cu
}  // namespace TU

#endif
