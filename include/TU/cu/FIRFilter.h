/*
 * TU/cu/FIRFilter.h -- TU::cu::FIRFilter2 over the GB300 C ABI.
 *
 * Same class name, members and argument meaning as the reference's
 * FIRFilter2<T, BLOCK_TRAITS> (TU/cu/FIRFilter.h:18-52, 245-377): lobes of
 * at most 17 taps,
 * outermost tap first; convolve(ib, ie, out, shift) writes the valid region
 * (rows-2*LS_V) x (cols-2*LS_H) at (LS_V, LS_H) when shift, LS = size & ~1;
 * an image smaller than the support is a silent no-op; lobes that are too
 * long throw std::runtime_error.  The work runs on the current stream
 * (default: the legacy default stream) through tucu_fir_convolve.
 */
#ifndef TUCU_CXX_FIRFILTER_H
#define TUCU_CXX_FIRFILTER_H

#include <cstddef>

#include "detail/tucu_cxx.h"

namespace TU
{
namespace cu
{

template <class T = float, class BLOCK_TRAITS = BlockTraits<>>
class FIRFilter2 : public BLOCK_TRAITS
{
  public:
    using value_type = T;
    constexpr static size_t LobeSizeMax = TUCU_LOBE_MAX;

    FIRFilter2() { detail::check(tucu_fir_create(&h_), "FIRFilter2"); }
    ~FIRFilter2() { tucu_fir_destroy(h_); }
    FIRFilter2(const FIRFilter2&) = delete;
    FIRFilter2& operator=(const FIRFilter2&) = delete;

    /* Any contiguous containers of float (std::vector, std::array, ...). */
    template <class LH, class LV>
    FIRFilter2& initialize(const LH& lobeH, const LV& lobeV)
    {
        detail::check(tucu_fir_initialize(h_, lobeH.data(), (int)lobeH.size(), lobeV.data(),
                                          (int)lobeV.size()),
                      "FIRFilter2::initialize");
        sizeH_ = (int)lobeH.size();
        sizeV_ = (int)lobeV.size();
        return *this;
    }

    size_t lobeSizeH() const { return sizeH_; }
    size_t lobeSizeV() const { return sizeV_; }
    size_t offsetH() const { return sizeH_ & ~1; }
    size_t offsetV() const { return sizeV_ & ~1; }
    size_t outSizeH(size_t inSize) const { return inSize - 2 * offsetH(); }
    size_t outSizeV(size_t inSize) const { return inSize - 2 * offsetV(); }

    template <class S, class D>
    void convolve(RowIterator<S> ib, RowIterator<S> ie, RowIterator<D> out, bool shift = true) const
    {
        detail::check(tucu_fir_convolve(h_, ib.ptr(), ib.pitch(), (int)(ie - ib), ib.cols(),
                                        detail::dtype_of<S>(), out.ptr(), out.pitch(),
                                        detail::dtype_of<D>(), shift ? 1 : 0, stream_),
                      "FIRFilter2::convolve");
    }

    /* Not in the reference: true runs later calls with an f16 input (rows on
     * 16-byte boundaries), an f16 or f32 output and at most 33 taps per
     * direction on the tensor cores, FP32-accurate but not bit-equal to the
     * reference arithmetic. */
    FIRFilter2& setTensorCores(bool on)
    {
        detail::check(tucu_fir_set_tensor_cores(h_, on ? 1 : 0), "FIRFilter2::setTensorCores");
        return *this;
    }

    /* Stream the convolutions run on (nullptr: the legacy default stream). */
    void setStream(cudaStream_t s) { stream_ = s; }

  private:
    tucu_fir* h_ = nullptr;
    int sizeH_ = 0, sizeV_ = 0;
    cudaStream_t stream_ = nullptr;
};

}  // namespace cu
}  // namespace TU

#endif
