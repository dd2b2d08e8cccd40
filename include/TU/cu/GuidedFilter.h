/*
 * TU/cu/GuidedFilter.h -- TU::cu::GuidedFilter2 over the GB300 C ABI.
 *
 * Same class name, template parameters, members and argument meaning as the
 * reference's GuidedFilter2<T, BLOCK_TRAITS, WMAX, CLOCK>
 * (TU/cu/GuidedFilter.h:134-344): windows wrow x wcol, e squared internally,
 * output (rows-2(w-1)) x (cols-2(w-1)) at (wV-1, wH-1) when shift;
 * convolve(ib, ie, gb, ge, out, shift) with a guide and convolve(ib, ie, out,
 * shift) guided by the input itself (the reference's self-guided offset term
 * kept).  BLOCK_TRAITS is inherited and otherwise ignored; CLOCK times the
 * convolve calls (print()).  Runs on the current stream through
 * tucu_guided_convolve; the coefficient scratch belongs to the object.
 */
#ifndef TUCU_CXX_GUIDEDFILTER_H
#define TUCU_CXX_GUIDEDFILTER_H

#include <cstddef>

#include "detail/tucu_cxx.h"

namespace TU
{
namespace cu
{

template <class T = float, class BLOCK_TRAITS = BlockTraits<>, size_t WMAX = TUCU_WIN_MAX_DEFAULT,
          class CLOCK = void>
class GuidedFilter2 : public BLOCK_TRAITS, public detail::CallTimer<CLOCK>
{
  public:
    using element_type = T;

    GuidedFilter2(size_t wrow, size_t wcol, T e)
    {
        detail::check(tucu_guided_create((int)wrow, (int)wcol, (float)e, (int)WMAX, &h_), "GuidedFilter2");
        wV_ = wrow;
        wH_ = wcol;
    }
    ~GuidedFilter2() { tucu_guided_destroy(h_); }
    GuidedFilter2(const GuidedFilter2&) = delete;
    GuidedFilter2& operator=(const GuidedFilter2&) = delete;

    T epsilon() const { return (T)tucu_guided_epsilon(h_); }
    GuidedFilter2& setEpsilon(T e)
    {
        detail::check(tucu_guided_set_epsilon(h_, (float)e), "GuidedFilter2::setEpsilon");
        return *this;
    }
    size_t winSizeV() const { return wV_; }
    size_t winSizeH() const { return wH_; }
    GuidedFilter2& setWinSizeV(size_t w)
    {
        detail::check(tucu_guided_set_window(h_, (int)w, (int)wH_), "GuidedFilter2::setWinSizeV");
        wV_ = w;
        return *this;
    }
    GuidedFilter2& setWinSizeH(size_t w)
    {
        detail::check(tucu_guided_set_window(h_, (int)wV_, (int)w), "GuidedFilter2::setWinSizeH");
        wH_ = w;
        return *this;
    }
    size_t outSizeV(size_t nrow) const { return nrow - 2 * (wV_ - 1); }
    size_t outSizeH(size_t ncol) const { return ncol - 2 * (wH_ - 1); }
    size_t offsetV() const { return wV_ - 1; }
    size_t offsetH() const { return wH_ - 1; }

    template <class S, class G, class D>
    void convolve(RowIterator<S> ib, RowIterator<S> ie, RowIterator<G> gb, RowIterator<G> ge,
                  RowIterator<D> out, bool shift = true) const
    {
        static_assert(detail::dtype_of<S>() == detail::dtype_of<G>(), "input and guide share a pixel type");
        if ((ge - gb) != (ie - ib) || gb.cols() != ib.cols())
            throw std::runtime_error("GuidedFilter2::convolve: guide and input differ in size");
        [[maybe_unused]] const auto timing = this->timed();
        detail::check(tucu_guided_convolve(h_, ib.ptr(), ib.pitch(), gb.ptr(), gb.pitch(), (int)(ie - ib),
                                           ib.cols(), detail::dtype_of<S>(), out.ptr(), out.pitch(),
                                           detail::dtype_of<D>(), shift ? 1 : 0, stream_),
                      "GuidedFilter2::convolve");
    }

    template <class S, class D>
    void convolve(RowIterator<S> ib, RowIterator<S> ie, RowIterator<D> out, bool shift = true) const
    {
        [[maybe_unused]] const auto timing = this->timed();
        detail::check(tucu_guided_convolve(h_, ib.ptr(), ib.pitch(), nullptr, 0, (int)(ie - ib), ib.cols(),
                                           detail::dtype_of<S>(), out.ptr(), out.pitch(),
                                           detail::dtype_of<D>(), shift ? 1 : 0, stream_),
                      "GuidedFilter2::convolve");
    }

    void setStream(cudaStream_t s) { stream_ = s; }

  private:
    tucu_guided* h_ = nullptr;
    size_t wV_ = 0, wH_ = 0;
    cudaStream_t stream_ = nullptr;
};

}  // namespace cu
}  // namespace TU

#endif
