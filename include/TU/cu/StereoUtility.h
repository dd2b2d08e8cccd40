/*
 * TU/cu/StereoUtility.h -- TU::cu::DisparitySelector over the GB300 C ABI.
 *
 * Same class name, constructor and select() as the reference's
 * DisparitySelector<T, BLOCK_TRAITS> (TU/cu/StereoUtility.h:109-217): winner-
 * take-all disparities of a disparity-major cost volume (Array3<T> of
 * disparitySearchWidth x rows x cols, as BoxFilter2's stereo convolve fills
 * it) with the left-right consistency check; out = disparityMax - d, or 0 when
 * the check fails.  select() takes the region to select over (the valid cost
 * region, outSizeV x outSizeH of the box filter) and the output row iterator
 * at the position it is written to.  The reference's right-image minima are
 * computed by unsynchronised blocks; here they are exact (see
 * tucu_disparity_select).  Runs on the current stream.
 */
#ifndef TUCU_CXX_STEREOUTILITY_H
#define TUCU_CXX_STEREOUTILITY_H

#include <cstddef>

#include "Array++.h"
#include "detail/tucu_cxx.h"

namespace TU
{
namespace cu
{

template <class T>
class DisparitySelector
{
  public:
    using value_type = T;

    DisparitySelector(int disparityMax, int disparityInconsistency)
    {
        detail::check(tucu_disparity_create(disparityMax, disparityInconsistency, &h_),
                      "DisparitySelector");
    }
    ~DisparitySelector() { tucu_disparity_destroy(h_); }
    DisparitySelector(const DisparitySelector&) = delete;
    DisparitySelector& operator=(const DisparitySelector&) = delete;

    template <class D>
    void select(const Array3<T>& costs, RowIterator<D> rowD, size_t nrow, size_t ncol) const
    {
        const SliceIterator<const T> c = costs.cbegin();
        detail::check(tucu_disparity_select(h_, c.ptr(), c.pitch(), c.slice_pitch(), costs.size(),
                                            (int)nrow, (int)ncol, detail::dtype_of<T>(), rowD.ptr(),
                                            rowD.pitch(), detail::dtype_of<D>(), 0, 0, stream_),
                      "DisparitySelector::select");
    }

    void setStream(cudaStream_t s) { stream_ = s; }

  private:
    tucu_disparity* h_ = nullptr;
    cudaStream_t stream_ = nullptr;
};

}  // namespace cu
}  // namespace TU

#endif
