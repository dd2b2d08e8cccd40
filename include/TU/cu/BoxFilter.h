/*
 * TU/cu/BoxFilter.h -- TU::cu::BoxFilter2 over the GB300 C ABI.
 *
 * Same class name, members and argument meaning as the reference's
 * BoxFilter2 (TU/cu/BoxFilter.h:416-583): window sums (not means) of
 * winSizeV x winSizeH, output (rows+1-wV) x (cols+1-wH) at (wV/2, wH/2) when
 * shift, windows above WMAX throw std::runtime_error, an image smaller than
 * the window is a silent no-op.  The reference's first template parameter
 * (the convolver type) becomes the accumulation implied by the pixel types:
 * integer inputs sum in int32 (exact), float inputs in FP32.  Runs on the
 * current stream through tucu_box_convolve.
 */
#ifndef TUCU_CXX_BOXFILTER_H
#define TUCU_CXX_BOXFILTER_H

#include <cstddef>

#include "detail/tucu_cxx.h"

namespace TU
{
namespace cu
{

/* The thresholded difference min(|x - y|, thresh) of the reference's stereo
 * cost (TU/cu/functional.h:385-398), as the op argument of
 * BoxFilter2::convolve(rowL, rowLe, rowR, costs, op, disparitySearchWidth). */
template <class T>
class diff
{
  public:
    diff(T thresh) : thresh_(thresh) {}
    T thresh() const { return thresh_; }

  private:
    T thresh_;
};

template <class T = float, size_t WMAX = TUCU_WIN_MAX_DEFAULT>
class BoxFilter2
{
  public:
    constexpr static size_t WinSizeMax = WMAX;

    BoxFilter2(size_t winSizeV, size_t winSizeH)
    {
        detail::check(tucu_box_create((int)winSizeV, (int)winSizeH, (int)WMAX, &h_), "BoxFilter2");
        wV_ = winSizeV;
        wH_ = winSizeH;
    }
    ~BoxFilter2() { tucu_box_destroy(h_); }
    BoxFilter2(const BoxFilter2&) = delete;
    BoxFilter2& operator=(const BoxFilter2&) = delete;

    size_t winSizeV() const { return wV_; }
    size_t winSizeH() const { return wH_; }
    BoxFilter2& setWinSizeV(size_t w)
    {
        detail::check(tucu_box_set_window(h_, (int)w, (int)wH_), "BoxFilter2::setWinSizeV");
        wV_ = w;
        return *this;
    }
    BoxFilter2& setWinSizeH(size_t w)
    {
        detail::check(tucu_box_set_window(h_, (int)wV_, (int)w), "BoxFilter2::setWinSizeH");
        wH_ = w;
        return *this;
    }
    size_t outSizeV(size_t nrow) const { return nrow + 1 - wV_; }
    size_t outSizeH(size_t ncol) const { return ncol + 1 - wH_; }
    size_t offsetV() const { return wV_ / 2; }
    size_t offsetH() const { return wH_ / 2; }

    template <class S, class D>
    void convolve(RowIterator<S> row, RowIterator<S> rowe, RowIterator<D> rowO, bool shift = true) const
    {
        detail::check(tucu_box_convolve(h_, row.ptr(), row.pitch(), (int)(rowe - row), row.cols(),
                                        detail::dtype_of<S>(), rowO.ptr(), rowO.pitch(),
                                        detail::dtype_of<D>(), shift ? 1 : 0, 0, stream_),
                      "BoxFilter2::convolve");
    }

    /* box_convolver<vec<float, N>> (TU/cu/BoxFilter.h:175-194): window sums of
     * vector pixels, here CUDA's float2 / float3 / float4 (N = 2, 3, 4), the
     * filter SuperPixels runs over its feature vectors.  Rows must start on
     * 16-byte boundaries (Array2's 256-byte rows do). */
    void convolve(RowIterator<const float2> row, RowIterator<const float2> rowe, RowIterator<float2> rowO,
                  bool shift = true) const
    {
        vec(row.ptr(), row.pitch(), (int)(rowe - row), row.cols(), 2, rowO.ptr(), rowO.pitch(), shift);
    }
    void convolve(RowIterator<const float3> row, RowIterator<const float3> rowe, RowIterator<float3> rowO,
                  bool shift = true) const
    {
        vec(row.ptr(), row.pitch(), (int)(rowe - row), row.cols(), 3, rowO.ptr(), rowO.pitch(), shift);
    }
    void convolve(RowIterator<const float4> row, RowIterator<const float4> rowe, RowIterator<float4> rowO,
                  bool shift = true) const
    {
        vec(row.ptr(), row.pitch(), (int)(rowe - row), row.cols(), 4, rowO.ptr(), rowO.pitch(), shift);
    }

    /* Stereo cost aggregation (TU/cu/BoxFilter.h:585-746) in the
     * disparity-major layout: costs slice d, (y, x) = window sum of
     * op(L, R shifted left by d) for d < disparitySearchWidth; int32 costs for
     * integer images, float for float images. */
    template <class S, class C>
    void convolve(RowIterator<S> rowL, RowIterator<S> rowLe, RowIterator<S> rowR,
                  SliceIterator<C> costs, diff<typename std::remove_const<S>::type> op,
                  size_t disparitySearchWidth) const
    {
        detail::check(tucu_box_stereo(h_, rowL.ptr(), rowL.pitch(), rowR.ptr(), rowR.pitch(),
                                      (int)(rowLe - rowL), rowL.cols(), detail::dtype_of<S>(),
                                      (float)op.thresh(), (int)disparitySearchWidth, costs.ptr(),
                                      costs.pitch(), costs.slice_pitch(), detail::dtype_of<C>(),
                                      stream_),
                      "BoxFilter2::convolve (stereo)");
    }

    /* Not in the reference: true runs later calls with an f16 input (rows on
     * 16-byte boundaries), an f16 or f32 output and windows up to 33 on the tensor cores, FP32-accurate but not bit-equal to the
     * reference arithmetic. */
    BoxFilter2& setTensorCores(bool on)
    {
        detail::check(tucu_box_set_tensor_cores(h_, on ? 1 : 0), "BoxFilter2::setTensorCores");
        return *this;
    }

    void setStream(cudaStream_t s) { stream_ = s; }

  private:
    void vec(const void* in, size_t ip, int rows, int cols, int n, void* out, size_t op, bool shift) const
    {
        detail::check(tucu_box_convolve_vec(h_, in, ip, rows, cols, n, out, op, shift ? 1 : 0, 0, stream_),
                      "BoxFilter2::convolve (vector pixels)");
    }

    tucu_box* h_ = nullptr;
    size_t wV_ = 0, wH_ = 0;
    cudaStream_t stream_ = nullptr;
};

/*
 * BoxFilter2 with the extrema_finder convolver (TU/cu/BoxFilter.h:196-233):
 * the reference's BoxFilter2<device::extrema_finder<OP>> with OP =
 * extrema_value<COMP> (convolve into an image of T), extrema_position<COMP>
 * (into an image of int2 (x, y) input positions; the reference's
 * vec<int, 2>) or extrema_value_position<COMP> (both).  COMP = thrust::less
 * is MAX = false (window minima), thrust::greater is MAX = true.  Same
 * geometry, WMAX check and no-op as BoxFilter2; windows up to 64.
 */
template <class T = float, bool MAX = false, size_t WMAX = TUCU_WIN_MAX_DEFAULT>
class ExtremaFilter2
{
  public:
    constexpr static size_t WinSizeMax = WMAX;

    ExtremaFilter2(size_t winSizeV, size_t winSizeH)
    {
        detail::check(tucu_extrema_create((int)winSizeV, (int)winSizeH, (int)WMAX, &h_),
                      "ExtremaFilter2");
        wV_ = winSizeV;
        wH_ = winSizeH;
    }
    ~ExtremaFilter2() { tucu_extrema_destroy(h_); }
    ExtremaFilter2(const ExtremaFilter2&) = delete;
    ExtremaFilter2& operator=(const ExtremaFilter2&) = delete;

    size_t winSizeV() const { return wV_; }
    size_t winSizeH() const { return wH_; }
    ExtremaFilter2& setWinSizeV(size_t w)
    {
        detail::check(tucu_extrema_set_window(h_, (int)w, (int)wH_), "ExtremaFilter2::setWinSizeV");
        wV_ = w;
        return *this;
    }
    ExtremaFilter2& setWinSizeH(size_t w)
    {
        detail::check(tucu_extrema_set_window(h_, (int)wV_, (int)w), "ExtremaFilter2::setWinSizeH");
        wH_ = w;
        return *this;
    }
    size_t outSizeV(size_t nrow) const { return nrow + 1 - wV_; }
    size_t outSizeH(size_t ncol) const { return ncol + 1 - wH_; }
    size_t offsetV() const { return wV_ / 2; }
    size_t offsetH() const { return wH_ / 2; }

    /* extrema_value: window extrema into rowO (pixels of T). */
    void convolve(RowIterator<const T> row, RowIterator<const T> rowe, RowIterator<T> rowO,
                  bool shift = true) const
    {
        run(row, rowe, rowO.ptr(), rowO.pitch(), nullptr, 0, shift);
    }
    /* extrema_position: (x, y) input positions of the window extrema. */
    void convolve(RowIterator<const T> row, RowIterator<const T> rowe, RowIterator<int2> rowP,
                  bool shift = true) const
    {
        run(row, rowe, nullptr, 0, rowP.ptr(), rowP.pitch(), shift);
    }
    /* extrema_value_position: both. */
    void convolve(RowIterator<const T> row, RowIterator<const T> rowe, RowIterator<T> rowO,
                  RowIterator<int2> rowP, bool shift = true) const
    {
        run(row, rowe, rowO.ptr(), rowO.pitch(), rowP.ptr(), rowP.pitch(), shift);
    }

    void setStream(cudaStream_t s) { stream_ = s; }

  private:
    void run(RowIterator<const T> row, RowIterator<const T> rowe, void* val, size_t vpitch,
             void* pos, size_t ppitch, bool shift) const
    {
        detail::check(tucu_extrema_convolve(h_, MAX ? TUCU_EXTREMA_MAX : TUCU_EXTREMA_MIN,
                                            row.ptr(), row.pitch(), (int)(rowe - row), row.cols(),
                                            detail::dtype_of<T>(), val, vpitch, pos, ppitch,
                                            shift ? 1 : 0, stream_),
                      "ExtremaFilter2::convolve");
    }

    tucu_extrema* h_ = nullptr;
    size_t wV_ = 0, wH_ = 0;
    cudaStream_t stream_ = nullptr;
};

}  // namespace cu
}  // namespace TU

#endif
