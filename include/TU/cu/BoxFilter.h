/*
 * TU/cu/BoxFilter.h -- TU::cu::BoxFilter2 over the GB300 C ABI.
 *
 * Same class name, template parameters, members and argument meaning as the
 * reference's BoxFilter2<CONVOLVER, BLOCK_TRAITS, WMAX, CLOCK>
 * (TU/cu/BoxFilter.h:414-583): window sums (not means) of winSizeV x
 * winSizeH, output (rows+1-wV) x (cols+1-wH) at (wV/2, wH/2) when shift,
 * windows above WMAX throw std::runtime_error, an image smaller than the
 * window is a silent no-op.  CONVOLVER is device::box_convolver<T> (window
 * sums: integer inputs sum in int32, float inputs in FP32, which equals the
 * reference's sums in T for every input it accepts) or
 * device::extrema_finder<OP> (window minima / maxima and their positions,
 * TU/cu/BoxFilter.h:196-233).  BLOCK_TRAITS is inherited and otherwise
 * ignored; CLOCK times the convolve calls (print()).  Runs on the current
 * stream through tucu_box_convolve / tucu_extrema_convolve.
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

namespace device
{
/* The convolver types the reference's BoxFilter2 takes (TU/cu/BoxFilter.h:
 * 96-233).  Here they only select what BoxFilter2 computes; the kernels are
 * the library's. */
template <class T>
struct box_convolver
{
    using value_type = T;
    using result_type = T;
};

/* extrema_value<COMP>: the window extremum; extrema_position<COMP>: its
 * (x, y) input position as vec<int, 2>; extrema_value_position<COMP>: both.
 * COMP orders the values: less (std::less, thrust::less) finds minima,
 * greater finds maxima; ties resolve as in the reference. */
template <class COMP>
struct compared_type;  // T of a comparison functor COMP<T> (less<T>, greater<T>, ...)
template <template <class> class C, class T>
struct compared_type<C<T>>
{
    using type = T;
};

template <class COMP>
struct extrema_value
{
    using compare_type = COMP;
    using value_type = typename compared_type<COMP>::type;
    using result_type = value_type;
};
template <class COMP>
struct extrema_position
{
    using compare_type = COMP;
    using value_type = typename compared_type<COMP>::type;
    using result_type = vec<int, 2>;
};
template <class COMP>
struct extrema_value_position
{
    using compare_type = COMP;
    using value_type = typename compared_type<COMP>::type;
    using result_type = vec<int, 2>;
};

template <class OP, size_t WMAX = 23>
struct extrema_finder
{
    using value_type = typename OP::value_type;
    using result_type = typename OP::result_type;
};
}  // namespace device

template <class CONVOLVER = device::box_convolver<float>, class BLOCK_TRAITS = BlockTraits<>,
          size_t WMAX = TUCU_WIN_MAX_DEFAULT, class CLOCK = void>
class BoxFilter2 : public BLOCK_TRAITS, public detail::CallTimer<CLOCK>
{
  public:
    using convolver_type = CONVOLVER;
    using value_type = typename CONVOLVER::value_type;
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
        [[maybe_unused]] const auto timing = this->timed();
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
        [[maybe_unused]] const auto timing = this->timed();
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
        [[maybe_unused]] const auto timing = this->timed();
        detail::check(tucu_box_convolve_vec(h_, in, ip, rows, cols, n, out, op, shift ? 1 : 0, 0, stream_),
                      "BoxFilter2::convolve (vector pixels)");
    }

    tucu_box* h_ = nullptr;
    size_t wV_ = 0, wH_ = 0;
    cudaStream_t stream_ = nullptr;
};

/*
 * BoxFilter2<device::extrema_finder<OP>, ...>: window extrema of a T image
 * (TU/cu/BoxFilter.h:196-233) with the box geometry; OP = extrema_value<COMP>
 * writes the extrema, extrema_position<COMP> their (x, y) input positions,
 * extrema_value_position<COMP> both, into two images (the reference zips the
 * two output rows into one iterator instead).
 */
template <class OP, size_t W, class BLOCK_TRAITS, size_t WMAX, class CLOCK>
class BoxFilter2<device::extrema_finder<OP, W>, BLOCK_TRAITS, WMAX, CLOCK>
    : public BLOCK_TRAITS, public detail::CallTimer<CLOCK>
{
  public:
    using convolver_type = device::extrema_finder<OP, W>;
    using value_type = typename OP::value_type;
    constexpr static size_t WinSizeMax = WMAX;

    BoxFilter2(size_t winSizeV, size_t winSizeH)
    {
        using C = typename OP::compare_type;
        max_ = C()(value_type(1), value_type(0));  // a greater-than order finds maxima
        detail::check(tucu_extrema_create((int)winSizeV, (int)winSizeH, (int)WMAX, &h_), "BoxFilter2");
        wV_ = winSizeV;
        wH_ = winSizeH;
    }
    ~BoxFilter2() { tucu_extrema_destroy(h_); }
    BoxFilter2(const BoxFilter2&) = delete;
    BoxFilter2& operator=(const BoxFilter2&) = delete;

    size_t winSizeV() const { return wV_; }
    size_t winSizeH() const { return wH_; }
    BoxFilter2& setWinSizeV(size_t w)
    {
        detail::check(tucu_extrema_set_window(h_, (int)w, (int)wH_), "BoxFilter2::setWinSizeV");
        wV_ = w;
        return *this;
    }
    BoxFilter2& setWinSizeH(size_t w)
    {
        detail::check(tucu_extrema_set_window(h_, (int)wV_, (int)w), "BoxFilter2::setWinSizeH");
        wH_ = w;
        return *this;
    }
    size_t outSizeV(size_t nrow) const { return nrow + 1 - wV_; }
    size_t outSizeH(size_t ncol) const { return ncol + 1 - wH_; }
    size_t offsetV() const { return wV_ / 2; }
    size_t offsetH() const { return wH_ / 2; }

    /* extrema_value: the extrema into rowO; extrema_position: the positions
     * into rowO (pixels of vec<int, 2>). */
    template <class S, class D>
    void convolve(RowIterator<S> row, RowIterator<S> rowe, RowIterator<D> rowO, bool shift = true) const
    {
        using V = typename std::remove_const<D>::type;
        constexpr bool positions = std::is_same<V, int2>::value;
        if (positions)
            run(row, rowe, nullptr, 0, rowO.ptr(), rowO.pitch(), shift);
        else
            run(row, rowe, rowO.ptr(), rowO.pitch(), nullptr, 0, shift);
    }
    /* extrema_value_position: extrema into rowO, positions into rowP. */
    template <class S, class D>
    void convolve(RowIterator<S> row, RowIterator<S> rowe, RowIterator<D> rowO, RowIterator<int2> rowP,
                  bool shift = true) const
    {
        run(row, rowe, rowO.ptr(), rowO.pitch(), rowP.ptr(), rowP.pitch(), shift);
    }

    void setStream(cudaStream_t s) { stream_ = s; }

  private:
    template <class S>
    void run(RowIterator<S> row, RowIterator<S> rowe, void* val, size_t vpitch, void* pos, size_t ppitch,
             bool shift) const
    {
        [[maybe_unused]] const auto timing = this->timed();
        detail::check(tucu_extrema_convolve(h_, max_ ? TUCU_EXTREMA_MAX : TUCU_EXTREMA_MIN, row.ptr(),
                                            row.pitch(), (int)(rowe - row), row.cols(),
                                            detail::dtype_of<S>(), val, vpitch, pos, ppitch,
                                            shift ? 1 : 0, stream_),
                      "BoxFilter2::convolve (extrema)");
    }

    tucu_extrema* h_ = nullptr;
    size_t wV_ = 0, wH_ = 0;
    bool max_ = false;
    cudaStream_t stream_ = nullptr;
};

/*
 * ExtremaFilter2<T, MAX, WMAX> (not in the reference): the extrema BoxFilter2
 * above under a shorter name, with the order as a flag (MAX = false: window
 * minima, true: maxima) instead of a comparison type.  Same geometry, WMAX
 * check and no-op; windows up to 64.
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
