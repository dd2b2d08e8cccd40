// Stand-in for the BoxFilter2 declarations GuidedFilter.h names.  No box
// arithmetic lives here; only the guided-filter functors are exercised.
#pragma once
#include "TU/shim_array.h"
namespace TU
{
template <class CLOCK>
class Profiler
{
  public:
    explicit Profiler(size_t) {}
    void start(int) const {}
    void nextFrame() const {}
};
namespace cu
{
template <size_t X = 32, size_t Y = 16>
struct BlockTraits
{
    constexpr static size_t BlockDimX = X, BlockDimY = Y, BlockDim = X * Y;
};
template <class T>
class Array2 : public TU::Array2<TU::Array<T>>
{
};
namespace device
{
template <class T>
struct box_convolver { using value_type = T; using result_type = T; };
}  // namespace device
template <class CONV, class BT = BlockTraits<>, size_t WMAX = 23, class CLOCK = void>
class BoxFilter2
{
  public:
    BoxFilter2(size_t v, size_t h) : _v(v), _h(h) {}
    size_t winSizeV() const { return _v; }
    size_t winSizeH() const { return _h; }
    BoxFilter2& setWinSizeV(size_t w) { _v = w; return *this; }
    BoxFilter2& setWinSizeH(size_t w) { _h = w; return *this; }
    template <class... A>
    void convolve(A...) const {}

  private:
    size_t _v, _h;
};
}  // namespace cu
}  // namespace TU
