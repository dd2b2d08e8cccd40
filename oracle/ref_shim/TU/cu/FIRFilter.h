// Stand-in for the FIRFilter2 base that FIRGaussianConvolver.h derives from:
// only the lobe-size limit and the two members the Gaussian convolver names.
// The lobe design and lobeSize() compiled against it are the reference's own.
#pragma once
#include "TU/shim_array.h"
namespace TU
{
namespace cu
{
template <class T = float, class BLOCK_TRAITS = void>
class FIRFilter2
{
  public:
    constexpr static size_t LobeSizeMax = 17;
    FIRFilter2& initialize(const TU::Array<float>&, const TU::Array<float>&) { return *this; }
    template <class IN, class OUT>
    void convolve(IN, IN, OUT, bool = true) const {}
};
}  // namespace cu
}  // namespace TU
