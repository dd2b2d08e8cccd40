// Stand-in for TU/cu/algorithm.h: the range types the kernels' signatures
// name and the block-size traits the filter classes derive from.
#pragma once
#include <cstddef>
namespace TU
{
template <class ITER>
class range;
template <class ITER>
class range_iterator;
namespace cu
{
template <size_t BLOCK_DIM_X = 32, size_t BLOCK_DIM_Y = 16>
struct BlockTraits
{
    constexpr static size_t BlockDimX = BLOCK_DIM_X;
    constexpr static size_t BlockDimY = BLOCK_DIM_Y;
};
using TU::range;
using TU::range_iterator;
}  // namespace cu
}  // namespace TU
