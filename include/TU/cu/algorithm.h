/*
 * TU/cu/algorithm.h -- the block-shape parameter of the reference's filter
 * classes (TU/cu/algorithm.h:56-67, BlockTraits<BLOCK_DIM_X, BLOCK_DIM_Y>).
 *
 * The classes of include/TU/cu/ accept it as their BLOCK_TRAITS template
 * argument and inherit it (BlockDimX, BlockDimY, BlockDim keep their values),
 * so the reference's instantiations compile unchanged.  The kernels choose
 * their own tiles: the block shape does not change what they compute.
 */
#ifndef TUCU_CXX_ALGORITHM_H
#define TUCU_CXX_ALGORITHM_H

#include <cstddef>

namespace TU
{
namespace cu
{

template <size_t BLOCK_DIM_X = 32, size_t BLOCK_DIM_Y = 16>
struct BlockTraits
{
    constexpr static size_t BlockDimX = BLOCK_DIM_X;
    constexpr static size_t BlockDimY = BLOCK_DIM_Y;
    constexpr static size_t BlockDim = BlockDimX * BlockDimY;
};

}  // namespace cu
}  // namespace TU

#endif
