// Stand-in for TU/cu/vec.h: the vector type the position functors name.
#pragma once
#include <cstddef>
#include <cuda/std/tuple>
namespace TU
{
namespace cu
{
template <class T, size_t N>
struct vec;
}  // namespace cu
}  // namespace TU
