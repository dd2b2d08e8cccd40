// Stand-in for TU/cu/vec.h: aggregate 2- and 4-vectors with x,y,z,w members.
#pragma once
#include <cstddef>
namespace TU
{
namespace cu
{
template <class T, size_t D>
struct vec;
template <class T>
struct vec<T, 2> { T x, y; };
template <class T>
struct vec<T, 4> { T x, y, z, w; };
}  // namespace cu
}  // namespace TU
