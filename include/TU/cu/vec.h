/*
 * TU/cu/vec.h -- TU::cu::vec<T, D>, the reference's short-vector pixel type
 * (TU/cu/vec.h:325), as the CUDA vector type it names: vec<float, 2..4> is
 * float2..float4, vec<int, 2> is int2 (the (x, y) positions of the extrema
 * finder), vec<T, 1> is T.  SuperPixels sums feature vectors of these types
 * with BoxFilter2<device::box_convolver<vec<float, N>>>.
 */
#ifndef TUCU_CXX_VEC_H
#define TUCU_CXX_VEC_H

#include <cuda_runtime.h>

#include <cstddef>

namespace TU
{
namespace cu
{
namespace detail
{
template <class T, size_t D> struct vec_type;
template <class T> struct vec_type<T, 1> { using type = T; };
template <> struct vec_type<float, 2> { using type = float2; };
template <> struct vec_type<float, 3> { using type = float3; };
template <> struct vec_type<float, 4> { using type = float4; };
template <> struct vec_type<int, 2> { using type = int2; };
}  // namespace detail

template <class T, size_t D>
using vec = typename detail::vec_type<T, D>::type;

}  // namespace cu
}  // namespace TU

#endif
