// box_ops.cuh -- producers and epilogues of the plain box filter on the
// window-sum strip (box_strip.cuh), shared by the single-image and the
// batched kernels.
#pragma once
#include <type_traits>

#include "box_strip.cuh"

namespace tucu
{
namespace box
{

// ---- raw pixel groups ------------------------------------------------------------

// Four consecutive pixels of one row as raw bits (zero outside the image).
template <class TIn> struct Raw4;
template <> struct Raw4<uint8_t> { uint32_t v; };
template <> struct Raw4<__half> { uint2 v; };
template <> struct Raw4<__nv_bfloat16> { uint2 v; };
template <> struct Raw4<float> { uint4 v; };
template <> struct Raw4<int32_t> { uint4 v; };

template <class TIn, bool VEC>
__device__ __forceinline__ Raw4<TIn> load_raw4(const void* base, size_t pitch, int rows, int cols,
                                              int y, int x)
{
    Raw4<TIn> r;
    memset(&r, 0, sizeof(r));
    if (y < 0 || y >= rows || x >= cols)
        return r;
    const TIn* row = reinterpret_cast<const TIn*>(row_ptr(base, pitch, y));
    if (VEC && x + kCPT <= cols) {
        r.v = __ldg(reinterpret_cast<const decltype(r.v)*>(row + x));
        return r;
    }
    TIn* e = reinterpret_cast<TIn*>(&r.v);
#pragma unroll
    for (int j = 0; j < kCPT; ++j)
        if (x + j < cols)
            e[j] = row[x + j];
    return r;
}

template <class TIn, class Acc>
__device__ __forceinline__ Acc raw_elem(const Raw4<TIn>& r, int j)
{
    const TIn* e = reinterpret_cast<const TIn*>(&r.v);
    if constexpr (std::is_same<TIn, uint8_t>::value)
        return Acc((r.v >> (8 * j)) & 0xffu);
    else if constexpr (std::is_same<TIn, int32_t>::value)
        return Acc(e[j]);
    else
        return Acc(to_float(e[j]));
}

// ---- producers ----------------------------------------------------------------

template <class TIn, class Acc, bool VEC>
struct PlainProd
{
    using Raw = Raw4<TIn>;
    const void* src;
    size_t pitch;
    int rows, cols;
    __device__ Raw load(int y, int x) const { return load_raw4<TIn, VEC>(src, pitch, rows, cols, y, x); }
    __device__ void expand(const Raw& r, int j, Acc (&q)[1]) const { q[0] = raw_elem<TIn, Acc>(r, j); }
};

// ---- epilogues --------------------------------------------------------------------

// Writes 4 converted values at row + x*es; vector store when all 4 are valid
// and the address allows it.
template <class T>
__device__ __forceinline__ void put4(char* row, int x, const T (&v)[4], unsigned mask)
{
    T* p = reinterpret_cast<T*>(row) + x;
    if (mask == 0xfu && (reinterpret_cast<uintptr_t>(p) % (4 * sizeof(T))) == 0) {
        if constexpr (sizeof(T) == 1) {
            uint32_t u;
            memcpy(&u, v, 4);
            *reinterpret_cast<uint32_t*>(p) = u;
        } else if constexpr (sizeof(T) == 2) {
            uint2 u;
            memcpy(&u, v, 8);
            *reinterpret_cast<uint2*>(p) = u;
        } else {
            uint4 u;
            memcpy(&u, v, 16);
            *reinterpret_cast<uint4*>(p) = u;
        }
        return;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if ((mask >> j) & 1u)
            p[j] = v[j];
}

// Converts 4 float results to the output type and stores them.
__device__ __forceinline__ void store4_float(char* row, int x, int dt, const float (&f)[4],
                                             unsigned mask)
{
    switch (dt) {
    case U8: {
        uint8_t v[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) v[j] = f2u8(f[j]);
        put4(row, x, v, mask);
        break;
    }
    case F16: {
        __half v[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) v[j] = __float2half_rn(f[j]);
        put4(row, x, v, mask);
        break;
    }
    case BF16: {
        __nv_bfloat16 v[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) v[j] = __float2bfloat16_rn(f[j]);
        put4(row, x, v, mask);
        break;
    }
    case I32: {
        int32_t v[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) v[j] = __float2int_rz(f[j]);
        put4(row, x, v, mask);
        break;
    }
    default: put4(row, x, f, mask); break;
    }
}

__device__ __forceinline__ unsigned valid_mask(int i, int two)
{
    unsigned m = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (i + j >= 0 && i + j < two)
            m |= 1u << j;
    return m;
}

template <class Acc>
struct PlainEpi
{
    void* dst;
    size_t pitch;
    int dtype, oy, ox;
    int normalize;
    float inv_n;  // 1/(wV*wH) rounded to float: a mean is sum * inv_n
    __device__ void store4(int y, int x, const Acc (&s)[4][1], int i, int two) const
    {
        char* row = row_ptr(dst, pitch, y + oy);
        const unsigned mask = valid_mask(i, two);
        if constexpr (std::is_same<Acc, int>::value) {
            if (!normalize && dtype == I32) {
                const int32_t v[4] = {s[0][0], s[1][0], s[2][0], s[3][0]};
                put4(row, x + ox, v, mask);
                return;
            }
            if (!normalize && dtype == U8) {
                uint8_t v[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) v[j] = (uint8_t)min(max(s[j][0], 0), 255);
                put4(row, x + ox, v, mask);
                return;
            }
        }
        float f[4];
#pragma unroll
        for (int j = 0; j < 4; ++j)
            f[j] = normalize ? __fmul_rn((float)s[j][0], inv_n) : (float)s[j][0];
        store4_float(row, x + ox, dtype, f, mask);
    }
};

// Rows fetched per batch: about 32 bytes of raw input per thread and row
// direction in flight, bounded by registers.
template <class TIn> struct BoxRows { static constexpr int value = sizeof(TIn) >= 4 ? 4 : 8; };

}  // namespace box
}  // namespace tucu
