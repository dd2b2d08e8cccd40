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
    // FP32 input keeps compensated sums; narrower pixels sum exactly enough.
    static constexpr bool kCompensate = std::is_same<TIn, float>::value;
    const void* src;
    size_t pitch;
    int rows, cols;
    __device__ Raw load(int y, int x) const { return load_raw4<TIn, VEC>(src, pitch, rows, cols, y, x); }
    __device__ void expand(const Raw& r, int j, Acc (&q)[1]) const { q[0] = raw_elem<TIn, Acc>(r, j); }
};

// ---- epilogues --------------------------------------------------------------------

// Stores n = sizeof(W)/sizeof(T) consecutive values of v from element k.
template <class W, class T>
__device__ __forceinline__ void put_w(T* p, const T (&v)[4], int k)
{
    W w;
    memcpy(&w, v + k, sizeof(W));
    *reinterpret_cast<W*>(p + k) = w;
}

template <int S> struct Word;
template <> struct Word<1> { using type = uint8_t; };
template <> struct Word<2> { using type = uint16_t; };
template <> struct Word<4> { using type = uint32_t; };
template <> struct Word<8> { using type = uint2; };
template <> struct Word<16> { using type = uint4; };

// Writes 4 converted values at row + x*es.  All four valid: one vector store
// where the address allows it, else (output columns shifted off the 4-element
// grid) one element, one aligned pair and one element, or two aligned pairs.
template <class T>
__device__ __forceinline__ void put4(char* row, int x, const T (&v)[4], unsigned mask)
{
    T* p = reinterpret_cast<T*>(row) + x;
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    using W4 = typename Word<4 * sizeof(T)>::type;
    using W2 = typename Word<2 * sizeof(T)>::type;
    using W1 = typename Word<sizeof(T)>::type;
    if (mask == 0xfu) {
        if (a % (4 * sizeof(T)) == 0) {
            put_w<W4>(p, v, 0);
        } else if (a % (2 * sizeof(T)) == 0) {
            put_w<W2>(p, v, 0);
            put_w<W2>(p, v, 2);
        } else {
            put_w<W1>(p, v, 0);
            put_w<W2>(p, v, 1);
            put_w<W1>(p, v, 3);
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

template <class Acc>
struct PlainEpi
{
    void* dst;
    size_t pitch;
    int dtype, oy, ox;
    int normalize;
    float inv_n;  // 1/(wV*wH) rounded to float: a mean is sum * inv_n
    __device__ void store4(int y, int x, const Acc (&s)[4][1], unsigned mask) const
    {
        char* row = row_ptr(dst, pitch, y + oy);
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

// Rows fetched per batch (entering and leaving rows each), bounded by
// registers: TUCU_BOX_ROWS for narrow pixels, half as many for 4-byte ones.
#ifndef TUCU_BOX_ROWS
#define TUCU_BOX_ROWS 4
#endif
template <class TIn>
struct BoxRows
{
    static constexpr int value = sizeof(TIn) >= 4 ? (TUCU_BOX_ROWS > 2 ? TUCU_BOX_ROWS / 2 : 1) : TUCU_BOX_ROWS;
};

}  // namespace box
}  // namespace tucu
