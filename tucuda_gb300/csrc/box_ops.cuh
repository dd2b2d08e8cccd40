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

// Columns x..x+3 of row y, checked against the image.
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
    static constexpr int kPlanes = 1;
    static constexpr int kPlaneBytes = 4 * sizeof(TIn);
    static constexpr bool kAsync = VEC;
    // FP32 input keeps compensated sums; narrower pixels sum exactly enough.
    static constexpr bool kCompensate = std::is_same<TIn, float>::value;
    const void* src;
    size_t pitch;
    int rows, cols;
    __device__ const void* plane_ptr(int, int y, int x) const
    {
        return row_ptr(src, pitch, y) + (size_t)x * sizeof(TIn);
    }
    __device__ int plane_bytes(int, int nvalid, int) const { return nvalid * (int)sizeof(TIn); }
    __device__ Raw load(int y, int x) const { return load_raw4<TIn, VEC>(src, pitch, rows, cols, y, x); }
    __device__ void finish(Raw&, int) const {}
    __device__ void expand(const Raw& r, int j, Acc (&q)[1]) const { q[0] = raw_elem<TIn, Acc>(r, j); }
};

// ---- stores -------------------------------------------------------------------

// Alignment of four consecutive output elements starting at column x + ox of
// any row (x a multiple of 4), computed on the host: 4 = one vector store,
// 2 = two aligned pairs, 1 = element, pair, element (odd start), 0 = look at
// each address.
inline int store_class(const void* dst, size_t pitch, int ox, int es)
{
    const uintptr_t a = reinterpret_cast<uintptr_t>(dst) + (uintptr_t)ox * es;
    if (a % es != 0)
        return 0;
    if (pitch % (4 * (size_t)es) == 0 && a % (4 * es) == 0)
        return 4;
    if (pitch % (2 * (size_t)es) == 0 && a % (2 * es) == 0)
        return 2;
    if (pitch % (2 * (size_t)es) == 0)
        return 1;
    return 0;
}

template <class T>
__device__ __forceinline__ uint32_t bits_of(T v)
{
    if constexpr (sizeof(T) == 1) {
        return (uint32_t)(uint8_t)v;
    } else if constexpr (sizeof(T) == 2) {
        uint16_t u;
        memcpy(&u, &v, 2);
        return u;
    } else {
        uint32_t u;
        memcpy(&u, &v, 4);
        return u;
    }
}

// Writes 4 values at row + x*es: bit j of mask set = value j is written.
// All four valid: one vector store where the address allows it, else two
// aligned pairs, or element, pair, element (cls from store_class; 0 = look
// at the address).  Words are assembled from the values' bits, so nothing
// goes through local memory.
template <class T>
__device__ __forceinline__ void put4(char* row, int x, const T (&v)[4], unsigned mask, int cls)
{
    T* p = reinterpret_cast<T*>(row) + x;
    if (mask != 0xfu) {
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if ((mask >> j) & 1u)
                p[j] = v[j];
        return;
    }
    if (cls == 0) {
        const uintptr_t a = reinterpret_cast<uintptr_t>(p);
        cls = a % (4 * sizeof(T)) == 0 ? 4 : a % (2 * sizeof(T)) == 0 ? 2 : 1;
    }
    const uint32_t b0 = bits_of(v[0]), b1 = bits_of(v[1]), b2 = bits_of(v[2]), b3 = bits_of(v[3]);
    if constexpr (sizeof(T) == 1) {
        if (cls == 4) {
            *reinterpret_cast<uint32_t*>(p) = b0 | b1 << 8 | b2 << 16 | b3 << 24;
        } else if (cls == 2) {
            *reinterpret_cast<uint16_t*>(p) = (uint16_t)(b0 | b1 << 8);
            *reinterpret_cast<uint16_t*>(p + 2) = (uint16_t)(b2 | b3 << 8);
        } else {
            *reinterpret_cast<uint8_t*>(p) = (uint8_t)b0;
            *reinterpret_cast<uint16_t*>(p + 1) = (uint16_t)(b1 | b2 << 8);
            *reinterpret_cast<uint8_t*>(p + 3) = (uint8_t)b3;
        }
    } else if constexpr (sizeof(T) == 2) {
        if (cls == 4) {
            *reinterpret_cast<uint2*>(p) = make_uint2(b0 | b1 << 16, b2 | b3 << 16);
        } else if (cls == 2) {
            *reinterpret_cast<uint32_t*>(p) = b0 | b1 << 16;
            *reinterpret_cast<uint32_t*>(p + 2) = b2 | b3 << 16;
        } else {
            *reinterpret_cast<uint16_t*>(p) = (uint16_t)b0;
            *reinterpret_cast<uint32_t*>(p + 1) = b1 | b2 << 16;
            *reinterpret_cast<uint16_t*>(p + 3) = (uint16_t)b3;
        }
    } else {
        if (cls == 4) {
            *reinterpret_cast<uint4*>(p) = make_uint4(b0, b1, b2, b3);
        } else if (cls == 2) {
            *reinterpret_cast<uint2*>(p) = make_uint2(b0, b1);
            *reinterpret_cast<uint2*>(p + 2) = make_uint2(b2, b3);
        } else {
            *reinterpret_cast<uint32_t*>(p) = b0;
            *reinterpret_cast<uint2*>(p + 1) = make_uint2(b1, b2);
            *reinterpret_cast<uint32_t*>(p + 3) = b3;
        }
    }
}

template <class T> __device__ __forceinline__ T from_float(float f);
template <> __device__ __forceinline__ uint8_t from_float<uint8_t>(float f) { return f2u8(f); }
template <> __device__ __forceinline__ __half from_float<__half>(float f) { return __float2half_rn(f); }
template <> __device__ __forceinline__ __nv_bfloat16 from_float<__nv_bfloat16>(float f)
{
    return __float2bfloat16_rn(f);
}
template <> __device__ __forceinline__ float from_float<float>(float f) { return f; }
template <> __device__ __forceinline__ int32_t from_float<int32_t>(float f) { return __float2int_rz(f); }

// Converts 4 float results to the output dtype (known at run time) and
// stores them.
__device__ __forceinline__ void store4_float(char* row, int x, int dt, const float (&f)[4],
                                             unsigned mask, int cls)
{
    auto put = [&](auto tag) {
        using T = decltype(tag);
        T v[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) v[j] = from_float<T>(f[j]);
        put4(row, x, v, mask, cls);
    };
    switch (dt) {
    case U8: put(uint8_t()); break;
    case F16: put(__half()); break;
    case BF16: put(__nv_bfloat16()); break;
    case I32: put(int32_t()); break;
    default: put4(row, x, f, mask, cls); break;
    }
}

// ---- epilogue -------------------------------------------------------------------

// Writes window sums (or means) at (y + oy, x + ox).  TOut = void: output
// dtype read at run time; otherwise the kernel is compiled for it.
template <class Acc, class TOut>
struct PlainEpi
{
    void* dst;
    size_t pitch;
    int dtype, oy, ox;
    int normalize;
    float inv_n;  // 1/(wV*wH) rounded to float: a mean is sum * inv_n
    int cls;      // store_class of dst, pitch, ox
    __device__ void store4(int y, int x, const Acc (&s)[4][1], unsigned mask) const
    {
        char* row = row_ptr(dst, pitch, y + oy);
        if constexpr (!std::is_void<TOut>::value) {
            TOut v[4];
            if constexpr (std::is_same<Acc, int>::value && std::is_same<TOut, int32_t>::value) {
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    v[j] = normalize ? __float2int_rz(__fmul_rn((float)s[j][0], inv_n)) : s[j][0];
            } else if constexpr (std::is_same<Acc, int>::value && std::is_same<TOut, uint8_t>::value) {
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    v[j] = normalize ? f2u8(__fmul_rn((float)s[j][0], inv_n))
                                     : (uint8_t)min(max(s[j][0], 0), 255);
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    v[j] = from_float<TOut>(normalize ? __fmul_rn((float)s[j][0], inv_n)
                                                      : (float)s[j][0]);
            }
            put4(row, x + ox, v, mask, cls);
        } else {
            if constexpr (std::is_same<Acc, int>::value) {
                if (!normalize && dtype == I32) {
                    const int32_t v[4] = {s[0][0], s[1][0], s[2][0], s[3][0]};
                    put4(row, x + ox, v, mask, cls);
                    return;
                }
                if (!normalize && dtype == U8) {
                    uint8_t v[4];
#pragma unroll
                    for (int j = 0; j < 4; ++j) v[j] = (uint8_t)min(max(s[j][0], 0), 255);
                    put4(row, x + ox, v, mask, cls);
                    return;
                }
            }
            float f[4];
#pragma unroll
            for (int j = 0; j < 4; ++j)
                f[j] = normalize ? __fmul_rn((float)s[j][0], inv_n) : (float)s[j][0];
            store4_float(row, x + ox, dtype, f, mask, cls);
        }
    }
};

// Output type the box kernels are compiled for, given the input type (the
// sums of u8 pixels are int32, every other type keeps its own); other
// outputs take the run-time dtype path.
template <class TIn> struct NaturalOut { using type = TIn; };
template <> struct NaturalOut<uint8_t> { using type = int32_t; };


}  // namespace box
}  // namespace tucu
