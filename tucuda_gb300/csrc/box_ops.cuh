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

// N consecutive pixels of one row as raw bits (zero outside the image): one
// word of 4, 8 or 16 bytes, or several 16-byte words.
template <class TIn, int N>
struct RawN
{
    static constexpr int kBytes = N * (int)sizeof(TIn);
    static constexpr int kWords = kBytes > 16 ? kBytes / 16 : 1;
    using W = std::conditional_t<kBytes == 4, uint32_t, std::conditional_t<kBytes == 8, uint2, uint4>>;
    W v[kWords];
};
template <class TIn> using Raw4 = RawN<TIn, 4>;

// Columns x..x+N-1 of row y, checked against the image (VEC: row + x is
// aligned to the raw words).
template <class TIn, bool VEC, int N = kCPT>
__device__ __forceinline__ RawN<TIn, N> load_raw(const void* base, size_t pitch, int rows, int cols,
                                                 int y, int x)
{
    using R = RawN<TIn, N>;
    R r;
    memset(&r, 0, sizeof(r));
    if (y < 0 || y >= rows || x >= cols)
        return r;
    const TIn* row = reinterpret_cast<const TIn*>(row_ptr(base, pitch, y));
    if (VEC && x + N <= cols) {
#pragma unroll
        for (int k = 0; k < R::kWords; ++k)
            r.v[k] = __ldg(reinterpret_cast<const typename R::W*>(row + x) + k);
        return r;
    }
    TIn* e = reinterpret_cast<TIn*>(r.v);
#pragma unroll
    for (int j = 0; j < N; ++j)
        if (x + j < cols)
            e[j] = row[x + j];
    return r;
}
template <class TIn, bool VEC>
__device__ __forceinline__ Raw4<TIn> load_raw4(const void* base, size_t pitch, int rows, int cols,
                                              int y, int x)
{
    return load_raw<TIn, VEC, 4>(base, pitch, rows, cols, y, x);
}

template <class TIn, class Acc, int N>
__device__ __forceinline__ Acc raw_elem(const RawN<TIn, N>& r, int j)
{
    const TIn* e = reinterpret_cast<const TIn*>(r.v);
    if constexpr (std::is_same<TIn, uint8_t>::value)
        return Acc((reinterpret_cast<const uint32_t*>(r.v)[j >> 2] >> (8 * (j & 3))) & 0xffu);
    else if constexpr (std::is_same<TIn, int32_t>::value)
        return Acc(e[j]);
    else
        return Acc(to_float(e[j]));
}

// ---- producers ----------------------------------------------------------------

// CPT columns per lane: one plane of CPT pixels, or 16-byte planes where the
// pixels of a lane span more than 16 bytes (FP32 and int32 at 8 columns).
template <class TIn, class Acc, bool VEC, int CPT = kCPT>
struct PlainProd
{
    using Raw = RawN<TIn, CPT>;
    static constexpr int kCols = CPT;
    static constexpr int kPlaneBytes = CPT * (int)sizeof(TIn) > 16 ? 16 : CPT * (int)sizeof(TIn);
    static constexpr int kPlanes = CPT * (int)sizeof(TIn) / kPlaneBytes;
    static constexpr bool kAsync = VEC;
    // FP32 input keeps compensated sums; narrower pixels sum exactly enough.
    static constexpr bool kCompensate = std::is_same<TIn, float>::value;
    const void* src;
    size_t pitch;
    int rows, cols;
    __device__ const void* plane_ptr(int p, int y, int x) const
    {
        return row_ptr(src, pitch, y) + (size_t)x * sizeof(TIn) + p * kPlaneBytes;
    }
    __device__ int plane_bytes(int p, int nvalid, int) const
    {
        return min(max(nvalid * (int)sizeof(TIn) - p * kPlaneBytes, 0), kPlaneBytes);
    }
    __device__ Raw load(int y, int x) const { return load_raw<TIn, VEC, CPT>(src, pitch, rows, cols, y, x); }
    __device__ void finish(Raw&, int) const {}
    __device__ void expand(const Raw& r, int j, Acc (&q)[1]) const { q[0] = raw_elem<TIn, Acc>(r, j); }
};

// ---- stores -------------------------------------------------------------------

// Alignment of four consecutive output elements starting at column x + ox of
// any row (x a multiple of 4), computed on the host: 4 = one vector store
// (8 = also eight elements at x a multiple of 8), 2 = two aligned pairs, 1 =
// element, pair, element (odd start), 0 = look at each address.
inline int store_class(const void* dst, size_t pitch, int ox, int es)
{
    const uintptr_t a = reinterpret_cast<uintptr_t>(dst) + (uintptr_t)ox * es;
    if (a % es != 0)
        return 0;
    if (pitch % (8 * (size_t)es) == 0 && a % (8 * es) == 0)
        return 8;
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
// aligned pairs, or element, pair, element (cls from store_class, 8 counts
// as 4; 0 = look at the address).  Words are assembled from the values' bits, so nothing
// goes through local memory.
template <class T>
__device__ __forceinline__ void put4p(T* p, const T (&v)[4], unsigned mask, int cls)
{
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
        if (cls >= 4) {
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
        if (cls >= 4) {
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
        if (cls >= 4) {
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

template <class T>
__device__ __forceinline__ void put4(char* row, int x, const T (&v)[4], unsigned mask, int cls)
{
    put4p(reinterpret_cast<T*>(row) + x, v, mask, cls);
}

// Writes 8 values at row + x*es (x a multiple of 8): one 8- or 16-byte
// store for 1- and 2-byte values at cls 8, else two groups of four.
template <class T>
__device__ __forceinline__ void put8(char* row, int x, const T (&v)[8], unsigned mask, int cls)
{
    if constexpr (sizeof(T) <= 2) {
        if (mask == 0xffu && cls == 8) {
            uint32_t b[8];
#pragma unroll
            for (int j = 0; j < 8; ++j)
                b[j] = bits_of(v[j]);
            T* p = reinterpret_cast<T*>(row) + x;
            if constexpr (sizeof(T) == 1)
                *reinterpret_cast<uint2*>(p) = make_uint2(b[0] | b[1] << 8 | b[2] << 16 | b[3] << 24,
                                                          b[4] | b[5] << 8 | b[6] << 16 | b[7] << 24);
            else
                *reinterpret_cast<uint4*>(p) = make_uint4(b[0] | b[1] << 16, b[2] | b[3] << 16,
                                                          b[4] | b[5] << 16, b[6] | b[7] << 16);
            return;
        }
    }
    const T lo[4] = {v[0], v[1], v[2], v[3]}, hi[4] = {v[4], v[5], v[6], v[7]};
    if (mask & 0xfu)
        put4(row, x, lo, mask & 0xfu, cls);
    if (mask >> 4)
        put4(row, x + 4, hi, mask >> 4, cls);
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

    // A float sum times scale(): inv_n for means, exactly itself otherwise.
    __device__ __forceinline__ float scale() const { return normalize ? inv_n : 1.0f; }

    // One window sum in the compiled output type.
    template <class T = TOut>
    __device__ __forceinline__ T out_of(Acc s) const
    {
        if constexpr (std::is_same<Acc, int>::value && std::is_same<T, int32_t>::value)
            return normalize ? __float2int_rz(__fmul_rn((float)s, inv_n)) : s;
        else if constexpr (std::is_same<Acc, int>::value && std::is_same<T, uint8_t>::value)
            return normalize ? f2u8(__fmul_rn((float)s, inv_n)) : sum2u8(s);
        else
            return from_float<T>(__fmul_rn((float)s, scale()));
    }
    // Four window sums in the output dtype read at run time.
    __device__ __forceinline__ void store4_rt(char* row, int x, const Acc (&s)[4], unsigned mask) const
    {
        if constexpr (std::is_same<Acc, int>::value) {
            if (!normalize && dtype == I32) {
                const int32_t v[4] = {s[0], s[1], s[2], s[3]};
                put4(row, x, v, mask, cls);
                return;
            }
            if (!normalize && dtype == U8) {
                uint8_t v[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) v[j] = sum2u8(s[j]);
                put4(row, x, v, mask, cls);
                return;
            }
        }
        float f[4];
#pragma unroll
        for (int j = 0; j < 4; ++j)
            f[j] = __fmul_rn((float)s[j], scale());
        store4_float(row, x, dtype, f, mask, cls);
    }
    // Four sums at p (compiled output type).
    __device__ __forceinline__ void put_typed4(TOut* p, const Acc (&s)[4][1], unsigned mask) const
    {
        if constexpr (std::is_same<Acc, float>::value &&
                      (std::is_same<TOut, __half>::value || std::is_same<TOut, __nv_bfloat16>::value)) {
            // FP32 sums to f16 / bf16 in packed pairs: the same roundings as
            // out_of (multiply by the scale, then round to nearest even).
            const float k = scale();
            const float2 a = __fmul2_rn(make_float2(s[0][0], s[1][0]), make_float2(k, k));
            const float2 b = __fmul2_rn(make_float2(s[2][0], s[3][0]), make_float2(k, k));
            uint32_t w0, w1;
            if constexpr (std::is_same<TOut, __half>::value) {
                const __half2 h0 = __float22half2_rn(a), h1 = __float22half2_rn(b);
                memcpy(&w0, &h0, 4);
                memcpy(&w1, &h1, 4);
            } else {
                const __nv_bfloat162 h0 = __float22bfloat162_rn(a), h1 = __float22bfloat162_rn(b);
                memcpy(&w0, &h0, 4);
                memcpy(&w1, &h1, 4);
            }
            if (mask == 0xfu && cls >= 4) {
                *reinterpret_cast<uint2*>(p) = make_uint2(w0, w1);
                return;
            }
            TOut v[4];
            const uint16_t u[4] = {(uint16_t)w0, (uint16_t)(w0 >> 16), (uint16_t)w1, (uint16_t)(w1 >> 16)};
            memcpy(v, u, 8);
            put4p(p, v, mask, cls);
        } else {
            TOut v[4];
#pragma unroll
            for (int j = 0; j < 4; ++j)
                v[j] = out_of(s[j][0]);
            put4p(p, v, mask, cls);
        }
    }
    __device__ void store4(int y, int x, const Acc (&s)[4][1], unsigned mask) const
    {
        char* row = row_ptr(dst, pitch, y + oy);
        if constexpr (!std::is_void<TOut>::value) {
            put_typed4(reinterpret_cast<TOut*>(row) + x + ox, s, mask);
        } else {
            const Acc a[4] = {s[0][0], s[1][0], s[2][0], s[3][0]};
            store4_rt(row, x + ox, a, mask);
        }
    }
    __device__ void store8(int y, int x, const Acc (&s)[8][1], unsigned mask) const
    {
        char* row = row_ptr(dst, pitch, y + oy);
        if constexpr (!std::is_void<TOut>::value) {
            TOut v[8];
#pragma unroll
            for (int j = 0; j < 8; ++j)
                v[j] = out_of(s[j][0]);
            put8(row, x + ox, v, mask, cls);
        } else {
            const Acc a[4] = {s[0][0], s[1][0], s[2][0], s[3][0]}, b[4] = {s[4][0], s[5][0], s[6][0], s[7][0]};
            if (mask & 0xfu)
                store4_rt(row, x + ox, a, mask & 0xfu);
            if (mask >> 4)
                store4_rt(row, x + ox + 4, b, mask >> 4);
        }
    }

    // Row cursor of the compiled-type 4-column stores: output (y, x) of the
    // first row a strip block writes, then one pitch further per row.
    struct Cursor
    {
        char* p;
        size_t pitch;
        __device__ __forceinline__ void next() { p += pitch; }
    };
    template <class T = TOut, class = std::enable_if_t<!std::is_void<T>::value>>
    __device__ Cursor cursor(int y, int x) const
    {
        return Cursor{row_ptr(dst, pitch, y + oy) + (size_t)(x + ox) * sizeof(T), pitch};
    }
    template <class T = TOut, class = std::enable_if_t<!std::is_void<T>::value>>
    __device__ void store4(const Cursor& c, const Acc (&s)[4][1], unsigned mask) const
    {
        put_typed4(reinterpret_cast<TOut*>(c.p), s, mask);
    }
};

// Output type the box kernels are compiled for, given the input type (the
// sums of u8 pixels are int32, every other type keeps its own); other
// outputs take the run-time dtype path.
template <class TIn> struct NaturalOut { using type = TIn; };
template <> struct NaturalOut<uint8_t> { using type = int32_t; };


}  // namespace box
}  // namespace tucu
