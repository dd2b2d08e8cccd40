// stereo.cuh -- the stereo cost kernel on the window-sum strip: producer,
// ring and kernel templates, instantiated for 4 columns per lane in
// box_stereo.cu and for 8 (windows wider than 125 columns) in
// box_stereo_wide.cu.
#pragma once
#include "box_kernels.h"
#include "box_plain.cuh"

namespace tucu
{
namespace box
{

// 4 pixels starting `sh` pixels into the 8 pixels (a, b).
__device__ __forceinline__ uint32_t shift4(uint32_t a, uint32_t b, int sh)
{
    return __funnelshift_r(a, b, 8 * sh);
}
__device__ __forceinline__ uint2 shift4(uint2 a, uint2 b, int sh)
{
    const bool w = sh >= 2;
    const uint32_t w0 = w ? a.y : a.x, w1 = w ? b.x : a.y, w2 = w ? b.y : b.x;
    const int bo = 16 * (sh & 1);
    return make_uint2(__funnelshift_r(w0, w1, bo), __funnelshift_r(w1, w2, bo));
}
__device__ __forceinline__ uint4 shift4(uint4 a, uint4 b, int sh)
{
    switch (sh) {
    case 0: return a;
    case 1: return make_uint4(a.y, a.z, a.w, b.x);
    case 2: return make_uint4(a.z, a.w, b.x, b.y);
    default: return make_uint4(a.w, b.x, b.y, b.z);
    }
}

// 8 pixels starting `sh` pixels into the 16 pixels (a, b), as 32-bit words:
// word i of the result is bits [bits, bits+32) of words ws+i, ws+i+1 of
// (a, b), with ws = sh*es/4 < K and bits = 8*(sh*es mod 4).
template <class TIn>
__device__ __forceinline__ RawN<TIn, 8> shift8(const RawN<TIn, 8>& a, const RawN<TIn, 8>& b, int sh)
{
    constexpr int K = 8 * (int)sizeof(TIn) / 4;  // words per group
    uint32_t w[2 * K];
    memcpy(w, a.v, 4 * K);
    memcpy(w + K, b.v, 4 * K);
    const int ws = sh * (int)sizeof(TIn) / 4, bits = 8 * (sh * (int)sizeof(TIn) % 4);
    uint32_t o[K];
#pragma unroll
    for (int s = 0; s < K; ++s)
        if (ws == s) {
#pragma unroll
            for (int i = 0; i < K; ++i)
                o[i] = __funnelshift_r(w[s + i], w[s + i + 1], bits);
        }
    RawN<TIn, 8> r;
    memcpy(r.v, o, 4 * K);
    return r;
}

// Producer: planes left (x..x+CPT-1), right aligned group (xa..xa+CPT-1) and
// the next one, xa = (x + d) rounded down to a multiple of CPT; 16-byte
// planes where a group spans more (FP32 and int32 at 8 columns).
template <class TIn, class Acc, bool VEC, int CPT = kCPT>
struct StereoProd
{
    struct Raw
    {
        RawN<TIn, CPT> l, ra, rb;
    };
    static constexpr int kCols = CPT;
    static constexpr int kPlaneBytes = CPT * (int)sizeof(TIn) > 16 ? 16 : CPT * (int)sizeof(TIn);
    static constexpr int kPerGroup = CPT * (int)sizeof(TIn) / kPlaneBytes;
    static constexpr int kPlanes = 3 * kPerGroup;
    static constexpr bool kAsync = VEC;
    static constexpr bool kCompensate = std::is_same<TIn, float>::value;
    const void* left;
    size_t lpitch;
    const void* right;
    size_t rpitch;
    int rows, cols, d;
    Acc thresh;

    // First column of group g (0 left, 1 right aligned, 2 the next one).
    __device__ int ralign(int x, int g) const { return ((x + d) & ~(CPT - 1)) + (g == 2 ? CPT : 0); }
    __device__ const void* plane_ptr(int p, int y, int x) const
    {
        const int g = p / kPerGroup, off = (p % kPerGroup) * kPlaneBytes;
        if (g == 0)
            return row_ptr(left, lpitch, y) + (size_t)x * sizeof(TIn) + off;
        const int xa = ralign(x, g);
        // a group wholly past the row reads nothing: any valid address
        return row_ptr(right, rpitch, y) + (size_t)(xa < cols ? xa : 0) * sizeof(TIn) + (xa < cols ? off : 0);
    }
    __device__ int plane_bytes(int p, int nvalid, int x) const
    {
        const int g = p / kPerGroup, off = (p % kPerGroup) * kPlaneBytes;
        const int n = g == 0 || nvalid == 0 ? nvalid : max(0, min(CPT, cols - ralign(x, g)));
        return min(max(n * (int)sizeof(TIn) - off, 0), kPlaneBytes);
    }
    __device__ Raw load(int y, int x) const
    {
        Raw r;
        r.l = load_raw<TIn, false, CPT>(left, lpitch, rows, cols, y, x);
        const int xa = ralign(x, 1);
        r.ra = load_raw<TIn, false, CPT>(right, rpitch, rows, cols, y, xa);
        r.rb = load_raw<TIn, false, CPT>(right, rpitch, rows, cols, y, xa + CPT);
        return r;
    }
    __device__ void finish(Raw& r, int) const
    {
        if constexpr (CPT == 4)
            r.ra.v[0] = shift4(r.ra.v[0], r.rb.v[0], d & 3);
        else
            r.ra = shift8(r.ra, r.rb, d & 7);
    }
    __device__ void expand(const Raw& r, int j, Acc (&q)[1]) const
    {
        const Acc a = raw_elem<TIn, Acc>(r.l, j), b = raw_elem<TIn, Acc>(r.ra, j);
        const Acc c = a > b ? a - b : b - a;
        q[0] = c < thresh ? c : thresh;
    }
};

// 8 pixels starting `sh` (< 4) pixels into the 12 pixels of three aligned
// 4-pixel groups (a, b, c), as 32-bit words: word i of the result is bits
// [bits, bits+32) of words ws+i, ws+i+1, with ws = sh*es/4 and
// bits = 8*(sh*es mod 4).
template <class TIn>
__device__ __forceinline__ RawN<TIn, 8> window8(const RawN<TIn, 4>& a, const RawN<TIn, 4>& b,
                                                const RawN<TIn, 4>& c, int sh)
{
    constexpr int G = (int)sizeof(TIn);  // words per 4-pixel group
    uint32_t w[3 * G];
    memcpy(w, a.v, 4 * G);
    memcpy(w + G, b.v, 4 * G);
    memcpy(w + 2 * G, c.v, 4 * G);
    const int ws = sh * (int)sizeof(TIn) / 4, bits = 8 * (sh * (int)sizeof(TIn) % 4);
    uint32_t o[2 * G];
#pragma unroll
    for (int s = 0; s < G; ++s)
        if (ws == s) {
#pragma unroll
            for (int i = 0; i < 2 * G; ++i)
                o[i] = __funnelshift_r(w[s + i], w[s + i + 1], bits);
        }
    RawN<TIn, 8> r;
    memcpy(r.v, o, 8 * G);
    return r;
}

// Producer of K consecutive disparities d0..d0+K-1 at once (K summed
// quantities per pixel, 1- and 2-byte input, 4 columns per lane): planes
// left (x..x+3) and the three aligned right groups from xa = (x + d0)
// rounded down to a multiple of 4; finish() cuts the right pixels x+d0 ..
// x+d0+7 out of them, and quantity k of column j is the cost of right pixel
// j + k.  Each disparity's sums are those of the one-disparity producer.
template <class TIn, class Acc, bool VEC, int K>
struct StereoProdK
{
    static_assert(sizeof(TIn) <= 2 && K >= 1 && K <= 4, "1- and 2-byte input, up to 4 disparities");
    struct Raw
    {
        RawN<TIn, 4> l, r0, r1, r2;  // the planes copied through the ring
        RawN<TIn, 8> w;              // right pixels x+d0 .. x+d0+7
    };
    static constexpr int kPlanes = 4;
    static constexpr int kPlaneBytes = 4 * (int)sizeof(TIn);
    static constexpr bool kAsync = VEC;
    static constexpr bool kCompensate = false;
    const void* left;
    size_t lpitch;
    const void* right;
    size_t rpitch;
    int rows, cols, d;  // d: the group's first disparity d0
    Acc thresh;

    // First column of right group g (1..3).
    __device__ int ralign(int x, int g) const { return ((x + d) & ~3) + 4 * (g - 1); }
    __device__ const void* plane_ptr(int p, int y, int x) const
    {
        if (p == 0)
            return row_ptr(left, lpitch, y) + (size_t)x * sizeof(TIn);
        const int xa = ralign(x, p);
        // a group wholly past the row reads nothing: any valid address
        return row_ptr(right, rpitch, y) + (size_t)(xa < cols ? xa : 0) * sizeof(TIn);
    }
    __device__ int plane_bytes(int p, int nvalid, int x) const
    {
        if (p == 0 || nvalid == 0)
            return nvalid * (int)sizeof(TIn);
        return max(0, min(4, cols - ralign(x, p))) * (int)sizeof(TIn);
    }
    __device__ Raw load(int y, int x) const
    {
        Raw r;
        r.l = load_raw<TIn, false, 4>(left, lpitch, rows, cols, y, x);
        const int xa = ralign(x, 1);
        r.r0 = load_raw<TIn, false, 4>(right, rpitch, rows, cols, y, xa);
        r.r1 = load_raw<TIn, false, 4>(right, rpitch, rows, cols, y, xa + 4);
        r.r2 = load_raw<TIn, false, 4>(right, rpitch, rows, cols, y, xa + 8);
        return r;
    }
    __device__ void finish(Raw& r, int) const { r.w = window8(r.r0, r.r1, r.r2, d & 3); }
    __device__ void expand(const Raw& r, int j, Acc (&q)[K]) const
    {
        const Acc a = raw_elem<TIn, Acc>(r.l, j);
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const Acc b = raw_elem<TIn, Acc>(r.w, j + k);
            const Acc c = a > b ? a - b : b - a;
            q[k] = c < thresh ? c : thresh;
        }
    }
};

// Cost type: int32 for integer images, float32 for float ones (the only
// pairs the launcher accepts), so the stores are compiled for it.
template <class Acc>
using CostOf = std::conditional_t<std::is_same<Acc, int>::value, int32_t, float>;

// Stores the K cost slices of a disparity group (the first nk of them: the
// last group may be short).
template <class Acc, int K>
struct StereoEpiK
{
    char* costs;  // slice of the group's first disparity
    size_t pitch, slice;
    int dtype, cls, nk;
    __device__ void store4(int y, int x, const Acc (&s)[4][K], unsigned mask) const
    {
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (k < nk) {
                const PlainEpi<Acc, CostOf<Acc>> e{costs + (size_t)k * slice, pitch, dtype, 0, 0, 0, 1.0f, cls};
                const Acc a[4][1] = {{s[0][k]}, {s[1][k]}, {s[2][k]}, {s[3][k]}};
                e.store4(y, x, a, mask);
            }
    }
};

// Disparities per warp task: groups of 4 for 1- and 2-byte input (4 columns
// per lane), one otherwise.
template <class TIn, int CPT>
struct StereoGroup
{
    static constexpr int K = (sizeof(TIn) <= 2 && CPT == kCPT) ? 4 : 1;
};

// CTAs per SM: disparity groups (4 x 4 running sums, 128 registers) and
// 8-column strips (wide windows only) run two, single disparities three.
template <class TIn, int CPT>
struct StereoCfg
{
    static constexpr int kCtas = (StereoGroup<TIn, CPT>::K > 1 || CPT == 8) ? 2 : 3;
};
constexpr int kStereoWarpBytes = 6144;  // 48 KB per CTA: no opt-in needed

template <class TIn, bool VEC, int CPT>
struct StereoRing
{
    static constexpr int K = StereoGroup<TIn, CPT>::K;
    using Acc = typename AccOf<TIn>::type;
    using Prod = std::conditional_t<(K > 1), StereoProdK<TIn, Acc, VEC, K>, StereoProd<TIn, Acc, VEC, CPT>>;
    // Grouped disparities copy four planes per row: a deeper budget keeps the
    // same rows in flight.
    static constexpr int kDepth = Ring<Prod>::depth(K > 1 ? 2 * kStereoWarpBytes : kStereoWarpBytes);
    static constexpr int kSmem = kWarps * kDepth * Ring<Prod>::kStepBytes;
};

struct StereoArgs
{
    const void* left;
    size_t lpitch;
    const void* right;
    size_t rpitch;
    int rows, cols;
    float thresh;
    int ndisp;
    char* costs;
    size_t cost_pitch, slice_pitch;
    int out_dtype;
    int cls;
};

// Warp task t: disparity group t / ntask (K disparities from K * group),
// then the image's task t mod ntask.
template <class TIn, bool VEC, int CPT>
__global__ void __launch_bounds__(kThreads, StereoCfg<TIn, CPT>::kCtas)
    stereo_kernel(const __grid_constant__ Geo G, const __grid_constant__ StereoArgs A)
{
    using Acc = typename AccOf<TIn>::type;
    using R = StereoRing<TIn, VEC, CPT>;
    constexpr int K = R::K;
    char* ring = warp_ring(R::kSmem / kWarps);
    with_c<CPT>(G.wH, [&](auto cc) {
        const int tw = out_cols_per_warp(G.wH, CPT);
        const int nw = gridDim.x * kWarps;
        const int ngroups = (A.ndisp + K - 1) / K;
        const long ntot = (long)G.tg.ntask * ngroups;
        for (long t = blockIdx.x * kWarps + (threadIdx.x >> 5); t < ntot; t += nw) {
            const int g = (int)(t / G.tg.ntask), u = (int)(t - (long)g * G.tg.ntask);
            const int b = u / G.tg.nwc, c = u - b * G.tg.nwc;
            const int y0 = b * G.tg.strip_rows, d = g * K;
            const typename R::Prod prod{A.left, A.lpitch, A.right, A.rpitch, A.rows, A.cols, d,
                                        Acc(A.thresh)};
            char* const slice = A.costs + (size_t)d * A.slice_pitch;
            if constexpr (K > 1) {
                const StereoEpiK<Acc, K> epi{slice, A.cost_pitch, A.slice_pitch, A.out_dtype, A.cls,
                                             min(K, A.ndisp - d)};
                strip_body<decltype(cc)::value, K, Acc, R::kDepth>(prod, epi, G.wV, G.wH, c * tw, y0,
                                                                   min(G.tg.strip_rows, G.orows - y0),
                                                                   G.ocols, ring, A.cols, G.tg.restart);
            } else {
                const PlainEpi<Acc, CostOf<Acc>> epi{slice, A.cost_pitch, A.out_dtype, 0, 0, 0, 1.0f, A.cls};
                strip_body<decltype(cc)::value, 1, Acc, R::kDepth>(prod, epi, G.wV, G.wH, c * tw, y0,
                                                                   min(G.tg.strip_rows, G.orows - y0),
                                                                   G.ocols, ring, A.cols, G.tg.restart);
            }
        }
    });
}

template <class TIn, int CPT>
cudaError_t launch_stereo_c(const Geo& G, const StereoArgs& A, bool vec, long grid,
                                   cudaStream_t st)
{
    // Rings above 48 KB per CTA (8-column groups of 4-byte pixels) need the
    // opt-in.
    constexpr size_t smem = StereoRing<TIn, true, CPT>::kSmem;
    // Wide windows (8 columns per lane) run the synchronous loads only.
    if constexpr (CPT == kCPT) {
        if (vec) {
            const cudaError_t e = smem_opt_in<stereo_kernel<TIn, true, CPT>>(smem);
            if (e != cudaSuccess)
                return e;
            stereo_kernel<TIn, true, CPT><<<(unsigned)grid, kThreads, smem, st>>>(G, A);
            return cudaGetLastError();
        }
    }
    const cudaError_t e = smem_opt_in<stereo_kernel<TIn, false, CPT>>(smem);
    if (e != cudaSuccess)
        return e;
    stereo_kernel<TIn, false, CPT><<<(unsigned)grid, kThreads, smem, st>>>(G, A);
    return cudaGetLastError();
}

// Disparities per warp task and CTAs per SM for an input type (StereoGroup,
// StereoCfg).
inline int stereo_group(int dtype, int cpt)
{
    return cpt == kCPT && dtype_size(dtype) <= 2 ? 4 : 1;
}
inline int stereo_ctas(int dtype, int cpt)
{
    return stereo_group(dtype, cpt) > 1 || cpt == 8 ? 2 : 3;
}

template <int CPT>
cudaError_t launch_stereo_cpt(const Geo& G, const StereoArgs& A, int dtype, bool vec, long grid,
                              cudaStream_t st)
{
    switch (dtype) {
    case U8: return launch_stereo_c<uint8_t, CPT>(G, A, vec, grid, st);
    case F16: return launch_stereo_c<__half, CPT>(G, A, vec, grid, st);
    case BF16: return launch_stereo_c<__nv_bfloat16, CPT>(G, A, vec, grid, st);
    case F32: return launch_stereo_c<float, CPT>(G, A, vec, grid, st);
    case I32: return launch_stereo_c<int32_t, CPT>(G, A, vec, grid, st);
    default: return cudaErrorInvalidValue;
    }
}
// The 8-column instantiations (box_stereo_wide.cu).
cudaError_t launch_stereo_wide(const Geo& G, const StereoArgs& A, int dtype, bool vec, long grid,
                               cudaStream_t st);

}  // namespace box
}  // namespace tucu
