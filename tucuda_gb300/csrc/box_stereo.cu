// box_stereo.cu -- stereo cost aggregation: BoxFilter2::convolve(rowL, rowLe,
// rowR, rowO, op, disparitySearchWidth) (TU/cu/BoxFilter.h:585-746) with the
// thresholded difference op diff<T> (TU/cu/functional.h:385-398), in the
// reference's disparity-major layout (DISPARITY_MAJOR): for every disparity
// d < D,
//
//   costs[d][y][x] = sum over the wV x wH window at (y, x) of
//                    min(|L[y'][x'] - R[y'][x' + d]|, thresh)
//
// for the (rows+1-wV) x (cols+1-wH) window origins, written at (y, x).
// Right-image pixels past the last column count as 0 (the reference reads
// them from its zero-filled row padding).
//
// The reference runs a horizontal pass (box_filterH, a running sum of the
// costs) into a cost volume and a vertical pass over it (box_filterV), with
// device-wide synchronisation between them.  Here every (disparity, warp
// column, row band) is one warp task of the one-pass window-sum strip
// (box_strip.cuh): the producer forms the costs as it expands each input row,
// so no cost volume is stored, and each output element is written once.
// The right image of disparity d starts d columns to the right of the left
// one, which breaks the 4-pixel alignment the lanes' asynchronous copies
// need; each lane copies two aligned 4-pixel groups of the right row and
// shifts them by d mod 4 pixels (the same for the whole warp).  Windows
// wider than a 4-column warp tile holds (wH > 125) run 8 columns per lane,
// with 8-pixel groups shifted by d mod 8.
#include <algorithm>

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

// CTAs per SM: 8-column strips (wide windows only) hold twice the sums.
template <int CPT>
struct StereoCfg
{
    static constexpr int kCtas = CPT == 8 ? 2 : 3;
};
constexpr int kStereoWarpBytes = 6144;  // 48 KB per CTA: no opt-in needed

template <class TIn, bool VEC, int CPT>
struct StereoRing
{
    using Prod = StereoProd<TIn, typename AccOf<TIn>::type, VEC, CPT>;
    static constexpr int kDepth = Ring<Prod>::depth(kStereoWarpBytes);
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

// Warp task t: disparity t / ntask, then the image's task t mod ntask.
template <class TIn, bool VEC, int CPT>
__global__ void __launch_bounds__(kThreads, StereoCfg<CPT>::kCtas)
    stereo_kernel(const __grid_constant__ Geo G, const __grid_constant__ StereoArgs A)
{
    using Acc = typename AccOf<TIn>::type;
    using R = StereoRing<TIn, VEC, CPT>;
    char* ring = warp_ring(R::kSmem / kWarps);
    with_c<CPT>(G.wH, [&](auto cc) {
        const int tw = out_cols_per_warp(G.wH, CPT);
        const int nw = gridDim.x * kWarps;
        const long ntot = (long)G.tg.ntask * A.ndisp;
        for (long t = blockIdx.x * kWarps + (threadIdx.x >> 5); t < ntot; t += nw) {
            const int d = (int)(t / G.tg.ntask), u = (int)(t - (long)d * G.tg.ntask);
            const int b = u / G.tg.nwc, c = u - b * G.tg.nwc;
            const int y0 = b * G.tg.strip_rows;
            const typename R::Prod prod{A.left, A.lpitch, A.right, A.rpitch, A.rows, A.cols, d,
                                        Acc(A.thresh)};
            const PlainEpi<Acc, void> epi{A.costs + (size_t)d * A.slice_pitch, A.cost_pitch, A.out_dtype,
                                          0, 0, 0, 1.0f, A.cls};
            strip_body<decltype(cc)::value, 1, Acc, R::kDepth>(prod, epi, G.wV, G.wH, c * tw, y0,
                                                               min(G.tg.strip_rows, G.orows - y0),
                                                               G.ocols, ring, A.cols, G.tg.restart);
        }
    });
}

template <class TIn, int CPT>
static cudaError_t launch_stereo_c(const Geo& G, const StereoArgs& A, bool vec, long grid,
                                   cudaStream_t st)
{
    // Rings above 48 KB per CTA (8-column groups of 4-byte pixels) need the
    // opt-in.
    constexpr size_t smem = StereoRing<TIn, true, CPT>::kSmem;
    const cudaError_t e = vec ? smem_opt_in<stereo_kernel<TIn, true, CPT>>(smem)
                              : smem_opt_in<stereo_kernel<TIn, false, CPT>>(smem);
    if (e != cudaSuccess)
        return e;
    if (vec)
        stereo_kernel<TIn, true, CPT><<<(unsigned)grid, kThreads, smem, st>>>(G, A);
    else
        stereo_kernel<TIn, false, CPT><<<(unsigned)grid, kThreads, smem, st>>>(G, A);
    return cudaGetLastError();
}

template <class TIn>
static cudaError_t launch_stereo_t(const Geo& G, const StereoArgs& A, bool vec, long grid, int cpt,
                                   cudaStream_t st)
{
    return cpt == 8 ? launch_stereo_c<TIn, 8>(G, A, vec, grid, st) : launch_stereo_c<TIn, 4>(G, A, vec, grid, st);
}

cudaError_t launch_stereo(const StereoLaunch& L, cudaStream_t st)
{
    if (L.wV < 1 || L.wH < 1 || L.ndisp < 1)
        return cudaErrorInvalidValue;
    Geo G;
    G.wV = L.wV;
    G.wH = L.wH;
    G.orows = L.rows + 1 - L.wV;
    G.ocols = L.cols + 1 - L.wH;
    if (G.orows <= 0 || G.ocols <= 0)
        return cudaSuccess;
    const bool integral = L.dtype == U8 || L.dtype == I32;
    const int cpt = out_cols_per_warp(L.wH, 4) > 0 ? 4 : 8;
    const int ctas = cpt == 8 ? StereoCfg<8>::kCtas : StereoCfg<4>::kCtas;
    // Band height: the whole-rounds rule of the box filter over the warp
    // tasks of all disparities.
    G.tg = plan_tasks(G.orows, G.ocols, L.wV, L.wH, 0, ctas, integral ? 16 : kRestart, L.ndisp, cpt);
    const TaskGrid& tg = G.tg;
    StereoArgs A;
    A.left = L.left;
    A.lpitch = L.left_pitch;
    A.right = L.right;
    A.rpitch = L.right_pitch;
    A.rows = L.rows;
    A.cols = L.cols;
    A.thresh = L.thresh;
    A.ndisp = L.ndisp;
    A.costs = static_cast<char*>(L.costs);
    A.cost_pitch = L.cost_pitch;
    A.slice_pitch = L.slice_pitch;
    A.out_dtype = L.cost_dtype;
    const int es = dtype_size(L.cost_dtype);
    A.cls = L.slice_pitch % (4 * (size_t)es) == 0 ? store_class(L.costs, L.cost_pitch, 0, es) : 0;
    const bool vec = plain_vec(L.left, L.left_pitch, L.dtype, cpt) && plain_vec(L.right, L.right_pitch, L.dtype, cpt);
    const long want = ((long)tg.ntask * L.ndisp + kWarps - 1) / kWarps;
    const long grid = std::max(1L, std::min(want, (long)ctas * sm_count()));
    switch (L.dtype) {
    case U8: return launch_stereo_t<uint8_t>(G, A, vec, grid, cpt, st);
    case F16: return launch_stereo_t<__half>(G, A, vec, grid, cpt, st);
    case BF16: return launch_stereo_t<__nv_bfloat16>(G, A, vec, grid, cpt, st);
    case F32: return launch_stereo_t<float>(G, A, vec, grid, cpt, st);
    case I32: return launch_stereo_t<int32_t>(G, A, vec, grid, cpt, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace box
}  // namespace tucu
