// box_vec.cu -- box sums of vector-valued pixels: BoxFilter2 with
// box_convolver<vec<float, N>> (TU/cu/BoxFilter.h:175-194, 542-583), the
// filter SuperPixels runs over its per-pixel feature vectors
// (TU/cu/SuperPixels.h:596-597, 806-812).  Pixels are N = 2, 3 or 4
// interleaved float32 channels; each channel's window sum is the box filter's
// FP32 sum of that channel (compensated, restarted every 64 rows), so the
// result equals N separate box filters of the channel planes.
//
// One pass on the window-sum strip (box_strip.cuh) with NQ = N quantities per
// pixel: a lane's four pixels are 16N bytes, copied as N 16-byte planes; the
// epilogue writes the four pixels' N sums as one run of 4N floats.  Windows
// wider than a 4-column warp tile holds (wH > 125) run eight pixels per lane
// (2N planes), one CTA per SM.
#include <algorithm>

#include "box_kernels.h"
#include "box_plain.cuh"

namespace tucu
{
namespace box
{

template <int N, int CPT = kCPT>
struct VecProd
{
    struct Raw
    {
        float v[CPT * N];  // pixel j, channel c at v[j*N + c]
    };
    static constexpr int kCols = CPT;
    static constexpr int kPlanes = CPT * N / 4;
    static constexpr int kPlaneBytes = 16;
    static constexpr bool kAsync = true;  // rows and images 16-byte aligned (checked on the host)
    static constexpr bool kCompensate = true;
    const float* src;
    size_t pitch;
    int rows, cols;
    __device__ const void* plane_ptr(int p, int y, int x) const
    {
        return reinterpret_cast<const float*>(row_ptr(src, pitch, y)) + (size_t)x * N + 4 * p;
    }
    __device__ int plane_bytes(int p, int nvalid, int) const
    {
        return max(0, min(16, nvalid * N * 4 - 16 * p));
    }
    __device__ Raw load(int, int) const { return Raw{}; }  // never called: kAsync
    __device__ void finish(Raw&, int) const {}
    __device__ void expand(const Raw& r, int j, float (&q)[N]) const
    {
#pragma unroll
        for (int c = 0; c < N; ++c)
            q[c] = r.v[j * N + c];
    }
};

// Writes the N sums (or means) of pixels x..x+P-1 (P = 4 or 8) at
// (y + oy, x + ox).
template <int N>
struct VecEpi
{
    float* dst;
    size_t pitch;
    int oy, ox;
    int normalize;
    float inv_n;
    int aligned;  // dst rows and (x + ox) * N * 4 bytes 16-byte aligned for every x % 4 == 0
    template <int P>
    __device__ __forceinline__ void store(int y, int x, const float (&s)[P][N], unsigned mask) const
    {
        float* row = reinterpret_cast<float*>(row_ptr(dst, pitch, y + oy)) + (size_t)(x + ox) * N;
        float v[P * N];
#pragma unroll
        for (int j = 0; j < P; ++j)
#pragma unroll
            for (int c = 0; c < N; ++c)
                v[j * N + c] = normalize ? __fmul_rn(s[j][c], inv_n) : s[j][c];
        if (mask == (1u << P) - 1u && aligned) {
#pragma unroll
            for (int k = 0; k < P * N / 4; ++k)
                reinterpret_cast<float4*>(row)[k] =
                    make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
            return;
        }
#pragma unroll
        for (int j = 0; j < P; ++j)
            if ((mask >> j) & 1u)
#pragma unroll
                for (int c = 0; c < N; ++c)
                    row[j * N + c] = v[j * N + c];
    }
    __device__ void store4(int y, int x, const float (&s)[4][N], unsigned mask) const { store<4>(y, x, s, mask); }
    __device__ void store8(int y, int x, const float (&s)[8][N], unsigned mask) const { store<8>(y, x, s, mask); }
};

// CTAs per SM and ring bytes per warp (opt-in above 48 KB per CTA).
template <int CPT>
struct VecCfg
{
    static constexpr int kCtas = CPT == 8 ? 1 : 2;
    static constexpr int kWarpBytes = CPT == 8 ? 16384 : 12288;
};

template <int N, int CPT>
struct VecRing
{
    static constexpr int kDepth = Ring<VecProd<N, CPT>>::depth(VecCfg<CPT>::kWarpBytes);
    static constexpr int kSmem = kWarps * kDepth * Ring<VecProd<N, CPT>>::kStepBytes;
};

template <int N, int CPT>
__global__ void __launch_bounds__(kThreads, VecCfg<CPT>::kCtas)
    vec_box_kernel(const __grid_constant__ Geo G, const __grid_constant__ VecProd<N, CPT> prod,
                   const __grid_constant__ VecEpi<N> epi)
{
    using R = VecRing<N, CPT>;
    char* ring = warp_ring(R::kSmem / kWarps);
    for_each_task<CPT>(G, [&](auto cc, int xw, int y0, int nrows) {
        strip_body<decltype(cc)::value, N, float, R::kDepth>(prod, epi, G.wV, G.wH, xw, y0, nrows, G.ocols,
                                                              ring, prod.cols, G.tg.restart);
    });
}

template <int N, int CPT>
static cudaError_t launch_vec_c(const VecLaunch& L, cudaStream_t st)
{
    using R = VecRing<N, CPT>;
    constexpr int kCtas = VecCfg<CPT>::kCtas;
    cudaError_t e = smem_opt_in<vec_box_kernel<N, CPT>>(R::kSmem);
    if (e != cudaSuccess)
        return e;
    Geo G;
    G.wV = L.wV;
    G.wH = L.wH;
    G.orows = L.rows + 1 - L.wV;
    G.ocols = L.cols + 1 - L.wH;
    if (G.orows <= 0 || G.ocols <= 0)
        return cudaSuccess;
    G.tg = plan_tasks(G.orows, G.ocols, L.wV, L.wH, 0, kCtas, kRestart, 1, CPT);
    const VecProd<N, CPT> prod{static_cast<const float*>(L.src), L.src_pitch, L.rows, L.cols};
    const uintptr_t d0 = reinterpret_cast<uintptr_t>(L.dst) + (uintptr_t)L.ox * N * 4;
    const VecEpi<N> epi{static_cast<float*>(L.dst), L.dst_pitch, L.oy, L.ox, L.normalize,
                        1.0f / (float)(L.wV * L.wH), d0 % 16 == 0 && L.dst_pitch % 16 == 0};
    const long want = (G.tg.ntask + kWarps - 1) / kWarps;
    const dim3 grid((unsigned)std::max(1L, std::min(want, (long)kCtas * sm_count())));
    vec_box_kernel<N, CPT><<<grid, kThreads, R::kSmem, st>>>(G, prod, epi);
    return cudaGetLastError();
}

template <int N>
static cudaError_t launch_vec_n(const VecLaunch& L, cudaStream_t st)
{
    return out_cols_per_warp(L.wH, 4) > 0 ? launch_vec_c<N, 4>(L, st) : launch_vec_c<N, 8>(L, st);
}

cudaError_t launch_vec(const VecLaunch& L, cudaStream_t st)
{
    if (reinterpret_cast<uintptr_t>(L.src) % 16 != 0 || L.src_pitch % 16 != 0)
        return cudaErrorInvalidValue;
    switch (L.channels) {
    case 2: return launch_vec_n<2>(L, st);
    case 3: return launch_vec_n<3>(L, st);
    case 4: return launch_vec_n<4>(L, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace box
}  // namespace tucu
