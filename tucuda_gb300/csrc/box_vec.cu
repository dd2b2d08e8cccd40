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
// epilogue writes the four pixels' N sums as one run of 4N floats.
#include <algorithm>

#include "box_kernels.h"
#include "box_plain.cuh"

namespace tucu
{
namespace box
{

template <int N>
struct VecProd
{
    struct Raw
    {
        float v[4 * N];  // pixel j, channel c at v[j*N + c]
    };
    static constexpr int kPlanes = N;
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

// Writes the N sums (or means) of pixels x..x+3 at (y + oy, x + ox).
template <int N>
struct VecEpi
{
    float* dst;
    size_t pitch;
    int oy, ox;
    int normalize;
    float inv_n;
    int aligned;  // dst rows and (x + ox) * N * 4 bytes 16-byte aligned for every x % 4 == 0
    __device__ void store4(int y, int x, const float (&s)[4][N], unsigned mask) const
    {
        float* row = reinterpret_cast<float*>(row_ptr(dst, pitch, y + oy)) + (size_t)(x + ox) * N;
        float v[4 * N];
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int c = 0; c < N; ++c)
                v[j * N + c] = normalize ? __fmul_rn(s[j][c], inv_n) : s[j][c];
        if (mask == 0xfu && aligned) {
#pragma unroll
            for (int k = 0; k < N; ++k)
                reinterpret_cast<float4*>(row)[k] =
                    make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
            return;
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if ((mask >> j) & 1u)
#pragma unroll
                for (int c = 0; c < N; ++c)
                    row[j * N + c] = v[j * N + c];
    }
};

constexpr int kVecCtas = 2;
constexpr int kVecWarpBytes = 12288;  // 96 KB per CTA (opt-in)

template <int N>
struct VecRing
{
    static constexpr int kDepth = Ring<VecProd<N>>::depth(kVecWarpBytes);
    static constexpr int kSmem = kWarps * kDepth * Ring<VecProd<N>>::kStepBytes;
};

template <int N>
__global__ void __launch_bounds__(kThreads, kVecCtas)
    vec_box_kernel(const __grid_constant__ Geo G, const __grid_constant__ VecProd<N> prod,
                   const __grid_constant__ VecEpi<N> epi)
{
    char* ring = warp_ring(VecRing<N>::kSmem / kWarps);
    for_each_task(G, [&](auto cc, int xw, int y0, int nrows) {
        strip_body<decltype(cc)::value, N, float, VecRing<N>::kDepth>(prod, epi, G.wV, G.wH, xw, y0,
                                                                       nrows, G.ocols, ring, prod.cols,
                                                                       G.tg.restart);
    });
}

template <int N>
static cudaError_t launch_vec_n(const VecLaunch& L, cudaStream_t st)
{
    auto kern = vec_box_kernel<N>;
    static DeviceOnce attr_once;
    cudaError_t e = attr_once.run([&] {
        return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, VecRing<N>::kSmem);
    });
    if (e != cudaSuccess)
        return e;
    Geo G;
    G.wV = L.wV;
    G.wH = L.wH;
    G.orows = L.rows + 1 - L.wV;
    G.ocols = L.cols + 1 - L.wH;
    if (G.orows <= 0 || G.ocols <= 0)
        return cudaSuccess;
    G.tg = plan_tasks(G.orows, G.ocols, L.wV, L.wH, 0, kVecCtas, kRestart);
    const VecProd<N> prod{static_cast<const float*>(L.src), L.src_pitch, L.rows, L.cols};
    const uintptr_t d0 = reinterpret_cast<uintptr_t>(L.dst) + (uintptr_t)L.ox * N * 4;
    const VecEpi<N> epi{static_cast<float*>(L.dst), L.dst_pitch, L.oy, L.ox, L.normalize,
                        1.0f / (float)(L.wV * L.wH), d0 % 16 == 0 && L.dst_pitch % 16 == 0};
    const long want = (G.tg.ntask + kWarps - 1) / kWarps;
    const dim3 grid((unsigned)std::max(1L, std::min(want, (long)kVecCtas * sm_count())));
    kern<<<grid, kThreads, VecRing<N>::kSmem, st>>>(G, prod, epi);
    return cudaGetLastError();
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
