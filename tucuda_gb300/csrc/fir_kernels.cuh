// fir_kernels.cuh -- the single-job FIR strip kernel and its launcher,
// instantiated once per input type by fir_<type>.cu (split so the
// instantiations compile in parallel).
#pragma once
#include "fir_strip.cuh"
#include "tucu_internal.h"

namespace tucu
{
namespace fir
{

struct KParams
{
    FirJob job;
    LobeSet lobes;
    int strip_rows;  // output rows per CTA (multiple of CH)
    int use_tma;
};

template <int RH, int RV, int NH, int CH, class TIn>
__global__ void __launch_bounds__(kThreads)
    fir_strip_kernel(const __grid_constant__ KParams P, const __grid_constant__ CUtensorMap tmap)
{
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
    if (P.use_tma && threadIdx.x == 0) {
        tma_prefetch_desc(&tmap);
        for (int s = 0; s < StripCfg<RH, RV, NH, CH, TIn>::NSTAGE; ++s)
            mbar_init(&bars[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    const int x0 = blockIdx.x * kTW;
    const int y0 = blockIdx.y * P.strip_rows;
    const int nrows = min(P.strip_rows, P.job.orows - y0);
    if (nrows <= 0)
        return;
    Pipe pipe{0};
    run_strip<RH, RV, NH, CH, TIn>(P.job, P.lobes, P.use_tma ? &tmap : nullptr, x0, y0,
                                   (nrows + CH - 1) / CH, smem, pipe);
}

template <int RH, int RV, int NH, int CH, class TIn>
static cudaError_t launch_cfg(const FirLaunch& L, cudaStream_t stream)
{
    using Cfg = StripCfg<RH, RV, NH, CH, TIn>;
    auto kern = fir_strip_kernel<RH, RV, NH, CH, TIn>;
    static DeviceOnce attr_once;  // one attribute call per device
    cudaError_t e = attr_once.run([&] {
        return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)Cfg::SMEM);
    });
    if (e != cudaSuccess)
        return e;
    KParams P;
    P.job = L.job;
    P.lobes = L.lobes;
    P.use_tma = L.use_tma;
    int strip = L.strip_rows > 0 ? L.strip_rows : CH * 4;
    strip = (strip + CH - 1) / CH * CH;
    P.strip_rows = strip;
    const dim3 grid((L.job.ocols + kTW - 1) / kTW, (L.job.orows + strip - 1) / strip);
    kern<<<grid, kThreads, Cfg::SMEM, stream>>>(P, L.tmap);
    return cudaGetLastError();
}

// Dispatch on (RH, RV) for one input type.
template <int NH, int CH, class TIn>
static cudaError_t launch_for_type(const FirLaunch& L, cudaStream_t stream)
{
#define TUCU_FIR_CASE(A, B)                                                             \
    if (L.rh == A && L.rv == B)                                                         \
        return launch_cfg<A, B, NH, CH, TIn>(L, stream);
    if (NH == 1) {
        TUCU_FIR_CASE(2, 2) TUCU_FIR_CASE(2, 4) TUCU_FIR_CASE(2, 8) TUCU_FIR_CASE(2, 16)
        TUCU_FIR_CASE(4, 2) TUCU_FIR_CASE(4, 4) TUCU_FIR_CASE(4, 8) TUCU_FIR_CASE(4, 16)
        TUCU_FIR_CASE(8, 2) TUCU_FIR_CASE(8, 4) TUCU_FIR_CASE(8, 8) TUCU_FIR_CASE(8, 16)
        TUCU_FIR_CASE(16, 2) TUCU_FIR_CASE(16, 4) TUCU_FIR_CASE(16, 8) TUCU_FIR_CASE(16, 16)
    } else {
        TUCU_FIR_CASE(2, 2) TUCU_FIR_CASE(4, 4) TUCU_FIR_CASE(8, 8) TUCU_FIR_CASE(16, 16)
    }
#undef TUCU_FIR_CASE
    return cudaErrorInvalidValue;
}

template <class TIn>
static cudaError_t launch_typed(const FirLaunch& L, cudaStream_t stream)
{
    if (L.nh == 1)
        return launch_for_type<1, 32, TIn>(L, stream);
    return launch_for_type<3, 16, TIn>(L, stream);
}

template <class TIn>
static size_t smem_typed(int rh, int rv, int nh)
{
#define TUCU_FIR_SMEM(r1, r2, n, c)                                                        \
    if (rh == r1 && rv == r2 && nh == n)                                                   \
        return StripCfg<r1, r2, n, c, TIn>::SMEM;
    TUCU_FIR_SMEM(16, 16, 3, 16) TUCU_FIR_SMEM(8, 8, 3, 16) TUCU_FIR_SMEM(4, 4, 3, 16)
    TUCU_FIR_SMEM(2, 2, 3, 16)
    TUCU_FIR_SMEM(16, 16, 1, 32) TUCU_FIR_SMEM(8, 8, 1, 32) TUCU_FIR_SMEM(4, 4, 1, 32)
    TUCU_FIR_SMEM(2, 2, 1, 32)
#undef TUCU_FIR_SMEM
    return 0;
}

}  // namespace fir
}  // namespace tucu

#define TUCU_FIR_INSTANTIATE(suffix, T)                                                   \
    namespace tucu                                                                        \
    {                                                                                     \
    namespace fir                                                                         \
    {                                                                                     \
    cudaError_t launch_##suffix(const FirLaunch& L, cudaStream_t stream)                  \
    {                                                                                     \
        return launch_typed<T>(L, stream);                                                \
    }                                                                                     \
    size_t smem_##suffix(int rh, int rv, int nh) { return smem_typed<T>(rh, rv, nh); }    \
    }                                                                                     \
    }                                                                                     \
    TUCU_DEFINE_ERROR_ACCESSOR(tucu_fir_##suffix##_tu_error)
