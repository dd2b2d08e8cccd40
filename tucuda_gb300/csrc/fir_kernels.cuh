// fir_kernels.cuh -- the multi-lobe FIR strip kernel (fir_strip.cuh) and its
// launcher, instantiated once per input type by fir_<type>.cu.  Used for the
// Gaussian multi-operator pass (up to three horizontal lobes, six outputs)
// and for single lobe pairs of unequal radii (padded to the larger one).
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

template <int R, int CH, class TIn>
__global__ void __launch_bounds__(kThreads)
    fir_multi_kernel(const __grid_constant__ KParams P, const __grid_constant__ CUtensorMap tmap)
{
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
    if (P.use_tma && threadIdx.x == 0) {
        tma_prefetch_desc(&tmap);
        for (int s = 0; s < StripCfg<R, R, 3, CH, TIn>::NSTAGE; ++s)
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
    run_strip<R, R, 3, CH, TIn>(P.job, P.lobes, P.use_tma ? &tmap : nullptr, x0, y0,
                                (nrows + CH - 1) / CH, smem, pipe);
}

template <int R, class TIn>
static cudaError_t launch_multi_r(const FirLaunch& L, cudaStream_t stream)
{
    constexpr int CH = 16;
    using Cfg = StripCfg<R, R, 3, CH, TIn>;
    auto kern = fir_multi_kernel<R, CH, TIn>;
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
    const int ncx = (L.job.ocols + kTW - 1) / kTW;
    int strip = L.strip_rows;
    if (strip <= 0) {
        static int resident = 0;  // CTAs per SM (the same on every device of one type)
        if (resident == 0)
            resident = ctas_per_sm((const void*)kern, kThreads, Cfg::SMEM);
        strip = plan_strip_rows(L.job.orows, ncx, (long)resident * sm_count(), CH, R, 1024);
    }
    strip = (strip + CH - 1) / CH * CH;
    P.strip_rows = strip;
    const dim3 grid(ncx, (L.job.orows + strip - 1) / strip);
    kern<<<grid, kThreads, Cfg::SMEM, stream>>>(P, L.tmap);
    return cudaGetLastError();
}

template <class TIn>
static cudaError_t launch_typed(const FirLaunch& L, cudaStream_t stream)
{
    if (L.rh != L.rv)
        return cudaErrorInvalidValue;
    switch (L.rh) {
    case 2: return launch_multi_r<2, TIn>(L, stream);
    case 4: return launch_multi_r<4, TIn>(L, stream);
    case 8: return launch_multi_r<8, TIn>(L, stream);
    case 16: return launch_multi_r<16, TIn>(L, stream);
    default: return cudaErrorInvalidValue;
    }
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
    }                                                                                     \
    }                                                                                     \
    TUCU_DEFINE_ERROR_ACCESSOR(tucu_fir_##suffix##_tu_error)
