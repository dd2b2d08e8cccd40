// fir_kernels.cuh -- the single-job FIR strip kernel and its launcher,
// instantiated once per input type by fir_<type>.cu (split so the
// instantiations compile in parallel).
#pragma once
#include "fir_strip.cuh"
#include "fir_v3.cuh"
#include "batch_types.h"
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

// Single-operator FIR: warp-specialised strips of 128 columns (fir_v3.cuh).
template <int RH, int RV, class TIn>
__global__ void __launch_bounds__(fir3::kThreads, 2)
    fir3_kernel(const __grid_constant__ KParams P, const __grid_constant__ CUtensorMap tmap)
{
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
    if (P.use_tma && threadIdx.x == 0) {
        tma_prefetch_desc(&tmap);
        for (int s = 0; s < fir3::Cfg<RH, RV, TIn>::NSTAGE; ++s)
            mbar_init(&bars[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    const int x0 = blockIdx.x * fir3::kTW;
    const int y0 = blockIdx.y * P.strip_rows;
    const int nrows = min(P.strip_rows, P.job.orows - y0);
    if (nrows <= 0)
        return;
    Pipe pipe{0};
    fir3::run_strip<RH, RV, TIn>(P.job, P.lobes, P.use_tma ? &tmap : nullptr, x0, y0, nrows,
                                 smem, pipe);
}

// One CTA per work item of a batch class (radius R, input type TIn).
template <int R, class TIn>
__global__ void __launch_bounds__(fir3::kThreads, 2)
    fir3_batch_kernel(const batch::FirJobD* __restrict__ jobs, const CUtensorMap* __restrict__ tmaps,
                      const batch::Item* __restrict__ items)
{
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
    const batch::Item it = items[blockIdx.x];
    const batch::FirJobD& J = jobs[it.job];
    if (threadIdx.x == 0) {
        for (int s = 0; s < fir3::Cfg<R, R, TIn>::NSTAGE; ++s)
            mbar_init(&bars[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    Pipe pipe{0};
    fir3::run_strip<R, R, TIn>(J.fir, J.lobes, J.has_tmap ? &tmaps[it.job] : nullptr, it.x0, it.y0,
                               it.nrows, smem, pipe);
}

template <class TIn>
static const void* batch_kernel_typed(int r, size_t* smem)
{
    switch (r) {
    case 2: *smem = fir3::Cfg<2, 2, TIn>::SMEM; return (const void*)fir3_batch_kernel<2, TIn>;
    case 4: *smem = fir3::Cfg<4, 4, TIn>::SMEM; return (const void*)fir3_batch_kernel<4, TIn>;
    case 8: *smem = fir3::Cfg<8, 8, TIn>::SMEM; return (const void*)fir3_batch_kernel<8, TIn>;
    case 16: *smem = fir3::Cfg<16, 16, TIn>::SMEM; return (const void*)fir3_batch_kernel<16, TIn>;
    default: return nullptr;
    }
}

template <int RH, int RV, class TIn>
static cudaError_t launch_cfg3(const FirLaunch& L, cudaStream_t stream)
{
    using Cfg = fir3::Cfg<RH, RV, TIn>;
    auto kern = fir3_kernel<RH, RV, TIn>;
    static DeviceOnce attr_once;
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
    int strip = L.strip_rows > 0 ? L.strip_rows : 256;
    strip = (strip + fir3::kCH - 1) / fir3::kCH * fir3::kCH;
    P.strip_rows = strip;
    const dim3 grid((L.job.ocols + fir3::kTW - 1) / fir3::kTW, (L.job.orows + strip - 1) / strip);
    kern<<<grid, fir3::kThreads, Cfg::SMEM, stream>>>(P, L.tmap);
    return cudaGetLastError();
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
#define TUCU_FIR3_CASE(A, B)                                                            \
    if (L.rh == A && L.rv == B)                                                         \
        return launch_cfg3<A, B, TIn>(L, stream);
#define TUCU_FIR_CASE(A, B)                                                             \
    if (L.rh == A && L.rv == B)                                                         \
        return launch_cfg<A, B, NH, CH, TIn>(L, stream);
    if constexpr (NH == 1) {
        TUCU_FIR3_CASE(2, 2) TUCU_FIR3_CASE(2, 4) TUCU_FIR3_CASE(2, 8) TUCU_FIR3_CASE(2, 16)
        TUCU_FIR3_CASE(4, 2) TUCU_FIR3_CASE(4, 4) TUCU_FIR3_CASE(4, 8) TUCU_FIR3_CASE(4, 16)
        TUCU_FIR3_CASE(8, 2) TUCU_FIR3_CASE(8, 4) TUCU_FIR3_CASE(8, 8) TUCU_FIR3_CASE(8, 16)
        TUCU_FIR3_CASE(16, 2) TUCU_FIR3_CASE(16, 4) TUCU_FIR3_CASE(16, 8) TUCU_FIR3_CASE(16, 16)
    } else {
        TUCU_FIR_CASE(2, 2) TUCU_FIR_CASE(4, 4) TUCU_FIR_CASE(8, 8) TUCU_FIR_CASE(16, 16)
    }
#undef TUCU_FIR_CASE
#undef TUCU_FIR3_CASE
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
#undef TUCU_FIR_SMEM
    if (nh == 1 && rh == rv) {
        switch (rh) {
        case 2: return fir3::Cfg<2, 2, TIn>::SMEM;
        case 4: return fir3::Cfg<4, 4, TIn>::SMEM;
        case 8: return fir3::Cfg<8, 8, TIn>::SMEM;
        case 16: return fir3::Cfg<16, 16, TIn>::SMEM;
        default: break;
        }
    }
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
    const void* batch_kernel_##suffix(int r, size_t* smem) { return batch_kernel_typed<T>(r, smem); } \
    }                                                                                     \
    }                                                                                     \
    TUCU_DEFINE_ERROR_ACCESSOR(tucu_fir_##suffix##_tu_error)
