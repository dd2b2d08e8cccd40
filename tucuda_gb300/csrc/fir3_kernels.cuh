// fir3_kernels.cuh -- kernels and launchers of the warp-specialised
// single-operator FIR strip (fir_v3.cuh), instantiated once per (input type,
// output type) by the fir3_<in>_<out>.cu translation units so that they
// compile in parallel.  Equal horizontal and vertical radii only (every
// Gaussian smooth and most operators); other lobe pairs use the padded
// multi-lobe kernel of fir_kernels.cuh.
#pragma once
#include "batch_types.h"
#include "fir_v3.cuh"
#include "tucu_internal.h"

namespace tucu
{
namespace fir
{

struct K3Params
{
    FirJob job;
    LobeSet lobes;
    int strip_rows;  // output rows per CTA (multiple of 32)
    int use_tma;
};

template <int R, class TIn, class TOut>
__global__ void __launch_bounds__(fir3::kThreads, 2)
    fir3_kernel(const __grid_constant__ K3Params P, const __grid_constant__ CUtensorMap tmap)
{
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
    if (P.use_tma && threadIdx.x == 0) {
        tma_prefetch_desc(&tmap);
        for (int s = 0; s < fir3::Cfg<R, R, TIn>::NSTAGE; ++s)
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
    fir3::run_strip<R, R, TIn, TOut>(P.job, P.lobes, P.use_tma ? &tmap : nullptr, x0, y0, nrows,
                                     smem, pipe);
}

// One CTA per work item of a batch class.
template <int R, class TIn, class TOut>
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
    fir3::run_strip<R, R, TIn, TOut>(J.fir, J.lobes, J.has_tmap ? &tmaps[it.job] : nullptr, it.x0,
                                     it.y0, it.nrows, smem, pipe);
}

template <int R, class TIn, class TOut>
static cudaError_t launch3_r(const FirLaunch& L, cudaStream_t stream)
{
    using Cfg = fir3::Cfg<R, R, TIn>;
    auto kern = fir3_kernel<R, TIn, TOut>;
    static DeviceOnce attr_once;
    cudaError_t e = attr_once.run([&] {
        return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)Cfg::SMEM);
    });
    if (e != cudaSuccess)
        return e;
    K3Params P;
    P.job = L.job;
    P.lobes = L.lobes;
    P.use_tma = L.use_tma;
    const int ncx = (L.job.ocols + fir3::kTW - 1) / fir3::kTW;
    int strip = L.strip_rows;
    if (strip <= 0) {
        static int resident = 0;  // CTAs per SM (the same on every device of one type)
        if (resident == 0)
            resident = ctas_per_sm((const void*)kern, fir3::kThreads, Cfg::SMEM);
        strip = plan_strip_rows(L.job.orows, ncx, (long)resident * sm_count(), fir3::kCH, R, 2048);
    }
    strip = (strip + fir3::kCH - 1) / fir3::kCH * fir3::kCH;
    P.strip_rows = strip;
    const dim3 grid(ncx, (L.job.orows + strip - 1) / strip);
    kern<<<grid, fir3::kThreads, Cfg::SMEM, stream>>>(P, L.tmap);
    return cudaGetLastError();
}

template <class TIn, class TOut>
static cudaError_t launch3_typed(const FirLaunch& L, cudaStream_t stream)
{
    if (L.rh != L.rv)
        return cudaErrorInvalidValue;
    switch (L.rh) {
    case 2: return launch3_r<2, TIn, TOut>(L, stream);
    case 4: return launch3_r<4, TIn, TOut>(L, stream);
    case 8: return launch3_r<8, TIn, TOut>(L, stream);
    case 16: return launch3_r<16, TIn, TOut>(L, stream);
    default: return cudaErrorInvalidValue;
    }
}

template <class TIn, class TOut>
static const void* batch3_typed(int r, size_t* smem)
{
    switch (r) {
    case 2: *smem = fir3::Cfg<2, 2, TIn>::SMEM; return (const void*)fir3_batch_kernel<2, TIn, TOut>;
    case 4: *smem = fir3::Cfg<4, 4, TIn>::SMEM; return (const void*)fir3_batch_kernel<4, TIn, TOut>;
    case 8: *smem = fir3::Cfg<8, 8, TIn>::SMEM; return (const void*)fir3_batch_kernel<8, TIn, TOut>;
    case 16: *smem = fir3::Cfg<16, 16, TIn>::SMEM; return (const void*)fir3_batch_kernel<16, TIn, TOut>;
    default: return nullptr;
    }
}

}  // namespace fir
}  // namespace tucu

#define TUCU_FIR3_INSTANTIATE(in, TIn, out, TOut)                                           \
    namespace tucu                                                                          \
    {                                                                                       \
    namespace fir                                                                           \
    {                                                                                       \
    cudaError_t launch3_##in##_##out(const FirLaunch& L, cudaStream_t stream)               \
    {                                                                                       \
        return launch3_typed<TIn, TOut>(L, stream);                                         \
    }                                                                                       \
    const void* batch3_##in##_##out(int r, size_t* smem) { return batch3_typed<TIn, TOut>(r, smem); } \
    }                                                                                       \
    }                                                                                       \
    TUCU_DEFINE_ERROR_ACCESSOR(tucu_fir3_##in##_##out##_tu_error)
