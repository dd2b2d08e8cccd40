// guided.cuh -- GuidedFilter2's two passes on the window-sum strip
// (box_strip.cuh): producers, epilogues, kernels and the launcher template,
// instantiated for 4 columns per lane in guided_narrow.cu and for 8 (windows
// wider than 125 columns) in guided_wide.cu.
#pragma once
#include <algorithm>

#include "box_kernels.h"
#include "box_plain.cuh"

namespace tucu
{
namespace box
{

// Guided pass A: sums of (p', g', p'g', g'g') with p' = p - Kp, g' = g - Kg
// (per-strip anchors, so the variance term does not cancel); the epilogue
// turns them into the coefficients (a, b) of init_coeffs
// (TU/cu/GuidedFilter.h:74-105), written as float2.  CPT = 8 only for
// windows wider than a 4-column warp tile holds.
template <class TIn, bool VEC, int CPT = kCPT>
struct GuidedAProd
{
    static constexpr bool kCompensate = true;
    static constexpr int kCols = CPT;
    // The p planes, then the g planes, of at most 16 bytes each.
    static constexpr int kPlaneBytes = CPT * (int)sizeof(TIn) > 16 ? 16 : CPT * (int)sizeof(TIn);
    static constexpr int kPerImage = CPT * (int)sizeof(TIn) / kPlaneBytes;
    static constexpr int kPlanes = 2 * kPerImage;
    static constexpr bool kAsync = VEC;
    struct Raw
    {
        RawN<TIn, CPT> p, g;
        uint32_t valid;  // bit j: column j lies inside the image
    };
    const void* p;
    size_t p_pitch;
    const void* g;
    size_t g_pitch;
    int rows, cols;
    float kp, kg;
    __device__ const void* plane_ptr(int k, int y, int x) const
    {
        const int off = (k % kPerImage) * kPlaneBytes;
        return k < kPerImage ? row_ptr(p, p_pitch, y) + (size_t)x * sizeof(TIn) + off
                             : row_ptr(g, g_pitch, y) + (size_t)x * sizeof(TIn) + off;
    }
    __device__ int plane_bytes(int k, int nvalid, int) const
    {
        return min(max(nvalid * (int)sizeof(TIn) - (k % kPerImage) * kPlaneBytes, 0), kPlaneBytes);
    }
    __device__ void finish(Raw& r, int nvalid) const { r.valid = (1u << nvalid) - 1u; }
    __device__ Raw load(int y, int x) const
    {
        Raw r;
        r.p = load_raw<TIn, VEC, CPT>(p, p_pitch, rows, cols, y, x);
        r.g = load_raw<TIn, VEC, CPT>(g, g_pitch, rows, cols, y, x);
        const bool in = y >= 0 && y < rows;
        const int n = in ? max(0, min(CPT, cols - x)) : 0;
        r.valid = (1u << n) - 1u;
        return r;
    }
    __device__ void expand(const Raw& r, int j, float (&q)[4]) const
    {
        const bool ok = (r.valid >> j) & 1u;
        const float pv = ok ? raw_elem<TIn, float>(r.p, j) - kp : 0.0f;
        const float gv = ok ? raw_elem<TIn, float>(r.g, j) - kg : 0.0f;
        q[0] = pv;
        q[1] = gv;
        q[2] = pv * gv;
        q[3] = gv * gv;
    }
};

// Guided pass B: sums of (a, b) over the coefficient image.
template <int CPT = kCPT>
struct GuidedBProd
{
    static constexpr bool kCompensate = true;
    static constexpr int kCols = CPT;
    static constexpr int kPlanes = CPT / 2;  // columns 2k, 2k+1
    static constexpr int kPlaneBytes = 16;
    static constexpr bool kAsync = true;  // coefficient rows are 16-byte aligned
    struct Raw
    {
        float4 q[CPT / 2];  // (a0,b0,a1,b1), (a2,b2,a3,b3), ...
    };
    const float2* coef;
    size_t pitch;
    int rows, cols;
    __device__ const void* plane_ptr(int k, int y, int x) const
    {
        return reinterpret_cast<const float2*>(row_ptr(coef, pitch, y)) + x + 2 * k;
    }
    __device__ int plane_bytes(int k, int nvalid, int) const { return min(max(nvalid - 2 * k, 0), 2) * 8; }
    __device__ void finish(Raw&, int) const {}
    __device__ Raw load(int y, int x) const
    {
        Raw r;
#pragma unroll
        for (int k = 0; k < CPT / 2; ++k)
            r.q[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (y < 0 || y >= rows || x >= cols)
            return r;
        const float2* row = reinterpret_cast<const float2*>(row_ptr(coef, pitch, y));
        if (x + CPT <= cols) {
#pragma unroll
            for (int k = 0; k < CPT / 2; ++k)
                r.q[k] = __ldg(reinterpret_cast<const float4*>(row + x) + k);
            return r;
        }
        float2* e = reinterpret_cast<float2*>(&r);
#pragma unroll
        for (int j = 0; j < CPT; ++j)
            if (x + j < cols)
                e[j] = row[x + j];
        return r;
    }
    __device__ void expand(const Raw& r, int j, float (&q)[2]) const
    {
        const float2* e = reinterpret_cast<const float2*>(&r);
        q[0] = e[j].x;
        q[1] = e[j].y;
    }
};

// ---- guided epilogues -------------------------------------------------------------

struct GuidedAEpi
{
    float2* coef;
    size_t pitch;  // bytes
    float n, inv_n, sq_e, kp, kg;
    int self;
    // Every operation is an explicitly rounded intrinsic, so no kernel
    // instantiation contracts it differently (results are bit-identical
    // whichever load path ran).
    __device__ float2 coeffs(const float (&s)[4]) const
    {
        const float mp = __fmul_rn(s[0], inv_n), mg = __fmul_rn(s[1], inv_n);
        const float cov = __fmaf_rn(-mp, mg, __fmul_rn(s[2], inv_n));
        const float var = fmaxf(__fmaf_rn(-mg, mg, __fmul_rn(s[3], inv_n)), 0.0f);
        float a, b;
        if (self) {
            // a = var/(var + e^2); b = (Sp - a*Spp)/n as the reference writes it
            // (GuidedFilter.h:94-97): E[p^2] = var + mean^2.
            a = __fdiv_rn(var, __fadd_rn(var, sq_e));
            const float mean = __fadd_rn(mp, kp);
            b = __fmaf_rn(-a, __fmaf_rn(mean, mean, var), mean);
        } else {
            a = __fdiv_rn(cov, __fadd_rn(var, sq_e));
            b = __fmaf_rn(-a, __fadd_rn(mg, kg), __fadd_rn(mp, kp));
        }
        return make_float2(a, b);
    }
    template <int N>
    __device__ __forceinline__ void store(int y, int x, const float (&s)[N][4], unsigned mask) const
    {
        float2* row = reinterpret_cast<float2*>(row_ptr(coef, pitch, y)) + x;
        float2 c[N];
#pragma unroll
        for (int j = 0; j < N; ++j)
            c[j] = coeffs(s[j]);
        if (mask == (1u << N) - 1u && (reinterpret_cast<uintptr_t>(row) & 15) == 0) {
#pragma unroll
            for (int k = 0; k < N / 2; ++k)
                reinterpret_cast<float4*>(row)[k] = make_float4(c[2 * k].x, c[2 * k].y, c[2 * k + 1].x, c[2 * k + 1].y);
            return;
        }
#pragma unroll
        for (int j = 0; j < N; ++j)
            if ((mask >> j) & 1u)
                row[j] = c[j];
    }
    __device__ void store4(int y, int x, const float (&s)[4][4], unsigned mask) const { store<4>(y, x, s, mask); }
    __device__ void store8(int y, int x, const float (&s)[8][4], unsigned mask) const { store<8>(y, x, s, mask); }
};

// out = (A*g + B)/n with g at the window centre (trans_guides,
// TU/cu/GuidedFilter.h:107-125).
template <class TIn>
struct GuidedBEpi
{
    const void* g;
    size_t g_pitch;
    void* dst;
    size_t pitch;
    int dtype, oy, ox, gy, gx;
    float n;
    // The guide pixels of output row y into L1 ahead of store4.
    __device__ void prefetch(int y, int x) const
    {
        const char* p = row_ptr(g, g_pitch, y + gy) + (size_t)(x + gx) * sizeof(TIn);
        asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
    }
    __device__ void store4(int y, int x, const float (&s)[4][2], unsigned mask) const
    {
        const char* grow = row_ptr(g, g_pitch, y + gy);
        float f[4];
#pragma unroll
        for (int j = 0; j < 4; ++j)
            f[j] = ((mask >> j) & 1u)
                       ? __fdiv_rn(fmaf(s[j][0], load_px<TIn>(grow, x + gx + j), s[j][1]), n)
                       : 0.0f;
        store4_float(row_ptr(dst, pitch, y + oy), x + ox, dtype, f, mask, cls);
    }
    __device__ void store8(int y, int x, const float (&s)[8][2], unsigned mask) const
    {
        const float lo[4][2] = {{s[0][0], s[0][1]}, {s[1][0], s[1][1]}, {s[2][0], s[2][1]}, {s[3][0], s[3][1]}};
        const float hi[4][2] = {{s[4][0], s[4][1]}, {s[5][0], s[5][1]}, {s[6][0], s[6][1]}, {s[7][0], s[7][1]}};
        if (mask & 0xfu)
            store4(y, x, lo, mask & 0xfu);
        if (mask >> 4)
            store4(y, x + 4, hi, mask >> 4);
    }
    int cls;  // store_class of dst, pitch, ox
};

// ---- kernels --------------------------------------------------------------------

// CTAs per SM of the guided kernels; 8-column strips (wide windows only)
// hold twice the compensated sums and run one CTA per SM.
template <int CPT>
struct GuidedCfg
{
    static constexpr int kCtas = CPT == 8 ? 1 : 2;
};
constexpr int kGuidedWarpBytes = 6144;  // 48 KB per CTA: no opt-in needed

template <class Prod>
struct GuidedRing
{
    static constexpr int kDepth = Ring<Prod>::depth(kGuidedWarpBytes);
    static constexpr int kSmem = kWarps * kDepth * Ring<Prod>::kStepBytes;
};

template <class TIn, bool VEC, int CPT>
__global__ void __launch_bounds__(kThreads, GuidedCfg<CPT>::kCtas)
    guided_a_kernel(const __grid_constant__ Geo G, const __grid_constant__ GuidedAProd<TIn, VEC, CPT> prod0,
                    const __grid_constant__ GuidedAEpi epi0)
{
    using R = GuidedRing<GuidedAProd<TIn, VEC, CPT>>;
    char* ring = warp_ring(R::kSmem / kWarps);
    for_each_task<CPT>(G, [&](auto cc, int xw, int y0, int nrows) {
        // Per-task anchors: the task's first pixel (any constant works; a
        // local one keeps the shifted values small).
        GuidedAProd<TIn, VEC, CPT> prod = prod0;
        GuidedAEpi epi = epi0;
        const int ay = min(y0, prod.rows - 1), ax = min(xw, prod.cols - 1);
        prod.kp = load_px<TIn>(row_ptr(prod.p, prod.p_pitch, ay), ax);
        prod.kg = load_px<TIn>(row_ptr(prod.g, prod.g_pitch, ay), ax);
        epi.kp = prod.kp;
        epi.kg = prod.kg;
        strip_body<decltype(cc)::value, 4, float, R::kDepth>(prod, epi, G.wV, G.wH, xw, y0, nrows, G.ocols,
                                                               ring, prod.cols, G.tg.restart);
    });
}

template <class TIn, int CPT>
__global__ void __launch_bounds__(kThreads, GuidedCfg<CPT>::kCtas)
    guided_b_kernel(const __grid_constant__ Geo G, const __grid_constant__ GuidedBProd<CPT> prod,
                    const __grid_constant__ GuidedBEpi<TIn> epi)
{
    using R = GuidedRing<GuidedBProd<CPT>>;
    char* ring = warp_ring(R::kSmem / kWarps);
    for_each_task<CPT>(G, [&](auto cc, int xw, int y0, int nrows) {
        strip_body<decltype(cc)::value, 2, float, R::kDepth>(prod, epi, G.wV, G.wH, xw, y0, nrows, G.ocols,
                                                               ring, prod.cols, G.tg.restart);
    });
}

// Grid of the guided passes: the warp tasks' CTAs, at most the resident ones.
inline dim3 guided_grid(const Geo& G, int ctas_per_sm)
{
    const long want = (G.tg.ntask + kWarps - 1) / kWarps;
    return dim3((unsigned)std::max(1L, std::min(want, (long)ctas_per_sm * sm_count())));
}

// Rows of es-byte pixels aligned for the copies of cpt-pixel groups.
inline bool guided_rows_aligned(const void* p, size_t pitch, size_t es, int cpt)
{
    const size_t a = std::min<size_t>((size_t)cpt * es, 16);
    return (reinterpret_cast<uintptr_t>(p) % a) == 0 && (pitch % a) == 0;
}

// Float restart period of the guided passes, from the image size alone
// (every caller of the same image gets the same bits): small images take
// short restart blocks, so they split into enough warp tasks to fill the GPU;
// large ones long blocks, so the window set-up rows stay a small fraction.
inline int guided_restart(int rows, int cols)
{
    const long px = (long)rows * cols;
    return px >= 16000000 ? 64 : px >= 4000000 ? 32 : 8;
}

template <class TIn, int CPT>
cudaError_t launch_guided_t(const GuidedLaunch& L, cudaStream_t st)
{
    constexpr int kCtas = GuidedCfg<CPT>::kCtas;
    const int restart = guided_restart(L.rows, L.cols);
    const int n = L.wV * L.wH;
    // Pass A over the input grid -> coefficient grid (rows+1-wV) x (cols+1-wH).
    Geo A;
    A.wV = L.wV;
    A.wH = L.wH;
    A.orows = L.rows + 1 - L.wV;
    A.ocols = L.cols + 1 - L.wH;
    GuidedAEpi ea{static_cast<float2*>(L.coef), L.coef_pitch, (float)n, 1.0f / (float)n, L.e * L.e, 0.0f, 0.0f,
                  L.guide == nullptr};
    const void* g = L.guide ? L.guide : L.src;
    const size_t gp = L.guide ? L.guide_pitch : L.src_pitch;
    // Wide windows (8 columns per lane) run the synchronous loads only.
    const bool vec = CPT == kCPT && guided_rows_aligned(L.src, L.src_pitch, sizeof(TIn), CPT) &&
                     guided_rows_aligned(g, gp, sizeof(TIn), CPT);
    A.tg = plan_tasks(A.orows, A.ocols, L.wV, L.wH, 0, kCtas, restart, 1, CPT);
    // Rings above 48 KB per CTA (8-column strips) need the opt-in.
    cudaError_t e;
    if constexpr (CPT == kCPT) {
        if (vec) {
            GuidedAProd<TIn, true, CPT> pa{L.src, L.src_pitch, g, gp, L.rows, L.cols, 0.0f, 0.0f};
            constexpr size_t smem = GuidedRing<GuidedAProd<TIn, true, CPT>>::kSmem;
            if ((e = smem_opt_in<guided_a_kernel<TIn, true, CPT>>(smem)) != cudaSuccess)
                return e;
            guided_a_kernel<TIn, true, CPT><<<guided_grid(A, kCtas), kThreads, smem, st>>>(A, pa, ea);
        }
    }
    if (!vec) {
        GuidedAProd<TIn, false, CPT> pa{L.src, L.src_pitch, g, gp, L.rows, L.cols, 0.0f, 0.0f};
        constexpr size_t smem = GuidedRing<GuidedAProd<TIn, false, CPT>>::kSmem;
        if ((e = smem_opt_in<guided_a_kernel<TIn, false, CPT>>(smem)) != cudaSuccess)
            return e;
        guided_a_kernel<TIn, false, CPT><<<guided_grid(A, kCtas), kThreads, smem, st>>>(A, pa, ea);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    // Pass B over the coefficient grid -> output grid.
    Geo B;
    B.wV = L.wV;
    B.wH = L.wH;
    B.orows = A.orows + 1 - L.wV;
    B.ocols = A.ocols + 1 - L.wH;
    B.tg = plan_tasks(B.orows, B.ocols, L.wV, L.wH, 0, kCtas, restart, 1, CPT);
    GuidedBProd<CPT> pb{reinterpret_cast<const float2*>(L.coef), L.coef_pitch, A.orows, A.ocols};
    GuidedBEpi<TIn> eb{g, gp, L.dst, L.dst_pitch, L.out_dtype, L.oy, L.ox,
                       L.wV - 1, L.wH - 1, (float)n,
                       store_class(L.dst, L.dst_pitch, L.ox, dtype_size(L.out_dtype))};
    constexpr size_t smem_b = GuidedRing<GuidedBProd<CPT>>::kSmem;
    if ((e = smem_opt_in<guided_b_kernel<TIn, CPT>>(smem_b)) != cudaSuccess)
        return e;
    guided_b_kernel<TIn, CPT><<<guided_grid(B, kCtas), kThreads, smem_b, st>>>(B, pb, eb);
    return cudaGetLastError();
}

template <int CPT>
cudaError_t launch_guided_cpt(const GuidedLaunch& L, cudaStream_t st)
{
    switch (L.in_dtype) {
    case U8: return launch_guided_t<uint8_t, CPT>(L, st);
    case F16: return launch_guided_t<__half, CPT>(L, st);
    case BF16: return launch_guided_t<__nv_bfloat16, CPT>(L, st);
    case F32: return launch_guided_t<float, CPT>(L, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace box
}  // namespace tucu
