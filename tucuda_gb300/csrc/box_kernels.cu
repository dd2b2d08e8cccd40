// box_kernels.cu -- BoxFilter2 and GuidedFilter2 kernels built on the
// one-pass window-sum strip (box_strip.cuh), and their launchers.
#include "box_kernels.h"
#include "batch_types.h"
#include "box_ops.cuh"

namespace tucu
{
namespace box
{

// Guided pass A: sums of (p', g', p'g', g'g') with p' = p - Kp, g' = g - Kg
// (per-strip anchors, so the variance term does not cancel); the epilogue
// turns them into the coefficients (a, b) of init_coeffs
// (TU/cu/GuidedFilter.h:74-105), written as float2.
template <class TIn, bool VEC>
struct GuidedAProd
{
    struct Raw
    {
        Raw4<TIn> p, g;
        uint32_t valid;  // bit j: column j lies inside the image
    };
    const void* p;
    size_t p_pitch;
    const void* g;
    size_t g_pitch;
    int rows, cols;
    float kp, kg;
    __device__ Raw load(int y, int x) const
    {
        Raw r;
        r.p = load_raw4<TIn, VEC>(p, p_pitch, rows, cols, y, x);
        r.g = load_raw4<TIn, VEC>(g, g_pitch, rows, cols, y, x);
        const bool in = y >= 0 && y < rows;
        const int n = in ? max(0, min(kCPT, cols - x)) : 0;
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
struct GuidedBProd
{
    struct Raw
    {
        float4 lo, hi;  // (a0,b0,a1,b1), (a2,b2,a3,b3)
    };
    const float2* coef;
    size_t pitch;
    int rows, cols;
    __device__ Raw load(int y, int x) const
    {
        Raw r;
        r.lo = r.hi = make_float4(0.f, 0.f, 0.f, 0.f);
        if (y < 0 || y >= rows || x >= cols)
            return r;
        const float2* row = reinterpret_cast<const float2*>(row_ptr(coef, pitch, y));
        if (x + kCPT <= cols) {
            r.lo = __ldg(reinterpret_cast<const float4*>(row + x));
            r.hi = __ldg(reinterpret_cast<const float4*>(row + x + 2));
            return r;
        }
        float2* e = reinterpret_cast<float2*>(&r);
#pragma unroll
        for (int j = 0; j < kCPT; ++j)
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
    __device__ float2 coeffs(const float (&s)[4]) const
    {
        const float mp = s[0] * inv_n, mg = s[1] * inv_n;
        const float cov = fmaf(-mp, mg, s[2] * inv_n);
        const float var = fmaxf(fmaf(-mg, mg, s[3] * inv_n), 0.0f);
        float a, b;
        if (self) {
            // a = var/(var + e^2); b = (Sp - a*Spp)/n as the reference writes it
            // (GuidedFilter.h:94-97): E[p^2] = var + mean^2.
            a = var / (var + sq_e);
            const float mean = mp + kp;
            b = mean - a * fmaf(mean, mean, var);
        } else {
            a = cov / (var + sq_e);
            b = (mp + kp) - a * (mg + kg);
        }
        return make_float2(a, b);
    }
    __device__ void store4(int y, int x, const float (&s)[4][4], int i, int two) const
    {
        float2* row = reinterpret_cast<float2*>(row_ptr(coef, pitch, y)) + x;
        const unsigned mask = valid_mask(i, two);
        float2 c[4];
#pragma unroll
        for (int j = 0; j < 4; ++j)
            c[j] = coeffs(s[j]);
        if (mask == 0xfu && (reinterpret_cast<uintptr_t>(row) & 15) == 0) {
            reinterpret_cast<float4*>(row)[0] = make_float4(c[0].x, c[0].y, c[1].x, c[1].y);
            reinterpret_cast<float4*>(row)[1] = make_float4(c[2].x, c[2].y, c[3].x, c[3].y);
            return;
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if ((mask >> j) & 1u)
                row[j] = c[j];
    }
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
    __device__ void store4(int y, int x, const float (&s)[4][2], int i, int two) const
    {
        const unsigned mask = valid_mask(i, two);
        const char* grow = row_ptr(g, g_pitch, y + gy);
        float f[4];
#pragma unroll
        for (int j = 0; j < 4; ++j)
            f[j] = ((mask >> j) & 1u)
                       ? __fdiv_rn(fmaf(s[j][0], load_px<TIn>(grow, x + gx + j), s[j][1]), n)
                       : 0.0f;
        store4_float(row_ptr(dst, pitch, y + oy), x + ox, dtype, f, mask);
    }
};

// ---- kernels --------------------------------------------------------------------

struct Geo
{
    int wV, wH;
    int orows, ocols;   // output extent (valid coords)
    int strip_rows;
    int ox_align;       // (output column offset) mod 4
};

template <class TIn, class Acc, bool VEC>
__global__ void __launch_bounds__(kThreads, 2)
    box_kernel(const __grid_constant__ Geo G, const __grid_constant__ PlainProd<TIn, Acc, VEC> prod,
               const __grid_constant__ PlainEpi<Acc> epi)
{
    constexpr int U = BoxRows<TIn>::value;
    __shared__ __align__(16) unsigned char smem[sizeof(Smem<1, Acc, U>)];
    const int x0 = blockIdx.x * out_cols_per_cta(G.wH);
    const int y0 = blockIdx.y * G.strip_rows;
    const int nrows = min(G.strip_rows, G.orows - y0);
    run_strip<1, Acc, U>(prod, epi, G.wV, G.wH, x0, y0, nrows, G.ocols, G.ox_align, smem);
}

template <class TIn, bool VEC>
__global__ void __launch_bounds__(kThreads, 2)
    guided_a_kernel(const __grid_constant__ Geo G, GuidedAProd<TIn, VEC> prod, GuidedAEpi epi)
{
    constexpr int U = 2;
    __shared__ __align__(16) unsigned char smem[sizeof(Smem<4, float, U>)];
    const int x0 = blockIdx.x * out_cols_per_cta(G.wH);
    const int y0 = blockIdx.y * G.strip_rows;
    const int nrows = min(G.strip_rows, G.orows - y0);
    // Per-strip anchors: the first pixel of the strip (any constant works;
    // a local one keeps the shifted values small).
    const int ay = min(y0, prod.rows - 1), ax = min(x0, prod.cols - 1);
    prod.kp = load_px<TIn>(row_ptr(prod.p, prod.p_pitch, ay), ax);
    prod.kg = load_px<TIn>(row_ptr(prod.g, prod.g_pitch, ay), ax);
    epi.kp = prod.kp;
    epi.kg = prod.kg;
    run_strip<4, float, U>(prod, epi, G.wV, G.wH, x0, y0, nrows, G.ocols, 0, smem);
}

template <class TIn>
__global__ void __launch_bounds__(kThreads, 2)
    guided_b_kernel(const __grid_constant__ Geo G, const __grid_constant__ GuidedBProd prod,
                    const __grid_constant__ GuidedBEpi<TIn> epi)
{
    constexpr int U = 2;
    __shared__ __align__(16) unsigned char smem[sizeof(Smem<2, float, U>)];
    const int x0 = blockIdx.x * out_cols_per_cta(G.wH);
    const int y0 = blockIdx.y * G.strip_rows;
    const int nrows = min(G.strip_rows, G.orows - y0);
    run_strip<2, float, U>(prod, epi, G.wV, G.wH, x0, y0, nrows, G.ocols, G.ox_align, smem);
}

// One CTA per work item of a box batch class.
template <class TIn, class Acc, bool VEC>
__global__ void __launch_bounds__(kThreads, 2)
    box_batch_kernel(const batch::BoxJobD* __restrict__ jobs, const batch::Item* __restrict__ items)
{
    constexpr int U = BoxRows<TIn>::value;
    __shared__ __align__(16) unsigned char smem[sizeof(Smem<1, Acc, U>)];
    const batch::Item it = items[blockIdx.x];
    const batch::BoxJobD& J = jobs[it.job];
    PlainEpi<Acc> epi{J.dst, J.dst_pitch, J.out_dtype, J.oy, J.ox, J.normalize,
                      1.0f / (float)(J.wV * J.wH)};
    PlainProd<TIn, Acc, VEC> prod{J.src, J.src_pitch, J.rows, J.cols};
    run_strip<1, Acc, U>(prod, epi, J.wV, J.wH, it.x0, it.y0, it.nrows, J.ocols, J.ox & 3, smem);
}

const void* batch_kernel(int in_dtype, bool vec)
{
#define TUCU_BOX_BK(T, A)                                                                 \
    return vec ? (const void*)box_batch_kernel<T, A, true> : (const void*)box_batch_kernel<T, A, false>;
    switch (in_dtype) {
    case U8: TUCU_BOX_BK(uint8_t, int)
    case I32: TUCU_BOX_BK(int32_t, int)
    case F16: TUCU_BOX_BK(__half, float)
    case BF16: TUCU_BOX_BK(__nv_bfloat16, float)
    case F32: TUCU_BOX_BK(float, float)
    default: return nullptr;
    }
#undef TUCU_BOX_BK
}

// ---- launchers ------------------------------------------------------------------

static bool vec_ok(const void* p, size_t pitch, int es)
{
    const size_t a = (size_t)kCPT * es;
    return (reinterpret_cast<uintptr_t>(p) % a) == 0 && (pitch % a) == 0;
}

static dim3 grid_for(const Geo& G)
{
    return dim3((G.ocols + out_cols_per_cta(G.wH) - 1) / out_cols_per_cta(G.wH),
                (G.orows + G.strip_rows - 1) / G.strip_rows);
}

template <class TIn, class Acc>
static cudaError_t launch_box_t(const BoxLaunch& L, const Geo& G, cudaStream_t st)
{
    PlainEpi<Acc> epi{L.dst, L.dst_pitch, L.out_dtype, L.oy, L.ox, L.normalize,
                      1.0f / (float)(L.wV * L.wH)};
    if (vec_ok(L.src, L.src_pitch, sizeof(TIn))) {
        PlainProd<TIn, Acc, true> prod{L.src, L.src_pitch, L.rows, L.cols};
        box_kernel<TIn, Acc, true><<<grid_for(G), kThreads, 0, st>>>(G, prod, epi);
    } else {
        PlainProd<TIn, Acc, false> prod{L.src, L.src_pitch, L.rows, L.cols};
        box_kernel<TIn, Acc, false><<<grid_for(G), kThreads, 0, st>>>(G, prod, epi);
    }
    return cudaGetLastError();
}

static int default_strip(int orows, int ncx, int wV)
{
    // Aim for about four CTAs per SM; keep strips long enough that the
    // wV-row window set-up stays a small fraction of the strip.
    const int want = 4 * sm_count();
    const int nsy = (want + ncx - 1) / ncx;
    int strip = (orows + nsy - 1) / nsy;
    strip = max(strip, 2 * wV);
    // Strips start on multiples of the float restart period (box_strip.cuh),
    // so results do not depend on the strip height.
    strip = (strip + kRestart - 1) / kRestart * kRestart;
    return min(strip, 1024);
}

cudaError_t launch_box(const BoxLaunch& L, cudaStream_t st)
{
    Geo G;
    G.wV = L.wV;
    G.wH = L.wH;
    G.orows = L.rows + 1 - L.wV;
    G.ocols = L.cols + 1 - L.wH;
    const int ncx = (G.ocols + out_cols_per_cta(G.wH) - 1) / out_cols_per_cta(G.wH);
    G.strip_rows = L.strip_rows > 0 ? (L.strip_rows + kRestart - 1) / kRestart * kRestart
                                    : default_strip(G.orows, ncx, L.wV);
    G.ox_align = L.ox & 3;
    switch (L.in_dtype) {
    case U8: return launch_box_t<uint8_t, int>(L, G, st);
    case I32: return launch_box_t<int32_t, int>(L, G, st);
    case F16: return launch_box_t<__half, float>(L, G, st);
    case BF16: return launch_box_t<__nv_bfloat16, float>(L, G, st);
    case F32: return launch_box_t<float, float>(L, G, st);
    default: return cudaErrorInvalidValue;
    }
}

template <class TIn>
static cudaError_t launch_guided_t(const GuidedLaunch& L, cudaStream_t st)
{
    const int n = L.wV * L.wH;
    // Pass A over the input grid -> coefficient grid (rows+1-wV) x (cols+1-wH).
    Geo A;
    A.wV = L.wV;
    A.wH = L.wH;
    A.orows = L.rows + 1 - L.wV;
    A.ocols = L.cols + 1 - L.wH;
    const int ncxa = (A.ocols + out_cols_per_cta(A.wH) - 1) / out_cols_per_cta(A.wH);
    A.strip_rows = default_strip(A.orows, ncxa, L.wV);
    A.ox_align = 0;
    GuidedAEpi ea{static_cast<float2*>(L.coef), L.coef_pitch, (float)n, 1.0f / (float)n, L.e * L.e, 0.0f, 0.0f,
                  L.guide == nullptr};
    const void* g = L.guide ? L.guide : L.src;
    const size_t gp = L.guide ? L.guide_pitch : L.src_pitch;
    if (vec_ok(L.src, L.src_pitch, sizeof(TIn)) && vec_ok(g, gp, sizeof(TIn))) {
        GuidedAProd<TIn, true> pa{L.src, L.src_pitch, g, gp, L.rows, L.cols, 0.0f, 0.0f};
        guided_a_kernel<TIn, true><<<grid_for(A), kThreads, 0, st>>>(A, pa, ea);
    } else {
        GuidedAProd<TIn, false> pa{L.src, L.src_pitch, g, gp, L.rows, L.cols, 0.0f, 0.0f};
        guided_a_kernel<TIn, false><<<grid_for(A), kThreads, 0, st>>>(A, pa, ea);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    // Pass B over the coefficient grid -> output grid.
    Geo B;
    B.wV = L.wV;
    B.wH = L.wH;
    B.orows = A.orows + 1 - L.wV;
    B.ocols = A.ocols + 1 - L.wH;
    const int ncxb = (B.ocols + out_cols_per_cta(B.wH) - 1) / out_cols_per_cta(B.wH);
    B.strip_rows = default_strip(B.orows, ncxb, L.wV);
    B.ox_align = L.ox & 3;
    GuidedBProd pb{reinterpret_cast<const float2*>(L.coef), L.coef_pitch, A.orows, A.ocols};
    GuidedBEpi<TIn> eb{g, gp, L.dst, L.dst_pitch, L.out_dtype, L.oy, L.ox,
                       L.wV - 1, L.wH - 1, (float)n};
    guided_b_kernel<TIn><<<grid_for(B), kThreads, 0, st>>>(B, pb, eb);
    return cudaGetLastError();
}

cudaError_t launch_guided(const GuidedLaunch& L, cudaStream_t st)
{
    switch (L.in_dtype) {
    case U8: return launch_guided_t<uint8_t>(L, st);
    case F16: return launch_guided_t<__half>(L, st);
    case BF16: return launch_guided_t<__nv_bfloat16>(L, st);
    case F32: return launch_guided_t<float>(L, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace box
}  // namespace tucu

TUCU_DEFINE_ERROR_ACCESSOR(tucu_box_tu_error)
