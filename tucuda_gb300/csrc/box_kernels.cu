// box_kernels.cu -- BoxFilter2 and GuidedFilter2 kernels built on the
// one-pass window-sum strip (box_strip.cuh), and their launchers.
#include "box_kernels.h"
#include "box_strip.cuh"

namespace tucu
{
namespace box
{

// ---- producers ----------------------------------------------------------------

// Four consecutive pixels of row y starting at x as Acc, zero outside.
template <class TIn, class Acc, bool VEC>
__device__ __forceinline__ void load_row4(const void* base, size_t pitch, int rows, int cols,
                                          int y, int x, Acc (&v)[kCPT])
{
    if (y < 0 || y >= rows || x >= cols) {
#pragma unroll
        for (int j = 0; j < kCPT; ++j)
            v[j] = Acc(0);
        return;
    }
    const TIn* row = reinterpret_cast<const TIn*>(row_ptr(base, pitch, y));
    if (VEC && x + kCPT <= cols) {
        if constexpr (sizeof(TIn) == 1) {
            const uint32_t u = __ldg(reinterpret_cast<const uint32_t*>(row + x));
#pragma unroll
            for (int j = 0; j < kCPT; ++j)
                v[j] = Acc((u >> (8 * j)) & 0xff);
        } else if constexpr (sizeof(TIn) == 2) {
            const uint2 u = __ldg(reinterpret_cast<const uint2*>(row + x));
            const TIn* h = reinterpret_cast<const TIn*>(&u);
#pragma unroll
            for (int j = 0; j < kCPT; ++j)
                v[j] = Acc(to_float(h[j]));
        } else {
            if constexpr (sizeof(Acc) == 4 && std::is_same<TIn, int32_t>::value) {
                const int4 u = __ldg(reinterpret_cast<const int4*>(row + x));
                v[0] = Acc(u.x); v[1] = Acc(u.y); v[2] = Acc(u.z); v[3] = Acc(u.w);
            } else {
                const float4 u = __ldg(reinterpret_cast<const float4*>(row + x));
                v[0] = Acc(u.x); v[1] = Acc(u.y); v[2] = Acc(u.z); v[3] = Acc(u.w);
            }
        }
        return;
    }
#pragma unroll
    for (int j = 0; j < kCPT; ++j) {
        if constexpr (std::is_same<TIn, int32_t>::value || std::is_same<TIn, uint8_t>::value)
            v[j] = (x + j < cols) ? Acc(row[x + j]) : Acc(0);
        else
            v[j] = (x + j < cols) ? Acc(to_float(row[x + j])) : Acc(0);
    }
}

template <class TIn, class Acc, bool VEC>
struct PlainProd
{
    const void* src;
    size_t pitch;
    int rows, cols;
    __device__ void load(int y, int x, Acc (&raw)[1][kCPT]) const
    {
        load_row4<TIn, Acc, VEC>(src, pitch, rows, cols, y, x, raw[0]);
    }
    __device__ void expand(const Acc (&r)[1], Acc (&q)[1]) const { q[0] = r[0]; }
};

template <class Acc>
struct PlainEpi
{
    void* dst;
    size_t pitch;
    int dtype, oy, ox;
    int normalize;
    float n;
    __device__ void store(int y, int x, const Acc (&s)[1]) const
    {
        char* row = row_ptr(dst, pitch, y + oy);
        if (normalize)
            store_px(row, x + ox, dtype, __fdiv_rn((float)s[0], n));
        else if constexpr (std::is_same<Acc, int>::value)
            store_i32(row, x + ox, dtype, s[0]);
        else
            store_px(row, x + ox, dtype, s[0]);
    }
};

// Guided pass A: sums of (p', g', p'g', g'g') with p' = p - Kp, g' = g - Kg
// (per-strip anchors, so the variance term does not cancel); the epilogue
// turns them into the coefficients (a, b) of init_coeffs
// (TU/cu/GuidedFilter.h:74-105), written as float2.
template <class TIn, bool VEC>
struct GuidedAProd
{
    const void* p;
    size_t p_pitch;
    const void* g;
    size_t g_pitch;
    int rows, cols;
    float kp, kg;
    __device__ void load(int y, int x, float (&raw)[2][kCPT]) const
    {
        load_row4<TIn, float, VEC>(p, p_pitch, rows, cols, y, x, raw[0]);
        load_row4<TIn, float, VEC>(g, g_pitch, rows, cols, y, x, raw[1]);
        // Outside the image p' and g' must be zero, not -K.
        const bool in = y >= 0 && y < rows;
#pragma unroll
        for (int j = 0; j < kCPT; ++j) {
            const bool ok = in && x + j < cols;
            raw[0][j] = ok ? raw[0][j] - kp : 0.0f;
            raw[1][j] = ok ? raw[1][j] - kg : 0.0f;
        }
    }
    __device__ void expand(const float (&r)[2], float (&q)[4]) const
    {
        q[0] = r[0];
        q[1] = r[1];
        q[2] = r[0] * r[1];
        q[3] = r[1] * r[1];
    }
};

struct GuidedAEpi
{
    float2* coef;
    size_t pitch;  // bytes
    float n, inv_n, sq_e, kp, kg;
    int self;
    __device__ void store(int y, int x, const float (&s)[4]) const
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
        reinterpret_cast<float2*>(row_ptr(coef, pitch, y))[x] = make_float2(a, b);
    }
};

// Guided pass B: sums of (a, b); out = (A*g + B)/n with g at the window
// centre (trans_guides, TU/cu/GuidedFilter.h:107-125).
struct GuidedBProd
{
    const float2* coef;
    size_t pitch;
    int rows, cols;
    __device__ void load(int y, int x, float (&raw)[2][kCPT]) const
    {
        if (y < 0 || y >= rows) {
#pragma unroll
            for (int j = 0; j < kCPT; ++j)
                raw[0][j] = raw[1][j] = 0.0f;
            return;
        }
        const float2* row = reinterpret_cast<const float2*>(row_ptr(coef, pitch, y));
        if (x + kCPT <= cols) {
            const float4 a = __ldg(reinterpret_cast<const float4*>(row + x));
            const float4 b = __ldg(reinterpret_cast<const float4*>(row + x + 2));
            raw[0][0] = a.x; raw[1][0] = a.y; raw[0][1] = a.z; raw[1][1] = a.w;
            raw[0][2] = b.x; raw[1][2] = b.y; raw[0][3] = b.z; raw[1][3] = b.w;
            return;
        }
#pragma unroll
        for (int j = 0; j < kCPT; ++j) {
            const float2 v = (x + j < cols) ? row[x + j] : make_float2(0.0f, 0.0f);
            raw[0][j] = v.x;
            raw[1][j] = v.y;
        }
    }
    __device__ void expand(const float (&r)[2], float (&q)[2]) const
    {
        q[0] = r[0];
        q[1] = r[1];
    }
};

template <class TIn>
struct GuidedBEpi
{
    const void* g;
    size_t g_pitch;
    void* dst;
    size_t pitch;
    int dtype, oy, ox, gy, gx;
    float n;
    __device__ void store(int y, int x, const float (&s)[2]) const
    {
        const float gv = load_px<TIn>(row_ptr(g, g_pitch, y + gy), x + gx);
        store_px(row_ptr(dst, pitch, y + oy), x + ox, dtype, __fdiv_rn(fmaf(s[0], gv, s[1]), n));
    }
};

// ---- kernels --------------------------------------------------------------------

struct Geo
{
    int wV, wH;
    int orows, ocols;   // output extent (valid coords)
    int strip_rows;
};

template <class TIn, class Acc, bool VEC>
__global__ void __launch_bounds__(kThreads)
    box_kernel(const __grid_constant__ Geo G, const __grid_constant__ PlainProd<TIn, Acc, VEC> prod,
               const __grid_constant__ PlainEpi<Acc> epi)
{
    __shared__ __align__(16) unsigned char smem[sizeof(Smem<1, Acc>)];
    const int x0 = blockIdx.x * out_cols_per_cta(G.wH);
    const int y0 = blockIdx.y * G.strip_rows;
    const int nrows = min(G.strip_rows, G.orows - y0);
    run_strip<1, 1, Acc, 8>(prod, epi, G.wV, G.wH, x0, y0, nrows, G.ocols, smem);
}

template <class TIn, bool VEC>
__global__ void __launch_bounds__(kThreads)
    guided_a_kernel(const __grid_constant__ Geo G, GuidedAProd<TIn, VEC> prod, GuidedAEpi epi)
{
    __shared__ __align__(16) unsigned char smem[sizeof(Smem<4, float>)];
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
    run_strip<4, 2, float, 2>(prod, epi, G.wV, G.wH, x0, y0, nrows, G.ocols, smem);
}

template <class TIn>
__global__ void __launch_bounds__(kThreads)
    guided_b_kernel(const __grid_constant__ Geo G, const __grid_constant__ GuidedBProd prod,
                    const __grid_constant__ GuidedBEpi<TIn> epi)
{
    __shared__ __align__(16) unsigned char smem[sizeof(Smem<2, float>)];
    const int x0 = blockIdx.x * out_cols_per_cta(G.wH);
    const int y0 = blockIdx.y * G.strip_rows;
    const int nrows = min(G.strip_rows, G.orows - y0);
    run_strip<2, 2, float, 4>(prod, epi, G.wV, G.wH, x0, y0, nrows, G.ocols, smem);
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
                      (float)(L.wV * L.wH)};
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
    strip = max(strip, 16);
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
    G.strip_rows = L.strip_rows > 0 ? L.strip_rows : default_strip(G.orows, ncx, L.wV);
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
    A.strip_rows = L.strip_rows > 0 ? L.strip_rows : default_strip(A.orows, ncxa, L.wV);
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
    B.strip_rows = L.strip_rows > 0 ? L.strip_rows : default_strip(B.orows, ncxb, L.wV);
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
