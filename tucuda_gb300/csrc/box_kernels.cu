// box_kernels.cu -- BoxFilter2 and GuidedFilter2 kernels built on the
// one-pass window-sum strip (box_strip.cuh), and their launchers.
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
// (TU/cu/GuidedFilter.h:74-105), written as float2.
template <class TIn, bool VEC>
struct GuidedAProd
{
    static constexpr bool kCompensate = true;
    static constexpr int kPlanes = 2;  // p, g
    static constexpr int kPlaneBytes = 4 * sizeof(TIn);
    static constexpr bool kAsync = VEC;
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
    __device__ const void* plane_ptr(int k, int y, int x) const
    {
        return k == 0 ? row_ptr(p, p_pitch, y) + (size_t)x * sizeof(TIn)
                      : row_ptr(g, g_pitch, y) + (size_t)x * sizeof(TIn);
    }
    __device__ int plane_bytes(int, int nvalid, int) const { return nvalid * (int)sizeof(TIn); }
    __device__ void finish(Raw& r, int nvalid) const { r.valid = (1u << nvalid) - 1u; }
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
    static constexpr bool kCompensate = true;
    static constexpr int kPlanes = 2;  // columns 0-1, columns 2-3
    static constexpr int kPlaneBytes = 16;
    static constexpr bool kAsync = true;  // coefficient rows are 16-byte aligned
    struct Raw
    {
        float4 lo, hi;  // (a0,b0,a1,b1), (a2,b2,a3,b3)
    };
    const float2* coef;
    size_t pitch;
    int rows, cols;
    __device__ const void* plane_ptr(int k, int y, int x) const
    {
        return reinterpret_cast<const float2*>(row_ptr(coef, pitch, y)) + x + 2 * k;
    }
    __device__ int plane_bytes(int k, int nvalid, int) const
    {
        return k == 0 ? min(nvalid, 2) * 8 : max(nvalid - 2, 0) * 8;
    }
    __device__ void finish(Raw&, int) const {}
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
    __device__ void store4(int y, int x, const float (&s)[4][4], unsigned mask) const
    {
        float2* row = reinterpret_cast<float2*>(row_ptr(coef, pitch, y)) + x;
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
    int cls;  // store_class of dst, pitch, ox
};

// ---- kernels --------------------------------------------------------------------

constexpr int kGuidedCtas = 2;
constexpr int kGuidedWarpBytes = 6144;  // 48 KB per CTA: no opt-in needed

template <class Prod>
struct GuidedRing
{
    static constexpr int kDepth = Ring<Prod>::depth(kGuidedWarpBytes);
    static constexpr int kSmem = kWarps * kDepth * Ring<Prod>::kStepBytes;
};

template <class TIn, bool VEC>
__global__ void __launch_bounds__(kThreads, kGuidedCtas)
    guided_a_kernel(const __grid_constant__ Geo G, const __grid_constant__ GuidedAProd<TIn, VEC> prod0,
                    const __grid_constant__ GuidedAEpi epi0)
{
    using R = GuidedRing<GuidedAProd<TIn, VEC>>;
    char* ring = warp_ring(R::kSmem / kWarps);
    for_each_task(G, [&](auto cc, int xw, int y0, int nrows) {
        // Per-task anchors: the task's first pixel (any constant works; a
        // local one keeps the shifted values small).
        GuidedAProd<TIn, VEC> prod = prod0;
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

template <class TIn>
__global__ void __launch_bounds__(kThreads, kGuidedCtas)
    guided_b_kernel(const __grid_constant__ Geo G, const __grid_constant__ GuidedBProd prod,
                    const __grid_constant__ GuidedBEpi<TIn> epi)
{
    using R = GuidedRing<GuidedBProd>;
    char* ring = warp_ring(R::kSmem / kWarps);
    for_each_task(G, [&](auto cc, int xw, int y0, int nrows) {
        strip_body<decltype(cc)::value, 2, float, R::kDepth>(prod, epi, G.wV, G.wH, xw, y0, nrows, G.ocols,
                                                               ring, prod.cols, G.tg.restart);
    });
}

size_t plain_smem_bytes(int in_dtype)
{
    switch (in_dtype) {
    case U8: return PlainRing<uint8_t, true>::kSmem;
    case I32: return PlainRing<int32_t, true>::kSmem;
    case F16: return PlainRing<__half, true>::kSmem;
    case BF16: return PlainRing<__nv_bfloat16, true>::kSmem;
    case F32: return PlainRing<float, true>::kSmem;
    default: return 0;
    }
}

const void* batch_kernel(int in_dtype, int out_dtype, bool vec)
{
    const void* fn = vec ? typed_kernel(in_dtype, out_dtype, true) : nullptr;
    return fn ? fn : generic_kernel(in_dtype, vec, true);
}

// ---- launchers ------------------------------------------------------------------

static bool vec_ok(const void* p, size_t pitch, int es)
{
    const size_t a = (size_t)kCPT * es;
    return (reinterpret_cast<uintptr_t>(p) % a) == 0 && (pitch % a) == 0;
}

// Warp tasks for an image: the strip height (a multiple of the restart
// period) that minimises rounds x (strip + window set-up), where a round is
// one task for every warp the grid keeps resident.
TaskGrid plan_tasks(int orows, int ocols, int wV, int wH, int strip_rows, int ctas_per_sm,
                    int restart, int copies)
{
    TaskGrid t;
    t.restart = restart;
    t.nwc = (ocols + out_cols_per_warp(wH) - 1) / out_cols_per_warp(wH);
    const long warps = (long)ctas_per_sm * sm_count() * kWarps;
    auto tasks_of = [&](int strip) { return (long)t.nwc * ((orows + strip - 1) / strip) * copies; };
    if (strip_rows > 0) {
        t.strip_rows = (strip_rows + 15) / 16 * 16;
    } else {
        // Bands that are multiples of the restart period: whole rounds of
        // warp tasks x (band + wV).
        t.strip_rows = restart;
        double best = 1e300;
        for (int k = 1; k <= 32; ++k) {
            const int strip = k * restart;
            const long rounds = (tasks_of(strip) + warps - 1) / warps;
            const double cost = (double)rounds * (std::min(strip, orows) + wV);
            if (cost < best) {
                best = cost;
                t.strip_rows = strip;
            }
            if (strip >= orows)
                break;
        }
        // An image too small to give every SM a CTA of warp tasks gets bands
        // shorter than the restart period (halves, quarters, down to 16
        // rows): a band inside a restart block replays the rows of the block
        // above it, which costs little next to the idle SMs it fills.
        const long fill = (long)sm_count() * kWarps * 3 / 4;
        while (t.strip_rows > 16 && t.strip_rows <= restart && tasks_of(t.strip_rows) < fill)
            t.strip_rows /= 2;
    }
    t.ntask = (int)tasks_of(t.strip_rows) / copies;
    return t;
}

static dim3 grid_for(const Geo& G, int ctas_per_sm)
{
    const long want = (G.tg.ntask + kWarps - 1) / kWarps;
    return dim3((unsigned)std::max(1L, std::min(want, (long)ctas_per_sm * sm_count())));
}

cudaError_t launch_box(const BoxLaunch& L, cudaStream_t st)
{
    Geo G;
    G.wV = L.wV;
    G.wH = L.wH;
    G.orows = L.rows + 1 - L.wV;
    G.ocols = L.cols + 1 - L.wH;
    if (L.in_dtype < U8 || L.in_dtype > I32)
        return cudaErrorInvalidValue;
    const bool vec = vec_ok(L.src, L.src_pitch, dtype_size(L.in_dtype));
    // Integer sums are exact in any order, so their strips may be as short
    // as 16 rows (more warp tasks for small images); float sums keep the
    // 64-row restart grid the batched launch uses, so both agree bit for bit.
    const bool integral = L.in_dtype == U8 || L.in_dtype == I32;
    G.tg = plan_tasks(G.orows, G.ocols, L.wV, L.wH, L.strip_rows, kBoxCtas, integral ? 16 : kRestart);
    const void* fn = vec ? typed_kernel(L.in_dtype, L.out_dtype, false) : nullptr;
    if (!fn)
        fn = generic_kernel(L.in_dtype, vec, false);
    BoxArgs A;
    A.src = L.src;
    A.src_pitch = L.src_pitch;
    A.rows = L.rows;
    A.cols = L.cols;
    A.dst = L.dst;
    A.dst_pitch = L.dst_pitch;
    A.out_dtype = L.out_dtype;
    A.oy = L.oy;
    A.ox = L.ox;
    A.normalize = L.normalize;
    A.inv_n = 1.0f / (float)(L.wV * L.wH);
    A.cls = store_class(L.dst, L.dst_pitch, L.ox, dtype_size(L.out_dtype));
    void* args[] = {&G, &A};
    return cudaLaunchKernel(fn, grid_for(G, kBoxCtas), dim3(kThreads), args, plain_smem_bytes(L.in_dtype), st);
}

// Float restart period of the guided passes, from the image size alone
// (every caller of the same image gets the same bits): small images take
// short restart blocks, so they split into enough warp tasks to fill the GPU;
// large ones long blocks, so the window set-up rows stay a small fraction.
static int guided_restart(int rows, int cols)
{
    const long px = (long)rows * cols;
    return px >= 16000000 ? 64 : px >= 4000000 ? 32 : 16;
}

template <class TIn>
static cudaError_t launch_guided_t(const GuidedLaunch& L, cudaStream_t st)
{
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
    const bool vec = vec_ok(L.src, L.src_pitch, sizeof(TIn)) && vec_ok(g, gp, sizeof(TIn));
    A.tg = plan_tasks(A.orows, A.ocols, L.wV, L.wH, 0, kGuidedCtas, restart);
    if (vec) {
        GuidedAProd<TIn, true> pa{L.src, L.src_pitch, g, gp, L.rows, L.cols, 0.0f, 0.0f};
        guided_a_kernel<TIn, true><<<grid_for(A, kGuidedCtas), kThreads, GuidedRing<GuidedAProd<TIn, true>>::kSmem, st>>>(A, pa, ea);
    } else {
        GuidedAProd<TIn, false> pa{L.src, L.src_pitch, g, gp, L.rows, L.cols, 0.0f, 0.0f};
        guided_a_kernel<TIn, false><<<grid_for(A, kGuidedCtas), kThreads, GuidedRing<GuidedAProd<TIn, false>>::kSmem, st>>>(A, pa, ea);
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
    B.tg = plan_tasks(B.orows, B.ocols, L.wV, L.wH, 0, kGuidedCtas, restart);
    GuidedBProd pb{reinterpret_cast<const float2*>(L.coef), L.coef_pitch, A.orows, A.ocols};
    GuidedBEpi<TIn> eb{g, gp, L.dst, L.dst_pitch, L.out_dtype, L.oy, L.ox,
                       L.wV - 1, L.wH - 1, (float)n,
                       store_class(L.dst, L.dst_pitch, L.ox, dtype_size(L.out_dtype))};
    guided_b_kernel<TIn><<<grid_for(B, kGuidedCtas), kThreads, GuidedRing<GuidedBProd>::kSmem, st>>>(B, pb, eb);
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
