/*
 * tucu_oracle.c -- CPU oracle for the TUCuda 2D-filter hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, on the CPU, the arithmetic of
 * libTUCuda's separable FIR convolver, Gaussian lobe design, running-sum box
 * filter and guided filter.  It is the checker for the CUDA kernels in
 * tucuda_gb300/csrc and the timed CPU baseline of bench.py.  Nothing on the
 * product path links, loads or calls it.
 *
 * Three variants are provided:
 *   - "ref-faithful" float32: same float lobes, same tap pairing and the same
 *     per-output evaluation order as the reference's device code
 *     (TU/cu/FIRFilter.h:66-176), with each "sum + product" step written as an
 *     explicit fmaf() the way the CUDA kernels evaluate it; box sums in the
 *     reference's 16-row / 16-column tile order (TU/cu/BoxFilter.h:175-194,
 *     246-296, 542-583); guided coefficients with the reference's formula
 *     (TU/cu/GuidedFilter.h:59-125).
 *   - FP64: lobes designed in double (sizes from the reference's truncation
 *     rule) and every sum accumulated in double.  This is the error oracle.
 *   - exact integer box sums (int64) for bit-exact checks of int32 output.
 *
 * Parity pins: the lobe design and truncation rule, the FIR index convention
 * for symmetric lobes and the guided-filter coefficient functors are checked
 * against fixtures produced by compiling the reference's own host code
 * (tests/golden/make_golden.py).  The box and guided window geometry and the
 * antisymmetric FIR sign convention are restated from reading the reference
 * and checked by known-answer tests only.
 *
 * Build with -ffp-contract=off so that x86-64 and aarch64 give identical
 * results: every fused multiply-add here is an explicit fmaf()/fma().
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define TUO_LOBE_MAX 17

static void set_threads(int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0)
        omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

int tuo_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------
 * Lobe design
 * ---------------------------------------------------------------------- */

/* Truncation rule of detail::lobeSize (FIRGaussianConvolver.cu:52-98).
 * Threshold = 1% of the largest |lobe[i]| over all 17 entries; the kept length
 * is one past the last entry strictly above it, rounded up to 2^n+1 (even
 * kernels) or 2^n (odd kernels).  size_t arithmetic is kept on purpose: an
 * all-zero lobe wraps the index and yields the largest size, as there. */
size_t tuo_lobe_size(const float* lobe, int even)
{
    const size_t sizMax = TUO_LOBE_MAX;
    const float  epsilon = 0.01f;
    float th = 0.0f;
    for (size_t i = sizMax; i-- > 0;)
        if (fabsf(lobe[i]) >= th)
            th = fabsf(lobe[i]);
    th *= epsilon;

    size_t siz;
    for (siz = sizMax; siz-- > 0;)
        if (fabsf(lobe[siz]) > th) {
            ++siz;
            break;
        }

    if (even)
        return siz <= 2 ? 3 : siz <= 5 ? 5 : siz <= 9 ? 9 : 17;
    return siz <= 1 ? 2 : siz <= 4 ? 4 : siz <= 8 ? 8 : 16;
}

/* Float lobe design of FIRGaussianConvolver2<T>::initialize(sigma, lobe0,
 * lobe1, lobe2) (FIRGaussianConvolver.h:123-170).  Lobes are stored outermost
 * tap first.  lobe1 takes lb1[L..1] but is normalised by sum_{i<L} 2 i lb1[i],
 * which leaves lb1[L] out of the norm exactly as the reference does. */
void tuo_gauss_lobes(float sigma, float* lobe0, int* n0, float* lobe1, int* n1,
                     float* lobe2, int* n2)
{
    float lb0[TUO_LOBE_MAX], lb1[TUO_LOBE_MAX], lb2[TUO_LOBE_MAX];
    for (size_t i = 0; i < TUO_LOBE_MAX; ++i) {
        const float dx = (float)i / sigma, dxdx = dx * dx;
        lb0[i] = expf(-0.5f * dxdx);
        lb1[i] = -dx * lb0[i];
        lb2[i] = (dxdx - 1.0f) * lb0[i];
    }

    size_t L = tuo_lobe_size(lb0, 1);
    float sum = lb0[0];
    for (size_t i = 1; i < L; ++i)
        sum += 2.0f * lb0[i];
    for (size_t i = 0; i < L; ++i)
        lobe0[i] = lb0[L - 1 - i] / fabsf(sum);
    *n0 = (int)L;

    L = tuo_lobe_size(lb1, 0);
    sum = 0.0f;
    for (size_t i = 0; i < L; ++i)
        sum += 2.0f * (float)i * lb1[i];
    for (size_t i = 0; i < L; ++i)
        lobe1[i] = lb1[L - i] / fabsf(sum);
    *n1 = (int)L;

    L = tuo_lobe_size(lb2, 1);
    sum = 0.0f;
    for (size_t i = 1; i < L; ++i)
        sum += (float)(i * i) * lb2[i];
    for (size_t i = 0; i < L; ++i)
        lobe2[i] = lb2[L - 1 - i] / fabsf(sum);
    *n2 = (int)L;
}

/* The same lobes designed in double.  Lengths come from the reference's float
 * truncation rule so that the FP64 filter has the same support. */
void tuo_gauss_lobes_f64(float sigma, double* lobe0, int* n0, double* lobe1,
                         int* n1, double* lobe2, int* n2)
{
    float f0[TUO_LOBE_MAX], f1[TUO_LOBE_MAX], f2[TUO_LOBE_MAX];
    tuo_gauss_lobes(sigma, f0, n0, f1, n1, f2, n2);

    double lb0[TUO_LOBE_MAX], lb1[TUO_LOBE_MAX], lb2[TUO_LOBE_MAX];
    for (int i = 0; i < TUO_LOBE_MAX; ++i) {
        const double dx = (double)i / (double)sigma, dxdx = dx * dx;
        lb0[i] = exp(-0.5 * dxdx);
        lb1[i] = -dx * lb0[i];
        lb2[i] = (dxdx - 1.0) * lb0[i];
    }
    int L = *n0;
    double sum = lb0[0];
    for (int i = 1; i < L; ++i)
        sum += 2.0 * lb0[i];
    for (int i = 0; i < L; ++i)
        lobe0[i] = lb0[L - 1 - i] / fabs(sum);

    L = *n1;
    sum = 0.0;
    for (int i = 0; i < L; ++i)
        sum += 2.0 * i * lb1[i];
    for (int i = 0; i < L; ++i)
        lobe1[i] = lb1[L - i] / fabs(sum);

    L = *n2;
    sum = 0.0;
    for (int i = 1; i < L; ++i)
        sum += (double)(i * i) * lb2[i];
    for (int i = 0; i < L; ++i)
        lobe2[i] = lb2[L - 1 - i] / fabs(sum);
}

/* ------------------------------------------------------------------------
 * Separable FIR (FIRFilter2)
 * ---------------------------------------------------------------------- */

/* One output of device::convolve (FIRFilter.h:66-176).  v points at the
 * outermost left tap; the window is v[0 .. 2*LS].  Lobe lengths 3,5,9,17 are
 * symmetric (centre tap lobe[LS]); 2,4,8,16 antisymmetric with no centre.
 * Evaluation: acc = lobe[0]*pair0, then acc = fma(lobe[k], pair_k, acc),
 * centre last. */
static inline float fir_tap_f32(const float* v, long step, const float* lobe, int L)
{
    const int LS = L & ~1;
    const int sym = L & 1;
    float pair = sym ? v[0] + v[2 * LS * step] : v[0] - v[2 * LS * step];
    float acc = lobe[0] * pair;
    for (int k = 1; k < LS; ++k) {
        pair = sym ? v[k * step] + v[(2 * LS - k) * step]
                   : v[k * step] - v[(2 * LS - k) * step];
        acc = fmaf(lobe[k], pair, acc);
    }
    if (sym)
        acc = fmaf(lobe[LS], v[LS * step], acc);
    return acc;
}

/* The reference's tap expression (FIRFilter.h:66-176) as nvcc 13.0 compiles
 * it for sm_103a with its default flags, measured on a GB300 with the
 * reference's own device code (oracle/ref_device.cu,
 * tests/golden/ref_device_vectors.json): the second pair's product is
 * rounded, the outermost pair is fused into it, and every further pair and
 * the centre tap follow as FMAs.  (fir_tap_f32 above rounds the outermost
 * product instead and fuses the second pair into it: one rounding of the first
 * step apart.)  out[i] = taps of in[i .. i + 2LS] for i < n - 2LS; returns -1
 * for an unsupported lobe length. */
int tuo_fir_row_nvcc_f32(const float* in, int n, const float* lobe, int L, float* out)
{
    if (!(L == 2 || L == 3 || L == 4 || L == 5 || L == 8 || L == 9 || L == 16 || L == 17))
        return -1;
    const int LS = L & ~1;
    const int sym = L & 1;
    for (int i = 0; i + 2 * LS < n; ++i) {
        const float* v = in + i;
        float pr[17];
        for (int k = 0; k < LS; ++k)
            pr[k] = sym ? v[k] + v[2 * LS - k] : v[k] - v[2 * LS - k];
        float acc = fmaf(lobe[0], pr[0], lobe[1] * pr[1]);
        for (int k = 2; k < LS; ++k)
            acc = fmaf(lobe[k], pr[k], acc);
        if (sym)
            acc = fmaf(lobe[LS], v[LS], acc);
        out[i] = acc;
    }
    return 0;
}

static inline double fir_tap_f64(const double* v, long step, const double* lobe, int L)
{
    const int LS = L & ~1;
    const int sym = L & 1;
    double acc = 0.0;
    for (int k = 0; k < LS; ++k) {
        const double pair = sym ? v[k * step] + v[(2 * LS - k) * step]
                                : v[k * step] - v[(2 * LS - k) * step];
        acc += lobe[k] * pair;
    }
    if (sym)
        acc += lobe[LS] * v[LS * step];
    return acc;
}

static int lobe_ok(int L)
{
    return L == 2 || L == 3 || L == 4 || L == 5 || L == 8 || L == 9 || L == 16 ||
           L == 17;
}

/* FIRFilter2::convolve (FIRFilter.h:298-377): returns without touching out
 * when rows <= 2*LS_V or cols <= 2*LS_H; otherwise writes the valid region
 * (rows-2LS_V) x (cols-2LS_H) at (LS_V, LS_H) when shift, else at (0,0).
 * Strides are in elements.  Returns 0 on success, 1 when nothing was written,
 * -1 for an unsupported lobe length. */
int tuo_fir_f32(const float* in, long in_stride, int rows, int cols,
                const float* lobeH, int LH, const float* lobeV, int LV,
                float* out, long out_stride, int shift, int nthreads)
{
    if (!lobe_ok(LH) || !lobe_ok(LV))
        return -1;
    const int lsH = LH & ~1, lsV = LV & ~1;
    if (rows <= 2 * lsV || cols <= 2 * lsH)
        return 1;
    const int mc = cols - 2 * lsH, orows = rows - 2 * lsV;
    float* mid = (float*)malloc(sizeof(float) * (size_t)rows * mc);
    if (!mid)
        return -2;
    set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < rows; ++y)
        for (int x = 0; x < mc; ++x)
            mid[(size_t)y * mc + x] = fir_tap_f32(in + (size_t)y * in_stride + x, 1, lobeH, LH);
    const int oy = shift ? lsV : 0, ox = shift ? lsH : 0;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < orows; ++y)
        for (int x = 0; x < mc; ++x)
            out[(size_t)(y + oy) * out_stride + x + ox] =
                fir_tap_f32(mid + (size_t)y * mc + x, mc, lobeV, LV);
    free(mid);
    return 0;
}

int tuo_fir_f64(const double* in, long in_stride, int rows, int cols,
                const double* lobeH, int LH, const double* lobeV, int LV,
                double* out, long out_stride, int shift, int nthreads)
{
    if (!lobe_ok(LH) || !lobe_ok(LV))
        return -1;
    const int lsH = LH & ~1, lsV = LV & ~1;
    if (rows <= 2 * lsV || cols <= 2 * lsH)
        return 1;
    const int mc = cols - 2 * lsH, orows = rows - 2 * lsV;
    double* mid = (double*)malloc(sizeof(double) * (size_t)rows * mc);
    if (!mid)
        return -2;
    set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < rows; ++y)
        for (int x = 0; x < mc; ++x)
            mid[(size_t)y * mc + x] = fir_tap_f64(in + (size_t)y * in_stride + x, 1, lobeH, LH);
    const int oy = shift ? lsV : 0, ox = shift ? lsH : 0;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < orows; ++y)
        for (int x = 0; x < mc; ++x)
            out[(size_t)(y + oy) * out_stride + x + ox] =
                fir_tap_f64(mid + (size_t)y * mc + x, mc, lobeV, LV);
    free(mid);
    return 0;
}

/* ------------------------------------------------------------------------
 * Box filter (BoxFilter2 with box_convolver)
 * ---------------------------------------------------------------------- */

/* Exact window sums: out[y][x] = sum_{dy<wV, dx<wH} in[y+dy][x+dx] for the
 * (rows+1-wV) x (cols+1-wH) valid outputs, placed at (wV/2, wH/2) when shift
 * (BoxFilter.h:487-509, 542-583).  No-op when the image is smaller than the
 * window.  Integer input, int64 output. */
int tuo_box_i64(const int32_t* in, long in_stride, int rows, int cols, int wV,
                int wH, int64_t* out, long out_stride, int shift, int nthreads)
{
    if (wV < 1 || wH < 1)
        return -1;
    if (rows < wV || cols < wH)
        return 1;
    const int orows = rows + 1 - wV, ocols = cols + 1 - wH;
    int64_t* vs = (int64_t*)malloc(sizeof(int64_t) * (size_t)orows * cols);
    if (!vs)
        return -2;
    set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < orows; ++y)
        for (int x = 0; x < cols; ++x) {
            int64_t s = 0;
            for (int k = 0; k < wV; ++k)
                s += in[(size_t)(y + k) * in_stride + x];
            vs[(size_t)y * cols + x] = s;
        }
    const int oy = shift ? wV / 2 : 0, ox = shift ? wH / 2 : 0;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < orows; ++y) {
        const int64_t* v = vs + (size_t)y * cols;
        int64_t s = 0;
        for (int k = 0; k < wH; ++k)
            s += v[k];
        out[(size_t)(y + oy) * out_stride + ox] = s;
        for (int x = 1; x < ocols; ++x) {
            s += v[x - 1 + wH] - v[x - 1];
            out[(size_t)(y + oy) * out_stride + x + ox] = s;
        }
    }
    free(vs);
    return 0;
}

/* One column of box_convolver::operator() (BoxFilter.h:181-193) over a tile
 * of up to 16 outputs: out[0] = sum_{y<w} in[y] left to right, then
 * out[y] = (out[y-1] + in[y-1+w]) - in[y-1]. */
static inline void box_tile_f32(const float* in, long step, int w, int ye,
                                float* out, long ostep)
{
    float s = in[0];
    for (int y = 1; y < w; ++y)
        s += in[y * step];
    out[0] = s;
    for (int y = 1; y < ye; ++y) {
        s = (s + in[(y - 1 + w) * step]) - in[(y - 1) * step];
        out[y * ostep] = s;
    }
}

/* One box_filter pass (BoxFilter.h:246-296): for every column of `in`
 * (rows x cols), window sums of w rows restarted on every 16-row tile, written
 * transposed into out (cols x (rows+1-w)). */
static void box_pass_f32(const float* in, long in_stride, int rows, int cols, int w,
                         float* out, long out_stride)
{
    const int T = 16;
    const int orows = rows + 1 - w;
#pragma omp parallel for schedule(static)
    for (int x = 0; x < cols; ++x)
        for (int y0 = 0; y0 < orows; y0 += T) {
            const int ysiz = (T + w - 1 < rows - y0) ? T + w - 1 : rows - y0;
            const int ye = ysiz - w + 1;
            box_tile_f32(in + (size_t)y0 * in_stride + x, in_stride, w, ye,
                         out + (size_t)x * out_stride + y0, 1);
        }
}

/* One vertical pass alone (the first half of tuo_box_f32): window sums of w
 * rows of every column of in (rows x cols) in the reference's 16-row tiles,
 * written transposed into out (cols x (rows+1-w), out_stride elements per
 * column).  Returns 1 without writing when rows < w. */
int tuo_box_pass_f32(const float* in, long in_stride, int rows, int cols, int w, float* out,
                     long out_stride, int nthreads)
{
    if (w < 1)
        return -1;
    if (rows < w)
        return 1;
    set_threads(nthreads);
    box_pass_f32(in, in_stride, rows, cols, w, out, out_stride);
    return 0;
}

/* Float box sums in the reference's order: vertical pass into a transposed
 * buffer, then the same kernel horizontally (BoxFilter.h:542-583). */
int tuo_box_f32(const float* in, long in_stride, int rows, int cols, int wV,
                int wH, float* out, long out_stride, int shift, int nthreads)
{
    if (wV < 1 || wH < 1)
        return -1;
    if (rows < wV || cols < wH)
        return 1;
    const int orows = rows + 1 - wV, ocols = cols + 1 - wH;
    float* buf = (float*)malloc(sizeof(float) * (size_t)cols * orows);
    float* res = (float*)malloc(sizeof(float) * (size_t)ocols * orows);
    if (!buf || !res) {
        free(buf);
        free(res);
        return -2;
    }
    set_threads(nthreads);
    box_pass_f32(in, in_stride, rows, cols, wV, buf, orows);   /* buf: cols x orows */
    box_pass_f32(buf, orows, cols, orows, wH, res, ocols);     /* res: orows x ocols */
    const int oy = shift ? wV / 2 : 0, ox = shift ? wH / 2 : 0;
    for (int y = 0; y < orows; ++y)
        memcpy(out + (size_t)(y + oy) * out_stride + ox, res + (size_t)y * ocols,
               sizeof(float) * ocols);
    free(buf);
    free(res);
    return 0;
}

int tuo_box_f64(const double* in, long in_stride, int rows, int cols, int wV,
                int wH, double* out, long out_stride, int shift, int nthreads)
{
    if (wV < 1 || wH < 1)
        return -1;
    if (rows < wV || cols < wH)
        return 1;
    const int orows = rows + 1 - wV, ocols = cols + 1 - wH;
    const int oy = shift ? wV / 2 : 0, ox = shift ? wH / 2 : 0;
    set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < orows; ++y)
        for (int x = 0; x < ocols; ++x) {
            double s = 0.0;
            for (int dy = 0; dy < wV; ++dy)
                for (int dx = 0; dx < wH; ++dx)
                    s += in[(size_t)(y + dy) * in_stride + x + dx];
            out[(size_t)(y + oy) * out_stride + x + ox] = s;
        }
    return 0;
}

/* ------------------------------------------------------------------------
 * Guided filter (GuidedFilter2)
 * ---------------------------------------------------------------------- */

/* init_coeffs<T>(n, e) (GuidedFilter.h:74-105) on window sums
 * (Sp, Sg, Spg, Sgg): e is squared internally, n = wV*wH. */
static inline void guided_coeffs_f32(size_t n, float sq_e, const float* s, float* a, float* b)
{
    const float fn = (float)n;
    const float num = fn * s[2] - s[0] * s[1];
    const float den = fn * (s[3] + fn * sq_e) - s[1] * s[1];
    *a = num / den;
    *b = (s[0] - *a * s[1]) / fn;
}

/* Self-guided overload on (Sp, Spp).  The reference's b uses Spp
 * (params.y), not Sp (GuidedFilter.h:97); that is reproduced here. */
static inline void guided_self_coeffs_f32(size_t n, float sq_e, const float* s, float* a, float* b)
{
    const float fn = (float)n;
    const float var = fn * s[1] - s[0] * s[0];
    *a = var / (var + (float)(n * n) * sq_e);
    *b = (s[0] - *a * s[1]) / fn;
}

/* Reference-faithful float guided filter (GuidedFilter.h:224-344).
 * guide == NULL selects the self-guided overload.  Output
 * (rows-2(wV-1)) x (cols-2(wH-1)) at (wV-1, wH-1) when shift, else (0,0):
 * out = (sum(a)*g + sum(b)) / n with g at the window centre.  No-op when
 * rows == 0; returns 1 without writing when the image is smaller than
 * 2w-1 in either direction. */
int tuo_guided_f32(const float* p, long p_stride, const float* g, long g_stride,
                   int rows, int cols, int wV, int wH, float e, float* out,
                   long out_stride, int shift, int nthreads)
{
    if (wV < 1 || wH < 1)
        return -1;
    if (rows <= 0 || rows < 2 * wV - 1 || cols < 2 * wH - 1)
        return 1;
    const int self = (g == NULL);
    const int nq = self ? 2 : 4;
    const size_t n = (size_t)wV * wH;
    const float sq_e = e * e;
    const int cr = rows + 1 - wV, cc = cols + 1 - wH;     /* coefficient grid */
    const int orr = cr + 1 - wV, oc = cc + 1 - wH;        /* output grid */
    set_threads(nthreads);

    float* q = (float*)malloc(sizeof(float) * (size_t)rows * cols);
    float* sums[4] = {0, 0, 0, 0};
    float* ab[2];
    float* abs_[2];
    for (int i = 0; i < nq; ++i)
        sums[i] = (float*)malloc(sizeof(float) * (size_t)cr * cc);
    for (int i = 0; i < 2; ++i) {
        ab[i] = (float*)malloc(sizeof(float) * (size_t)cr * cc);
        abs_[i] = (float*)malloc(sizeof(float) * (size_t)orr * oc);
    }
    /* init_params (GuidedFilter.h:59-72) per quantity, box-summed one at a time
     * (the vec components are independent sums). */
    for (int qi = 0; qi < nq; ++qi) {
#pragma omp parallel for schedule(static)
        for (int y = 0; y < rows; ++y)
            for (int x = 0; x < cols; ++x) {
                const float pv = p[(size_t)y * p_stride + x];
                const float gv = self ? pv : g[(size_t)y * g_stride + x];
                float v;
                if (self)
                    v = qi == 0 ? pv : pv * pv;
                else
                    v = qi == 0 ? pv : qi == 1 ? gv : qi == 2 ? pv * gv : gv * gv;
                q[(size_t)y * cols + x] = v;
            }
        tuo_box_f32(q, cols, rows, cols, wV, wH, sums[qi], cc, 0, nthreads);
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < cr * cc; ++i) {
        float s[4] = {0.0f, 0.0f, 0.0f, 0.0f}, a, b;
        for (int qi = 0; qi < nq; ++qi)
            s[qi] = sums[qi][i];
        if (self)
            guided_self_coeffs_f32(n, sq_e, s, &a, &b);
        else
            guided_coeffs_f32(n, sq_e, s, &a, &b);
        ab[0][i] = a;
        ab[1][i] = b;
    }
    tuo_box_f32(ab[0], cc, cr, cc, wV, wH, abs_[0], oc, 0, nthreads);
    tuo_box_f32(ab[1], cc, cr, cc, wV, wH, abs_[1], oc, 0, nthreads);

    const int offV = wV - 1, offH = wH - 1;
    const int oy = shift ? offV : 0, ox = shift ? offH : 0;
    const float* gg = self ? p : g;
    const long gs = self ? p_stride : g_stride;
    const float fn = (float)n;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < orr; ++y)
        for (int x = 0; x < oc; ++x) {
            const float gv = gg[(size_t)(y + offV) * gs + x + offH];
            const float A = abs_[0][(size_t)y * oc + x], B = abs_[1][(size_t)y * oc + x];
            out[(size_t)(y + oy) * out_stride + x + ox] = (A * gv + B) / fn;
        }

    free(q);
    for (int i = 0; i < 4; ++i)
        free(sums[i]);
    for (int i = 0; i < 2; ++i) {
        free(ab[i]);
        free(abs_[i]);
    }
    return 0;
}

/* FP64 guided filter: the same definition (including the self-guided b
 * formula) with window sums taken directly in double. */
int tuo_guided_f64(const double* p, long p_stride, const double* g, long g_stride,
                   int rows, int cols, int wV, int wH, double e, double* out,
                   long out_stride, int shift, int nthreads)
{
    if (wV < 1 || wH < 1)
        return -1;
    if (rows <= 0 || rows < 2 * wV - 1 || cols < 2 * wH - 1)
        return 1;
    const int self = (g == NULL);
    const double n = (double)wV * wH, sq_e = e * e;
    const int cr = rows + 1 - wV, cc = cols + 1 - wH;
    const int orr = cr + 1 - wV, oc = cc + 1 - wH;
    set_threads(nthreads);
    double* A = (double*)malloc(sizeof(double) * (size_t)cr * cc);
    double* B = (double*)malloc(sizeof(double) * (size_t)cr * cc);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < cr; ++y)
        for (int x = 0; x < cc; ++x) {
            double sp = 0, sg = 0, spg = 0, sgg = 0;
            for (int dy = 0; dy < wV; ++dy)
                for (int dx = 0; dx < wH; ++dx) {
                    const double pv = p[(size_t)(y + dy) * p_stride + x + dx];
                    const double gv = self ? pv : g[(size_t)(y + dy) * g_stride + x + dx];
                    sp += pv;
                    sg += gv;
                    spg += pv * gv;
                    sgg += gv * gv;
                }
            double a, b;
            if (self) {
                const double var = n * spg - sp * sp;
                a = var / (var + n * n * sq_e);
                b = (sp - a * spg) / n;
            } else {
                a = (n * spg - sp * sg) / (n * (sgg + n * sq_e) - sg * sg);
                b = (sp - a * sg) / n;
            }
            A[(size_t)y * cc + x] = a;
            B[(size_t)y * cc + x] = b;
        }
    const int offV = wV - 1, offH = wH - 1;
    const int oy = shift ? offV : 0, ox = shift ? offH : 0;
    const double* gg = self ? p : g;
    const long gs = self ? p_stride : g_stride;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < orr; ++y)
        for (int x = 0; x < oc; ++x) {
            double sa = 0, sb = 0;
            for (int dy = 0; dy < wV; ++dy)
                for (int dx = 0; dx < wH; ++dx) {
                    sa += A[(size_t)(y + dy) * cc + x + dx];
                    sb += B[(size_t)(y + dy) * cc + x + dx];
                }
            const double gv = gg[(size_t)(y + offV) * gs + x + offH];
            out[(size_t)(y + oy) * out_stride + x + ox] = (sa * gv + sb) / n;
        }
    free(A);
    free(B);
    return 0;
}

/* Exposes the two coefficient functors for the fixture cross-check. */
void tuo_guided_coeffs(int self, size_t n, float e, const float* sums, float* a, float* b)
{
    if (self)
        guided_self_coeffs_f32(n, e * e, sums, a, b);
    else
        guided_coeffs_f32(n, e * e, sums, a, b);
}

/* trans_guides<T>(n) (GuidedFilter.h:107-125). */
float tuo_guided_trans(size_t n, float A, float B, float g)
{
    return (A * g + B) / (float)n;
}

/* Sliding-window extrema: the monotone deque of extrema_finder::operator()
 * (BoxFilter.h:196-233) run down every column, then along every row of the
 * column results, as BoxFilter2::convolve's two box_filter passes do
 * (BoxFilter.h:542-583).  A value enters the deque after popping the values
 * it beats (less<> for the minimum, greater<> for the maximum), so the front
 * is the earliest of the window's best values; the row pass compares values
 * only and reports (column of the front, row that the column pass recorded
 * for it).  Two departures from the reference's device code, both where it
 * does not compute the window extremum: the deque here holds w+1 entries
 * (the reference's ring of WMAX slots holds WMAX-1, which monotone runs
 * overflow when w >= WMAX-1), and element 0 goes through the same loop as
 * the others (the reference writes no output for it when w = 1).  Values
 * compare as double, exact for every storage type.  val (may be NULL) gets
 * the extrema, pos (may be NULL) int32 (x, y) pairs, pos_stride counting
 * pairs; outputs at (wV/2, wH/2) when shift.  No-op when the image is
 * smaller than the window. */
static void extrema_line(const double* v, long step, int n, int w, int is_max, double* ov,
                         int* oi, int* q)
{
    int front = 0, back = 0; /* q[front..back) */
    for (int y = 0; y < n; ++y) {
        while (back > front &&
               (is_max ? v[(long)y * step] > v[(long)q[back - 1] * step]
                       : v[(long)y * step] < v[(long)q[back - 1] * step]))
            --back;
        q[back++] = y;
        if (y == q[front] + w)
            ++front;
        if (y >= w - 1) {
            ov[y - (w - 1)] = v[(long)q[front] * step];
            oi[y - (w - 1)] = q[front];
        }
    }
}

int tuo_extrema(const double* in, long in_stride, int rows, int cols, int wV, int wH,
                int is_max, double* val, long val_stride, int32_t* pos, long pos_stride,
                int shift, int nthreads)
{
    if (wV < 1 || wH < 1)
        return -1;
    if (rows < wV || cols < wH)
        return 1;
    const int orows = rows + 1 - wV, ocols = cols + 1 - wH;
    double* cv = (double*)malloc(sizeof(double) * (size_t)orows * cols);
    int* cr = (int*)malloc(sizeof(int) * (size_t)orows * cols);
    if (!cv || !cr) {
        free(cv);
        free(cr);
        return -2;
    }
    set_threads(nthreads);
    /* column pass: cv[y][x], cr[y][x] = extremum of rows y..y+wV-1, its row */
#pragma omp parallel
    {
        double* ov = (double*)malloc(sizeof(double) * (size_t)orows);
        int* oi = (int*)malloc(sizeof(int) * (size_t)orows);
        int* q = (int*)malloc(sizeof(int) * (size_t)rows);
#pragma omp for schedule(static)
        for (int x = 0; x < cols; ++x) {
            extrema_line(in + x, in_stride, rows, wV, is_max, ov, oi, q);
            for (int y = 0; y < orows; ++y) {
                cv[(size_t)y * cols + x] = ov[y];
                cr[(size_t)y * cols + x] = oi[y];
            }
        }
        free(ov);
        free(oi);
        free(q);
    }
    const int oy = shift ? wV / 2 : 0, ox = shift ? wH / 2 : 0;
    /* row pass over the column results */
#pragma omp parallel
    {
        double* ov = (double*)malloc(sizeof(double) * (size_t)ocols);
        int* oi = (int*)malloc(sizeof(int) * (size_t)ocols);
        int* q = (int*)malloc(sizeof(int) * (size_t)cols);
#pragma omp for schedule(static)
        for (int y = 0; y < orows; ++y) {
            extrema_line(cv + (size_t)y * cols, 1, cols, wH, is_max, ov, oi, q);
            for (int x = 0; x < ocols; ++x) {
                if (val)
                    val[(size_t)(y + oy) * val_stride + x + ox] = ov[x];
                if (pos) {
                    int32_t* p = pos + 2 * ((size_t)(y + oy) * pos_stride + x + ox);
                    p[0] = oi[x];
                    p[1] = cr[(size_t)y * cols + oi[x]];
                }
            }
        }
        free(ov);
        free(oi);
        free(q);
    }
    free(cv);
    free(cr);
    return 0;
}

/* Stereo cost aggregation (BoxFilter.h:585-746 with diff<T>(thresh),
 * functional.h:385-398), disparity-major: for d < ndisp, window origins
 * y < rows+1-wV, x < cols+1-wH,
 *   costs[d][y][x] = sum over the window of min(|L[y'][x'] - R[y'][x'+d]|, t)
 * with right pixels past the last column taken as 0.  Sums in double (exact
 * for integer images); out is ndisp slices of rows x cols, each stored at
 * (y, x).  No-op when the image is smaller than the window. */
int tuo_stereo(const double* left, const double* right, long stride, int rows, int cols,
               int wV, int wH, double thresh, int ndisp, double* out, int nthreads)
{
    if (wV < 1 || wH < 1 || ndisp < 1)
        return -1;
    if (rows < wV || cols < wH)
        return 1;
    const int orows = rows + 1 - wV, ocols = cols + 1 - wH;
    set_threads(nthreads);
#pragma omp parallel
    {
        double* c = (double*)malloc(sizeof(double) * (size_t)rows * cols);
        double* v = (double*)malloc(sizeof(double) * (size_t)orows * cols);
#pragma omp for schedule(dynamic)
        for (int d = 0; d < ndisp; ++d) {
            for (int y = 0; y < rows; ++y)
                for (int x = 0; x < cols; ++x) {
                    const double a = left[(size_t)y * stride + x];
                    const double b = x + d < cols ? right[(size_t)y * stride + x + d] : 0.0;
                    const double e = a > b ? a - b : b - a;
                    c[(size_t)y * cols + x] = e < thresh ? e : thresh;
                }
            for (int y = 0; y < orows; ++y)
                for (int x = 0; x < cols; ++x) {
                    double s = 0.0;
                    for (int k = 0; k < wV; ++k)
                        s += c[(size_t)(y + k) * cols + x];
                    v[(size_t)y * cols + x] = s;
                }
            double* o = out + (size_t)d * rows * cols;
            for (int y = 0; y < orows; ++y)
                for (int x = 0; x < ocols; ++x) {
                    double s = 0.0;
                    for (int k = 0; k < wH; ++k)
                        s += v[(size_t)y * cols + x + k];
                    o[(size_t)y * cols + x] = s;
                }
        }
        free(c);
        free(v);
    }
    return 0;
}

/* ------------------------------------------------------------------------
 * DisparitySelector (StereoUtility.h:56-107)
 * ---------------------------------------------------------------------- */

/* costs: D slices of rows x cols (the selected region, row-major, doubles).
 * Per pixel: dL = first d with the smallest cost; dR(xr) = first d <= xr
 * with the smallest costs[d][y][xr - d]; out = dmax - dL when xr = x + dL is
 * inside the row and |dL - dR(xr)| < inc, else 0.  The minima use strict
 * "<" as select_disparity does (the smallest disparity wins ties); the right
 * minima are taken over every d (the reference's blocks race on them). */
int tuo_select_disparity(const double* costs, int D, int rows, int cols, int dmax, int inc,
                         double* out, int nthreads)
{
    if (D < 1 || rows < 1 || cols < 1)
        return -1;
    set_threads(nthreads);
#pragma omp parallel
    {
        int* dR = (int*)malloc(sizeof(int) * (size_t)cols);
#pragma omp for schedule(static)
        for (int y = 0; y < rows; ++y) {
            for (int xr = 0; xr < cols; ++xr) {
                double best = INFINITY;
                int db = 0;
                for (int d = 0; d < D && d <= xr; ++d) {
                    const double c = costs[((size_t)d * rows + y) * cols + xr - d];
                    if (c < best) {
                        best = c;
                        db = d;
                    }
                }
                dR[xr] = db;
            }
            for (int x = 0; x < cols; ++x) {
                double best = INFINITY;
                int dl = 0;
                for (int d = 0; d < D; ++d) {
                    const double c = costs[((size_t)d * rows + y) * cols + x];
                    if (c < best) {
                        best = c;
                        dl = d;
                    }
                }
                const int xr = x + dl;
                const int diff = xr < cols ? abs(dl - dR[xr]) : inc;
                out[(size_t)y * cols + x] = diff < inc ? (double)(dmax - dl) : 0.0;
            }
        }
        free(dR);
    }
    return 0;
}
