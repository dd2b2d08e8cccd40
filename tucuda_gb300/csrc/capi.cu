// capi.cu -- the C ABI of include/tucu_gb300.h for the four filters: handle
// state, argument checks with the reference's error behaviour, the FP64
// Gaussian lobe design, and dispatch to the kernels.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <string>

#include "box_kernels.h"
#include "fir_tc.h"
#include "stereo_select.h"
#include "extrema.h"
#include "fir3_dispatch.h"
#include "fir_strip.cuh"
#include "fir_v3.cuh"
#include "tucu_internal.h"

int tucu_box_tu_error(bool clear);
int tucu_fir_u8_tu_error(bool clear);
int tucu_fir_f16_tu_error(bool clear);
int tucu_fir_bf16_tu_error(bool clear);
int tucu_fir_f32_tu_error(bool clear);
int tucu_tc_tu_error(bool clear);

namespace tucu
{

// ---- errors ---------------------------------------------------------------------

static thread_local std::string g_last_error;

void set_last_error(const std::string& msg) { g_last_error = msg; }

int fail(int status, const std::string& msg)
{
    g_last_error = msg;
    return status;
}

int cuda_fail(cudaError_t e, const char* what)
{
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return TUCU_ERR_CUDA;
}

// ---- device facts ---------------------------------------------------------------

int sm_count()
{
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return 148;
    int& c = cache[dev & 63];
    if (c == 0) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        c = v > 0 ? v : 148;
    }
    return c;
}

// ---- TMA descriptors ------------------------------------------------------------

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn()
{
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

bool make_tmap_2d(CUtensorMap* map, const void* base, int dtype, int cols, int rows,
                  size_t pitch, int box_w, int box_h, bool swizzle128)
{
    EncodeTiledFn fn = encode_fn();
    if (!fn || !base || (reinterpret_cast<uintptr_t>(base) & 15) || (pitch & 15) || rows < 1 ||
        cols < 1 || pitch >= (1ull << 40))
        return false;
    CUtensorMapDataType t;
    switch (dtype) {
    case U8: t = CU_TENSOR_MAP_DATA_TYPE_UINT8; break;
    case F16: t = CU_TENSOR_MAP_DATA_TYPE_FLOAT16; break;
    case BF16: t = CU_TENSOR_MAP_DATA_TYPE_BFLOAT16; break;
    case F32: t = CU_TENSOR_MAP_DATA_TYPE_FLOAT32; break;
    case I32: t = CU_TENSOR_MAP_DATA_TYPE_INT32; break;
    default: return false;
    }
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)pitch};
    const cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_h};
    const cuuint32_t estr[2] = {1, 1};
    return fn(map, t, 2, const_cast<void*>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE,
              swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
           CUDA_SUCCESS;
}

// ---- Gaussian lobe design ---------------------------------------------------------

static bool lobe_len_ok(int L)
{
    return L == 2 || L == 3 || L == 4 || L == 5 || L == 8 || L == 9 || L == 16 || L == 17;
}

// detail::lobeSize's rule (FIRGaussianConvolver.cu:52-98), size_t arithmetic
// kept so that an all-zero lobe yields the largest size as there.
static size_t lobe_size_rule(const float* lobe, bool even)
{
    const size_t sizMax = TUCU_LOBE_MAX;
    float th = 0.0f;
    for (size_t i = sizMax; i-- > 0;)
        if (std::fabs(lobe[i]) >= th)
            th = std::fabs(lobe[i]);
    th *= 0.01f;
    size_t siz;
    for (siz = sizMax; siz-- > 0;)
        if (std::fabs(lobe[siz]) > th) {
            ++siz;
            break;
        }
    if (even)
        return siz <= 2 ? 3 : siz <= 5 ? 5 : siz <= 9 ? 9 : 17;
    return siz <= 1 ? 2 : siz <= 4 ? 4 : siz <= 8 ? 8 : 16;
}

// The Gaussian, first- and second-derivative lobes of
// FIRGaussianConvolver2::initialize (FIRGaussianConvolver.h:123-170).  The
// lengths come from the reference's float computation so that they agree
// with it exactly; the coefficients are computed and normalised in FP64 and
// rounded once.  lobe1 keeps the reference's normalisation, which takes
// lb1[1..L] into the kernel but only lb1[0..L-1] into the norm.
static int design_lobes(float sigma, float* l0, int* n0, float* l1, int* n1, float* l2, int* n2)
{
    if (!(sigma > 0.0f) || !std::isfinite(sigma))
        return fail(TUCU_ERR_ARG, "sigma must be positive and finite");
    float f0[TUCU_LOBE_MAX], f1[TUCU_LOBE_MAX], f2[TUCU_LOBE_MAX];
    double d0[TUCU_LOBE_MAX], d1[TUCU_LOBE_MAX], d2[TUCU_LOBE_MAX];
    for (int i = 0; i < TUCU_LOBE_MAX; ++i) {
        const float dx = (float)i / sigma, dxdx = dx * dx;
        f0[i] = std::exp(-0.5f * dxdx);
        f1[i] = -dx * f0[i];
        f2[i] = (dxdx - 1.0f) * f0[i];
        const double Dx = (double)i / (double)sigma, DxDx = Dx * Dx;
        d0[i] = std::exp(-0.5 * DxDx);
        d1[i] = -Dx * d0[i];
        d2[i] = (DxDx - 1.0) * d0[i];
    }
    const int L0 = (int)lobe_size_rule(f0, true);
    const int L1 = (int)lobe_size_rule(f1, false);
    const int L2 = (int)lobe_size_rule(f2, true);
    double s = d0[0];
    for (int i = 1; i < L0; ++i)
        s += 2.0 * d0[i];
    for (int i = 0; i < L0; ++i)
        l0[i] = (float)(d0[L0 - 1 - i] / std::fabs(s));
    s = 0.0;
    for (int i = 0; i < L1; ++i)
        s += 2.0 * i * d1[i];
    for (int i = 0; i < L1; ++i)
        l1[i] = (float)(d1[L1 - i] / std::fabs(s));
    s = 0.0;
    for (int i = 1; i < L2; ++i)
        s += (double)i * i * d2[i];
    for (int i = 0; i < L2; ++i)
        l2[i] = (float)(d2[L2 - 1 - i] / std::fabs(s));
    *n0 = L0;
    *n1 = L1;
    *n2 = L2;
    return TUCU_OK;
}

// The same lobes in the reference's own float arithmetic
// (FIRGaussianConvolver.h:123-170): float samples, float normalisation sums in
// the reference's order, one float division per tap.  Each product is held in
// a volatile before it is added, so no compiler contracts a multiply-add into
// an FMA (the reference's host build has none on x86), and the result is the
// same on x86 and aarch64.
static int design_lobes_float(float sigma, float* l0, int* n0, float* l1, int* n1, float* l2,
                              int* n2)
{
    if (!(sigma > 0.0f) || !std::isfinite(sigma))
        return fail(TUCU_ERR_ARG, "sigma must be positive and finite");
    float f0[TUCU_LOBE_MAX], f1[TUCU_LOBE_MAX], f2[TUCU_LOBE_MAX];
    for (int i = 0; i < TUCU_LOBE_MAX; ++i) {
        const float dx = (float)i / sigma, dxdx = dx * dx;
        f0[i] = std::exp(-0.5f * dxdx);
        f1[i] = -dx * f0[i];
        f2[i] = (dxdx - 1.0f) * f0[i];
    }
    volatile float term;
    const size_t L0 = lobe_size_rule(f0, true);
    float sum = f0[0];
    for (size_t i = 1; i < L0; ++i) {
        term = 2.0f * f0[i];
        sum += term;
    }
    for (size_t i = 0; i < L0; ++i)
        l0[i] = f0[L0 - 1 - i] / std::fabs(sum);
    const size_t L1 = lobe_size_rule(f1, false);
    sum = 0.0f;
    for (size_t i = 0; i < L1; ++i) {
        term = 2.0f * (float)i * f1[i];
        sum += term;
    }
    for (size_t i = 0; i < L1; ++i)
        l1[i] = f1[L1 - i] / std::fabs(sum);
    const size_t L2 = lobe_size_rule(f2, true);
    sum = 0.0f;
    for (size_t i = 1; i < L2; ++i) {
        term = (float)(i * i) * f2[i];
        sum += term;
    }
    for (size_t i = 0; i < L2; ++i)
        l2[i] = f2[L2 - 1 - i] / std::fabs(sum);
    *n0 = (int)L0;
    *n1 = (int)L1;
    *n2 = (int)L2;
    return TUCU_OK;
}

// Pads a lobe of length L (outermost first) on its outer side to radius R:
// result index R is the centre (zero for antisymmetric lobes).
static void pad_lobe(const float* lobe, int L, int R, float* out)
{
    const int r = L & ~1;
    for (int k = 0; k <= R; ++k)
        out[k] = 0.0f;
    for (int k = 0; k < L; ++k)
        out[R - r + k] = lobe[k];
}

// ---- shared argument checks -------------------------------------------------------

static bool dtype_ok(int dt) { return dt >= U8 && dt <= I32; }

static int check_image(const void* p, size_t pitch, int rows, int cols, int dt, const char* what)
{
    if (!dtype_ok(dt))
        return fail(TUCU_ERR_DTYPE, std::string(what) + ": unknown dtype");
    if (!p)
        return fail(TUCU_ERR_ARG, std::string(what) + ": null pointer");
    if (rows < 0 || cols < 0)
        return fail(TUCU_ERR_ARG, std::string(what) + ": negative size");
    if (rows > 0 && pitch < (size_t)cols * dtype_size(dt))
        return fail(TUCU_ERR_ARG, std::string(what) + ": pitch smaller than a row");
    return TUCU_OK;
}

int plan_strip_rows(int orows, int ncx, long slots, int ch, int rv, int max_strip)
{
    // The 4R floor keeps the 2R halo rows at most half of a strip's
    // horizontal work; outputs do not depend on the strip height.
    const int lo = (std::max(ch, 4 * rv) + ch - 1) / ch * ch;
    const int hi = std::max(lo, max_strip / ch * ch);
    slots = std::max(1L, slots);
    int best_strip = lo;
    double best = 1e300;
    for (int strip = lo; strip <= hi; strip += ch) {
        const long strips = (long)ncx * ((orows + strip - 1) / strip);
        const long rounds = (strips + slots - 1) / slots;
        const double cost = (double)rounds * (2.0 * std::min(strip, orows) + 2 * rv + ch);
        if (cost < best) {
            best = cost;
            best_strip = strip;
        }
        if (strip >= orows)
            break;
    }
    return best_strip;
}

int ctas_per_sm(const void* kernel, int threads, size_t smem)
{
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem) != cudaSuccess)
        return 1;
    return std::max(n, 1);
}

static cudaError_t fir_dispatch(fir::FirLaunch& L, cudaStream_t st)
{
    switch (L.in_dtype) {
    case U8: return fir::launch_u8(L, st);
    case F16: return fir::launch_f16(L, st);
    case BF16: return fir::launch_bf16(L, st);
    case F32: return fir::launch_f32(L, st);
    default: return cudaErrorInvalidValue;
    }
}

// One separable FIR with lobes (lh, nh) / (lv, nv) through the single-lobe
// strip kernel.
// The tensor-core kernel for one image (fir_tc.cu), when the handle asked for
// it and the job qualifies: f16 input whose rows TMA can address, f16 or f32
// output, at most 33 taps per direction.  Returns 1 when it launched (e holds
// the launch status), 0 when the caller should take the FP32-pipe path.
static int try_tensor(const float* th, int nth, const float* tv, int ntv, float post, const void* in,
                      size_t in_pitch, int rows, int cols, int in_dtype, void* out,
                      size_t out_pitch, int out_dtype, int oy, int ox, void* stream, cudaError_t* e)
{
    if (!tcf::eligible(in_dtype, out_dtype, nth, ntv))
        return 0;
    tcf::TcJob J;
    if (!tcf::fill_job(&J, in, in_pitch, rows, cols, out, out_pitch, out_dtype, oy, ox, th, nth, tv,
                       ntv, post))
        return 0;
    *e = tcf::launch_single(J, static_cast<cudaStream_t>(stream));
    return 1;
}

static int run_fir(const float* lh, int nH, const float* lv, int nV, const void* in,
                   size_t in_pitch, int rows, int cols, int in_dtype, void* out, size_t out_pitch,
                   int out_dtype, int shift, void* stream, int strip_rows = 0, int tensor = 0)
{
    int rc = check_image(in, in_pitch, rows, cols, in_dtype, "input");
    if (rc)
        return rc;
    rc = check_image(out, out_pitch, rows, cols, out_dtype, "output");
    if (rc)
        return rc;
    if (in_dtype == I32)
        return fail(TUCU_ERR_DTYPE, "FIR input must be u8, f16, bf16 or f32");
    const int lsV = nV & ~1, lsH = nH & ~1;
    // The reference returns silently on small images before it looks at the
    // lobe lengths (FIRFilter.h:304-312), then throws on an unsupported one.
    if (rows <= 2 * lsV || cols <= 2 * lsH)
        return TUCU_NOOP;
    if (!lobe_len_ok(nH))
        return fail(TUCU_ERR_LOBE, "unsupported horizontal lobe size " + std::to_string(nH));
    if (!lobe_len_ok(nV))
        return fail(TUCU_ERR_LOBE, "unsupported vertical lobe size " + std::to_string(nV));
    if (tensor) {
        float th[tcf::kMaxTaps], tv[tcf::kMaxTaps];
        const int nth = tcf::full_taps(lh, nH, th), ntv = tcf::full_taps(lv, nV, tv);
        cudaError_t e = cudaSuccess;
        if (try_tensor(th, nth, tv, ntv, 1.0f, in, in_pitch, rows, cols, in_dtype, out, out_pitch,
                       out_dtype, shift ? lsV : 0, shift ? lsH : 0, stream, &e))
            return e == cudaSuccess ? TUCU_OK : cuda_fail(e, "tensor-core FIR launch");
    }
    fir::FirLaunch L;
    std::memset(&L, 0, sizeof(L));
    L.in_dtype = in_dtype;
    fir::FirJob& J = L.job;
    J.src = in;
    J.src_pitch = in_pitch;
    J.rows = rows;
    J.cols = cols;
    J.orows = rows - 2 * lsV;
    J.ocols = cols - 2 * lsH;
    J.oy = shift ? lsV : 0;
    J.ox = shift ? lsH : 0;
    J.nh = 1;
    J.nout = 1;
    J.out_dtype = out_dtype;
    J.dst[0] = out;
    J.dst_pitch[0] = out_pitch;
    L.lobes.sym_h = nH & 1;
    L.lobes.sym_v = nV & 1;
    cudaError_t e;
    if (lsH == lsV) {
        // Equal radii: the warp-specialised kernel.
        L.rh = L.rv = lsH;
        pad_lobe(lh, nH, lsH, L.lobes.h[0]);
        pad_lobe(lv, nV, lsV, L.lobes.v[0]);
        L.strip_rows = strip_rows;  // 0: the launcher plans
        L.use_tma = make_tmap_2d(&L.tmap, in, in_dtype, cols, rows, in_pitch,
                                 fir::round_up(fir3::kTW + 2 * lsH, 16), fir3::kCH);
        fir::Launch3Fn fn = fir::launch3_fn(in_dtype, out_dtype);
        if (!fn)
            return fail(TUCU_ERR_DTYPE, "unsupported FIR type pair");
        e = fn(L, static_cast<cudaStream_t>(stream));
    } else {
        // Unequal radii: both lobes zero-padded to the larger radius R over a
        // virtual input with (R - r) zero rows/columns on each side, so the
        // R-valid region is the operator's own valid region and the padded
        // taps only ever meet zeros.
        const int R = std::max(lsH, lsV);
        L.rh = L.rv = R;
        pad_lobe(lh, nH, R, L.lobes.h[0]);
        pad_lobe(lv, nV, R, L.lobes.v[0]);
        J.pad_y = R - lsV;
        J.pad_x = R - lsH;
        L.use_tma = 0;
        L.strip_rows = strip_rows;  // 0: the launcher plans
        e = fir_dispatch(L, static_cast<cudaStream_t>(stream));
    }
    return e == cudaSuccess ? TUCU_OK : cuda_fail(e, "FIR launch");
}

}  // namespace tucu

using namespace tucu;

// ==== C ABI ========================================================================

struct tucu_fir
{
    float lobeH[TUCU_LOBE_MAX];
    float lobeV[TUCU_LOBE_MAX];
    int nH, nV;
    int tensor = 0;  // f16 images on the tensor cores (tucu_fir_set_tensor_cores)
};

struct tucu_gauss
{
    float sigma;
    float lobe[3][TUCU_LOBE_MAX];
    int n[3];
    int tensor = 0;
    int ref_lobes = 0;  // lobes in the reference's float arithmetic
};

struct tucu_box
{
    int winV, winH, winMax;
    int tensor = 0;
};

struct tucu_disparity
{
    int disparity_max, inconsistency;
};

struct tucu_extrema
{
    int winV, winH, winMax;
};

struct tucu_guided
{
    int winV, winH, winMax;
    float e;
    void* coef;          // scratch coefficient image (float2)
    size_t coef_bytes;
    int coef_device;
};

extern "C" {

int tucu_version(void) { return 10000; }

const char* tucu_status_string(int status)
{
    switch (status) {
    case TUCU_OK: return "ok";
    case TUCU_NOOP: return "image smaller than the filter support; nothing written";
    case TUCU_ERR_ARG: return "invalid argument";
    case TUCU_ERR_LOBE: return "unsupported lobe size";
    case TUCU_ERR_WINDOW: return "window size out of range";
    case TUCU_ERR_DTYPE: return "unsupported pixel type";
    case TUCU_ERR_CUDA: return "CUDA runtime error";
    case TUCU_ERR_NOMEM: return "out of memory";
    case TUCU_ERR_BUDGET: return "request exceeds the memory budget";
    case TUCU_ERR_TIMEOUT: return "bounded wait ran out";
    case TUCU_ERR_STATE: return "invalid state";
    case TUCU_ERR_CANCELLED: return "cancelled";
    default: return "unknown status";
    }
}

const char* tucu_last_error(void) { return g_last_error.c_str(); }

int tucu_device_error(int* code)
{
    if (!code)
        return fail(TUCU_ERR_ARG, "null code");
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaDeviceSynchronize");
    int v = 0;
    int (*readers[])(bool) = {
        tucu_box_tu_error, tucu_fir_u8_tu_error, tucu_fir_f16_tu_error, tucu_fir_bf16_tu_error,
        tucu_fir_f32_tu_error, tucu_tc_tu_error,
#define TUCU_R(a) tucu_fir3_##a##_u8_tu_error, tucu_fir3_##a##_f16_tu_error, \
    tucu_fir3_##a##_bf16_tu_error, tucu_fir3_##a##_f32_tu_error, tucu_fir3_##a##_i32_tu_error,
        TUCU_R(u8) TUCU_R(f16) TUCU_R(bf16) TUCU_R(f32)
#undef TUCU_R
    };
    for (auto r : readers) {
        const int x = r(true);
        if (x < 0)
            return cuda_fail(cudaGetLastError(), "reading the device error word");
        if (x && !v)
            v = x;
    }
    *code = v;
    return TUCU_OK;
}

// ---- FIRFilter2 ------------------------------------------------------------------

int tucu_fir_create(tucu_fir** out)
{
    if (!out)
        return fail(TUCU_ERR_ARG, "null handle pointer");
    auto* h = new (std::nothrow) tucu_fir;
    if (!h)
        return fail(TUCU_ERR_NOMEM, "host allocation");
    *h = tucu_fir{};
    *out = h;
    return TUCU_OK;
}

int tucu_fir_initialize(tucu_fir* h, const float* lobeH, int nH, const float* lobeV, int nV)
{
    if (!h || (nH > 0 && !lobeH) || (nV > 0 && !lobeV) || nH < 0 || nV < 0)
        return fail(TUCU_ERR_ARG, "null handle or lobe");
    if (nH > TUCU_LOBE_MAX || nV > TUCU_LOBE_MAX)
        return fail(TUCU_ERR_LOBE, "FIRFilter2::initialize: too large lobe size!");
    std::memset(h->lobeH, 0, sizeof(h->lobeH));
    std::memset(h->lobeV, 0, sizeof(h->lobeV));
    if (nH)
        std::memcpy(h->lobeH, lobeH, sizeof(float) * nH);
    if (nV)
        std::memcpy(h->lobeV, lobeV, sizeof(float) * nV);
    h->nH = nH;
    h->nV = nV;
    return TUCU_OK;
}

int tucu_fir_offsets(const tucu_fir* h, int* offV, int* offH)
{
    if (!h || !offV || !offH)
        return fail(TUCU_ERR_ARG, "null argument");
    *offV = h->nV & ~1;
    *offH = h->nH & ~1;
    return TUCU_OK;
}

int tucu_fir_convolve(tucu_fir* h, const void* in, size_t in_pitch, int rows, int cols,
                      int in_dtype, void* out, size_t out_pitch, int out_dtype, int shift,
                      void* stream)
{
    if (!h)
        return fail(TUCU_ERR_ARG, "null handle");
    return run_fir(h->lobeH, h->nH, h->lobeV, h->nV, in, in_pitch, rows, cols, in_dtype, out,
                   out_pitch, out_dtype, shift, stream, 0, h->tensor);
}

int tucu_fir_set_tensor_cores(tucu_fir* h, int on)
{
    if (!h)
        return fail(TUCU_ERR_ARG, "null handle");
    h->tensor = on ? 1 : 0;
    return TUCU_OK;
}

void tucu_fir_destroy(tucu_fir* h) { delete h; }

// ---- FIRGaussianConvolver2 -------------------------------------------------------

int tucu_gauss_design(float sigma, float* lobe0, int* n0, float* lobe1, int* n1, float* lobe2,
                      int* n2)
{
    if (!lobe0 || !n0 || !lobe1 || !n1 || !lobe2 || !n2)
        return fail(TUCU_ERR_ARG, "null argument");
    return design_lobes(sigma, lobe0, n0, lobe1, n1, lobe2, n2);
}

int tucu_gauss_design_reference(float sigma, float* lobe0, int* n0, float* lobe1, int* n1,
                                float* lobe2, int* n2)
{
    if (!lobe0 || !n0 || !lobe1 || !n1 || !lobe2 || !n2)
        return fail(TUCU_ERR_ARG, "null argument");
    return design_lobes_float(sigma, lobe0, n0, lobe1, n1, lobe2, n2);
}

int tucu_gauss_create(float sigma, tucu_gauss** out)
{
    if (!out)
        return fail(TUCU_ERR_ARG, "null handle pointer");
    auto* h = new (std::nothrow) tucu_gauss;
    if (!h)
        return fail(TUCU_ERR_NOMEM, "host allocation");
    *h = tucu_gauss{};
    const int rc = tucu_gauss_initialize(h, sigma);
    if (rc != TUCU_OK) {
        delete h;
        return rc;
    }
    *out = h;
    return TUCU_OK;
}

int tucu_gauss_initialize(tucu_gauss* h, float sigma)
{
    if (!h)
        return fail(TUCU_ERR_ARG, "null handle");
    const int rc = (h->ref_lobes ? design_lobes_float : design_lobes)(
        sigma, h->lobe[0], &h->n[0], h->lobe[1], &h->n[1], h->lobe[2], &h->n[2]);
    if (rc == TUCU_OK)
        h->sigma = sigma;
    return rc;
}

int tucu_gauss_set_reference_lobes(tucu_gauss* h, int on)
{
    if (!h)
        return fail(TUCU_ERR_ARG, "null handle");
    h->ref_lobes = on ? 1 : 0;
    return tucu_gauss_initialize(h, h->sigma);
}

float tucu_gauss_sigma(const tucu_gauss* h) { return h ? h->sigma : 0.0f; }

int tucu_gauss_lobes(const tucu_gauss* h, float* lobe0, int* n0, float* lobe1, int* n1,
                     float* lobe2, int* n2)
{
    if (!h || !lobe0 || !n0 || !lobe1 || !n1 || !lobe2 || !n2)
        return fail(TUCU_ERR_ARG, "null argument");
    std::memcpy(lobe0, h->lobe[0], sizeof(float) * h->n[0]);
    std::memcpy(lobe1, h->lobe[1], sizeof(float) * h->n[1]);
    std::memcpy(lobe2, h->lobe[2], sizeof(float) * h->n[2]);
    *n0 = h->n[0];
    *n1 = h->n[1];
    *n2 = h->n[2];
    return TUCU_OK;
}

// (horizontal lobe, vertical lobe) of each operator (FIRGaussianConvolver.h:178-242).
static const int kOpLobes[6][2] = {{0, 0}, {1, 0}, {0, 1}, {2, 0}, {1, 1}, {0, 2}};

int tucu_gauss_offsets(const tucu_gauss* h, int op, int* offV, int* offH)
{
    if (!h || !offV || !offH || op < 0 || op > 5)
        return fail(TUCU_ERR_ARG, "bad argument");
    *offH = h->n[kOpLobes[op][0]] & ~1;
    *offV = h->n[kOpLobes[op][1]] & ~1;
    return TUCU_OK;
}

int tucu_gauss_convolve(tucu_gauss* h, int op, const void* in, size_t in_pitch, int rows,
                        int cols, int in_dtype, void* out, size_t out_pitch, int out_dtype,
                        int shift, void* stream)
{
    if (!h)
        return fail(TUCU_ERR_ARG, "null handle");
    if (op < 0 || op > 5)
        return fail(TUCU_ERR_ARG, "unknown Gaussian operator");
    const int lh = kOpLobes[op][0], lv = kOpLobes[op][1];
    return run_fir(h->lobe[lh], h->n[lh], h->lobe[lv], h->n[lv], in, in_pitch, rows, cols,
                   in_dtype, out, out_pitch, out_dtype, shift, stream, 0, h->tensor);
}

int tucu_gauss_set_tensor_cores(tucu_gauss* h, int on)
{
    if (!h)
        return fail(TUCU_ERR_ARG, "null handle");
    h->tensor = on ? 1 : 0;
    return TUCU_OK;
}

int tucu_gauss_convolve_multi(tucu_gauss* h, unsigned op_mask, const void* in, size_t in_pitch,
                              int rows, int cols, int in_dtype, void* const* outs,
                              const size_t* out_pitches, int out_dtype, int shift, void* stream)
{
    if (!h || !outs || !out_pitches)
        return fail(TUCU_ERR_ARG, "null argument");
    if (op_mask == 0 || op_mask > 0x3f)
        return fail(TUCU_ERR_ARG, "op_mask must select operators 0..5");
    int rc = check_image(in, in_pitch, rows, cols, in_dtype, "input");
    if (rc)
        return rc;
    if (in_dtype == I32)
        return fail(TUCU_ERR_DTYPE, "Gaussian input must be u8, f16, bf16 or f32");
    // Lobes in use and the common radius.
    bool hneed[3] = {false, false, false}, vneed[3] = {false, false, false};
    for (int op = 0; op < 6; ++op)
        if (op_mask & (1u << op)) {
            rc = check_image(outs[op], out_pitches[op], rows, cols, out_dtype, "output");
            if (rc)
                return rc;
            hneed[kOpLobes[op][0]] = true;
            vneed[kOpLobes[op][1]] = true;
        }
    int R = 0;
    for (int l = 0; l < 3; ++l)
        if (hneed[l] || vneed[l])
            R = std::max(R, h->n[l] & ~1);
    // Every selected output has the geometry of its own operator; the common
    // strip uses radius R, so outputs are computed on the R-valid region and
    // each operator's own valid region must coincide with it.  With lobes of
    // different radii the per-operator launch is used instead.
    bool uniform = true;
    for (int l = 0; l < 3; ++l)
        if ((hneed[l] || vneed[l]) && (h->n[l] & ~1) != R)
            uniform = false;
    if (!uniform) {
        for (int op = 0; op < 6; ++op)
            if (op_mask & (1u << op)) {
                rc = tucu_gauss_convolve(h, op, in, in_pitch, rows, cols, in_dtype, outs[op],
                                         out_pitches[op], out_dtype, shift, stream);
                if (rc < 0)
                    return rc;
            }
        return rc;
    }
    if (rows <= 2 * R || cols <= 2 * R)
        return TUCU_NOOP;
    fir::FirLaunch L;
    std::memset(&L, 0, sizeof(L));
    L.rh = L.rv = R;
    L.in_dtype = in_dtype;
    int hidx[3] = {-1, -1, -1}, nh = 0;
    for (int l = 0; l < 3; ++l)
        if (hneed[l]) {
            hidx[l] = nh;
            pad_lobe(h->lobe[l], h->n[l], R, L.lobes.h[nh]);
            if (h->n[l] & 1)
                L.lobes.sym_h |= 1 << nh;
            ++nh;
        }
    for (int l = 0; l < 3; ++l) {
        pad_lobe(h->lobe[l], h->n[l], R, L.lobes.v[l]);
        if (h->n[l] & 1)
            L.lobes.sym_v |= 1 << l;
    }
    fir::FirJob& J = L.job;
    J.src = in;
    J.src_pitch = in_pitch;
    J.rows = rows;
    J.cols = cols;
    J.orows = rows - 2 * R;
    J.ocols = cols - 2 * R;
    J.oy = J.ox = shift ? R : 0;
    J.nh = nh;
    J.out_dtype = out_dtype;
    for (int op = 0; op < 6; ++op)
        if (op_mask & (1u << op)) {
            J.dst[J.nout] = outs[op];
            J.dst_pitch[J.nout] = out_pitches[op];
            J.hsel[J.nout] = (unsigned char)hidx[kOpLobes[op][0]];
            J.vsel[J.nout] = (unsigned char)kOpLobes[op][1];
            ++J.nout;
        }
    L.strip_rows = 0;  // the launcher plans
    L.use_tma = make_tmap_2d(&L.tmap, in, in_dtype, cols, rows, in_pitch,
                             fir::round_up(fir::kTW + 2 * R, 16), 16);
    const cudaError_t e = fir_dispatch(L, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? TUCU_OK : cuda_fail(e, "Gaussian multi-operator launch");
}

void tucu_gauss_destroy(tucu_gauss* h) { delete h; }

// ---- BoxFilter2 --------------------------------------------------------------------

static int check_window(int wV, int wH, int wmax)
{
    if (wV < 1 || wH < 1 || wV > wmax || wH > wmax)
        return fail(TUCU_ERR_WINDOW, "Too large window size!");
    return TUCU_OK;
}

static int norm_wmax(int wmax)
{
    return wmax <= 0 ? TUCU_WIN_MAX_DEFAULT : std::min(wmax, TUCU_WIN_LIMIT);
}

int tucu_box_create(int winV, int winH, int win_max, tucu_box** out)
{
    if (!out)
        return fail(TUCU_ERR_ARG, "null handle pointer");
    if (win_max > TUCU_WIN_LIMIT)
        return fail(TUCU_ERR_WINDOW, "window limit above " + std::to_string(TUCU_WIN_LIMIT));
    const int wmax = norm_wmax(win_max);
    const int rc = check_window(winV, winH, wmax);
    if (rc)
        return rc;
    auto* h = new (std::nothrow) tucu_box;
    if (!h)
        return fail(TUCU_ERR_NOMEM, "host allocation");
    h->winV = winV;
    h->winH = winH;
    h->winMax = wmax;
    *out = h;
    return TUCU_OK;
}

int tucu_box_set_window(tucu_box* h, int winV, int winH)
{
    if (!h)
        return fail(TUCU_ERR_ARG, "null handle");
    const int rc = check_window(winV, winH, h->winMax);
    if (rc)
        return rc;
    h->winV = winV;
    h->winH = winH;
    return TUCU_OK;
}

int tucu_box_offsets(const tucu_box* h, int* offV, int* offH)
{
    if (!h || !offV || !offH)
        return fail(TUCU_ERR_ARG, "null argument");
    *offV = h->winV / 2;
    *offH = h->winH / 2;
    return TUCU_OK;
}

int tucu_box_convolve(tucu_box* h, const void* in, size_t in_pitch, int rows, int cols,
                      int in_dtype, void* out, size_t out_pitch, int out_dtype, int shift,
                      int normalize, void* stream)
{
    if (!h)
        return fail(TUCU_ERR_ARG, "null handle");
    int rc = check_image(in, in_pitch, rows, cols, in_dtype, "input");
    if (rc)
        return rc;
    rc = check_image(out, out_pitch, rows, cols, out_dtype, "output");
    if (rc)
        return rc;
    if (rows < h->winV || cols < h->winH)
        return TUCU_NOOP;  // BoxFilter.h:551-557
    if (h->tensor) {
        float ones[tcf::kMaxTaps];
        std::fill(ones, ones + tcf::kMaxTaps, 1.0f);
        const float post = normalize ? 1.0f / (float)(h->winV * h->winH) : 1.0f;
        cudaError_t e = cudaSuccess;
        if (try_tensor(ones, h->winH, ones, h->winV, post, in, in_pitch, rows, cols, in_dtype, out,
                       out_pitch, out_dtype, shift ? h->winV / 2 : 0, shift ? h->winH / 2 : 0,
                       stream, &e))
            return e == cudaSuccess ? TUCU_OK : cuda_fail(e, "tensor-core box launch");
    }
    box::BoxLaunch L;
    std::memset(&L, 0, sizeof(L));
    L.src = in;
    L.src_pitch = in_pitch;
    L.rows = rows;
    L.cols = cols;
    L.in_dtype = in_dtype;
    L.wV = h->winV;
    L.wH = h->winH;
    L.dst = out;
    L.dst_pitch = out_pitch;
    L.out_dtype = out_dtype;
    L.oy = shift ? h->winV / 2 : 0;
    L.ox = shift ? h->winH / 2 : 0;
    L.normalize = normalize ? 1 : 0;
    const cudaError_t e = box::launch_box(L, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? TUCU_OK : cuda_fail(e, "box launch");
}

int tucu_box_set_tensor_cores(tucu_box* h, int on)
{
    if (!h)
        return fail(TUCU_ERR_ARG, "null handle");
    h->tensor = on ? 1 : 0;
    return TUCU_OK;
}

int tucu_box_convolve_vec(tucu_box* h, const void* in, size_t in_pitch, int rows, int cols,
                          int channels, void* out, size_t out_pitch, int shift, int normalize,
                          void* stream)
{
    if (!h)
        return fail(TUCU_ERR_ARG, "null handle");
    if (channels < 2 || channels > 4)
        return fail(TUCU_ERR_ARG, "channels must be 2, 3 or 4 (1: tucu_box_convolve)");
    if (!in || !out)
        return fail(TUCU_ERR_ARG, "null image");
    if (rows < 0 || cols < 0)
        return fail(TUCU_ERR_ARG, "negative size");
    const size_t row_bytes = (size_t)cols * channels * sizeof(float);
    if (rows > 0 && (in_pitch < row_bytes || out_pitch < row_bytes))
        return fail(TUCU_ERR_ARG, "pitch smaller than a row");
    if ((reinterpret_cast<uintptr_t>(in) & 15) || (in_pitch & 15))
        return fail(TUCU_ERR_ARG, "input rows must start on 16-byte boundaries");
    if (rows < h->winV || cols < h->winH)
        return TUCU_NOOP;
    box::VecLaunch L;
    std::memset(&L, 0, sizeof(L));
    L.src = in;
    L.src_pitch = in_pitch;
    L.rows = rows;
    L.cols = cols;
    L.channels = channels;
    L.wV = h->winV;
    L.wH = h->winH;
    L.dst = out;
    L.dst_pitch = out_pitch;
    L.oy = shift ? h->winV / 2 : 0;
    L.ox = shift ? h->winH / 2 : 0;
    L.normalize = normalize ? 1 : 0;
    const cudaError_t e = box::launch_vec(L, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? TUCU_OK : cuda_fail(e, "vector box launch");
}

// ---- DisparitySelector ---------------------------------------------------------

int tucu_disparity_create(int disparity_max, int inconsistency, tucu_disparity** out)
{
    if (!out)
        return fail(TUCU_ERR_ARG, "null handle pointer");
    auto* h = new (std::nothrow) tucu_disparity;
    if (!h)
        return fail(TUCU_ERR_NOMEM, "host allocation");
    h->disparity_max = disparity_max;
    h->inconsistency = inconsistency;
    *out = h;
    return TUCU_OK;
}

int tucu_disparity_select(tucu_disparity* h, const void* costs, size_t cost_pitch,
                          size_t slice_pitch, int disparities, int rows, int cols, int cost_dtype,
                          void* out, size_t out_pitch, int out_dtype, int oy, int ox, void* stream)
{
    if (!h)
        return fail(TUCU_ERR_ARG, "null handle");
    if (cost_dtype != I32 && cost_dtype != F32)
        return fail(TUCU_ERR_DTYPE, "costs are int32 or float32");
    if (out_dtype < TUCU_U8 || out_dtype > TUCU_I32)
        return fail(TUCU_ERR_DTYPE, "unknown output dtype");
    if (disparities < 1 || disparities > 256)
        return fail(TUCU_ERR_ARG, "disparity search width must be 1..256");
    if (rows < 1 || cols < 1)
        return TUCU_NOOP;
    if (oy < 0 || ox < 0)
        return fail(TUCU_ERR_ARG, "negative output offset");
    int rc = check_image(costs, cost_pitch, rows, cols, cost_dtype, "costs");
    if (rc)
        return rc;
    if (disparities > 1 && slice_pitch < (size_t)rows * cost_pitch)
        return fail(TUCU_ERR_ARG, "slice pitch smaller than a rows x cols slice");
    if ((rc = check_image(out, out_pitch, rows + oy, cols + ox, out_dtype, "disparity image")))
        return rc;
    sel::SelectLaunch L;
    L.costs = costs;
    L.cost_pitch = cost_pitch;
    L.slice_pitch = slice_pitch;
    L.rows = rows;
    L.cols = cols;
    L.cost_dtype = cost_dtype;
    L.disparities = disparities;
    L.disparity_max = h->disparity_max;
    L.inconsistency = h->inconsistency;
    L.out = out;
    L.out_pitch = out_pitch;
    L.out_dtype = out_dtype;
    L.oy = oy;
    L.ox = ox;
    const cudaError_t e = sel::launch_select(L, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? TUCU_OK : cuda_fail(e, "disparity selection launch");
}

void tucu_disparity_destroy(tucu_disparity* h) { delete h; }

int tucu_box_stereo(tucu_box* h, const void* left, size_t left_pitch, const void* right,
                    size_t right_pitch, int rows, int cols, int dtype, float thresh,
                    int disparities, void* costs, size_t cost_pitch, size_t slice_pitch,
                    int cost_dtype, void* stream)
{
    if (!h)
        return fail(TUCU_ERR_ARG, "null handle");
    int rc = check_image(left, left_pitch, rows, cols, dtype, "left image");
    if (rc)
        return rc;
    if ((rc = check_image(right, right_pitch, rows, cols, dtype, "right image")))
        return rc;
    if ((rc = check_image(costs, cost_pitch, rows, cols, cost_dtype, "costs")))
        return rc;
    const bool integral = dtype == U8 || dtype == I32;
    if (cost_dtype != (integral ? I32 : F32))
        return fail(TUCU_ERR_DTYPE, integral ? "costs of integer images are int32"
                                             : "costs of float images are float32");
    if (disparities < 1)
        return fail(TUCU_ERR_ARG, "disparity search width must be at least 1");
    if (!(thresh >= 0.0f) || !std::isfinite(thresh))
        return fail(TUCU_ERR_ARG, "threshold must be finite and non-negative");
    if (disparities > 1 && slice_pitch < (size_t)rows * cost_pitch)
        return fail(TUCU_ERR_ARG, "slice pitch smaller than a rows x cols slice");
    if (rows < h->winV || cols < h->winH)
        return TUCU_NOOP;  // BoxFilter.h:596-602
    box::StereoLaunch L;
    std::memset(&L, 0, sizeof(L));
    L.left = left;
    L.left_pitch = left_pitch;
    L.right = right;
    L.right_pitch = right_pitch;
    L.rows = rows;
    L.cols = cols;
    L.dtype = dtype;
    L.wV = h->winV;
    L.wH = h->winH;
    // diff<T>(thresh) (TU/cu/functional.h:385-398) holds the threshold as the
    // pixel type: an integer threshold becomes a u_char modulo 256 (C++'s
    // integer conversion), so thresholds from 256 on wrap for u8 images.
    L.thresh = dtype == U8 ? (float)std::fmod(std::floor((double)thresh), 256.0)
                           : integral ? std::floor(thresh) : thresh;
    L.ndisp = disparities;
    L.costs = costs;
    L.cost_pitch = cost_pitch;
    L.slice_pitch = slice_pitch;
    L.cost_dtype = cost_dtype;
    const cudaError_t e = box::launch_stereo(L, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? TUCU_OK : cuda_fail(e, "stereo launch");
}

void tucu_box_destroy(tucu_box* h) { delete h; }

// ---- BoxFilter2<extrema_finder<OP>> ------------------------------------------------

int tucu_extrema_create(int winV, int winH, int win_max, tucu_extrema** out)
{
    if (!out)
        return fail(TUCU_ERR_ARG, "null handle pointer");
    if (win_max > TUCU_EXTREMA_WIN_LIMIT)
        return fail(TUCU_ERR_WINDOW,
                    "extrema window limit above " + std::to_string(TUCU_EXTREMA_WIN_LIMIT));
    const int wmax = win_max <= 0 ? TUCU_WIN_MAX_DEFAULT : win_max;
    const int rc = check_window(winV, winH, wmax);
    if (rc)
        return rc;
    auto* h = new (std::nothrow) tucu_extrema;
    if (!h)
        return fail(TUCU_ERR_NOMEM, "host allocation");
    h->winV = winV;
    h->winH = winH;
    h->winMax = wmax;
    *out = h;
    return TUCU_OK;
}

int tucu_extrema_set_window(tucu_extrema* h, int winV, int winH)
{
    if (!h)
        return fail(TUCU_ERR_ARG, "null handle");
    const int rc = check_window(winV, winH, h->winMax);
    if (rc)
        return rc;
    h->winV = winV;
    h->winH = winH;
    return TUCU_OK;
}

int tucu_extrema_offsets(const tucu_extrema* h, int* offV, int* offH)
{
    if (!h || !offV || !offH)
        return fail(TUCU_ERR_ARG, "null argument");
    *offV = h->winV / 2;
    *offH = h->winH / 2;
    return TUCU_OK;
}

int tucu_extrema_convolve(tucu_extrema* h, int op, const void* in, size_t in_pitch, int rows,
                          int cols, int dtype, void* val, size_t val_pitch, void* pos,
                          size_t pos_pitch, int shift, void* stream)
{
    if (!h)
        return fail(TUCU_ERR_ARG, "null handle");
    if (op != TUCU_EXTREMA_MIN && op != TUCU_EXTREMA_MAX)
        return fail(TUCU_ERR_ARG, "op must be TUCU_EXTREMA_MIN or TUCU_EXTREMA_MAX");
    if (!val && !pos)
        return fail(TUCU_ERR_ARG, "no output: give values, positions or both");
    int rc = check_image(in, in_pitch, rows, cols, dtype, "input");
    if (rc)
        return rc;
    if (val && (rc = check_image(val, val_pitch, rows, cols, dtype, "values")))
        return rc;
    if (pos && rows > 0 && pos_pitch < (size_t)cols * 8)
        return fail(TUCU_ERR_ARG, "positions: pitch smaller than a row of (x, y) pairs");
    if (rows < h->winV || cols < h->winH)
        return TUCU_NOOP;  // BoxFilter.h:551-557
    ext::ExtremaLaunch L;
    std::memset(&L, 0, sizeof(L));
    L.src = in;
    L.src_pitch = in_pitch;
    L.rows = rows;
    L.cols = cols;
    L.dtype = dtype;
    L.wV = h->winV;
    L.wH = h->winH;
    L.is_max = op == TUCU_EXTREMA_MAX;
    L.val = val;
    L.val_pitch = val_pitch;
    L.pos = pos;
    L.pos_pitch = pos_pitch;
    L.oy = shift ? h->winV / 2 : 0;
    L.ox = shift ? h->winH / 2 : 0;
    const cudaError_t e = ext::launch_extrema(L, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? TUCU_OK : cuda_fail(e, "extrema launch");
}

void tucu_extrema_destroy(tucu_extrema* h) { delete h; }

// ---- GuidedFilter2 -----------------------------------------------------------------

int tucu_guided_create(int winV, int winH, float e, int win_max, tucu_guided** out)
{
    if (!out)
        return fail(TUCU_ERR_ARG, "null handle pointer");
    if (win_max > TUCU_WIN_LIMIT)
        return fail(TUCU_ERR_WINDOW, "window limit above " + std::to_string(TUCU_WIN_LIMIT));
    const int wmax = norm_wmax(win_max);
    const int rc = check_window(winV, winH, wmax);
    if (rc)
        return rc;
    if (!std::isfinite(e))
        return fail(TUCU_ERR_ARG, "epsilon must be finite");
    auto* h = new (std::nothrow) tucu_guided;
    if (!h)
        return fail(TUCU_ERR_NOMEM, "host allocation");
    std::memset(h, 0, sizeof(*h));
    h->winV = winV;
    h->winH = winH;
    h->winMax = wmax;
    h->e = e;
    *out = h;
    return TUCU_OK;
}

int tucu_guided_set_window(tucu_guided* h, int winV, int winH)
{
    if (!h)
        return fail(TUCU_ERR_ARG, "null handle");
    const int rc = check_window(winV, winH, h->winMax);
    if (rc)
        return rc;
    h->winV = winV;
    h->winH = winH;
    return TUCU_OK;
}

int tucu_guided_set_epsilon(tucu_guided* h, float e)
{
    if (!h || !std::isfinite(e))
        return fail(TUCU_ERR_ARG, "null handle or non-finite epsilon");
    h->e = e;
    return TUCU_OK;
}

float tucu_guided_epsilon(const tucu_guided* h) { return h ? h->e : 0.0f; }

int tucu_guided_offsets(const tucu_guided* h, int* offV, int* offH)
{
    if (!h || !offV || !offH)
        return fail(TUCU_ERR_ARG, "null argument");
    *offV = h->winV - 1;
    *offH = h->winH - 1;
    return TUCU_OK;
}

int tucu_guided_convolve(tucu_guided* h, const void* in, size_t in_pitch, const void* guide,
                         size_t guide_pitch, int rows, int cols, int in_dtype, void* out,
                         size_t out_pitch, int out_dtype, int shift, void* stream)
{
    if (!h)
        return fail(TUCU_ERR_ARG, "null handle");
    int rc = check_image(in, in_pitch, rows, cols, in_dtype, "input");
    if (rc)
        return rc;
    if (guide) {
        rc = check_image(guide, guide_pitch, rows, cols, in_dtype, "guide");
        if (rc)
            return rc;
    }
    rc = check_image(out, out_pitch, rows, cols, out_dtype, "output");
    if (rc)
        return rc;
    if (in_dtype == I32)
        return fail(TUCU_ERR_DTYPE, "guided input must be u8, f16, bf16 or f32");
    if (rows == 0 || rows < 2 * h->winV - 1 || cols < 2 * h->winH - 1)
        return TUCU_NOOP;
    const int cr = rows + 1 - h->winV, cc = cols + 1 - h->winH;
    const size_t cpitch = ((size_t)cc * sizeof(float2) + 255) / 256 * 256;
    const size_t need = cpitch * (size_t)cr;
    int dev = 0;
    cudaGetDevice(&dev);
    if (h->coef && (h->coef_bytes < need || h->coef_device != dev)) {
        cudaFree(h->coef);
        h->coef = nullptr;
        h->coef_bytes = 0;
    }
    if (!h->coef) {
        const cudaError_t e = cudaMalloc(&h->coef, need);
        if (e != cudaSuccess) {
            h->coef = nullptr;
            return e == cudaErrorMemoryAllocation ? fail(TUCU_ERR_NOMEM, "coefficient scratch")
                                                  : cuda_fail(e, "cudaMalloc");
        }
        h->coef_bytes = need;
        h->coef_device = dev;
    }
    box::GuidedLaunch L;
    std::memset(&L, 0, sizeof(L));
    L.src = in;
    L.src_pitch = in_pitch;
    L.guide = guide;
    L.guide_pitch = guide_pitch;
    L.rows = rows;
    L.cols = cols;
    L.in_dtype = in_dtype;
    L.wV = h->winV;
    L.wH = h->winH;
    L.e = h->e;
    L.coef = h->coef;
    L.coef_pitch = cpitch;
    L.dst = out;
    L.dst_pitch = out_pitch;
    L.out_dtype = out_dtype;
    L.oy = shift ? h->winV - 1 : 0;
    L.ox = shift ? h->winH - 1 : 0;
    const cudaError_t e = box::launch_guided(L, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? TUCU_OK : cuda_fail(e, "guided launch");
}

void tucu_guided_destroy(tucu_guided* h)
{
    if (!h)
        return;
    if (h->coef)
        cudaFree(h->coef);
    delete h;
}

}  // extern "C"
