/*
 * tucu_gb300.h -- C ABI of the GB300-native TUCuda 2D-filter path.
 *
 * Plain C: opaque handles, plain pointers, pitches in bytes, integer status
 * codes, CUDA streams passed as void* (a cudaStream_t; NULL = legacy default
 * stream).  No exception crosses this boundary and nothing here exits the
 * process.  Images are row-major pitched 2D arrays in device memory (or, for
 * the server, in host memory); `pitch` is the distance between rows in bytes.
 *
 * Each entry point names the reference interface it replaces (paths relative
 * to the t-ueshiba/TUCuda checkout).  The reference is a C++ template API
 * with no C ABI; the C++ drop-in headers in include/TU/cu/ sit on top of this
 * file and keep the reference's class interfaces.
 *
 * Geometry follows the reference exactly:
 *   FIR / Gaussian:  valid region (rows-2*LS_V) x (cols-2*LS_H), LS = L & ~1,
 *                    written at (LS_V, LS_H) when shift, else at (0,0)
 *                    (TU/cu/FIRFilter.h:37-40, 276-289, 298-312).
 *   Box:             (rows+1-wV) x (cols+1-wH) window SUMS at (wV/2, wH/2)
 *                    when shift (TU/cu/BoxFilter.h:487-509, 542-583).
 *   Guided:          (rows-2(wV-1)) x (cols-2(wH-1)) at (wV-1, wH-1) when
 *                    shift (TU/cu/GuidedFilter.h:202-205, 224-283).
 * Pixels outside the valid region are never written.  An image smaller than
 * the filter support is a silent no-op in the reference; here it returns
 * TUCU_NOOP and writes nothing.
 */
#ifndef TUCU_GB300_H
#define TUCU_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------
 * Reference: std::runtime_error for bad lobe / window sizes
 * (TU/cu/FIRFilter.h:250-251, 344, 375; TU/cu/BoxFilter.h:464-480) and
 * exit(EXIT_FAILURE) on CUDA errors (TU/cu/algorithm.h:86-95). */
typedef enum tucu_status {
    TUCU_OK = 0,
    TUCU_NOOP = 1,            /* image smaller than the filter support: nothing written */
    TUCU_ERR_ARG = -1,        /* null pointer, bad size, pitch or flag */
    TUCU_ERR_LOBE = -2,       /* lobe length not in {2,3,4,5,8,9,16,17} */
    TUCU_ERR_WINDOW = -3,     /* window size 0 or above the handle's maximum */
    TUCU_ERR_DTYPE = -4,      /* unsupported input/output type combination */
    TUCU_ERR_CUDA = -5,       /* a CUDA runtime call failed (see tucu_last_error) */
    TUCU_ERR_NOMEM = -6,      /* device or host allocation failed */
    TUCU_ERR_BUDGET = -7,     /* request larger than the server's memory budget */
    TUCU_ERR_TIMEOUT = -8,    /* a bounded wait ran out */
    TUCU_ERR_STATE = -9,      /* call not valid in the object's current state */
    TUCU_ERR_CANCELLED = -10  /* request cancelled before it ran */
} tucu_status;

/* Pixel storage types.  Arithmetic is FP32 for every float type and int32
 * for box sums of integer input. */
typedef enum tucu_dtype {
    TUCU_U8 = 0,
    TUCU_F16 = 1,
    TUCU_BF16 = 2,
    TUCU_F32 = 3,
    TUCU_I32 = 4
} tucu_dtype;

/* The six operators of FIRGaussianConvolver2 (TU/cu/FIRGaussianConvolver.h:178-242). */
typedef enum tucu_gauss_op {
    TUCU_SMOOTH = 0,  /* (lobe0 H, lobe0 V) */
    TUCU_DIFF_H = 1,  /* (lobe1, lobe0) */
    TUCU_DIFF_V = 2,  /* (lobe0, lobe1) */
    TUCU_DIFF_HH = 3, /* (lobe2, lobe0) */
    TUCU_DIFF_HV = 4, /* (lobe1, lobe1) */
    TUCU_DIFF_VV = 5  /* (lobe0, lobe2) */
} tucu_gauss_op;

#define TUCU_LOBE_MAX 17        /* FIRFilter2::LobeSizeMax (TU/cu/FIRFilter.h:26) */
#define TUCU_WIN_MAX_DEFAULT 23 /* BoxFilter2 / GuidedFilter2 WMAX default (TU/cu/BoxFilter.h:417) */
#define TUCU_WIN_LIMIT 129      /* largest window any handle accepts */

/* ---- library ------------------------------------------------------------- */

/* Library version as 10000*major + 100*minor + patch.  (No reference counterpart.) */
int tucu_version(void);

/* Text for a status code; never NULL.  (No reference counterpart.) */
const char* tucu_status_string(int status);

/* Message of the last failing call on this thread ("" if none).  Replaces the
 * stderr text of checkError (TU/cu/algorithm.h:86-95). */
const char* tucu_last_error(void);

/* Reads (and clears) the device-side error word that a kernel sets when one of
 * its bounded waits runs out (code 1), when a tensor-core batch job's
 * horizontal result leaves the f16 range (code 2) or when a kernel's shared
 * memory lacks the alignment its swizzled tiles need (code 3).  *code = 0
 * when no kernel has reported anything.  Synchronises the current device.
 * (No reference counterpart: the reference has no device-side checks.) */
int tucu_device_error(int* code);

/* Test hook of the tensor-core kernel's bounded waits: for tensor-core jobs
 * set up after this call (single-image calls, batches planned afterwards),
 * every barrier wait gives up after limit_ns nanoseconds (0 restores the
 * default of one second), and each input stage expects tx_pad bytes more
 * than its copies deliver.  0 in normal use; a non-zero pad makes the first
 * wait run out, so that a test can check that the kernel then reports code 1
 * through tucu_device_error and leaves the context usable.  Process-wide.
 * (No reference counterpart.) */
int tucu_debug_tc_wait(unsigned long long limit_ns, unsigned tx_pad);

/* ---- FIRFilter2 ----------------------------------------------------------
 * Replaces TU::cu::FIRFilter2<float, BlockTraits<>> (TU/cu/FIRFilter.h:18-52). */
typedef struct tucu_fir tucu_fir;

/* FIRFilter2::FIRFilter2() (TU/cu/FIRFilter.h:30). */
int tucu_fir_create(tucu_fir** out);

/* FIRFilter2::initialize(lobeH, lobeV) (TU/cu/FIRFilter.h:245-261).  Lobes are
 * stored outermost tap first; lengths 3,5,9,17 are symmetric (last entry =
 * centre), 2,4,8,16 antisymmetric.  The lobes are kept in the handle (not in
 * global __constant__ memory), so handles are independent.  A length above
 * 17 returns TUCU_ERR_LOBE; other unsupported lengths are accepted here and
 * rejected by convolve, as in the reference. */
int tucu_fir_initialize(tucu_fir* h, const float* lobeH, int nH, const float* lobeV, int nV);

/* FIRFilter2::offsetV/offsetH (TU/cu/FIRFilter.h:39-40). */
int tucu_fir_offsets(const tucu_fir* h, int* offV, int* offH);

/* FIRFilter2::convolve(ib, ie, out, shift) (TU/cu/FIRFilter.h:298-377), with
 * the reference's u8/f32 instantiations (FIRFilter.cu:49-68) widened to any
 * of u8/f16/bf16/f32 in and out.  One fused kernel: the horizontal pass stays
 * in shared memory; no intermediate image is written to HBM. */
int tucu_fir_convolve(tucu_fir* h, const void* in, size_t in_pitch, int rows, int cols,
                      int in_dtype, void* out, size_t out_pitch, int out_dtype, int shift,
                      void* stream);

/* on != 0: later convolve calls on this handle run on the tensor cores when
 * f16 input (rows on 16-byte boundaries), f16 or f32 output, at most 33 taps
 * per direction: one tcgen05 kernel (taps and horizontal results as f16 hi/lo
 * pairs, FP32 accumulation), FP32-accurate but not bit-equal to the reference
 * arithmetic; other calls keep the default path.  (No reference counterpart.) */
int tucu_fir_set_tensor_cores(tucu_fir* h, int on);

/* FIRFilter2::~FIRFilter2. */
void tucu_fir_destroy(tucu_fir* h);

/* ---- FIRGaussianConvolver2 -----------------------------------------------
 * Replaces TU::cu::FIRGaussianConvolver2<float> (TU/cu/FIRGaussianConvolver.h:56-90). */
typedef struct tucu_gauss tucu_gauss;

/* Static FIRGaussianConvolver2::initialize(sigma, lobe0, lobe1, lobe2)
 * (TU/cu/FIRGaussianConvolver.h:123-170) with detail::lobeSize
 * (FIRGaussianConvolver.cu:52-98).  Lobe arrays hold up to 17 floats; the
 * lengths are returned in n0/n1/n2.  The coefficients are designed in FP64
 * and rounded once to float; the lengths follow the reference's float rule. */
int tucu_gauss_design(float sigma, float* lobe0, int* n0, float* lobe1, int* n1,
                      float* lobe2, int* n2);

/* The same lobes computed the way the reference computes them
 * (TU/cu/FIRGaussianConvolver.h:123-170 with detail::lobeSize,
 * FIRGaussianConvolver.cu:52-98): float samples, float normalisation sums in
 * the reference's order, no fused multiply-adds.  These equal the reference's
 * lobes bit for bit (they differ from tucu_gauss_design's FP64-designed ones
 * by up to a few ulp of the peak tap). */
int tucu_gauss_design_reference(float sigma, float* lobe0, int* n0, float* lobe1, int* n1,
                                float* lobe2, int* n2);

/* FIRGaussianConvolver2(sigma) (TU/cu/FIRGaussianConvolver.h:96-101). */
int tucu_gauss_create(float sigma, tucu_gauss** out);

/* FIRGaussianConvolver2::initialize(sigma) (TU/cu/FIRGaussianConvolver.h:114-121). */
int tucu_gauss_initialize(tucu_gauss* h, float sigma);

/* on != 0: the handle's lobes (now and after every initialize) are those of
 * tucu_gauss_design_reference, bit-equal to the reference's; the default
 * path's outputs then follow the reference's FP32 tap arithmetic in the CPU
 * oracle's order (within one rounding of the first tap step of the
 * reference's as nvcc compiles it); on == 0 (the default): FP64-designed lobes
 * rounded once.  (No reference counterpart: the reference always designs in
 * float.) */
int tucu_gauss_set_reference_lobes(tucu_gauss* h, int on);

/* FIRGaussianConvolver2::sigma() (TU/cu/FIRGaussianConvolver.h:103-107). */
float tucu_gauss_sigma(const tucu_gauss* h);

/* Copies the handle's lobes (as tucu_gauss_design) for inspection. */
int tucu_gauss_lobes(const tucu_gauss* h, float* lobe0, int* n0, float* lobe1, int* n1,
                     float* lobe2, int* n2);

/* smooth/diffH/diffV/diffHH/diffHV/diffVV(in, ie, out, shift)
 * (TU/cu/FIRGaussianConvolver.h:178-242) selected by `op` (tucu_gauss_op).
 * No per-call lobe upload: the lobes travel as kernel parameters. */
int tucu_gauss_convolve(tucu_gauss* h, int op, const void* in, size_t in_pitch, int rows,
                        int cols, int in_dtype, void* out, size_t out_pitch, int out_dtype,
                        int shift, void* stream);

/* on != 0: later tucu_gauss_convolve calls on this handle run on the tensor
 * cores when the call has an
 * f16 input (rows on 16-byte boundaries), f16 or f32 output, at most 33 taps
 * per direction: one tcgen05 kernel (taps and horizontal results as f16 hi/lo
 * pairs, FP32 accumulation), FP32-accurate but not bit-equal to the reference
 * arithmetic; other calls keep the default path.  (No reference counterpart.) */
int tucu_gauss_set_tensor_cores(tucu_gauss* h, int on);

/* Several operators in ONE pass over the input: bit i of op_mask selects
 * operator i (tucu_gauss_op); outs[i] / out_pitches[i] are read for the
 * selected operators only.  Each output equals the single-operator call.
 * Lobes are zero-padded to the longest selected radius.  (No reference
 * counterpart: the reference reruns convolve per operator.) */
int tucu_gauss_convolve_multi(tucu_gauss* h, unsigned op_mask, const void* in, size_t in_pitch,
                              int rows, int cols, int in_dtype, void* const* outs,
                              const size_t* out_pitches, int out_dtype, int shift, void* stream);

/* Geometry of an operator: offsets of the valid region (TU/cu/FIRFilter.h:39-40). */
int tucu_gauss_offsets(const tucu_gauss* h, int op, int* offV, int* offH);

void tucu_gauss_destroy(tucu_gauss* h);

/* ---- BoxFilter2<box_convolver<S>> -----------------------------------------
 * Replaces TU::cu::BoxFilter2<device::box_convolver<S>, BT, WMAX>
 * (TU/cu/BoxFilter.h:416-539).  Sums are int32 for u8/i32 input (bit-exact,
 * order-free) and FP32 for f16/bf16/f32 input. */
typedef struct tucu_box tucu_box;

/* BoxFilter2(winSizeV, winSizeH) with WMAX = win_max
 * (TU/cu/BoxFilter.h:438-443, 464-480).  win_max <= 0 selects the reference's
 * default 23; windows above win_max return TUCU_ERR_WINDOW. */
int tucu_box_create(int winV, int winH, int win_max, tucu_box** out);

/* setWinSizeV / setWinSizeH (TU/cu/BoxFilter.h:462-480). */
int tucu_box_set_window(tucu_box* h, int winV, int winH);

/* offsetV/offsetH = w/2 (TU/cu/BoxFilter.h:502-509). */
int tucu_box_offsets(const tucu_box* h, int* offV, int* offH);

/* BoxFilter2::convolve(row, rowe, rowO, shift) (TU/cu/BoxFilter.h:542-583).
 * One kernel, no transposed intermediate, no device-wide synchronisation.
 * normalize != 0 writes window means, sum * fl(1/(wV*wH)) (the reciprocal
 * rounded to float), instead of sums -- an extension for FP16/BF16/u8
 * storage, where sums overflow. */
int tucu_box_convolve(tucu_box* h, const void* in, size_t in_pitch, int rows, int cols,
                      int in_dtype, void* out, size_t out_pitch, int out_dtype, int shift,
                      int normalize, void* stream);

/* on != 0: later tucu_box_convolve calls on this handle (windows up to 33)
 * run on the tensor cores when the call has an
 * f16 input (rows on 16-byte boundaries), f16 or f32 output, at most 33 taps
 * per direction: one tcgen05 kernel (taps and horizontal results as f16 hi/lo
 * pairs, FP32 accumulation), FP32-accurate but not bit-equal to the reference
 * arithmetic; other calls keep the default path.  (No reference counterpart.) */
int tucu_box_set_tensor_cores(tucu_box* h, int on);

/* BoxFilter2 with box_convolver<vec<float, N>> (TU/cu/BoxFilter.h:175-194,
 * 542-583): window sums of pixels of `channels` (2, 3 or 4) interleaved
 * float32 values -- the box filter SuperPixels runs over its feature vectors
 * (TU/cu/SuperPixels.h:596-597, 806-812).  Each channel's sum equals the
 * FP32 box sum of that channel plane (tucu_box_convolve on f32).  Rows of
 * both images must start on 16-byte boundaries (pointers and pitches); the
 * reference's Array2 rows are 256-byte aligned.  normalize != 0 writes
 * means. */
int tucu_box_convolve_vec(tucu_box* h, const void* in, size_t in_pitch, int rows, int cols,
                          int channels, void* out, size_t out_pitch, int shift, int normalize,
                          void* stream);

/* Stereo cost aggregation: BoxFilter2::convolve(rowL, rowLe, rowR, rowO, op,
 * disparitySearchWidth) (TU/cu/BoxFilter.h:585-746) with op = diff<T>(thresh)
 * (TU/cu/functional.h:385-398), in the disparity-major layout the reference
 * builds with DISPARITY_MAJOR: for d < disparities,
 *   costs[d][y][x] = sum over the winV x winH window at (y, x) of
 *                    min(|left[y'][x'] - right[y'][x' + d]|, thresh)
 * for y < rows+1-winV, x < cols+1-winH (written at (y, x); nothing else is
 * written).  Right pixels past the last column count as 0.  Slice d starts
 * at costs + d*slice_pitch bytes; each slice is rows x cols with cost_pitch.
 * u8/i32 images sum in int32 (cost_dtype TUCU_I32, exact); f16/bf16/f32 in
 * FP32 (cost_dtype TUCU_F32).  thresh is taken as the pixel type, as diff<T>
 * holds it: integer images use its integer part, and for u8 images that part
 * modulo 256 (thresholds from 256 on wrap).  One kernel, no cost volume
 * intermediate. */
int tucu_box_stereo(tucu_box* h, const void* left, size_t left_pitch, const void* right,
                    size_t right_pitch, int rows, int cols, int dtype, float thresh,
                    int disparities, void* costs, size_t cost_pitch, size_t slice_pitch,
                    int cost_dtype, void* stream);

/* ---- DisparitySelector ----------------------------------------------------
 * Replaces TU::cu::DisparitySelector<T> (TU/cu/StereoUtility.h:109-217): for
 * each pixel (y, x) of the rows x cols region of a disparity-major cost volume
 * (int32 or float32 costs, e.g. from tucu_box_stereo; slice d starts
 * slice_pitch bytes after slice d-1), dL = the first d < disparities with the
 * smallest cost, dR(xr) = the first d <= xr with the smallest C[d][y][xr - d]
 * (the right image's view), and out[oy + y][ox + x] = disparity_max - dL when
 * |dL - dR(x + dL)| < inconsistency, else 0 (StereoUtility.h:56-107).  Where
 * the reference's result is not defined (its right-image minima are updated by
 * unsynchronised blocks; x + dL past the row end reads outside the row) the
 * exact minima and 0 are written.  disparities 1..256; out as u8/f16/bf16/
 * f32/int32 (u8 keeps the low byte, as the reference's int to u_char
 * assignment does). */
typedef struct tucu_disparity tucu_disparity;
int tucu_disparity_create(int disparity_max, int inconsistency, tucu_disparity** out);
int tucu_disparity_select(tucu_disparity* h, const void* costs, size_t cost_pitch,
                          size_t slice_pitch, int disparities, int rows, int cols, int cost_dtype,
                          void* out, size_t out_pitch, int out_dtype, int oy, int ox, void* stream);
void tucu_disparity_destroy(tucu_disparity* h);

void tucu_box_destroy(tucu_box* h);

/* ---- BoxFilter2<extrema_finder<OP>> ----------------------------------------
 * Replaces TU::cu::BoxFilter2 with the convolver device::extrema_finder<OP>
 * (TU/cu/BoxFilter.h:196-233) and OP one of extrema_value<less/greater>,
 * extrema_position<...> or extrema_value_position<...>
 * (TU/cu/BoxFilter.h:100-170): the minimum (or maximum) of every
 * winV x winH window and/or the input position (x, y) where it lies, with the
 * box filter's geometry ((rows+1-wV) x (cols+1-wH) at (wV/2, wH/2) when
 * shift).  Among equal values the reference's two deque passes pick the
 * leftmost column and, in it, the topmost row; so does this one.  Windows up
 * to TUCU_EXTREMA_WIN_LIMIT. */
typedef struct tucu_extrema tucu_extrema;

#define TUCU_EXTREMA_MIN 0       /* extrema over thrust::less */
#define TUCU_EXTREMA_MAX 1       /* extrema over thrust::greater */
#define TUCU_EXTREMA_WIN_LIMIT 64

/* BoxFilter2(winSizeV, winSizeH) with WMAX = win_max (<= 0: 23). */
int tucu_extrema_create(int winV, int winH, int win_max, tucu_extrema** out);

int tucu_extrema_set_window(tucu_extrema* h, int winV, int winH);

/* offsetV/offsetH = w/2 (TU/cu/BoxFilter.h:502-509). */
int tucu_extrema_offsets(const tucu_extrema* h, int* offV, int* offH);

/* BoxFilter2::convolve(row, rowe, rowO, shift) (TU/cu/BoxFilter.h:542-583)
 * with extrema_finder.  `val` (input dtype, may be NULL) receives the window
 * extrema, `pos` (pairs of int32 (x, y), 8 bytes per pixel, may be NULL) the
 * input position of each; at least one must be given.  op is
 * TUCU_EXTREMA_MIN or TUCU_EXTREMA_MAX.  One kernel, no intermediate image. */
int tucu_extrema_convolve(tucu_extrema* h, int op, const void* in, size_t in_pitch, int rows,
                          int cols, int dtype, void* val, size_t val_pitch, void* pos,
                          size_t pos_pitch, int shift, void* stream);

void tucu_extrema_destroy(tucu_extrema* h);

/* ---- GuidedFilter2 ---------------------------------------------------------
 * Replaces TU::cu::GuidedFilter2<float, BT, WMAX> (TU/cu/GuidedFilter.h:134-214). */
typedef struct tucu_guided tucu_guided;

/* GuidedFilter2(wrow, wcol, e) (TU/cu/GuidedFilter.h:151-153).  As in the
 * reference, e is squared internally (a variance-scale epsilon E maps to
 * e = sqrt(E)).  win_max <= 0 selects 23. */
int tucu_guided_create(int winV, int winH, float e, int win_max, tucu_guided** out);

/* setWinSizeV/H and setEpsilon (TU/cu/GuidedFilter.h:172-194). */
int tucu_guided_set_window(tucu_guided* h, int winV, int winH);
int tucu_guided_set_epsilon(tucu_guided* h, float e);
float tucu_guided_epsilon(const tucu_guided* h);

/* offsetV/offsetH = w-1 (TU/cu/GuidedFilter.h:204-205). */
int tucu_guided_offsets(const tucu_guided* h, int* offV, int* offH);

/* GuidedFilter2::convolve(ib, ie, gb, ge, out, shift) (TU/cu/GuidedFilter.h:224-283);
 * guide == NULL selects the self-guided overload (TU/cu/GuidedFilter.h:292-344),
 * whose offset term is reproduced as the reference writes it (b uses the sum
 * of squares, TU/cu/GuidedFilter.h:97).  The input and the guide share
 * in_dtype.  Window sums are mean-shifted per strip and compensated, so the
 * variance term does not cancel.  Uses a scratch coefficient image owned by
 * the handle (grown on demand). */
int tucu_guided_convolve(tucu_guided* h, const void* in, size_t in_pitch, const void* guide,
                         size_t guide_pitch, int rows, int cols, int in_dtype, void* out,
                         size_t out_pitch, int out_dtype, int shift, void* stream);

void tucu_guided_destroy(tucu_guided* h);

/* Guided filter that allocates nothing.  The same computation and result as
 * tucu_guided_convolve, without a handle (window and e are passed directly),
 * for callers that cannot call cudaMalloc: applications whose memory manager
 * owns all of the GPU's memory and forbids further allocation, or loops that
 * cannot take the device-wide synchronisation cudaMalloc/cudaFree imply.
 * Its scratch (the coefficient image between the two window-sum passes) is a
 * 16 MiB file-scope device array that every GPU loading the library holds
 * until the process exits.  An image whose coefficient image
 * (rows+1-winV) x (cols+1-winH) x 8 bytes (rows padded to 16 bytes) exceeds
 * 16 MiB is rejected with TUCU_ERR_ARG and nothing is written.  The first
 * call on a device loads the library's device code there (which is when the
 * 16 MiB are taken) and looks up the array's device address: make that first
 * call at start-up, before the caller's memory manager takes the rest of the
 * GPU and before any stream capture.  The address is kept for the life of
 * the process, so a device reset (cudaDeviceReset) between calls is not
 * supported.  Every call shares the one array and it keeps the last call's
 * contents, so calls that overlap on the GPU (other streams or threads) race
 * and must be serialised by the caller.  No counterpart in the reference. */
int tucu_guided_convolve_noalloc(int winV, int winH, float e, const void* in, size_t in_pitch,
                                 const void* guide, size_t guide_pitch, int rows, int cols,
                                 int in_dtype, void* out, size_t out_pitch, int out_dtype,
                                 int shift, void* stream);

/* ---- batched launch -----------------------------------------------------------
 * Many images of uneven sizes, Gaussian operators and box filters mixed, run by
 * ONE CUDA-graph launch: one specialised kernel per class (operator x pixel type
 * x radius), one CTA per strip, all classes concurrent.  Each output equals the
 * single-image call.
 * (No reference counterpart: the reference launches per image and per pass,
 * TU/cu/FIRFilter.h:263-289, TU/cu/BoxFilter.h:562-582.) */
typedef struct tucu_batch tucu_batch;

typedef enum tucu_batch_op {
    TUCU_BATCH_GAUSS = 0, /* FIRGaussianConvolver2 operator `gauss_op` at `sigma` */
    TUCU_BATCH_BOX = 1    /* BoxFilter2 window sums (or means) of winV x winH */
} tucu_batch_op;

typedef struct tucu_batch_job {
    int op;            /* tucu_batch_op */
    int gauss_op;      /* tucu_gauss_op (TUCU_BATCH_GAUSS); the H and V lobes must
                          have equal radii (always true for smooth) */
    float sigma;       /* TUCU_BATCH_GAUSS */
    int winV, winH;    /* TUCU_BATCH_BOX, each 1..TUCU_WIN_LIMIT */
    int normalize;     /* TUCU_BATCH_BOX: window means instead of sums */
    const void* in;    /* device image */
    size_t in_pitch;
    int in_dtype;
    void* out;         /* device image of the same size */
    size_t out_pitch;
    int out_dtype;
    int rows, cols;
    int shift;         /* as in the single-image calls */
} tucu_batch_job;

int tucu_batch_create(tucu_batch** out);

/* Appends a job; returns its index (>= 0) or a negative status. */
int tucu_batch_add(tucu_batch* b, const tucu_batch_job* job);

/* on != 0: the next plan runs every job with an f16 input, an f16 or f32
 * output and at most 33 taps (Gaussian radius <= 16, box windows <= 33) on
 * the tensor cores (tcgen05): both passes as banded matrix products over
 * f16 hi/lo pairs with FP32 accumulation (about 22 significant bits before
 * the output rounding), instead of the FP32 pipe's bit-exact restatement of
 * the reference arithmetic.  Horizontal results must stay within the f16 range
 * (|value| <= 65504), else device error code 2.  Other jobs keep their
 * kernels.  (No reference counterpart.) */
int tucu_batch_set_tensor_cores(tucu_batch* b, int on);

/* Drops every job (device buffers are kept for reuse). */
int tucu_batch_clear(tucu_batch* b);

/* Builds the work list and uploads it.  fir_strip_rows / box_strip_rows are
 * the strip heights (tile shapes) per operator; <= 0 selects the defaults.
 * Must run after the last add and before a launch; pointers of the jobs are
 * captured here. */
int tucu_batch_plan(tucu_batch* b, int fir_strip_rows, int box_strip_rows);

/* The class kernels launched on `stream` one after another. */
int tucu_batch_launch(tucu_batch* b, void* stream);

/* The same as a CUDA graph: captured on first use after a plan, then
 * replayed on `stream`. */
int tucu_batch_graph_launch(tucu_batch* b, void* stream);

/* Planned jobs, work items (strips), kernels per launch (classes) and the
 * largest dynamic shared memory per CTA. */
int tucu_batch_info(const tucu_batch* b, int* njobs, int* nitems, int* nkernels, size_t* smem);

void tucu_batch_destroy(tucu_batch* b);

/* ---- batches on host images ----------------------------------------------------
 * A batch whose inputs and outputs live in host memory.  Each job names its
 * device buffers (as for tucu_batch_add) and the host images they mirror; one
 * run copies every input in, filters, and copies every valid output region
 * back (pixels outside it are left alone, as the single-image calls leave
 * them).  The jobs are cut into `chunks` groups of consecutive jobs with about
 * equal bytes, each planned as its own batch: the copies in of one group, the
 * kernels of another and the copies out of a third run on three streams at
 * once.  Host images in page-locked memory copy fastest.
 * (No reference counterpart: the reference filters device arrays only.) */
typedef struct tucu_pipe tucu_pipe;

int tucu_pipe_create(int chunks, tucu_pipe** out);

/* Span copies (flags = TUCU_PIPE_SPANS; 0 restores the default): for callers
 * whose host images mirror the device layout (consecutive jobs at the same
 * offsets from each other in host and device memory, equal pitches), a run
 * copies each group's inputs as one contiguous byte range and its outputs as
 * another instead of one pitched copy per image.  The ranges include what
 * lies between the images (row padding, gaps, and on the way out the output
 * pixels outside the valid regions, as the device buffers hold them), so the
 * caller must own those bytes on both sides.  Fewer, larger copies move
 * about 15% faster over the host link.  Set before tucu_pipe_plan. */
#define TUCU_PIPE_SPANS 1
/* Tensor cores (flags |= TUCU_PIPE_TENSOR): every group's batch as after
 * tucu_batch_set_tensor_cores(b, 1). */
#define TUCU_PIPE_TENSOR 2
int tucu_pipe_set_flags(tucu_pipe* p, int flags);

/* Appends a job (device in/out as in tucu_batch_job) with its host images;
 * returns its index (>= 0) or a negative status. */
int tucu_pipe_add(tucu_pipe* p, const tucu_batch_job* job, const void* host_in,
                  size_t host_in_pitch, void* host_out, size_t host_out_pitch);

/* Groups the jobs and plans each group (strip heights as tucu_batch_plan). */
int tucu_pipe_plan(tucu_pipe* p, int fir_strip_rows, int box_strip_rows);

/* One run, ordered after the work already on `stream`; `stream` waits for
 * the last copy out. */
int tucu_pipe_run(tucu_pipe* p, void* stream);

/* Jobs, groups, kernels per run and the bytes one run copies each way (once
 * planned, the planned copies: spans count whole). */
int tucu_pipe_info(const tucu_pipe* p, int* njobs, int* ngroups, int* nkernels,
                   size_t* h2d_bytes, size_t* d2h_bytes);

void tucu_pipe_destroy(tucu_pipe* p);

/* ---- serving ------------------------------------------------------------------
 * A request loop for filter requests on HOST images.  Requests are admitted
 * while their device buffers fit in a fixed budget (one device arena allocated
 * at creation; no allocation per request), grouped into waves as they arrive
 * (continuous batching: a wave forms whenever a stream slot is free, so
 * requests arriving while others run join the next wave), copied in, filtered
 * (Gaussian and box jobs of a wave as one batched launch, guided requests on
 * the same stream) and copied out on one of several streams, so the copies
 * and kernels of successive waves overlap.  Each result equals the single
 * call of the same filter.  (No reference counterpart.) */
typedef struct tucu_server tucu_server;

typedef enum tucu_request_op {
    TUCU_REQ_GAUSS = 0,  /* Gaussian smooth at `sigma` (FIRGaussianConvolver2::smooth) */
    TUCU_REQ_BOX = 1,    /* box sums (or means if normalize) of (2*radius+1)^2 */
    TUCU_REQ_GUIDED = 2  /* guided filter of `in` with `guide` (NULL: self-guided) */
} tucu_request_op;

typedef struct tucu_request {
    int op;              /* tucu_request_op */
    float sigma;         /* TUCU_REQ_GAUSS */
    int radius;          /* TUCU_REQ_BOX / TUCU_REQ_GUIDED: window 2*radius+1 */
    float e;             /* TUCU_REQ_GUIDED: epsilon (squared inside, as GuidedFilter2) */
    int normalize;       /* TUCU_REQ_BOX: window means instead of sums */
    const void* in;      /* HOST image; must stay valid until the request completes */
    size_t in_pitch;
    const void* guide;   /* TUCU_REQ_GUIDED: HOST guide image (NULL = self-guided) */
    size_t guide_pitch;
    int in_dtype;
    void* out;           /* HOST image of the same size, written on completion */
    size_t out_pitch;
    int out_dtype;
    int rows, cols;
} tucu_request;

typedef struct tucu_server_stats {
    uint64_t submitted, completed, rejected, cancelled, failed;
    double p50_ms, p99_ms, max_ms;   /* submit-to-completion latency */
    double gpix_per_s;               /* input pixels of completed requests / busy wall time */
    double wall_s;                   /* first submit to last completion */
    uint64_t waves;                  /* batched waves launched */
    double mean_wave_requests;
    size_t budget_bytes, peak_bytes; /* device arena size and peak use */
} tucu_server_stats;

/* budget_bytes: device memory for request images (and guided scratch);
 * streams: waves in flight at once (>= 1); max_wave: requests per wave. */
int tucu_server_create(size_t budget_bytes, int streams, int max_wave, tucu_server** out);

/* on != 0: Gaussian and box requests with f16 input (and f16/f32 output, at most
 * 33 taps) run on the tensor cores, as tucu_batch_set_tensor_cores.  Call before
 * the first submit (TUCU_ERR_STATE afterwards).  (No reference counterpart.) */
int tucu_server_set_tensor_cores(tucu_server* s, int on);

/* Queues a request (non-blocking).  TUCU_ERR_BUDGET if it can never fit the
 * budget, TUCU_ERR_ARG for a malformed request. */
int tucu_server_submit(tucu_server* s, const tucu_request* r, uint64_t* ticket);

/* Waits up to timeout_s seconds for a request; *status receives its outcome
 * (TUCU_OK, TUCU_ERR_CANCELLED, ...).  TUCU_ERR_TIMEOUT if it is still open. */
int tucu_server_wait(tucu_server* s, uint64_t ticket, double timeout_s, int* status);

/* Cancels a request that has not been admitted yet (TUCU_ERR_STATE otherwise). */
int tucu_server_cancel(tucu_server* s, uint64_t ticket);

/* Waits until every submitted request has finished (or timeout_s). */
int tucu_server_drain(tucu_server* s, double timeout_s);

int tucu_server_get_stats(tucu_server* s, tucu_server_stats* out);

/* Drains, stops the threads and frees the arena. */
void tucu_server_destroy(tucu_server* s);

#ifdef __cplusplus
}
#endif

#endif /* TUCU_GB300_H */
