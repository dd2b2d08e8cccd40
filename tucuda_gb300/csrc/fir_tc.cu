// fir_tc.cu -- separable FIR (FIRFilter2 / FIRGaussianConvolver2, taps up to
// 33) and box sums (BoxFilter2, windows up to 33) of 16-bit float images on
// the 5th-generation tensor cores.
//
// The FP32-pipe kernels (fir_v3.cuh) spend 2R+1 packed FMAs per pixel and
// direction, which caps a radius-16 Gaussian near 570 Gpix/s, a third of the
// HBM bound for 16-bit pixels.  Here both passes are banded matrix products:
//
//   H pass   D1[x'][n] = sum_k A1[x'][k] * B1[n][k]
//            B1 = 64 input rows x K1 input columns (TMA, exact f16 pixels)
//            A1[x'][k] = taps_h[k - (127 - x')]: a Toeplitz band over the
//            column index; with x' = 127 - x it is a Hankel matrix, so its
//            core matrices depend on (row group + column group) only and the
//            descriptor walks one array of 35 core matrices (SBO = LBO) instead
//            of a 128 x 160 matrix
//   V pass   D2[x'][m] = sum_k A2[x'][k] * B2[m][k]
//            A2 = H results transposed (column x', input row k): a ring of 128
//            input rows in tensor memory (the MMA's A operand read from tensor
//            memory, not shared memory), written by the epilogue warps
//            B2[m][k] = taps_v[k - m]: 32 output rows x K2 <= 64 input rows
//
// Precision: the pixels are exact in f16; each coefficient and each H result
// is carried as an f16 pair hi + lo (lo = the rounding error of hi), and the
// products hi*hi, lo*hi, hi*lo are accumulated in FP32 in tensor memory, so
// the sums carry about 22 significant bits (the FP32 pipe carries 24) before
// the output is rounded to its storage type.  Taps that are exact in f16
// (box windows: all ones) skip their lo products.  The H results must stay
// within the f16 range (|value| <= 65504); a larger one sets device error
// code 2.
//
// Roles (352 threads): warp 0 drives TMA (3 input stages of 64 rows), warp 1
// allocates tensor memory and one lane issues the H pass's MMAs, warp 10
// issues the V pass's, warps 2-5 (one per tensor-memory lane quadrant) move
// H results to the ring, warps 6-9 write the outputs, so the two epilogues
// overlap.  H chunks of 64 rows (the H MMAs' N: the tap band, read from shared
// memory by every H MMA, serves twice the rows of a 32-row chunk) feed V
// chunks of 32 rows; tensor memory holds one D1 of 64 columns, two D2 of 32
// and the ring (256 columns, two CTAs per SM).  Every mbarrier wait is
// bounded; when one runs out the CTA stops issuing, sets the error word and
// returns.
#include <algorithm>
#include <cstring>

#include "fir_tc.h"
#include "tucu_common.cuh"
#include "tucu_internal.h"
#include "tucu_tc.cuh"

namespace tucu
{
namespace tcf
{

constexpr int kNst = 3;     // input stages
constexpr int kHCH = 64;    // rows per H chunk (the H MMAs' N); V chunks are kCH = 32
constexpr int kRing = 128;  // H-filtered rows kept in tensor memory (two H chunks)
constexpr int kCmA1 = 16 + kK1Max / 8 - 1;  // core matrices of the Hankel H band
// An input stage: up to three 64-column atoms (the 128-byte swizzled layout,
// 64 rows x 128 bytes each), loaded as TMA boxes of 64 x 64.
constexpr uint32_t kAtomBytes = kHCH * 128;
constexpr int kNAtom = (kK1Max + 63) / 64;
constexpr uint32_t kStageBytes = kNAtom * kAtomBytes;
constexpr uint32_t kB2Sbo = kK2Max / 8 * 128;

// Shared memory map (bytes).
constexpr uint32_t kBarOff = 0;  // 16 mbarriers
constexpr uint32_t kSlotOff = 192;  // tensor-memory base
constexpr uint32_t kAbortOff = 196;
constexpr uint32_t kA1Off = 256;
constexpr uint32_t kA1Bytes = kCmA1 * 128;
constexpr uint32_t kB2Off = kA1Off + 2 * kA1Bytes;
constexpr uint32_t kB2Bytes = kCH * kK2Max * 2;
constexpr uint32_t kInOff = (kB2Off + 2 * kB2Bytes + 1023) / 1024 * 1024;  // swizzle atoms
constexpr uint32_t kSmem = kInOff + kNst * kStageBytes;
static_assert(kSmem <= 113 * 1024, "two CTAs per SM");

// Tensor-memory columns: D1 (one buffer of 64) at 0, D2[b] at 64 + 32b (f32),
// the ring of H results as the V pass's A operand (lane x', two input rows per
// column): hi parts at kRingHi + row / 2, lo parts at kRingLo + row / 2.
constexpr uint32_t kD2Col = 64;
constexpr uint32_t kRingHi = 128;
constexpr uint32_t kRingLo = kRingHi + kRing / 2;
constexpr uint32_t kTmemCols = 256;
static_assert(kRingLo + kRing / 2 <= kTmemCols, "tensor-memory columns");

// The ring is released in four quarters of 32 rows (one per half of an H
// chunk): V chunk c reads quarters c and c + 1 and is the last reader of
// quarter c, so each V chunk releases one quarter and each half of an H chunk
// waits only for its own quarter (the first half no longer waits for the V
// chunk that still reads the second).  Measured on the batched workload: 1183
// Gpix/s against 1164 when a whole H chunk's slot was released by its last
// reader.  Written quarters are still signalled per H chunk: signalling each
// one needs a store wait between the halves and measured 1111-1125.  The H
// epilogue reads both halves of a chunk out of D1 (the first one already
// split) before any quarter wait, so D1 is released without waiting for the
// ring: 1192-1194 against 1184-1186.
constexpr int kQuarters = kRing / kCH;
static_assert(kHCH == 2 * kCH, "two ring quarters per H chunk");

enum Bar : int {
    kFull = 0,                      // [kNst] TMA -> H MMAs
    kEmpty = kFull + kNst,          // [kNst] H MMAs -> TMA
    kD1Full = kEmpty + kNst,        // H MMAs -> H epilogue
    kD1Empty,                       // H epilogue -> H MMAs
    kA2Full,                        // [2] H epilogue -> V MMAs (both quarters of an H chunk written)
    kD2Full = kA2Full + 2,          // [2] V MMAs -> V epilogue
    kD2Empty = kD2Full + 2,         // [2] V epilogue -> V MMAs
    kA2Empty = kD2Empty + 2,        // [kQuarters] V MMAs -> H epilogue (ring quarter no longer read)
    kDrainH = kA2Empty + kQuarters, // the H issuer's MMAs have completed (CTA exit)
    kDrainV,                        // the V issuer's MMAs have completed (CTA exit)
    kNumBars
};
static_assert(kNumBars * 8 <= 192, "barrier slots");

__device__ __forceinline__ uint32_t pack_half2(float a, float b)
{
    const __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

template <class TOut> __device__ __forceinline__ TOut out_cvt(float v);
template <> __device__ __forceinline__ __half out_cvt<__half>(float v) { return __float2half_rn(v); }
template <> __device__ __forceinline__ float out_cvt<float>(float v) { return v; }

struct Ctx
{
    char* smem;
    uint64_t* bar;
    volatile int* abort;
    unsigned long long lim;  // limit of every wait (ns)
    __device__ bool wait(int b, uint32_t parity)
    {
        if (*abort)
            return false;
        if (mbar_wait(bar + b, parity, lim))
            return true;
        *abort = 1;
        raise_device_error(kErrWaitTimeout);
        return false;
    }
};

// 32 H results (two 16-column tensor-memory loads) -> f16 hi parts and the
// f16 rounding errors as lo parts, two rows per 32-bit word; hmax collects
// |hi| for the range check.
__device__ __forceinline__ void split16(const uint32_t (&r0)[16], const uint32_t (&r1)[16], uint32_t (&hi)[16],
                                        uint32_t (&lo)[16], __half2& hmax)
{
#pragma unroll
    for (int e = 0; e < 16; ++e) {
        const float2 v = make_float2(__uint_as_float(e < 8 ? r0[2 * e] : r1[2 * e - 16]),
                                     __uint_as_float(e < 8 ? r0[2 * e + 1] : r1[2 * e - 15]));
        const __half2 h = __float22half2_rn(v);
        hmax = __hmax2(hmax, __habs2(h));
        const float2 d = __fadd2_rn(v, make_float2(-__low2float(h), -__high2float(h)));
        hi[e] = *reinterpret_cast<const uint32_t*>(&h);
        lo[e] = pack_half2(d.x, d.y);
    }
}

// One strip (128 output columns x it.nrows rows from row it.y0) of job J.
template <class TOut>
__device__ __forceinline__ void tc_strip(const TcJob& J, const batch::Item it, char* smem)
{
    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    if (smem_addr(smem) & 1023) {  // the swizzled stages need 1024-byte alignment
        if (tid == 0)
            raise_device_error(kErrAlign);
        return;
    }
    Ctx cx{smem, reinterpret_cast<uint64_t*>(smem + kBarOff),
           reinterpret_cast<volatile int*>(smem + kAbortOff), J.wait_ns};
    const int th = J.th, tv = J.tv;
    const int K1 = (kTW + th - 1 + 15) / 16 * 16;
    const int K2 = (kCH + tv - 1 + 15) / 16 * 16;
    const int nV = (it.nrows + kCH - 1) / kCH;
    const int nH = (kCH * (nV - 1) + K2 - 1) / kHCH + 1;  // H chunks holding every row read

    const int natom = (K1 + 63) / 64;
    const uint32_t stage_bytes = (uint32_t)natom * kAtomBytes;
    const uint32_t expect_bytes = stage_bytes + J.tx_pad;  // tx_pad: 0 outside tests
    const int nfirst = min(nH, kNst);  // input stages loaded during the set-up
    auto load_stage = [&](int j) {
        const int s = j % kNst;
        mbar_arrive_expect_tx(cx.bar + kFull + s, expect_bytes);
        char* st = smem + kInOff + s * kStageBytes;
        for (int a = 0; a < natom; ++a)
            tma_load_2d(st + a * kAtomBytes, &J.tmap, it.x0 + 64 * a, it.y0 + kHCH * j, cx.bar + kFull + s);
    };

    // ---- set-up: barriers and the first input stages (their latency overlaps
    // the rest of the set-up), coefficient bands, tensor memory ----
    {
        if (tid == 0) {
            for (int b = 0; b < kNumBars; ++b) {
                const bool quad = b == kD1Empty || (b >= kA2Full && b < kA2Full + 2) ||
                                  (b >= kD2Empty && b < kD2Empty + 2);
                mbar_init(cx.bar + b, quad ? 4 : 1);
            }
            *cx.abort = 0;
            mbar_fence_init();
            tma_prefetch_desc(&J.tmap);
            for (int j = 0; j < nfirst; ++j)
                load_stage(j);
        }
        const int ncm = 16 + K1 / 8 - 1;
        for (int i = tid; i < ncm * 64; i += kThreads) {
            const int s = 8 * (i / 64) + (i / 8) % 8 + i % 8 - (kTW - 1);
            const float v = (s >= 0 && s < th) ? J.ch[s] : 0.0f;
            const __half hi = __float2half_rn(v);
            const __half lo = __float2half_rn(v - __half2float(hi));
            reinterpret_cast<__half*>(smem + kA1Off)[i] = hi;
            reinterpret_cast<__half*>(smem + kA1Off + kA1Bytes)[i] = lo;
        }
        for (int i = tid; i < kCH * kK2Max; i += kThreads) {
            const int m = i / kK2Max, k = i % kK2Max, s = k - m;
            const float v = (s >= 0 && s < tv) ? J.cv[s] : 0.0f;
            const __half hi = __float2half_rn(v);
            const __half lo = __float2half_rn(v - __half2float(hi));
            const uint32_t off = tc::core_offset(m, k, 128, kB2Sbo);
            *reinterpret_cast<__half*>(smem + kB2Off + off) = hi;
            *reinterpret_cast<__half*>(smem + kB2Off + kB2Bytes + off) = lo;
        }
        fence_proxy_async_smem();
        if (warp == 1)
            tc::tmem_alloc(reinterpret_cast<uint32_t*>(smem + kSlotOff), kTmemCols);
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
    }
    const uint32_t tbase = *reinterpret_cast<volatile uint32_t*>(smem + kSlotOff);

    if (warp == 0) {
        // ---- TMA producer ----
        if (lane == 0) {
            int issued = nfirst;
            for (int j = nfirst; j < nH; ++j, ++issued) {
                if (!cx.wait(kEmpty + j % kNst, ((j / kNst) - 1) & 1))
                    break;
                load_stage(j);
            }
            // the copies still in flight land before the CTA leaves (all
            // have landed already unless a wait ran out)
            for (int j = max(0, issued - kNst); j < issued; ++j)
                mbar_wait(cx.bar + kFull + j % kNst, (j / kNst) & 1, J.wait_ns);
        }
    } else if (warp == 1 || warp == kThreads / 32 - 1) {
        // ---- MMA issuers: warp 1 the H pass, the last warp the V pass.  Each
        // whole warp runs its loop (uniform control flow keeps the
        // descriptors in the uniform datapath) and one elected lane issues;
        // two issuing warps keep the tensor core fed, since each one's waits
        // queue behind its own outstanding MMAs. ----
        const uint32_t idH = tc::idesc_f16(kTW, kHCH), idV = tc::idesc_f16(kTW, kCH);
        // Descriptors are built once; a byte offset o moves one by o >> 4.
        const bool split_h = J.split_h, split_v = J.split_v;
        const uint64_t dA1 = tc::smem_desc(smem_addr(smem + kA1Off), 128, 128);
        const uint64_t dIn = tc::smem_desc_sw128(smem_addr(smem + kInOff), 1024);
        const uint64_t dB2 = tc::smem_desc(smem_addr(smem + kB2Off), 128, kB2Sbo);
        if (warp == 1) {
            // H(j): 64 input rows of the strip -> D1
            for (int j = 0; j < nH; ++j) {
                const int s = j % kNst;
                if (!__all_sync(0xffffffffu, cx.wait(kFull + s, (j / kNst) & 1)))
                    break;
                if (j >= 1 && !__all_sync(0xffffffffu, cx.wait(kD1Empty, (j - 1) & 1)))
                    break;
                tc::fence_after_sync();
                const uint64_t b0 = dIn + ((uint32_t)s * kStageBytes >> 4);
                uint64_t ad = dA1;
                for (int ks = 0; ks < K1 / 16; ++ks) {
                    // atom ks / 4, 32 bytes per K step inside it
                    const uint64_t bd = b0 + (((uint32_t)(ks >> 2) * kAtomBytes + (ks & 3) * 32) >> 4);
                    tc::mma_f16_w(tbase, ad, bd, idH, ks > 0);
                    if (split_h)
                        tc::mma_f16_w(tbase, ad + (kA1Bytes >> 4), bd, idH, 1);
                    ad += 256 >> 4;
                }
                tc::mma_commit_w(cx.bar + kEmpty + s);
                tc::mma_commit_w(cx.bar + kD1Full);
            }
            // every MMA of this warp completes before the tensor memory is freed
            tc::mma_commit_w(cx.bar + kDrainH);
            mbar_wait(cx.bar + kDrainH, 0, J.wait_ns);
        } else {
            // V(c): 32 output rows from ring rows 32c .. 32c + K2 - 1 -> D2[c % 2]
            int ready = 0;  // H chunks known to be written
            for (int c = 0; c < nV; ++c) {
                const int b = c % 2;
                const int last = (kCH * c + K2 - 1) / kHCH;
                bool ok = true;
                for (; ok && ready <= last; ++ready)
                    ok = __all_sync(0xffffffffu, cx.wait(kA2Full + ready % 2, (ready / 2) & 1));
                if (!ok || (c >= 2 && !__all_sync(0xffffffffu, cx.wait(kD2Empty + b, ((c / 2) - 1) & 1))))
                    break;
                tc::fence_after_sync();
                const uint32_t d = tbase + kD2Col + kCH * b;
                uint64_t bd = dB2;
                int p = (kCH * c) % kRing;
                for (int t = 0; t < K2 / 16; ++t) {
                    const uint32_t ahi = tbase + kRingHi + p / 2;
                    tc::mma_f16_ta_w(d, ahi, bd, idV, t > 0);
                    tc::mma_f16_ta_w(d, ahi + (kRingLo - kRingHi), bd, idV, 1);
                    if (split_v)
                        tc::mma_f16_ta_w(d, ahi, bd + (kB2Bytes >> 4), idV, 1);
                    bd += 256 >> 4;
                    p = p + 16 == kRing ? 0 : p + 16;
                }
                tc::mma_commit_w(cx.bar + kD2Full + b);
                tc::mma_commit_w(cx.bar + kA2Empty + c % kQuarters);  // the last reader of quarter c
            }
            tc::mma_commit_w(cx.bar + kDrainV);
            mbar_wait(cx.bar + kDrainV, 0, J.wait_ns);
        }
    } else if (warp < 6) {
        // ---- H epilogue (warps 2..5, tensor-memory lane quadrant warp % 4):
        // the 64 H results of a chunk -> f16 hi/lo pairs in the ring, in two
        // halves of 32 rows ----
        const int q = warp % 4;
        const uint32_t trow = tbase + ((uint32_t)(32 * q) << 16);
        __half2 hmax = __float2half2_rn(0.0f);
        bool ok = true;
        for (int j = 0; ok && j < nH; ++j) {
            if (!__all_sync(0xffffffffu, cx.wait(kD1Full, j & 1)))
                break;
            tc::fence_after_sync();
            // Both halves are read out of D1 (the first one already split into
            // hi / lo parts) before D1 is released, so the next chunk's H MMAs
            // do not wait for the ring quarters; then each half waits for its
            // own quarter and is stored.
            uint32_t hi[16], lo[16], r0[16], r1[16];
            tc::tmem_ld16(trow, r0);
            tc::tmem_ld16(trow + 16, r1);
            tc::wait_ld(r0);
            tc::wait_ld(r1);
            split16(r0, r1, hi, lo, hmax);
            tc::tmem_ld16(trow + 32, r0);
            tc::tmem_ld16(trow + 48, r1);
            tc::wait_ld(r0);
            tc::wait_ld(r1);
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0)
                mbar_arrive(cx.bar + kD1Empty);
            for (int half = 0; half < 2; ++half) {
                const int k = 2 * j + half;  // ring quarter (mod kQuarters) written
                if (k >= kQuarters) {
                    // the quarter is free once V(k - kQuarters), its last reader, has completed
                    if (!__all_sync(0xffffffffu, cx.wait(kA2Empty + k % kQuarters, ((k / kQuarters) - 1) & 1))) {
                        ok = false;
                        break;
                    }
                    tc::fence_after_sync();
                }
                if (half == 1)
                    split16(r0, r1, hi, lo, hmax);
                const int p0 = (kCH * k) % kRing;  // first ring row written
                tc::tmem_st16(trow + kRingHi + p0 / 2, hi);
                tc::tmem_st16(trow + kRingLo + p0 / 2, lo);
            }
            if (!ok)
                break;
            tc::wait_st();
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0)
                mbar_arrive(cx.bar + kA2Full + j % 2);
        }
        // an H result beyond the f16 range became infinite
        if (__hisinf(__low2half(hmax)) || __hisinf(__high2half(hmax)))
            raise_device_error(kErrRange);
    } else {
        // ---- V epilogue (warps 6..9): outputs of a chunk -> HBM ----
        const int q = warp % 4;
        const int xp = 32 * q + lane;
        const uint32_t trow = tbase + ((uint32_t)(32 * q) << 16);
        const int col = it.x0 + (kTW - 1) - xp;
        const bool col_ok = col < J.ocols;
        const float post = J.post;
        const size_t pitch = J.dst_pitch;
        char* p = static_cast<char*>(J.dst) + (size_t)(J.ox + col) * sizeof(TOut) +
                  (size_t)(J.oy + it.y0) * pitch;
        for (int c = 0; c < nV; ++c) {
            const int b = c % 2;
            if (!__all_sync(0xffffffffu, cx.wait(kD2Full + b, (c / 2) & 1)))
                break;
            tc::fence_after_sync();
            uint32_t r[32];
            tc::tmem_ld16(trow + kD2Col + 32 * b, *reinterpret_cast<uint32_t(*)[16]>(r));
            tc::tmem_ld16(trow + kD2Col + 32 * b + 16, *reinterpret_cast<uint32_t(*)[16]>(r + 16));
            tc::wait_ld(*reinterpret_cast<uint32_t(*)[16]>(r));
            tc::wait_ld(*reinterpret_cast<uint32_t(*)[16]>(r + 16));
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0)
                mbar_arrive(cx.bar + kD2Empty + b);
            const int m_end = min(kCH, it.nrows - kCH * c);
            if (col_ok) {
                if (post != 1.0f) {
#pragma unroll
                    for (int m = 0; m < kCH; ++m)
                        r[m] = __float_as_uint(__uint_as_float(r[m]) * post);
                }
                if (m_end == kCH) {
#pragma unroll
                    for (int m = 0; m < kCH; ++m)
                        *reinterpret_cast<TOut*>(p + (size_t)m * pitch) = out_cvt<TOut>(__uint_as_float(r[m]));
                } else {
#pragma unroll
                    for (int m = 0; m < kCH; ++m)
                        if (m < m_end)
                            *reinterpret_cast<TOut*>(p + (size_t)m * pitch) = out_cvt<TOut>(__uint_as_float(r[m]));
                }
            }
            p += (size_t)kCH * pitch;
        }
    }

    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 1)
        tc::tmem_free(tbase, kTmemCols);
}

// The batch's class kernel: one CTA per work item.
template <class TOut>
__global__ void __launch_bounds__(kThreads, 2)
    fir_tc_kernel(const TcJob* __restrict__ jobs, const batch::Item* __restrict__ items)
{
    extern __shared__ __align__(1024) char smem[];
    const batch::Item it = items[blockIdx.x];
    if (it.job >= 0)
        tc_strip<TOut>(jobs[it.job], it, smem);
}

// One image: CTA (x, y) takes column strip x and row band y of `band` rows.
template <class TOut>
__global__ void __launch_bounds__(kThreads, 2) fir_tc_single_kernel(const __grid_constant__ TcJob J, int band)
{
    extern __shared__ __align__(1024) char smem[];
    const int y0 = (int)blockIdx.y * band;
    const batch::Item it{0, (int)blockIdx.x * kTW, y0, min(band, J.orows - y0)};
    tc_strip<TOut>(J, it, smem);
}

const void* kernel_for(int out_dtype)
{
    switch (out_dtype) {
    case F16: return reinterpret_cast<const void*>(fir_tc_kernel<__half>);
    case F32: return reinterpret_cast<const void*>(fir_tc_kernel<float>);
    default: return nullptr;
    }
}

cudaError_t launch_single(const TcJob& J, cudaStream_t st)
{
    const void* fn = J.out_dtype == F16 ? reinterpret_cast<const void*>(fir_tc_single_kernel<__half>)
                                        : reinterpret_cast<const void*>(fir_tc_single_kernel<float>);
    static DeviceOnce attr16, attr32;
    cudaError_t e = (J.out_dtype == F16 ? attr16 : attr32).run([&] {
        return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
    });
    if (e != cudaSuccess)
        return e;
    if (J.orows <= 0 || J.ocols <= 0)
        return cudaSuccess;
    const int ncx = (J.ocols + kTW - 1) / kTW;
    const int band = plan_strip_rows(J.orows, ncx, 2L * sm_count(), kHCH, (J.tv - 1) / 2, 4096);
    const dim3 grid((unsigned)ncx, (unsigned)((J.orows + band - 1) / band));
    void* args[2] = {const_cast<TcJob*>(&J), const_cast<int*>(&band)};
    return cudaLaunchKernel(fn, grid, dim3(kThreads), args, kSmem, st);
}

int full_taps(const float* lobe, int L, float* taps)
{
    const int ls = L & ~1;
    const bool sym = L & 1;
    for (int k = 0; k < ls; ++k) {
        taps[k] = lobe[k];
        taps[2 * ls - k] = sym ? lobe[k] : -lobe[k];
    }
    taps[ls] = sym ? lobe[ls] : 0.0f;
    return 2 * ls + 1;
}

size_t smem_bytes() { return kSmem; }

bool eligible(int in_dtype, int out_dtype, int taps_h, int taps_v)
{
    return in_dtype == F16 && kernel_for(out_dtype) != nullptr && taps_h >= 1 && taps_v >= 1 &&
           taps_h <= kMaxTaps && taps_v <= kMaxTaps;
}

namespace
{
std::atomic<unsigned long long> g_wait_ns{kWaitLimitNs};
std::atomic<unsigned> g_tx_pad{0};
}  // namespace

bool fill_job(TcJob* J, const void* src, size_t src_pitch, int rows, int cols, void* dst,
              size_t dst_pitch, int out_dtype, int oy, int ox, const float* taps_h, int th,
              const float* taps_v, int tv, float post)
{
    std::memset(J, 0, sizeof(*J));
    J->wait_ns = g_wait_ns.load();
    J->tx_pad = g_tx_pad.load();
    if (!make_tmap_2d(&J->tmap, src, F16, cols, rows, src_pitch, 64, kHCH, true))
        return false;
    J->dst = dst;
    J->dst_pitch = dst_pitch;
    J->out_dtype = out_dtype;
    J->orows = rows + 1 - tv;
    J->ocols = cols + 1 - th;
    J->oy = oy;
    J->ox = ox;
    J->th = th;
    J->tv = tv;
    J->post = post;
    auto exact = [](float v) { return (float)__float2half_rn(v) == v; };
    for (int i = 0; i < th; ++i) {
        J->ch[i] = taps_h[i];
        J->split_h |= !exact(taps_h[i]);
    }
    for (int i = 0; i < tv; ++i) {
        J->cv[i] = taps_v[i];
        J->split_v |= !exact(taps_v[i]);
    }
    return true;
}

}  // namespace tcf
}  // namespace tucu

extern "C" int tucu_debug_tc_wait(unsigned long long limit_ns, unsigned tx_pad)
{
    tucu::tcf::g_wait_ns.store(limit_ns ? limit_ns : tucu::kWaitLimitNs);
    tucu::tcf::g_tx_pad.store(tx_pad);
    return TUCU_OK;
}

TUCU_DEFINE_ERROR_ACCESSOR(tucu_tc_tu_error)
