// fir_strip.cuh -- fused separable FIR over one vertical strip of an image.
//
// Restates FIRFilter2's two passes (TU/cu/FIRFilter.h:181-231) as one on-chip
// pipeline.  A CTA of 256 threads owns kTW = 64 output columns and walks down
// its strip in chunks of CH input rows:
//
//   HBM --TMA 2D box (CH x XW, zero fill at the edges)--> raw[stage]   (mbarrier)
//   raw --convert to float, row pairs interleaved------> stagef
//   stagef --horizontal taps (f32x2 over row pairs)----> ring of H-filtered rows
//   ring --vertical taps (f32x2 over column pairs)-----> registers --> HBM
//
// The ring holds CH + 2*RV H-filtered rows and is double-mapped (each row is
// stored at pos and pos+RING) so the vertical window is always contiguous.
// Nothing but the input and the output touches HBM.
//
// Per-output arithmetic is the reference's device::convolve
// (TU/cu/FIRFilter.h:66-176) in the CPU oracle's order: pair the taps
// symmetric about the centre (sum for odd lengths, difference for even
// lengths), multiply the outermost pair, then fuse each further pair in with
// an FMA, centre tap last.  __fmul2_rn / __ffma2_rn / __fadd2_rn round each
// lane exactly like the scalar instructions, so results match the oracle bit
// for bit.  (nvcc compiles the reference's expression with the outermost pair
// fused into the rounded second product instead, measured on the GPU: one
// rounding of the first step apart.  Lobes padded with leading zero taps give
// the same results in this order, which the batch relies on.)
#pragma once
#include "tucu_common.cuh"
#include "tucu_tma.cuh"

#include <type_traits>

namespace tucu
{
namespace fir
{

constexpr int kThreads = 256;
constexpr int kTW = 64;       // output columns per strip
constexpr int kMaxStage = 8;  // mbarriers reserved at the start of shared memory

__host__ __device__ constexpr int round_up(int v, int m) { return (v + m - 1) / m * m; }
__host__ __device__ constexpr size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Coefficients of up to three horizontal and three vertical lobes, each
// zero-padded on the outer side to the strip's radius and stored outermost
// tap first (index R = centre).  sym bit i set = lobe i is symmetric.
struct LobeSet
{
    float h[3][TUCU_LOBE_MAX];
    float v[3][TUCU_LOBE_MAX];
    int sym_h, sym_v;
};

// One FIR job: source image, outputs and their lobe selection.
struct FirJob
{
    const void* src;
    size_t src_pitch;
    int rows, cols;        // input extent
    int pad_y, pad_x;      // zero rows/columns assumed above/left of the input (plain loads only)
    int orows, ocols;      // valid output extent
    int oy, ox;            // placement of the valid region in the outputs
    int nh;                // horizontal lobes in use (1..NH)
    int nout;              // outputs (1..6)
    int out_dtype;
    void* dst[6];
    size_t dst_pitch[6];
    unsigned char hsel[6];  // horizontal lobe of each output
    unsigned char vsel[6];  // vertical lobe of each output
};

// Everything a host launcher needs for one FIR job.
struct FirLaunch
{
    FirJob job;
    LobeSet lobes;
    int rh, rv;      // strip radii (2, 4, 8 or 16)
    int in_dtype;
    int strip_rows;  // output rows per CTA; <= 0 picks a default
    int use_tma;
    CUtensorMap tmap;
};

cudaError_t launch_u8(const FirLaunch& L, cudaStream_t stream);
cudaError_t launch_f16(const FirLaunch& L, cudaStream_t stream);
cudaError_t launch_bf16(const FirLaunch& L, cudaStream_t stream);
cudaError_t launch_f32(const FirLaunch& L, cudaStream_t stream);

// Per-CTA pipeline state carried across strips (stage phase bits).
struct Pipe
{
    uint32_t phase_bits;
};

template <int RH, int RV, int NH, int CH, class TIn>
struct StripCfg
{
    static constexpr int XW = round_up(kTW + 2 * RH, 16);  // staged input columns
    static constexpr int RING = CH + 2 * RV;
    static constexpr int PRO = (2 * RV + CH - 1) / CH;     // chunks before the first output
    // TMA pipeline depth: fewer stages for wide types so that several CTAs
    // fit on an SM.
    static constexpr int NSTAGE = sizeof(TIn) == 1 ? 6 : sizeof(TIn) == 2 ? 4 : 3;
    static constexpr int VR = CH / 8;                      // output rows per thread (V pass)
    static constexpr int RAW_BYTES = CH * XW * (int)sizeof(TIn);
    // Staged row pairs are 16-byte units (two float2 = two columns of a row
    // pair) with one unit of padding after every 8, so that lanes reading
    // units 32 bytes apart hit distinct banks.
    static constexpr int UNITS = XW / 2;
    static constexpr int ROWU = UNITS + UNITS / 8;
    // mbarriers and lobe coefficients first (fixed places), then the buffers.
    static constexpr size_t BAR_OFF = 0;
    static constexpr size_t COEF_OFF = 128;  // float2 cH[3][17], cV[3][17]
    static constexpr size_t RAW_OFF = 1024;
    static constexpr size_t STAGE_OFF = RAW_OFF + (size_t)NSTAGE * align_up(RAW_BYTES, 128);
    static constexpr size_t RING_OFF = STAGE_OFF + align_up((size_t)(CH / 2) * ROWU * 16, 128);
    static constexpr size_t SMEM = RING_OFF + (size_t)NH * 2 * RING * kTW * sizeof(float);
    static_assert(CH % 16 == 0, "chunk must be a multiple of 16 rows");
    static_assert(NSTAGE <= kMaxStage, "barrier slots");
    static_assert(XW <= 256, "TMA box width");
    static_assert((XW * sizeof(TIn)) % 16 == 0, "TMA inner box bytes");
};

__device__ __forceinline__ int pad_unit(int u) { return u + (u >> 3); }

__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

// pair = a + b (symmetric) or a - b (antisymmetric).
template <bool SYM>
__device__ __forceinline__ float2 pair2(float2 a, float2 b)
{
    return SYM ? __fadd2_rn(a, b) : __fadd2_rn(a, neg2(b));
}

// One packed output pair: taps v(0..2R) through the splatted lobe c[0..R].
template <int R, bool SYM, class LD>
__device__ __forceinline__ float2 tap2(const float2 (&c)[R + 1], LD v)
{
    float2 acc = __fmul2_rn(c[0], pair2<SYM>(v(0), v(2 * R)));
#pragma unroll
    for (int k = 1; k < R; ++k)
        acc = __ffma2_rn(c[k], pair2<SYM>(v(k), v(2 * R - k)), acc);
    if (SYM)
        acc = __ffma2_rn(c[R], v(R), acc);
    return acc;
}

template <class TIn>
__device__ __forceinline__ float4 load4_to_float(const TIn* p);

template <>
__device__ __forceinline__ float4 load4_to_float<uint8_t>(const uint8_t* p)
{
    const uint32_t u = *reinterpret_cast<const uint32_t*>(p);
    return make_float4((float)(u & 0xff), (float)((u >> 8) & 0xff), (float)((u >> 16) & 0xff),
                       (float)(u >> 24));
}
template <>
__device__ __forceinline__ float4 load4_to_float<__half>(const __half* p)
{
    const uint2 u = *reinterpret_cast<const uint2*>(p);
    const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&u.x));
    const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&u.y));
    return make_float4(a.x, a.y, b.x, b.y);
}
template <>
__device__ __forceinline__ float4 load4_to_float<__nv_bfloat16>(const __nv_bfloat16* p)
{
    const uint2 u = *reinterpret_cast<const uint2*>(p);
    const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&u.x));
    const float2 b = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&u.y));
    return make_float4(a.x, a.y, b.x, b.y);
}
template <>
__device__ __forceinline__ float4 load4_to_float<float>(const float* p)
{
    return *reinterpret_cast<const float4*>(p);
}

// Stores VR rows of two adjacent outputs of type T (rows below nvalid skipped).
template <class T, int VR>
__device__ __forceinline__ void store_rows(void* base, size_t pitch, int y, int x,
                                           const float2 (&acc)[VR], int nvalid, bool both)
{
#pragma unroll
    for (int r = 0; r < VR; ++r) {
        if (r >= nvalid)
            break;
        T* p = reinterpret_cast<T*>(row_ptr(base, pitch, y + r)) + x;
        T a, b;
        if constexpr (std::is_same<T, uint8_t>::value) {
            a = f2u8(acc[r].x);
            b = f2u8(acc[r].y);
        } else if constexpr (std::is_same<T, __half>::value) {
            a = __float2half_rn(acc[r].x);
            b = __float2half_rn(acc[r].y);
        } else if constexpr (std::is_same<T, __nv_bfloat16>::value) {
            a = __float2bfloat16_rn(acc[r].x);
            b = __float2bfloat16_rn(acc[r].y);
        } else if constexpr (std::is_same<T, int32_t>::value) {
            a = __float2int_rz(acc[r].x);
            b = __float2int_rz(acc[r].y);
        } else {
            a = acc[r].x;
            b = acc[r].y;
        }
        if (both && (reinterpret_cast<uintptr_t>(p) % (2 * sizeof(T))) == 0) {
            struct alignas(2 * sizeof(T)) P2 { T a, b; };
            *reinterpret_cast<P2*>(p) = P2{a, b};
        } else {
            p[0] = a;
            if (both)
                p[1] = b;
        }
    }
}

// Runs one strip: output columns [x0, x0+64), output rows [y0, y0 + CH*nsteps)
// (clipped to the valid extent).  tmap == nullptr selects plain loads (images
// whose base or pitch is not 16-byte aligned).  Returns false if a bounded
// wait ran out; the error word is set and the CTA must stop.
template <int RH, int RV, int NH, int CH, class TIn>
__device__ bool run_strip(const FirJob& job, const LobeSet& lobes, const CUtensorMap* tmap,
                          int x0, int y0, int nsteps, unsigned char* smem, Pipe& pipe)
{
    using Cfg = StripCfg<RH, RV, NH, CH, TIn>;
    constexpr int XW = Cfg::XW, RING = Cfg::RING, VR = Cfg::VR, PRO = Cfg::PRO;
    constexpr int ROWU = Cfg::ROWU;
    constexpr int kNStage = Cfg::NSTAGE;
    TIn* raw = reinterpret_cast<TIn*>(smem + Cfg::RAW_OFF);
    float4* stage4 = reinterpret_cast<float4*>(smem + Cfg::STAGE_OFF);
    float* ring = reinterpret_cast<float*>(smem + Cfg::RING_OFF);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + Cfg::BAR_OFF);
    float2* cH = reinterpret_cast<float2*>(smem + Cfg::COEF_OFF);
    float2* cV = cH + 3 * TUCU_LOBE_MAX;
    constexpr int kRawStride = (int)(align_up(Cfg::RAW_BYTES, 128) / sizeof(TIn));

    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    // Chunk q covers input rows y0 + 2RV + CH*(q-PRO) + [0,CH); the first PRO
    // chunks only fill the ring with the 2*RV rows above the first output.
    const int nchunks = nsteps + PRO;

    auto chunk_row0 = [&](int q) { return y0 + 2 * RV + CH * (q - PRO); };

    // The previous strip of this CTA may still read the coefficients.
    __syncthreads();
    for (int i = tid; i < 3 * TUCU_LOBE_MAX; i += kThreads) {
        const float h = lobes.h[i / TUCU_LOBE_MAX][i % TUCU_LOBE_MAX];
        const float v = lobes.v[i / TUCU_LOBE_MAX][i % TUCU_LOBE_MAX];
        cH[i] = make_float2(h, h);
        cV[i] = make_float2(v, v);
    }

    // Prologue: put the first kNStage chunks in flight.
    if (tmap && tid == 0) {
        fence_proxy_async_smem();
        for (int q = 0; q < kNStage && q < nchunks; ++q) {
            mbar_arrive_expect_tx(&bars[q], (uint32_t)Cfg::RAW_BYTES);
            tma_load_2d(raw + q * kRawStride, tmap, x0, chunk_row0(q), &bars[q]);
        }
    }

    for (int q = 0; q < nchunks; ++q) {
        const int stage = q % kNStage;
        // ---- 1. stage chunk q as float row pairs --------------------------------
        bool failed = false;
        if (tmap) {
            const uint32_t parity = (pipe.phase_bits >> stage) & 1u;
            failed = !mbar_wait(&bars[stage], parity);
            if (!failed) {
                const TIn* src = raw + stage * kRawStride;
                constexpr int NV = (CH / 2) * (XW / 4);
                for (int i = tid; i < NV; i += kThreads) {
                    const int rp = i / (XW / 4), c4 = (i % (XW / 4)) * 4;
                    const float4 a = load4_to_float<TIn>(src + (2 * rp) * XW + c4);
                    const float4 b = load4_to_float<TIn>(src + (2 * rp + 1) * XW + c4);
                    float4* d = stage4 + rp * ROWU;
                    d[pad_unit(c4 / 2)] = make_float4(a.x, b.x, a.y, b.y);
                    d[pad_unit(c4 / 2 + 1)] = make_float4(a.z, b.z, a.w, b.w);
                }
            }
        } else {
            const int r0 = chunk_row0(q) - job.pad_y;
            constexpr int NE = (CH / 2) * XW;
            for (int i = tid; i < NE; i += kThreads) {
                const int rp = i / XW, c = i % XW;
                const int x = x0 + c - job.pad_x, ya = r0 + 2 * rp, yb = ya + 1;
                float a = 0.0f, b = 0.0f;
                if (x >= 0 && x < job.cols) {
                    if (ya >= 0 && ya < job.rows)
                        a = load_px<TIn>(row_ptr(job.src, job.src_pitch, ya), x);
                    if (yb >= 0 && yb < job.rows)
                        b = load_px<TIn>(row_ptr(job.src, job.src_pitch, yb), x);
                }
                reinterpret_cast<float2*>(stage4 + rp * ROWU + pad_unit(c / 2))[c & 1] =
                    make_float2(a, b);
            }
        }
        if (__syncthreads_or(failed)) {
            if (tid == 0)
                raise_device_error(kErrWaitTimeout);
            // Let any copy still in flight land before the CTA leaves.
            if (tmap)
                for (int s = 0; s < kNStage; ++s)
                    mbar_wait(&bars[s], (pipe.phase_bits >> s) & 1u);
            return false;
        }
        if (tmap) {
            pipe.phase_bits ^= (1u << stage);
            // ---- 2. refill this stage with chunk q + kNStage -------------------
            if (tid == 0 && q + kNStage < nchunks) {
                fence_proxy_async_smem();
                mbar_arrive_expect_tx(&bars[stage], (uint32_t)Cfg::RAW_BYTES);
                tma_load_2d(raw + stage * kRawStride, tmap, x0, chunk_row0(q + kNStage),
                            &bars[stage]);
            }
        }

        // ---- 3. horizontal pass: H-rows hbase + [0, CH) into the ring ---------------
        // Task = one row pair x four columns; a thread's columns c..c+2RH+3
        // are RH+2 staged units.
        const int hbase = 2 * RV + CH * (q - PRO);  // H-row index of chunk row 0
        for (int l = 0; l < NH && l < job.nh; ++l) {
            float2 c[RH + 1];
#pragma unroll
            for (int k = 0; k <= RH; ++k)
                c[k] = cH[l * TUCU_LOBE_MAX + k];
            const bool sym = (lobes.sym_h >> l) & 1;
            float* rl = ring + l * (2 * RING * kTW);
            for (int t = tid; t < (CH / 2) * (kTW / 4); t += kThreads) {
                const int rp = t / (kTW / 4), c4 = (t % (kTW / 4)) * 4;
                if (hbase + 2 * rp + 1 < 0)
                    continue;  // rows above the strip (first chunks only)
                const float4* srow = stage4 + rp * ROWU;
                float4 w[RH + 2];
#pragma unroll
                for (int i = 0; i < RH + 2; ++i)
                    w[i] = srow[pad_unit(c4 / 2 + i)];
                // v(j) = (row 2rp, row 2rp+1) at column c4 + j
                auto v = [&](int j) {
                    return (j & 1) ? make_float2(w[j >> 1].z, w[j >> 1].w)
                                   : make_float2(w[j >> 1].x, w[j >> 1].y);
                };
                float2 a[4];
                if (sym) {
#pragma unroll
                    for (int m = 0; m < 4; ++m)
                        a[m] = tap2<RH, true>(c, [&](int j) { return v(j + m); });
                } else {
#pragma unroll
                    for (int m = 0; m < 4; ++m)
                        a[m] = tap2<RH, false>(c, [&](int j) { return v(j + m); });
                }
                int h = hbase + 2 * rp;
                int pos = h % RING;
                if (pos < 0)
                    pos += RING;
                const float4 r0v = make_float4(a[0].x, a[1].x, a[2].x, a[3].x);
                const float4 r1v = make_float4(a[0].y, a[1].y, a[2].y, a[3].y);
                if (h >= 0) {
                    *reinterpret_cast<float4*>(rl + pos * kTW + c4) = r0v;
                    *reinterpret_cast<float4*>(rl + (pos + RING) * kTW + c4) = r0v;
                }
                pos = (pos + 1 == RING) ? 0 : pos + 1;
                *reinterpret_cast<float4*>(rl + pos * kTW + c4) = r1v;
                *reinterpret_cast<float4*>(rl + (pos + RING) * kTW + c4) = r1v;
            }
        }
        __syncthreads();

        // ---- 4. vertical pass for output chunk s = q - PRO -------------------------
        if (q < PRO)
            continue;
        const int s = q - PRO;
        const int p = (CH * s) % RING;     // ring position of H-row CH*s
        const int r0 = warp * VR;          // this thread's first row in the chunk
        const int cpos = lane * 2;         // its two columns
        const int ybase = y0 + CH * s + r0;  // its first output row (valid coords)
        const int xo = x0 + cpos;            // its first output column (valid coords)
        const int nvalid = min(VR, job.orows - ybase);
        const bool active = xo < job.ocols && nvalid > 0;
        const bool both = xo + 1 < job.ocols;
        for (int o = 0; o < job.nout; ++o) {
            const int hs = job.hsel[o], vs = job.vsel[o];
            float2 c[RV + 1];
#pragma unroll
            for (int k = 0; k <= RV; ++k)
                c[k] = cV[vs * TUCU_LOBE_MAX + k];
            const bool sym = (lobes.sym_v >> vs) & 1;
            const float* col = ring + hs * (2 * RING * kTW) + (p + r0) * kTW + cpos;
            float2 acc[VR];
            if (sym) {
#pragma unroll
                for (int r = 0; r < VR; ++r)
                    acc[r] = tap2<RV, true>(c, [&](int i) {
                        return *reinterpret_cast<const float2*>(col + (r + i) * kTW);
                    });
            } else {
#pragma unroll
                for (int r = 0; r < VR; ++r)
                    acc[r] = tap2<RV, false>(c, [&](int i) {
                        return *reinterpret_cast<const float2*>(col + (r + i) * kTW);
                    });
            }
            if (!active)
                continue;
            void* dst = job.dst[o];
            const size_t pitch = job.dst_pitch[o];
            const int y = ybase + job.oy, x = xo + job.ox;
            switch (job.out_dtype) {
            case U8: store_rows<uint8_t, VR>(dst, pitch, y, x, acc, nvalid, both); break;
            case F16: store_rows<__half, VR>(dst, pitch, y, x, acc, nvalid, both); break;
            case BF16: store_rows<__nv_bfloat16, VR>(dst, pitch, y, x, acc, nvalid, both); break;
            case I32: store_rows<int32_t, VR>(dst, pitch, y, x, acc, nvalid, both); break;
            default: store_rows<float, VR>(dst, pitch, y, x, acc, nvalid, both); break;
            }
        }
    }
    return true;
}

}  // namespace fir
}  // namespace tucu
