// fir_v3.cuh -- warp-specialised single-operator separable FIR strip.
//
// Same arithmetic as fir_strip.cuh (the reference's device::convolve,
// TU/cu/FIRFilter.h:66-176: paired taps, outermost first, FMA-fused, centre
// last, so results are bit-identical), organised so that nearly every
// instruction is a packed FP32 operation:
//
//   thread 0 ............ TMA producer: 2D boxes of kCH x XW input pixels into
//                         a ring of raw stages (mbarrier transaction counts)
//   warps 0-3 (H role) .. convert a stage to float row pairs (padded layout,
//                         conflict-free), then horizontal taps for tasks of
//                         one row pair x 8 columns (packed across the pair)
//                         into a double-buffered chunk of H-filtered rows
//   warps 4-7 (V role) .. one output column per thread for the whole strip:
//                         a register sliding window of H-filtered row pairs
//                         P_k = (H[2k], H[2k+1]) and Q_k = (H[2k+1], H[2k+2]),
//                         so an output row pair costs one shared load, two
//                         moves and 2R+1 packed FP operations
//
// The roles hand chunks over with named barriers (full[b] / empty[b], 128 H +
// 128 V arrivals per phase, balanced over the strip).  Every TMA wait is
// bounded; if one runs out the H warps keep to the barrier protocol without
// reading the stage, the V warps store nothing, the error word is set and
// the strip returns false.
#pragma once
#include <type_traits>

#include "fir_strip.cuh"

namespace tucu
{
namespace fir3
{

using fir::FirJob;
using fir::LobeSet;
using fir::Pipe;

constexpr int kThreads = 256;
constexpr int kTW = 128;    // output columns per strip
constexpr int kCH = 32;     // rows per chunk
constexpr int kHalf = 128;  // threads per role
constexpr int kHB = kCH / 2;  // row pairs per chunk

template <int RH, int RV, class TIn>
struct Cfg
{
    static constexpr int XW = fir::round_up(kTW + 2 * RH, 16);  // staged input columns
    static constexpr int PRO = (2 * RV + kCH - 1) / kCH;         // chunks before the first output
    static constexpr int NSTAGE = sizeof(TIn) == 1 ? 6 : sizeof(TIn) == 2 ? 4 : 2;
    static constexpr int RAW_BYTES = kCH * XW * (int)sizeof(TIn);
    // Staged row pairs: 16-byte units of two columns, one pad unit per 4.
    static constexpr int UNITS = XW / 2;
    static constexpr int ROWU = UNITS + UNITS / 4 + 1;
    // H-filtered chunk: kHB row pairs x kTW columns of float2 (row pair
    // packed), 16-byte units of two columns, one pad unit per 8.
    static constexpr int HROWU = kTW / 2 + kTW / 16;
    static constexpr size_t BAR_OFF = 0;
    static constexpr size_t FLAG_OFF = 96;   // shared failure flag
    static constexpr size_t COEF_OFF = 128;  // float2 cH[17], cV[17]
    static constexpr size_t RAW_OFF = 1024;
    static constexpr size_t STAGE_OFF = RAW_OFF + (size_t)NSTAGE * fir::align_up(RAW_BYTES, 128);
    static constexpr size_t HBUF_OFF = STAGE_OFF + fir::align_up((size_t)kHB * ROWU * 16, 128);
    static constexpr size_t SMEM = HBUF_OFF + (size_t)2 * kHB * HROWU * 16;
    static_assert(XW <= 256, "TMA box width");
    static_assert((XW * sizeof(TIn)) % 16 == 0, "TMA inner box bytes");
    static_assert(NSTAGE <= fir::kMaxStage, "barrier slots");
};

__device__ __forceinline__ int pad4(int u) { return u + (u >> 2); }
__device__ __forceinline__ int pad8(int u) { return u + (u >> 3); }

__device__ __forceinline__ void named_sync(int id, int count)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
__device__ __forceinline__ void named_arrive(int id, int count)
{
    asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// Barrier ids (0 is __syncthreads): 1 = H warps only; 2,3 = chunk buffer
// full[b]; 4,5 = chunk buffer empty[b].
constexpr int kBarH = 1, kBarFull = 2, kBarEmpty = 4;

__device__ __forceinline__ void store_one(void* row, int x, int dt, float v)
{
    switch (dt) {
    case U8: static_cast<uint8_t*>(row)[x] = f2u8(v); break;
    case F16: static_cast<__half*>(row)[x] = __float2half_rn(v); break;
    case BF16: static_cast<__nv_bfloat16*>(row)[x] = __float2bfloat16_rn(v); break;
    case I32: static_cast<int32_t*>(row)[x] = __float2int_rz(v); break;
    default: static_cast<float*>(row)[x] = v; break;
    }
}

// ---- V role ---------------------------------------------------------------------

// The window holds P_k and Q_k in slot k mod W, W = R + 2 (even).  Output
// pair m (strip rows 2m, 2m+1) needs T_i = (H[2m+i], H[2m+1+i]), i = 0..2R:
// T_i = P_{m+i/2} for even i and Q_{m+(i-1)/2} for odd i.  Each step produces
// the two pairs m and m+1 (two independent FMA chains); the loop is unrolled
// by W/2 steps so that every slot index is a compile-time constant.
template <int R, bool SYM>
struct VWin
{
    static constexpr int W = R + 2;
    float2 P[W], Q[W];

    template <int M>
    __device__ __forceinline__ float2 T(int i) const
    {
        return (i & 1) ? Q[(M + (i - 1) / 2) % W] : P[(M + i / 2) % W];
    }

    template <int M>
    __device__ __forceinline__ float2 tap(const float2 (&c)[R + 1]) const
    {
        float2 acc = __fmul2_rn(c[0], fir::pair2<SYM>(T<M>(0), T<M>(2 * R)));
#pragma unroll
        for (int k = 1; k < R; ++k)
            acc = __ffma2_rn(c[k], fir::pair2<SYM>(T<M>(k), T<M>(2 * R - k)), acc);
        if (SYM)
            acc = __ffma2_rn(c[R], T<M>(R), acc);
        return acc;
    }
};

template <int RH, int RV, class TIn, bool SYM>
__device__ void v_role(const FirJob& job, const float2* __restrict__ hbuf, const float2 (&c)[RV + 1],
                       int x0, int y0, int nrows, int nchunks, const volatile int* failed)
{
    using C = Cfg<RH, RV, TIn>;
    using Win = VWin<RV, SYM>;
    constexpr int W = Win::W;
    constexpr int HB0 = 2 * RV - kCH * C::PRO;  // H-row of chunk 0's first row (<= 0)
    const int col = threadIdx.x - kHalf;
    const int x = x0 + col;
    const bool col_ok = x < job.ocols;
    const int npairs = (nrows + 1) / 2;
    const int kmax = (HB0 + kCH * nchunks) / 2;       // row pairs the strip produces
    const int hoff = pad8(col >> 1) * 2 + (col & 1);  // float2 offset of this column in a row pair

    int cur = -1;  // chunk currently held
    const float2* cb = hbuf;
    auto move_to = [&](int q) {
        if (cur >= 0 && cur + 2 < nchunks)
            named_arrive(kBarEmpty + (cur & 1), 2 * kHalf);
        named_sync(kBarFull + (q & 1), 2 * kHalf);
        cur = q;
        cb = hbuf + (size_t)(q & 1) * kHB * C::HROWU * 2;
    };
    auto fetch = [&](int k) -> float2 {
        if (k >= kmax)
            return make_float2(0.0f, 0.0f);  // past the strip: feeds only discarded rows
        const int rel = 2 * k - HB0;          // >= 0
        const int q = rel / kCH;
        if (q != cur)
            move_to(q);
        return cb[((rel - q * kCH) >> 1) * (C::HROWU * 2) + hoff];
    };

    Win w;
    // Warm-up: P_0..P_{R-1}, Q_0..Q_{R-2}.
#pragma unroll
    for (int k = 0; k < RV; ++k) {
        w.P[k] = fetch(k);
        if (k > 0)
            w.Q[k - 1] = make_float2(w.P[k - 1].y, w.P[k].x);
    }
    const int dt = job.out_dtype;
    void* dst = job.dst[0];
    const size_t pitch = job.dst_pitch[0];
    auto put = [&](int m, float2 acc) {
        const int y = y0 + 2 * m;
        if (col_ok && !*failed) {
            if (2 * m < nrows && y < job.orows)
                store_one(row_ptr(dst, pitch, y + job.oy), x + job.ox, dt, acc.x);
            if (2 * m + 1 < nrows && y + 1 < job.orows)
                store_one(row_ptr(dst, pitch, y + 1 + job.oy), x + job.ox, dt, acc.y);
        }
    };
    auto step = [&](auto Mc, int m) {
        constexpr int M = decltype(Mc)::value;  // m mod W
        // P_{m+R}, P_{m+R+1} enter; Q_{m+R-1}, Q_{m+R} are completed.
        w.P[(M + RV) % W] = fetch(m + RV);
        w.P[(M + RV + 1) % W] = fetch(m + RV + 1);
        w.Q[(M + RV - 1) % W] = make_float2(w.P[(M + RV - 1) % W].y, w.P[(M + RV) % W].x);
        w.Q[(M + RV) % W] = make_float2(w.P[(M + RV) % W].y, w.P[(M + RV + 1) % W].x);
        const float2 a0 = w.template tap<M>(c);
        const float2 a1 = w.template tap<(M + 1) % W>(c);
        put(m, a0);
        put(m + 1, a1);
    };
    for (int m0 = 0; m0 < npairs; m0 += W) {
        // W/2 steps of two pairs each; slot indices fixed per step.
        step(std::integral_constant<int, 0>(), m0);
        if (m0 + 2 < npairs) step(std::integral_constant<int, 2 % W>(), m0 + 2); else continue;
        if (m0 + 4 < npairs && W > 4) step(std::integral_constant<int, 4 % W>(), m0 + 4); else continue;
        if constexpr (W > 6) {
            if (m0 + 6 < npairs) step(std::integral_constant<int, 6 % W>(), m0 + 6); else continue;
            if (m0 + 8 < npairs && W > 8) step(std::integral_constant<int, 8 % W>(), m0 + 8); else continue;
        }
        if constexpr (W > 10) {
            if (m0 + 10 < npairs) step(std::integral_constant<int, 10 % W>(), m0 + 10); else continue;
            if (m0 + 12 < npairs) step(std::integral_constant<int, 12 % W>(), m0 + 12); else continue;
            if (m0 + 14 < npairs) step(std::integral_constant<int, 14 % W>(), m0 + 14); else continue;
            if (m0 + 16 < npairs && W > 16) step(std::integral_constant<int, 16 % W>(), m0 + 16); else continue;
        }
    }
    // Take (and release) every remaining chunk so the barrier counts balance.
    for (int q = cur + 1; q < nchunks; ++q)
        move_to(q);
}

// ---- H role ---------------------------------------------------------------------

template <int RH, int RV, class TIn, bool SYM>
__device__ __forceinline__ void h_tasks(const float4* __restrict__ stage, float2* __restrict__ hb,
                                        const float2 (&c)[RH + 1], int hbase)
{
    using C = Cfg<RH, RV, TIn>;
    const int tid = threadIdx.x;
    const int o = tid & 15;  // column octet
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const int p = (tid >> 4) + 8 * i;  // row pair
        if (hbase + 2 * p + 1 < 0)
            continue;  // rows above the strip (first chunks only)
        // Columns 8o .. 8o + 2RH + 7: units 4o .. 4o + RH + 3 (padded: 5o + j + j/4).
        const float4* srow = stage + p * C::ROWU + 5 * o;
        float4 w[RH + 4];
#pragma unroll
        for (int j = 0; j < RH + 4; ++j)
            w[j] = srow[j + (j >> 2)];
        // v(t) = (row 2p, row 2p+1) at column 8o + t
        auto v = [&](int t) {
            return (t & 1) ? make_float2(w[t >> 1].z, w[t >> 1].w)
                           : make_float2(w[t >> 1].x, w[t >> 1].y);
        };
        float2* drow = hb + p * (C::HROWU * 2) + (4 * o + (o >> 1)) * 2;
#pragma unroll
        for (int jj = 0; jj < 8; jj += 2) {
            const float2 a0 = fir::tap2<RH, SYM>(c, [&](int t) { return v(t + jj); });
            const float2 a1 = fir::tap2<RH, SYM>(c, [&](int t) { return v(t + jj + 1); });
            *reinterpret_cast<float4*>(drow + jj) = make_float4(a0.x, a0.y, a1.x, a1.y);
        }
    }
}

// Runs one strip: output columns [x0, x0+128), output rows [y0, y0+nrows)
// (clipped to the valid extent).  tmap == nullptr selects plain loads.
// Returns false if a bounded wait ran out (the error word is set).
template <int RH, int RV, class TIn>
__device__ bool run_strip(const FirJob& job, const LobeSet& lobes, const CUtensorMap* tmap,
                          int x0, int y0, int nrows, unsigned char* smem, Pipe& pipe)
{
    using C = Cfg<RH, RV, TIn>;
    constexpr int XW = C::XW, PRO = C::PRO, NSTAGE = C::NSTAGE;
    TIn* raw = reinterpret_cast<TIn*>(smem + C::RAW_OFF);
    float4* stage = reinterpret_cast<float4*>(smem + C::STAGE_OFF);
    float2* hbuf = reinterpret_cast<float2*>(smem + C::HBUF_OFF);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + C::BAR_OFF);
    volatile int* failed = reinterpret_cast<volatile int*>(smem + C::FLAG_OFF);
    float2* cH = reinterpret_cast<float2*>(smem + C::COEF_OFF);
    float2* cV = cH + TUCU_LOBE_MAX;
    constexpr int kRawStride = (int)(fir::align_up(C::RAW_BYTES, 128) / sizeof(TIn));

    const int tid = threadIdx.x;
    const int nsteps = (nrows + kCH - 1) / kCH;
    const int nchunks = nsteps + PRO;
    auto chunk_row0 = [&](int q) { return y0 + 2 * RV + kCH * (q - PRO); };

    __syncthreads();  // the previous strip of this CTA is done with the buffers
    if (tid < TUCU_LOBE_MAX) {
        cH[tid] = make_float2(lobes.h[0][tid], lobes.h[0][tid]);
        cV[tid] = make_float2(lobes.v[0][tid], lobes.v[0][tid]);
    }
    if (tid == 0)
        *failed = 0;
    __syncthreads();

    if (tid >= kHalf) {
        // ---------------- V role ----------------
        if (nchunks > 0)
            named_arrive(kBarEmpty + 0, 2 * kHalf);
        if (nchunks > 1)
            named_arrive(kBarEmpty + 1, 2 * kHalf);
        float2 c[RV + 1];
#pragma unroll
        for (int k = 0; k <= RV; ++k)
            c[k] = cV[k];
        if ((lobes.sym_v & 1))
            v_role<RH, RV, TIn, true>(job, hbuf, c, x0, y0, nrows, nchunks, failed);
        else
            v_role<RH, RV, TIn, false>(job, hbuf, c, x0, y0, nrows, nchunks, failed);
    } else {
        // ---------------- H role (and TMA producer) ----------------
        bool ok = true;
        if (tmap && tid == 0) {
            fence_proxy_async_smem();
            for (int q = 0; q < NSTAGE && q < nchunks; ++q) {
                mbar_arrive_expect_tx(&bars[q], (uint32_t)C::RAW_BYTES);
                tma_load_2d(raw + q * kRawStride, tmap, x0, chunk_row0(q), &bars[q]);
            }
        }
        float2 c[RH + 1];
#pragma unroll
        for (int k = 0; k <= RH; ++k)
            c[k] = cH[k];
        const bool sym = lobes.sym_h & 1;
        for (int q = 0; q < nchunks; ++q) {
            const int st = q % NSTAGE;
            if (q > 0)
                named_sync(kBarH, kHalf);  // everyone is done reading the staged rows
            // ---- stage chunk q as float row pairs ----
            if (tmap) {
                bool got = false;
                if (ok)
                    got = mbar_wait(&bars[st], (pipe.phase_bits >> st) & 1u);
                if (!got && ok) {
                    ok = false;
                    *failed = 1;
                    raise_device_error(kErrWaitTimeout);
                }
                if (got) {
                    const TIn* src = raw + st * kRawStride;
                    constexpr int NV = kHB * (XW / 4);
                    for (int i = tid; i < NV; i += kHalf) {
                        const int rp = i / (XW / 4), g = i % (XW / 4);
                        const float4 a = fir::load4_to_float<TIn>(src + (2 * rp) * XW + 4 * g);
                        const float4 b = fir::load4_to_float<TIn>(src + (2 * rp + 1) * XW + 4 * g);
                        float4* d = stage + rp * C::ROWU;
                        d[pad4(2 * g)] = make_float4(a.x, b.x, a.y, b.y);
                        d[pad4(2 * g + 1)] = make_float4(a.z, b.z, a.w, b.w);
                    }
                }
            } else {
                const int r0 = chunk_row0(q);
                constexpr int NE = kHB * XW;
                for (int i = tid; i < NE; i += kHalf) {
                    const int rp = i / XW, cc = i % XW;
                    const int xx = x0 + cc, ya = r0 + 2 * rp, yb = ya + 1;
                    float a = 0.0f, b = 0.0f;
                    if (xx < job.cols) {
                        if (ya >= 0 && ya < job.rows)
                            a = load_px<TIn>(row_ptr(job.src, job.src_pitch, ya), xx);
                        if (yb >= 0 && yb < job.rows)
                            b = load_px<TIn>(row_ptr(job.src, job.src_pitch, yb), xx);
                    }
                    reinterpret_cast<float2*>(stage + rp * C::ROWU + pad4(cc >> 1))[cc & 1] =
                        make_float2(a, b);
                }
            }
            named_sync(kBarH, kHalf);  // staged rows complete; the raw stage is free
            if (tmap && ok) {
                pipe.phase_bits ^= 1u << st;
                if (tid == 0 && q + NSTAGE < nchunks) {
                    fence_proxy_async_smem();
                    mbar_arrive_expect_tx(&bars[st], (uint32_t)C::RAW_BYTES);
                    tma_load_2d(raw + st * kRawStride, tmap, x0, chunk_row0(q + NSTAGE), &bars[st]);
                }
            }
            // ---- horizontal taps into chunk buffer q&1 ----
            named_sync(kBarEmpty + (q & 1), 2 * kHalf);
            float2* hb = hbuf + (size_t)(q & 1) * kHB * C::HROWU * 2;
            const int hbase = 2 * RV + kCH * (q - PRO);
            if (ok) {
                if (sym)
                    h_tasks<RH, RV, TIn, true>(stage, hb, c, hbase);
                else
                    h_tasks<RH, RV, TIn, false>(stage, hb, c, hbase);
            }
            named_arrive(kBarFull + (q & 1), 2 * kHalf);
        }
        if (!ok && tmap) {
            // Let any copy still in flight land before the buffers are reused.
            if (tid == 0)
                for (int s = 0; s < NSTAGE; ++s)
                    mbar_wait(&bars[s], (pipe.phase_bits >> s) & 1u);
        }
    }
    __syncthreads();
    return *failed == 0;
}

}  // namespace fir3
}  // namespace tucu
