// fir_v3.cuh -- warp-specialised single-operator separable FIR strip.
//
// Same arithmetic as fir_strip.cuh (the reference's device::convolve,
// TU/cu/FIRFilter.h:66-176, in the oracle's order: paired taps, outermost
// first, FMA-fused, centre last, so results are bit-identical to the oracle's
// and within one rounding of the first step of the reference's as nvcc
// compiles it), organised so that nearly every instruction is a packed FP32
// operation:
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

// The window holds P_k and Q_k in slot k mod W.  Output pair m (strip rows
// 2m, 2m+1) needs T_i = (H[2m+i], H[2m+1+i]), i = 0..2R: T_i = P_{m+i/2} for
// even i and Q_{m+(i-1)/2} for odd i.  Pairs are consumed in blocks of kHB
// output pairs: block j takes the kHB new pairs k = 16j + R .. 16j + R + 15,
// which are exactly chunk PRO + j, so every shared-memory offset and every
// slot index is a compile-time constant (W = 16, or 32 with two blocks per
// unrolled iteration when R + 2 > 16).  Each step produces the two pairs m
// and m+1 (two independent FMA chains).
template <int R, bool SYM>
struct VWin
{
    static constexpr int W = R + 2 <= kHB ? kHB : R + 2;
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

template <class T> __device__ __forceinline__ T cvt_to(float v);
template <> __device__ __forceinline__ uint8_t cvt_to<uint8_t>(float v) { return f2u8(v); }
template <> __device__ __forceinline__ __half cvt_to<__half>(float v) { return __float2half_rn(v); }
template <> __device__ __forceinline__ __nv_bfloat16 cvt_to<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }
template <> __device__ __forceinline__ int32_t cvt_to<int32_t>(float v) { return __float2int_rz(v); }
template <> __device__ __forceinline__ float cvt_to<float>(float v) { return v; }

// Output column of one V thread: row 0 of the strip and the row pitch.
template <class TOut>
struct ColOut
{
    char* p;
    size_t pitch;
    __device__ __forceinline__ void put(int r, float v) const
    {
        *reinterpret_cast<TOut*>(p + (size_t)r * pitch) = cvt_to<TOut>(v);
    }
};

template <int RH, int RV, class TIn, class TOut, bool SYM>
__device__ void v_role(const FirJob& job, const float2* __restrict__ hbuf, const float2 (&c)[RV + 1],
                       int x0, int y0, int nrows, int nchunks, const volatile int* failed)
{
    using C = Cfg<RH, RV, TIn>;
    using Win = VWin<RV, SYM>;
    constexpr int W = Win::W;
    constexpr int PRO = C::PRO;
    constexpr int RS = C::HROWU * 2;                 // float2 per chunk row pair
    constexpr int CHUNK = kHB * RS;                  // float2 per chunk buffer
    constexpr int LOFF = kHB * PRO - RV;             // local pair of k = 0 in chunk 0
    const int col = threadIdx.x - kHalf;
    const int x = x0 + col;
    // rows of this strip this thread may write
    int nvalid = (x < job.ocols) ? min(nrows, job.orows - y0) : 0;
    const int npairs = (nrows + 1) / 2;
    const int hoff = pad8(col >> 1) * 2 + (col & 1);  // this column in a chunk row pair
    const float2* hcol = hbuf + hoff;
    const ColOut<TOut> out{row_ptr(job.dst[0], job.dst_pitch[0], y0 + job.oy) +
                               (size_t)(x + job.ox) * sizeof(TOut),
                           job.dst_pitch[0]};

    auto take = [&](int q) { named_sync(kBarFull + (q & 1), 2 * kHalf); };
    auto give = [&](int q) {
        if (q + 2 < nchunks)
            named_arrive(kBarEmpty + (q & 1), 2 * kHalf);
    };

    Win w;
    // Warm-up: P_0..P_{R-1} and Q_0..Q_{R-2} from the first PRO chunks.
    for (int q = 0; q < PRO; ++q)
        take(q);
#pragma unroll
    for (int k = 0; k < RV; ++k) {
        const int g = k + LOFF;  // pair index counted from chunk 0
        w.P[k % W] = hcol[((g / kHB) & 1) * CHUNK + (g % kHB) * RS];
        if (k > 0)
            w.Q[(k - 1) % W] = make_float2(w.P[(k - 1) % W].y, w.P[k % W].x);
    }
    for (int q = 0; q < PRO; ++q)
        give(q);

    // One step: pairs m and m+1 (m = 16j + 2s, M = m mod W).
    auto step = [&](auto Mc, const float2* cb, int m) {
        constexpr int M = decltype(Mc)::value;
        constexpr int s2 = M % kHB;  // local index of the new pair k = m + R
        const float2 n0 = cb[s2 * RS], n1 = cb[(s2 + 1) * RS];
        w.P[(M + RV) % W] = n0;
        w.P[(M + RV + 1) % W] = n1;
        w.Q[(M + RV - 1) % W] = make_float2(w.P[(M + RV - 1) % W].y, n0.x);
        w.Q[(M + RV) % W] = make_float2(n0.y, n1.x);
        const float2 a0 = w.template tap<M>(c);
        const float2 a1 = w.template tap<(M + 1) % W>(c);
        const int r = 2 * m;
        if (r + 3 < nvalid) {
            out.put(r, a0.x);
            out.put(r + 1, a0.y);
            out.put(r + 2, a1.x);
            out.put(r + 3, a1.y);
        } else {
            if (r < nvalid) out.put(r, a0.x);
            if (r + 1 < nvalid) out.put(r + 1, a0.y);
            if (r + 2 < nvalid) out.put(r + 2, a1.x);
            if (r + 3 < nvalid) out.put(r + 3, a1.y);
        }
    };
    auto block = [&](auto Base, int j) {
        constexpr int B = decltype(Base)::value;  // (16 j) mod W
        const int q = PRO + j;
        take(q);
        if (*failed)
            nvalid = 0;  // a stage never arrived: store nothing
        const float2* cb = hcol + (q & 1) * CHUNK;
        const int m0 = kHB * j;
        step(std::integral_constant<int, (B + 0) % W>(), cb, m0 + 0);
        step(std::integral_constant<int, (B + 2) % W>(), cb, m0 + 2);
        step(std::integral_constant<int, (B + 4) % W>(), cb, m0 + 4);
        step(std::integral_constant<int, (B + 6) % W>(), cb, m0 + 6);
        step(std::integral_constant<int, (B + 8) % W>(), cb, m0 + 8);
        step(std::integral_constant<int, (B + 10) % W>(), cb, m0 + 10);
        step(std::integral_constant<int, (B + 12) % W>(), cb, m0 + 12);
        step(std::integral_constant<int, (B + 14) % W>(), cb, m0 + 14);
        give(q);
    };
    const int nblocks = (npairs + kHB - 1) / kHB;  // == nchunks - PRO
    if constexpr (W == kHB) {
        for (int j = 0; j < nblocks; ++j)
            block(std::integral_constant<int, 0>(), j);
    } else {
        // W = R + 2 slots (R + 2 > kHB): W/2 steps per unrolled iteration and
        // a chunk pointer that moves when the local pair index passes kHB
        // (every kHB/2 steps), so the code stays small enough for the
        // instruction cache.
        int q = PRO;
        take(q);
        if (*failed)
            nvalid = 0;
        const float2* cb = hcol + (q & 1) * CHUNK;
        int lp = 0;  // local pair index of the next new pair in chunk q
        auto rstep = [&](auto Mc, int m) {
            constexpr int M = decltype(Mc)::value;
            if (lp == kHB) {
                give(q);
                ++q;
                take(q);
                if (*failed)
                    nvalid = 0;
                cb = hcol + (q & 1) * CHUNK;
                lp = 0;
            }
            const float2 n0 = cb[lp * RS], n1 = cb[(lp + 1) * RS];
            lp += 2;
            w.P[(M + RV) % W] = n0;
            w.P[(M + RV + 1) % W] = n1;
            w.Q[(M + RV - 1) % W] = make_float2(w.P[(M + RV - 1) % W].y, n0.x);
            w.Q[(M + RV) % W] = make_float2(n0.y, n1.x);
            const float2 a0 = w.template tap<M>(c);
            const float2 a1 = w.template tap<(M + 1) % W>(c);
            const int r = 2 * m;
            if (r + 3 < nvalid) {
                out.put(r, a0.x);
                out.put(r + 1, a0.y);
                out.put(r + 2, a1.x);
                out.put(r + 3, a1.y);
            } else {
                if (r < nvalid) out.put(r, a0.x);
                if (r + 1 < nvalid) out.put(r + 1, a0.y);
                if (r + 2 < nvalid) out.put(r + 2, a1.x);
                if (r + 3 < nvalid) out.put(r + 3, a1.y);
            }
        };
        const int nsteps2 = nblocks * (kHB / 2);  // every chunk's pairs are taken
        for (int t0 = 0; t0 < nsteps2; t0 += W / 2) {
            auto at = [&](auto Sc) {
                constexpr int S = decltype(Sc)::value;
                if (t0 + S < nsteps2)
                    rstep(std::integral_constant<int, (2 * S) % W>(), 2 * (t0 + S));
            };
            at(std::integral_constant<int, 0>());
            at(std::integral_constant<int, 1>());
            at(std::integral_constant<int, 2>());
            at(std::integral_constant<int, 3>());
            at(std::integral_constant<int, 4>());
            at(std::integral_constant<int, 5>());
            at(std::integral_constant<int, 6>());
            at(std::integral_constant<int, 7>());
            at(std::integral_constant<int, 8>());
        }
        give(q);
    }
}

// ---- H role ---------------------------------------------------------------------

template <int RH, int RV, class TIn, bool SYM>
__device__ __forceinline__ void h_tasks(const float4* __restrict__ stage, float2* __restrict__ hb,
                                        const float2 (&c)[RH + 1], int hbase)
{
    using C = Cfg<RH, RV, TIn>;
    const int tid = threadIdx.x;
    const int o = tid & 15;  // column octet
#pragma unroll 1
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
template <int RH, int RV, class TIn, class TOut>
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
            v_role<RH, RV, TIn, TOut, true>(job, hbuf, c, x0, y0, nrows, nchunks, failed);
        else
            v_role<RH, RV, TIn, TOut, false>(job, hbuf, c, x0, y0, nrows, nchunks, failed);
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
                    // (row pair, group of 4 columns) over a power-of-two grid
                    for (int i = tid; i < kHB * 64; i += kHalf) {
                        const int rp = i >> 6, g = i & 63;
                        if (g >= XW / 4)
                            continue;
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
