// box_strip.cuh -- window sums over one strip of an image, in one pass.
//
// Restates BoxFilter2's two box_filter launches (TU/cu/BoxFilter.h:246-296,
// 542-583: a vertical running sum into a transposed HBM buffer, then the same
// kernel horizontally) as a single kernel with no intermediate image:
//
//   * each thread keeps vertical window sums V for 4 adjacent columns and
//     slides them down the strip: V += in[y+wV-1] - in[y-1] (the rows leaving
//     the window are re-read; they are still in L2).  Rows are fetched U at a
//     time as raw bytes, so many loads are in flight per thread;
//   * the U rows of column sums are then prefix-scanned together within each
//     warp's 128-column segment (thread-local, then warp shuffles, U
//     independent chains), and each window sum is a difference of prefixes
//     in at most two adjacent segments:
//         H[x] = P[x+wH-1] - P[x-1]  (+ the left segment's total);
//   * outputs are written four at a time, realigned so that the stores are
//     vector stores whenever the output rows allow it.
//
// Integer input accumulates in int32 (exact, order-free, so bit-equal to the
// reference's sums); float input in FP32 with compensated (Kahan) vertical
// updates.  The kernel is generic over NQ quantities per pixel: the plain box
// filter (NQ=1) and both passes of the guided filter (NQ=4, NQ=2) use it with
// their own producer (what is summed) and epilogue (what is written).
#pragma once
#include <type_traits>

#include "tucu_common.cuh"

namespace tucu
{
namespace box
{

constexpr int kThreads = 256;
constexpr int kCPT = 4;                 // columns per thread
constexpr int kTWin = kThreads * kCPT;  // input columns per CTA (1024)
constexpr int kSeg = 128;               // columns per warp segment
constexpr int kRestart = 64;            // float vertical sums restart at multiples of this row

// Output columns per CTA for a window width (multiple of 4 so column groups
// stay 4-aligned).
__host__ __device__ inline int out_cols_per_cta(int wH) { return ((kTWin - (wH - 1)) / 4) * 4; }

template <class Acc>
struct Kahan
{
    Acc s;
    __device__ __forceinline__ void reset(Acc v) { s = v; }
    __device__ __forceinline__ void add(Acc v) { s += v; }
    __device__ __forceinline__ Acc value() const { return s; }
};

template <>
struct Kahan<float>
{
    float s, c;
    __device__ __forceinline__ void reset(float v)
    {
        s = v;
        c = 0.0f;
    }
    __device__ __forceinline__ void add(float v)
    {
        const float y = __fsub_rn(v, c);
        const float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
    __device__ __forceinline__ float value() const { return s; }
};

template <class Acc>
__device__ __forceinline__ Acc shfl_up(Acc v, int d)
{
    return __shfl_up_sync(0xffffffffu, v, d);
}

// Shared memory: U rows of per-segment prefixes and segment totals.
template <int NQ, class Acc, int U>
struct Smem
{
    Acc P[U][NQ][kTWin];
    Acc wt[U][NQ][kThreads / 32];
};

// Runs one strip: output rows [y0, y0+nrows) (y0 a multiple of kRestart for
// float sums, and U dividing kRestart), output columns
// [x0, x0 + out_cols_per_cta(wH)) clipped to ocols.
//   Prod::Raw                     : raw data of 4 columns of one input row
//   prod.load(y, x) -> Raw        : input row y, columns x..x+3 (zero / flagged
//                                   invalid outside the input)
//   prod.expand(raw, j, q[NQ])    : the NQ summed quantities of column j
//   epi.store4(y, x, s[4][NQ], i) : window sums of outputs (y, x..x+3); the
//                                   columns with index i+j outside
//                                   [0, ncols) are not written
template <int NQ, class Acc, int U, class Prod, class Epi>
__device__ void run_strip(const Prod& prod, const Epi& epi, int wV, int wH, int x0, int y0,
                          int nrows, int ocols, int ox_align, void* smem_raw)
{
    using Raw = typename Prod::Raw;
    auto& sm = *reinterpret_cast<Smem<NQ, Acc, U>*>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int xin = x0 + kCPT * tid;  // this thread's first input column
    const int two = min(out_cols_per_cta(wH), ocols - x0);

    auto accumulate = [&](Kahan<Acc> (&V)[NQ][kCPT], const Raw& raw, bool sub) {
#pragma unroll
        for (int j = 0; j < kCPT; ++j) {
            Acc qv[NQ];
            prod.expand(raw, j, qv);
#pragma unroll
            for (int q = 0; q < NQ; ++q)
                V[q][j].add(sub ? -qv[q] : qv[q]);
        }
    };

    // Vertical window sums of output row y: summed afresh (not slid) at the
    // strip start and, for float sums, at every absolute row that is a
    // multiple of kRestart, so that float results do not depend on how the
    // image is cut into strips (single call, batch and server agree bit for
    // bit) and compensated running sums never span more than kRestart rows.
    Kahan<Acc> V[NQ][kCPT];
    auto fresh_sums = [&](int y) {
#pragma unroll
        for (int q = 0; q < NQ; ++q)
#pragma unroll
            for (int j = 0; j < kCPT; ++j)
                V[q][j].reset(Acc(0));
        for (int dy0 = 0; dy0 < wV; dy0 += U) {
            Raw rb[U];
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (dy0 + u < wV)
                    rb[u] = prod.load(y + dy0 + u, xin);
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (dy0 + u < wV)
                    accumulate(V, rb[u], false);
        }
    };

    // Output columns of this thread in the store phase, realigned so that the
    // output address of the first one is a multiple of 4 elements
    // (ox_align = (x0 + ox) mod 4).
    const int ist = kCPT * tid - ox_align;

    for (int r0 = 0; r0 < nrows; r0 += U) {
        // ---- 1. rows entering / leaving the window, all loads first ----------
        const bool fresh = r0 == 0 || (!std::is_integral<Acc>::value && ((y0 + r0) % kRestart) == 0);
        if (fresh)
            fresh_sums(y0 + r0);
        Raw rin[U], rout[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int r = r0 + u;
            if ((u > 0 || !fresh) && r < nrows) {
                rin[u] = prod.load(y0 + r + wV - 1, xin);
                rout[u] = prod.load(y0 + r - 1, xin);
            }
        }
        // ---- 2. slide the vertical sums; snapshot each row ------------------
        // The entering and leaving quantities are combined first: for pixel
        // data (u8, f16, bf16 values well inside FP32 range) the difference is
        // exact, so each row costs one compensated add per column.
        Acc snap[U][NQ][kCPT];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int r = r0 + u;
            if ((u > 0 || !fresh) && r < nrows) {
#pragma unroll
                for (int j = 0; j < kCPT; ++j) {
                    Acc qi[NQ], qo[NQ];
                    prod.expand(rin[u], j, qi);
                    prod.expand(rout[u], j, qo);
#pragma unroll
                    for (int q = 0; q < NQ; ++q)
                        V[q][j].add(qi[q] - qo[q]);
                }
            }
#pragma unroll
            for (int q = 0; q < NQ; ++q)
#pragma unroll
                for (int j = 0; j < kCPT; ++j)
                    snap[u][q][j] = V[q][j].value();
        }
        // ---- 3. segment prefix scans of the U rows (independent chains) -----
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int q = 0; q < NQ; ++q) {
                Acc* pre = snap[u][q];
#pragma unroll
                for (int j = 1; j < kCPT; ++j)
                    pre[j] += pre[j - 1];
                Acc incl = pre[kCPT - 1];
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const Acc t = shfl_up(incl, d);
                    if (lane >= d)
                        incl += t;
                }
                Acc excl = shfl_up(incl, 1);
                if (lane == 0)
                    excl = Acc(0);
                if (lane == 31)
                    sm.wt[u][q][warp] = incl;
#pragma unroll
                for (int j = 0; j < kCPT; ++j)
                    sm.P[u][q][kCPT * tid + j] = pre[j] + excl;
            }
        __syncthreads();
        // ---- 4. window sums and stores -----------------------------------
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int r = r0 + u;
            if (r >= nrows)
                break;
            Acc s[kCPT][NQ];
            bool any = false;
#pragma unroll
            for (int j = 0; j < kCPT; ++j) {
                const int i = ist + j;
                if (i >= 0 && i < two) {
                    const int ie = i + wH - 1;
                    const int sa = i >> 7, sb = ie >> 7;
#pragma unroll
                    for (int q = 0; q < NQ; ++q) {
                        const Acc lo = (i & (kSeg - 1)) ? sm.P[u][q][i - 1] : Acc(0);
                        const Acc hi = sm.P[u][q][ie];
                        s[j][q] = sa == sb ? hi - lo : (sm.wt[u][q][sa] - lo) + hi;
                    }
                    any = true;
                } else {
#pragma unroll
                    for (int q = 0; q < NQ; ++q)
                        s[j][q] = Acc(0);
                }
            }
            if (any)
                epi.store4(y0 + r, x0 + ist, s, ist, two);
        }
        __syncthreads();
    }
}

}  // namespace box
}  // namespace tucu
