// box_strip.cuh -- window sums over one strip of an image, in one pass.
//
// Restates BoxFilter2's two box_filter launches (TU/cu/BoxFilter.h:246-296,
// 542-583: a vertical running sum into a transposed HBM buffer, then the same
// kernel horizontally) as a single kernel with no intermediate image, no
// shared memory and no block-wide barrier:
//
//   * every warp owns kSeg = 128 consecutive input columns (4 per lane) and
//     keeps their vertical window sums V, sliding them down the strip:
//     V += in[y+wV-1] - in[y-1] (the rows leaving the window are re-read;
//     they are still in L2).  Rows are fetched U at a time as raw bytes, so
//     several loads are in flight per thread;
//   * per row the warp prefix-scans its 128 column sums with shuffles
//     (thread-local, then across lanes) and each window sum is a difference
//     of two prefixes, H[i] = P[i+wH-1] - P[i-1].  Lane l computes outputs
//     i = 4l..4l+3: P[i-1] is its own (or, for i = 4l, the scan's exclusive
//     prefix), P[i+wH-1] comes from lane l + (i+wH-1)/4 by one shuffle.  The
//     element index (i+wH-1) mod 4 is the same in every lane; the strip is
//     compiled for each of its four values, so no lane selects at run time;
//   * a warp writes out_cols_per_warp(wH) output columns; the warps of a CTA
//     tile the strip side by side and overlap by the window width on the
//     input side, so warps never wait for one another.
//
// Integer input accumulates in int32 (exact, order-free, so bit-equal to the
// reference's sums).  Float sums run in FP32 and are summed afresh at every
// absolute row that is a multiple of kRestart, so float results do not depend
// on how an image is cut into strips.  A producer with kCompensate set (FP32
// input, the guided passes) gets compensated (Kahan) vertical updates; for
// f16/bf16 input the entering-minus-leaving difference is exact and the plain
// FP32 running sum over at most kRestart rows stays far inside the float
// tolerance.  The kernel is generic over NQ quantities per pixel: the plain
// box filter (NQ=1) and both passes of the guided filter (NQ=4, NQ=2) use it
// with their own producer (what is summed) and epilogue (what is written).
#pragma once
#include <type_traits>

#include "tucu_common.cuh"

namespace tucu
{
namespace box
{

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kCPT = 4;          // columns per lane
constexpr int kSeg = 32 * kCPT;  // input columns per warp (128)
constexpr int kRestart = 64;     // float vertical sums restart at multiples of this row

// Output columns per warp (a multiple of 4): output i of a warp needs the
// prefix i+wH-1 inside its 128 columns.
__host__ __device__ inline int out_cols_per_warp(int wH) { return ((kSeg + 1 - wH) / 4) * 4; }
__host__ __device__ inline int out_cols_per_cta(int wH) { return kWarps * out_cols_per_warp(wH); }

// Running sum: compensated (Kahan) or plain.
template <class Acc, bool COMP>
struct RunSum
{
    Acc s;
    __device__ __forceinline__ void reset(Acc v) { s = v; }
    __device__ __forceinline__ void add(Acc v) { s += v; }
    __device__ __forceinline__ Acc value() const { return s; }
};

template <>
struct RunSum<float, true>
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

template <>
struct RunSum<float, false>
{
    float s;
    __device__ __forceinline__ void reset(float v) { s = v; }
    __device__ __forceinline__ void add(float v) { s = __fadd_rn(s, v); }
    __device__ __forceinline__ float value() const { return s; }
};

// acc + t*m with m in {0, 1}: exact, and no predicate per scan step.
__device__ __forceinline__ float mask_add(float acc, float t, float m) { return __fmaf_rn(t, m, acc); }
__device__ __forceinline__ int mask_add(int acc, int t, int m) { return acc + (t & m); }

template <class Acc>
__device__ __forceinline__ Acc lane_mask(bool on)
{
    if constexpr (std::is_integral<Acc>::value)
        return on ? Acc(-1) : Acc(0);
    else
        return on ? Acc(1) : Acc(0);
}

// Window sums of one row from the column sums v of this lane's four columns.
// C = (wH-1) mod 4; hlane = lane + (wH-1)/4; m[k] = lane_mask(lane >= 2^k).
template <int C, int NQ, class Acc>
__device__ __forceinline__ void window_row(const Acc (&v)[NQ][kCPT], int hlane, const Acc (&m)[5],
                                           Acc (&s)[kCPT][NQ])
{
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        Acc p[kCPT];
        p[0] = v[q][0];
#pragma unroll
        for (int j = 1; j < kCPT; ++j)
            p[j] = p[j - 1] + v[q][j];
        Acc incl = p[kCPT - 1];
#pragma unroll
        for (int k = 0; k < 5; ++k)
            incl = mask_add(incl, __shfl_up_sync(0xffffffffu, incl, 1 << k), m[k]);
        // P[4*lane - 1]; lane 0 receives its own value, masked to zero.
        const Acc excl = mask_add(Acc(0), __shfl_up_sync(0xffffffffu, incl, 1), m[0]);
#pragma unroll
        for (int j = 0; j < kCPT; ++j)
            p[j] += excl;
#pragma unroll
        for (int j = 0; j < kCPT; ++j) {
            const Acc hi = __shfl_sync(0xffffffffu, p[(j + C) & 3], hlane + ((j + C) >> 2));
            const Acc lo = j == 0 ? excl : p[j > 0 ? j - 1 : 0];
            s[j][q] = hi - lo;
        }
    }
}

// Runs one warp's strip: output rows [y0, y0+nrows) (y0 a multiple of
// kRestart for float sums, U dividing kRestart), output columns
// [xw, xw + out_cols_per_warp(wH)) clipped to ocols.  Float results depend on
// xw (the origin of the warp's prefix sums): every caller places warps on
// the grid of multiples of out_cols_per_warp(wH).
//   Prod::Raw                      : raw data of 4 columns of one input row
//   Prod::kCompensate              : Kahan vertical updates (float sums)
//   prod.load(y, x) -> Raw         : input row y, columns x..x+3 (zero / flagged
//                                    invalid outside the input)
//   prod.expand(raw, j, q[NQ])     : the NQ summed quantities of column j
//   epi.store4(y, x, s[4][NQ], m)  : window sums of outputs (y, x..x+3); bit j
//                                    of m set = output x+j is to be written
template <int C, int NQ, class Acc, int U, class Prod, class Epi>
__device__ __forceinline__ void strip_body(const Prod& prod, const Epi& epi, int wV, int wH, int xw,
                                           int y0, int nrows, int ocols)
{
    using Raw = typename Prod::Raw;
    using Sum = RunSum<Acc, Prod::kCompensate>;
    const int lane = threadIdx.x & 31;
    const int nout = min(out_cols_per_warp(wH), ocols - xw);  // output columns of the warp
    if (nout <= 0)
        return;  // no barrier below: warps leave independently
    const int xin = xw + kCPT * lane;      // this lane's first input and output column
    const int hlane = lane + ((wH - 1) >> 2);
    Acc m[5];
#pragma unroll
    for (int k = 0; k < 5; ++k)
        m[k] = lane_mask<Acc>(lane >= (1 << k));
    unsigned mask = 0;
#pragma unroll
    for (int j = 0; j < kCPT; ++j)
        if (kCPT * lane + j < nout)
            mask |= 1u << j;

    Sum V[NQ][kCPT];
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
                if (dy0 + u < wV) {
#pragma unroll
                    for (int j = 0; j < kCPT; ++j) {
                        Acc qv[NQ];
                        prod.expand(rb[u], j, qv);
#pragma unroll
                        for (int q = 0; q < NQ; ++q)
                            V[q][j].add(qv[q]);
                    }
                }
        }
    };

    for (int r0 = 0; r0 < nrows; r0 += U) {
        // ---- 1. rows entering / leaving the window, all loads first ----------
        // Vertical sums are summed afresh (not slid) at the strip start and,
        // for float sums, at every absolute row that is a multiple of
        // kRestart: single call, batch and server agree bit for bit, and a
        // running sum never spans more than kRestart rows.
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
        // ---- 2. per row: slide the vertical sums, window sums, store --------
        // Entering and leaving quantities are combined first (exact for
        // pixel data), so each row costs one running-sum update per column.
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int r = r0 + u;
            if (r >= nrows)
                break;
            if (u > 0 || !fresh) {
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
            Acc v[NQ][kCPT];
#pragma unroll
            for (int q = 0; q < NQ; ++q)
#pragma unroll
                for (int j = 0; j < kCPT; ++j)
                    v[q][j] = V[q][j].value();
            Acc s[kCPT][NQ];
            window_row<C, NQ, Acc>(v, hlane, m, s);
            if (mask)
                epi.store4(y0 + r, xin, s, mask);
        }
    }
}

// One warp's strip (see strip_body), compiled for each value of (wH-1) mod 4.
template <int NQ, class Acc, int U, class Prod, class Epi>
__device__ __forceinline__ void run_strip(const Prod& prod, const Epi& epi, int wV, int wH, int xw,
                                          int y0, int nrows, int ocols)
{
    switch ((wH - 1) & 3) {
    case 0: strip_body<0, NQ, Acc, U>(prod, epi, wV, wH, xw, y0, nrows, ocols); break;
    case 1: strip_body<1, NQ, Acc, U>(prod, epi, wV, wH, xw, y0, nrows, ocols); break;
    case 2: strip_body<2, NQ, Acc, U>(prod, epi, wV, wH, xw, y0, nrows, ocols); break;
    default: strip_body<3, NQ, Acc, U>(prod, epi, wV, wH, xw, y0, nrows, ocols); break;
    }
}

// Calls f(std::integral_constant<int, (wH-1) mod 4>()): callers that loop
// over several strips put the loop inside f, one loop per variant.
template <class F>
__device__ __forceinline__ void with_c(int wH, F&& f)
{
    switch ((wH - 1) & 3) {
    case 0: f(std::integral_constant<int, 0>()); break;
    case 1: f(std::integral_constant<int, 1>()); break;
    case 2: f(std::integral_constant<int, 2>()); break;
    default: f(std::integral_constant<int, 3>()); break;
    }
}

// Warp tasks of one image: task t covers output rows
// [b*strip_rows, (b+1)*strip_rows) and warp column c (t = b*nwc + c, so
// neighbouring warps share their halo columns in L1).
struct TaskGrid
{
    int strip_rows;  // a multiple of kRestart
    int nwc;         // warp columns: ceil(ocols / out_cols_per_warp(wH))
    int ntask;
};

}  // namespace box
}  // namespace tucu
