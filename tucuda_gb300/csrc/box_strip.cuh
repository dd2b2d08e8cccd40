// box_strip.cuh -- window sums over one strip of an image, in one pass.
//
// Restates BoxFilter2's two box_filter launches (TU/cu/BoxFilter.h:246-296,
// 542-583: a vertical running sum into a transposed HBM buffer, then the same
// kernel horizontally) as a single kernel with no intermediate image:
//
//   * each thread keeps vertical window sums V for 4 adjacent columns and
//     slides them down the strip: V += in[y+wV-1] - in[y-1] (the rows leaving
//     the window are re-read; they are still in L2);
//   * per output row the CTA's 1024 column sums are prefix-scanned
//     (thread-local, then warp shuffles, then across warps), and each window
//     sum is a difference of two prefixes: H[x] = P[x+wH-1] - P[x-1].
//
// Integer input accumulates in int32 (exact, order-free, so bit-equal to the
// reference's sums); float input in FP32 with compensated (Kahan) vertical
// updates.  The kernel is generic over NQ quantities per pixel: the plain box
// filter (NQ=1) and both passes of the guided filter (NQ=4, NQ=2) use it with
// their own producer (what is summed) and epilogue (what is written).
#pragma once
#include "tucu_common.cuh"

namespace tucu
{
namespace box
{

constexpr int kThreads = 256;
constexpr int kCPT = 4;                     // columns per thread
constexpr int kTWin = kThreads * kCPT;      // input columns per CTA (1024)

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

// Shared memory: two prefix buffers (row parity) of NQ x 1024 and the warp
// totals of each.
template <int NQ, class Acc>
struct Smem
{
    Acc P[2][NQ][kTWin];
    Acc wt[2][NQ][kThreads / 32];
};

// Runs one strip: output rows [y0, y0+nrows), output columns
// [x0, x0 + out_cols_per_cta(wH)) clipped to ocols.
//   prod.load(y, x, raw[NR][4]) : raw values of input row y, columns x..x+3
//                                 (zero outside the input)
//   prod.expand(raw[NR], q[NQ]) : the NQ summed quantities of one pixel
//   epi.store(y, x, s[NQ])      : window sums of output (y, x)
template <int NQ, int NR, class Acc, int U, class Prod, class Epi>
__device__ void run_strip(const Prod& prod, const Epi& epi, int wV, int wH, int x0, int y0,
                          int nrows, int ocols, void* smem_raw)
{
    auto& sm = *reinterpret_cast<Smem<NQ, Acc>*>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int xin = x0 + kCPT * tid;  // this thread's first input column
    const int two = out_cols_per_cta(wH);

    auto accumulate = [&](Kahan<Acc> (&V)[NQ][kCPT], const Acc (&raw)[NR][kCPT], bool sub) {
#pragma unroll
        for (int j = 0; j < kCPT; ++j) {
            Acc rj[NR], qv[NQ];
#pragma unroll
            for (int k = 0; k < NR; ++k)
                rj[k] = raw[k][j];
            prod.expand(rj, qv);
#pragma unroll
            for (int q = 0; q < NQ; ++q)
                V[q][j].add(sub ? -qv[q] : qv[q]);
        }
    };

    // Vertical window sums of the first output row.
    Kahan<Acc> V[NQ][kCPT];
#pragma unroll
    for (int q = 0; q < NQ; ++q)
#pragma unroll
        for (int j = 0; j < kCPT; ++j)
            V[q][j].reset(Acc(0));
    for (int dy = 0; dy < wV; ++dy) {
        Acc v[NR][kCPT];
        prod.load(y0 + dy, xin, v);
        accumulate(V, v, false);
    }

    for (int r0 = 0; r0 < nrows; r0 += U) {
        // Rows entering / leaving the window for the next U output rows,
        // loaded together so their latencies overlap.
        Acc vin[U][NR][kCPT], vout[U][NR][kCPT];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int y = y0 + r0 + u;
            if ((u > 0 || r0 > 0) && r0 + u < nrows) {
                prod.load(y + wV - 1, xin, vin[u]);
                prod.load(y - 1, xin, vout[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int r = r0 + u;
            if (r >= nrows)
                break;
            if (r > 0) {
                accumulate(V, vin[u], false);
                accumulate(V, vout[u], true);
            }
            const int buf = r & 1;
            // ---- prefix scan of the column sums across the CTA -------------
            Acc pre[NQ][kCPT];
#pragma unroll
            for (int q = 0; q < NQ; ++q) {
                pre[q][0] = V[q][0].value();
#pragma unroll
                for (int j = 1; j < kCPT; ++j)
                    pre[q][j] = pre[q][j - 1] + V[q][j].value();
                Acc incl = pre[q][kCPT - 1];
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
                    sm.wt[buf][q][warp] = incl;
#pragma unroll
                for (int j = 0; j < kCPT; ++j)
                    pre[q][j] += excl;
            }
            __syncthreads();
#pragma unroll
            for (int q = 0; q < NQ; ++q) {
                Acc base = Acc(0);
                for (int w = 0; w < warp; ++w)
                    base += sm.wt[buf][q][w];
#pragma unroll
                for (int j = 0; j < kCPT; ++j)
                    sm.P[buf][q][kCPT * tid + j] = pre[q][j] + base;
            }
            __syncthreads();
            // ---- window sums of this thread's output columns ----------------
#pragma unroll
            for (int j = 0; j < kCPT; ++j) {
                const int i = kCPT * tid + j;  // column index within the CTA
                const int x = x0 + i;
                if (i < two && x < ocols) {
                    Acc s[NQ];
#pragma unroll
                    for (int q = 0; q < NQ; ++q) {
                        const Acc hi = sm.P[buf][q][i + wH - 1];
                        const Acc lo = i > 0 ? sm.P[buf][q][i - 1] : Acc(0);
                        s[q] = hi - lo;
                    }
                    epi.store(y0 + r, x, s);
                }
            }
        }
    }
}

}  // namespace box
}  // namespace tucu
