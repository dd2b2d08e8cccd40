// box_strip.cuh -- window sums over one strip of an image, in one pass.
//
// Restates BoxFilter2's two box_filter launches (TU/cu/BoxFilter.h:246-296,
// 542-583: a vertical running sum into a transposed HBM buffer, then the same
// kernel horizontally) as a single kernel with no intermediate image and no
// block-wide barrier:
//
//   * every warp owns 32*CPT consecutive input columns (CPT = 4 or 8 per
//     lane; 4 unless the producer declares kCols) and keeps their vertical
//     window sums V.  A strip is a stream of steps: step
//     s adds input row y0+s and, once the window is full (s >= wV), removes
//     row y0+s-wV; from step wV-1 on every step emits one output row;
//   * the rows of the next D-1 steps are in flight at all times: each lane
//     copies its own CPT columns of them with cp.async into a private ring in
//     shared memory (no registers held, no other lane involved, so the only
//     synchronisation is the lane's own cp.async.wait_group);
//   * per output row the warp prefix-scans its 32*CPT column sums with
//     shuffles (thread-local, then across lanes) and each window sum is a
//     difference of two prefixes, H[i] = P[i+wH-1] - P[i-1].  Lane l computes
//     outputs i = CPT*l..CPT*l+CPT-1: P[i-1] is its own (or, for i = CPT*l,
//     the scan's exclusive prefix), P[i+wH-1] comes from lane
//     l + (i+wH-1)/CPT by one shuffle.  The element index (i+wH-1) mod CPT is
//     the same in every lane; the strip is compiled for each of its values,
//     so no lane selects at run time;
//   * a warp writes out_cols_per_warp(wH) output columns; the warps of a CTA
//     tile the strip side by side and overlap by the window width on the
//     input side, so warps never wait for one another.
//
// Integer input accumulates in int32 (exact, order-free, so bit-equal to the
// reference's sums).  Float sums run in FP32 and start afresh at every
// absolute row that is a multiple of the restart period (kRestart = 64 for
// the box filter; the guided filter picks 8, 32 or 64 from the image size
// alone), so float results do not depend on how an image is cut into strips.  A producer with kCompensate set
// (FP32 input, the guided passes) gets compensated (Kahan) vertical updates;
// for f16/bf16 input the entering-minus-leaving difference is exact and the
// plain FP32 running sum over at most kRestart rows stays far inside the
// float tolerance.  The kernel is generic over NQ quantities per pixel: the
// plain box filter (NQ=1) and both passes of the guided filter (NQ=4, NQ=2)
// use it with their own producer (what is summed) and epilogue (what is
// written).
#pragma once
#include <string.h>

#include <type_traits>

#include "tucu_common.cuh"

namespace tucu
{
namespace box
{

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kCPT = 4;          // columns per lane, unless a producer declares kCols
constexpr int kRestart = 64;     // float vertical sums restart at multiples of this row

// Output columns per warp of a strip with cpt columns per lane (a multiple
// of cpt): output i of a warp needs the prefix i+wH-1 inside its 32*cpt
// columns.
__host__ __device__ inline int out_cols_per_warp(int wH, int cpt = kCPT)
{
    return ((32 * cpt + 1 - wH) / cpt) * cpt;
}
__host__ __device__ inline int out_cols_per_cta(int wH) { return kWarps * out_cols_per_warp(wH); }

// Columns per lane of a producer: Prod::kCols where it declares one, else kCPT.
template <class Prod, class = void>
struct ColsOf
{
    static constexpr int value = kCPT;
};
template <class Prod>
struct ColsOf<Prod, std::void_t<decltype(Prod::kCols)>>
{
    static constexpr int value = Prod::kCols;
};

// Window ring: Prod::kWindowRing set = the ring keeps the last ring_rows input
// rows (at least wV + D - 1), so a step copies only its entering row and reads
// the leaving one from the ring; otherwise each step copies both rows into a
// ring of D row pairs.
template <class Prod, class = void>
struct WinOf
{
    static constexpr bool value = false;
};
template <class Prod>
struct WinOf<Prod, std::void_t<decltype(Prod::kWindowRing)>>
{
    static constexpr bool value = Prod::kWindowRing;
};

// ---- per-lane asynchronous row copies --------------------------------------------

// Copies BYTES (4, 8 or 16) from global src to shared dst; only the first
// src_bytes come from src, the rest are zero-filled (src_bytes = 0 reads
// nothing).  Both addresses aligned to BYTES.
template <int BYTES>
__device__ __forceinline__ void cp_async(uint32_t dst, const void* src, int src_bytes)
{
    static_assert(BYTES == 4 || BYTES == 8 || BYTES == 16, "cp.async size");
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(dst), "l"(src), "n"(BYTES),
                 "r"(src_bytes)
                 : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

template <int N>
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Ring geometry of a producer: one row of a warp is kPlanes planes of 32
// lanes x kPlaneBytes; a step holds two rows (entering, leaving).
template <class Prod>
struct Ring
{
    static constexpr int kRowBytes = Prod::kPlanes * 32 * Prod::kPlaneBytes;
    static constexpr int kStepBytes = 2 * kRowBytes;
    // Steps in the ring for a budget of shared memory per warp.
    static constexpr int depth(int bytes_per_warp)
    {
        const int d = bytes_per_warp / kStepBytes;
        return d < 2 ? 2 : d > 16 ? 16 : d;
    }
};

// ---- running sums ------------------------------------------------------------------

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

// Window sums of one row from the column sums v of this lane's CPT columns.
// C = (wH-1) mod CPT; hlane = lane + (wH-1)/CPT; m[k] = lane_mask(lane >= 2^k).
template <int C, int NQ, class Acc, int CPT = kCPT>
__device__ __forceinline__ void window_row(const Acc (&v)[NQ][CPT], int hlane, const Acc (&m)[5],
                                           Acc (&s)[CPT][NQ])
{
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        Acc p[CPT];
        p[0] = v[q][0];
#pragma unroll
        for (int j = 1; j < CPT; ++j)
            p[j] = p[j - 1] + v[q][j];
        Acc incl = p[CPT - 1];
#pragma unroll
        for (int k = 0; k < 5; ++k)
            incl = mask_add(incl, __shfl_up_sync(0xffffffffu, incl, 1 << k), m[k]);
        // P[CPT*lane - 1]: the inclusive lane prefix less this lane's own
        // total (exactly 0 in lane 0; one rounding of the difference for
        // FP32 sums, where the lanes' prefixes are rounded sums already).
        const Acc excl = incl - p[CPT - 1];
        Acc hi[CPT], lo[CPT];
        if constexpr (std::is_same<Acc, float>::value) {
            // Packed pairs: each lane rounds exactly like the scalar add.
#pragma unroll
            for (int j = 0; j < CPT; j += 2) {
                const float2 t = __fadd2_rn(make_float2(p[j], p[j + 1]), make_float2(excl, excl));
                p[j] = t.x;
                p[j + 1] = t.y;
            }
        } else {
#pragma unroll
            for (int j = 0; j < CPT; ++j)
                p[j] += excl;
        }
#pragma unroll
        for (int j = 0; j < CPT; ++j) {
            hi[j] = __shfl_sync(0xffffffffu, p[(j + C) % CPT], hlane + (j + C) / CPT);
            lo[j] = j == 0 ? excl : p[j > 0 ? j - 1 : 0];
        }
        if constexpr (std::is_same<Acc, float>::value) {
#pragma unroll
            for (int j = 0; j < CPT; j += 2) {
                const float2 t = __fadd2_rn(make_float2(hi[j], hi[j + 1]), make_float2(-lo[j], -lo[j + 1]));
                s[j][q] = t.x;
                s[j + 1][q] = t.y;
            }
        } else {
#pragma unroll
            for (int j = 0; j < CPT; ++j)
                s[j][q] = hi[j] - lo[j];
        }
    }
}

// Epilogues that read global memory of their own (the guided pass B reads
// the guide at the window centre) may define prefetch(y, x): strip_body calls
// it for output row y as soon as the input rows of that row are requested,
// D-1 steps before the row is stored.
template <class E>
__device__ __forceinline__ auto epi_prefetch(const E& e, int y, int x, int) -> decltype(e.prefetch(y, x), void())
{
    e.prefetch(y, x);
}
template <class E>
__device__ __forceinline__ void epi_prefetch(const E&, int, int, long)
{
}

// Epilogues may define cursor(y, x), a row cursor with next(), and
// store4(cursor, s, mask): a 4-column strip then opens the cursor at the
// first row a block writes and moves it one row per step, so no step
// recomputes its output address.
struct NoCursor
{
    __device__ __forceinline__ void next() {}
};
template <class E>
__device__ __forceinline__ auto epi_cursor(const E& e, int y, int x, int) -> decltype(e.cursor(y, x))
{
    return e.cursor(y, x);
}
template <class E>
__device__ __forceinline__ NoCursor epi_cursor(const E&, int, int, long)
{
    return NoCursor{};
}

// Runs one warp's strip: output rows [y0, y0+nrows), output columns
// [xw, xw + out_cols_per_warp(wH)) clipped to ocols.  Float results depend
// on xw (the origin of the warp's
// prefix sums): every caller places warps on the grid of multiples of
// out_cols_per_warp(wH).  ring: this warp's Ring<Prod>::kStepBytes * D bytes
// of shared memory, 16-byte aligned.
//   Prod::Raw                      : raw data of CPT columns of one input row;
//                                    its first kPlanes*kPlaneBytes bytes are
//                                    the planes copied into the ring
//   Prod::kPlanes, kPlaneBytes     : planes per row, bytes per lane and plane
//                                    (4, 8 or 16)
//   Prod::kAsync                   : rows aligned for cp.async of the planes
//   Prod::kCompensate              : Kahan vertical updates (float sums)
//   prod.plane_ptr(p, y, x)        : global address of plane p, row y, column x
//   prod.plane_bytes(p, nvalid, x) : bytes of plane p inside the image when
//                                    nvalid of the CPT columns from x are
//   prod.load(y, x) -> Raw         : checked synchronous load (!kAsync)
//   prod.finish(raw, nvalid)       : completes a Raw read back from the ring
//   prod.expand(raw, j, q[NQ])     : the NQ summed quantities of column j
//   epi.store4(y, x, s[4][NQ], m)  : window sums of outputs (y, x..x+3); bit j
//                                    of m set = output x+j is to be written
//   epi.store8(...)                : the same for 8 outputs (producers of 8
//                                    columns per lane, Prod::kCols = 8)
template <int C, int NQ, class Acc, int D, class Prod, class Epi, int CPT = ColsOf<Prod>::value>
__device__ __forceinline__ void strip_body(const Prod& prod, const Epi& epi, int wV, int wH, int xw,
                                           int y0, int nrows, int ocols, char* ring, int cols,
                                           int restart = kRestart, int ring_rows = 0)
{
    constexpr bool kWin = WinOf<Prod>::value;
    using Raw = typename Prod::Raw;
    using Sum = RunSum<Acc, Prod::kCompensate>;
    constexpr int PB = Prod::kPlaneBytes, NP = Prod::kPlanes;
    constexpr int kRow = Ring<Prod>::kRowBytes;
    const int lane = threadIdx.x & 31;
    const int nout = min(out_cols_per_warp(wH, CPT), ocols - xw);  // output columns of the warp
    if (nout <= 0)
        return;  // no barrier below: warps leave independently
    const int xin = xw + CPT * lane;  // this lane's first input and output column
    const int nvalid = max(0, min(CPT, cols - xin));
    const int xsrc = nvalid > 0 ? xin : 0;  // a valid address when nothing is read
    const int hlane = lane + (wH - 1) / CPT;
    Acc m[5];
#pragma unroll
    for (int k = 0; k < 5; ++k)
        m[k] = lane_mask<Acc>(lane >= (1 << k));
    unsigned mask = 0;
#pragma unroll
    for (int j = 0; j < CPT; ++j)
        if (CPT * lane + j < nout)
            mask |= 1u << j;
    int pbytes[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p)
        pbytes[p] = prod.plane_bytes(p, nvalid, xin);
    const uint32_t ring_s = static_cast<uint32_t>(__cvta_generic_to_shared(ring)) + lane * PB;

    // Row y into ring row `slot` (0..2D-1) of this lane.
    auto issue = [&](int y, int slot) {
        const uint32_t dst = ring_s + slot * kRow;
        if constexpr (Prod::kAsync) {
#pragma unroll
            for (int p = 0; p < NP; ++p)
                cp_async<PB>(dst + p * 32 * PB, prod.plane_ptr(p, y, xsrc), pbytes[p]);
        } else {
            const Raw r = prod.load(y, xin);
            char* d = ring + slot * kRow + lane * PB;
#pragma unroll
            for (int p = 0; p < NP; ++p)
                memcpy(d + p * 32 * PB, reinterpret_cast<const char*>(&r) + p * PB, PB);
        }
    };
    // The row this lane copied to `src` (its first plane's bytes in a ring row).
    auto read = [&](const char* src) {
        Raw r;
#pragma unroll
        for (int p = 0; p < NP; ++p)
            memcpy(reinterpret_cast<char*>(&r) + p * PB, src + p * 32 * PB, PB);
        prod.finish(r, nvalid);
        return r;
    };

    // Float sums restart at the absolute rows that are multiples of
    // `restart`; a strip that starts inside a restart block first replays the
    // block's rows above y0 (running sums only, nothing written), so every
    // output is the same however an image is cut into strips.  Integer sums
    // run the whole strip.
    constexpr bool kInt = std::is_integral<Acc>::value;
    const int period = kInt ? nrows : restart;
    const int ystart = kInt ? y0 : y0 - y0 % restart;
    for (int yb = ystart; yb < y0 + nrows; yb += period) {
        const int nb = min(period, y0 + nrows - yb);  // rows of the block up to the strip end
        const int nsteps = wV + nb - 1;
        const int semit = max(0, y0 - yb) + wV - 1;   // first step that writes
        // Step s: entering row yb+s into ring row 2*(s%D), leaving row
        // yb+s-wV (s >= wV) into ring row 2*(s%D)+1.  Steps are issued in
        // order; with asynchronous copies the source addresses advance by one
        // row pitch per step (every producer's plane address is affine in the
        // row) and the ring offset cycles, so no step recomputes an address.
        const char* src_in[NP];  // plane p of the next entering row
        ptrdiff_t src_step[NP], src_back[NP];
        if constexpr (Prod::kAsync) {
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                src_in[p] = static_cast<const char*>(prod.plane_ptr(p, yb, xsrc));
                src_step[p] = static_cast<const char*>(prod.plane_ptr(p, yb + 1, xsrc)) - src_in[p];
                src_back[p] = src_step[p] * wV;
            }
        }
        // Pair ring: step s's rows in ring rows 2*(s%D), 2*(s%D)+1.  Window
        // ring: block row r (entering at step r) in ring row r % ring_rows.
        constexpr int kAdvance = kWin ? kRow : 2 * kRow;
        uint32_t ring_next = ring_s;  // ring row (pair) of the next step issued
        const uint32_t ring_end = ring_s + (kWin ? ring_rows * kRow : D * 2 * kRow);
        int next_row = 0;             // window ring: ring row of the next step issued
        auto issue_step = [&](int s) {
            if constexpr (Prod::kAsync) {
#pragma unroll
                for (int p = 0; p < NP; ++p) {
                    cp_async<PB>(ring_next + p * 32 * PB, src_in[p], pbytes[p]);
                    if (!kWin && s >= wV)
                        cp_async<PB>(ring_next + kRow + p * 32 * PB, src_in[p] - src_back[p], pbytes[p]);
                    src_in[p] += src_step[p];
                }
            } else if constexpr (kWin) {
                issue(yb + s, next_row);
                next_row = next_row + 1 == ring_rows ? 0 : next_row + 1;
            } else {
                const int k = s % D;
                issue(yb + s, 2 * k);
                if (s >= wV)
                    issue(yb + s - wV, 2 * k + 1);
            }
            ring_next += kAdvance;
            if (ring_next == ring_end)
                ring_next = ring_s;
        };
#pragma unroll
        for (int s = 0; s < D - 1; ++s) {
            if (s < nsteps)
                issue_step(s);
            cp_async_commit();
        }
        Sum V[NQ][CPT];
#pragma unroll
        for (int q = 0; q < NQ; ++q)
#pragma unroll
            for (int j = 0; j < CPT; ++j)
                V[q][j].reset(Acc(0));
        auto cur = [&] {
            if constexpr (CPT == kCPT)
                return epi_cursor(epi, yb + semit - wV + 1, xin, 0);
            else
                return NoCursor{};
        }();
        int row_in = 0;  // window ring: ring row of block row s
        for (int s = 0; s < nsteps; ++s) {
            // Step s's copies are done once at most D-2 younger groups remain.
            cp_async_wait<D - 2>();
            const int k = s % D;
            const int slot_in = kWin ? row_in : 2 * k;
            int slot_out = 2 * k + 1;
            if constexpr (kWin) {
                slot_out = row_in - wV;
                if (slot_out < 0)
                    slot_out += ring_rows;
                row_in = row_in + 1 == ring_rows ? 0 : row_in + 1;
            }
            const Raw rin = read(ring + slot_in * kRow + lane * PB);
            if (s >= wV) {
                const Raw rout = read(ring + slot_out * kRow + lane * PB);
#pragma unroll
                for (int j = 0; j < CPT; ++j) {
                    Acc qi[NQ], qo[NQ];
                    prod.expand(rin, j, qi);
                    prod.expand(rout, j, qo);
#pragma unroll
                    for (int q = 0; q < NQ; ++q)
                        V[q][j].add(qi[q] - qo[q]);
                }
            } else {
#pragma unroll
                for (int j = 0; j < CPT; ++j) {
                    Acc qi[NQ];
                    prod.expand(rin, j, qi);
#pragma unroll
                    for (int q = 0; q < NQ; ++q)
                        V[q][j].add(qi[q]);
                }
            }
            // Refill the ring rows step s-1 used: their values were consumed
            // by the previous step's arithmetic, which issued before this.
            if (s + D - 1 < nsteps) {
                issue_step(s + D - 1);
                if (s + D - 1 >= semit && mask)
                    epi_prefetch(epi, yb + s + D - wV, xin, 0);
            }
            cp_async_commit();
            if (s >= semit) {
                Acc v[NQ][CPT];
#pragma unroll
                for (int q = 0; q < NQ; ++q)
#pragma unroll
                    for (int j = 0; j < CPT; ++j)
                        v[q][j] = V[q][j].value();
                Acc sw[CPT][NQ];
                window_row<C, NQ, Acc, CPT>(v, hlane, m, sw);
                if (mask) {
                    if constexpr (CPT != kCPT)
                        epi.store8(yb + s - wV + 1, xin, sw, mask);
                    else if constexpr (std::is_same<decltype(cur), NoCursor>::value)
                        epi.store4(yb + s - wV + 1, xin, sw, mask);
                    else
                        epi.store4(cur, sw, mask);
                }
                cur.next();
            }
        }
        // Nothing of this strip may still be landing in the ring.
        cp_async_wait<0>();
    }
}

// Calls f(std::integral_constant<int, (wH-1) mod CPT>()): callers that loop
// over several strips put the loop inside f, one loop per variant.
template <int CPT = kCPT, class F>
__device__ __forceinline__ void with_c(int wH, F&& f)
{
    switch ((wH - 1) % CPT) {
    case 0: f(std::integral_constant<int, 0>()); break;
    case 1: f(std::integral_constant<int, 1>()); break;
    case 2: f(std::integral_constant<int, 2>()); break;
    case 3: f(std::integral_constant<int, 3 % CPT>()); break;
    case 4: f(std::integral_constant<int, 4 % CPT>()); break;
    case 5: f(std::integral_constant<int, 5 % CPT>()); break;
    case 6: f(std::integral_constant<int, 6 % CPT>()); break;
    default: f(std::integral_constant<int, 7 % CPT>()); break;
    }
}

// One warp's strip (see strip_body), compiled for each value of
// (wH-1) mod CPT.
template <int NQ, class Acc, int D, class Prod, class Epi>
__device__ __forceinline__ void run_strip(const Prod& prod, const Epi& epi, int wV, int wH, int xw,
                                          int y0, int nrows, int ocols, char* ring, int cols)
{
    with_c<ColsOf<Prod>::value>(wH, [&](auto cc) {
        strip_body<decltype(cc)::value, NQ, Acc, D>(prod, epi, wV, wH, xw, y0, nrows, ocols, ring, cols);
    });
}

// Warp tasks of one image: task t covers output rows
// [b*strip_rows, (b+1)*strip_rows) and warp column c (t = b*nwc + c, so
// neighbouring warps share their halo columns in L1).
struct TaskGrid
{
    int restart;     // float restart period (rows)
    int strip_rows;  // a multiple of 16 rows, or of a shorter restart period
    int nwc;         // warp columns: ceil(ocols / out_cols_per_warp(wH))
    int ntask;
};

}  // namespace box
}  // namespace tucu
