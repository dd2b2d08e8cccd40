// box_plain.cuh -- the plain box filter kernels (single image and batch
// class) on the window-sum strip, compiled per input type, vector-load
// flag and output type (TOut = void: output dtype read at run time).  The
// instantiations live in box_generic.cu and box_typed.cu.
#pragma once
#include "batch_types.h"
#include "box_ops.cuh"
#include "tucu_internal.h"

namespace tucu
{
namespace box
{

// CTAs per SM the plain box kernels with CPT columns per lane are compiled
// for (registers per thread at most 65536 / (256 * kCtas)), and the shared
// memory each warp gives its row ring (kCtas * kWarps * kWarpBytes per SM,
// at most 48 KB per CTA).  Eight columns per lane hold twice the running
// sums, so fewer CTAs share an SM.
template <int CPT>
struct PlainCfg
{
    static constexpr int kCtas = CPT == 8 ? 3 : 4;
    static constexpr int kWarpBytes = CPT == 8 ? 6144 : 4096;
};
constexpr int kBoxCtas = PlainCfg<kCPT>::kCtas;

template <class TIn> struct AccOf { using type = float; };
template <> struct AccOf<uint8_t> { using type = int; };
template <> struct AccOf<int32_t> { using type = int; };

// A producer whose strip keeps the window's rows in a ring (WinOf).
template <class P>
struct Windowed : P
{
    static constexpr bool kWindowRing = true;
};

// Window-ring geometry of the plain box kernels (1- and 2-byte input): a ring
// of kWinRows rows per warp, kWinDepth steps in flight, so windows up to
// kWinRows - kWinDepth + 1 rows tall.
constexpr int kWinRows = 24;
constexpr int kWinDepth = 8;
constexpr int kWinMaxV = kWinRows - kWinDepth + 1;

// Ring depth, rows and dynamic shared memory of the plain box kernels.
template <class TIn, bool VEC, int CPT = kCPT, bool WIN = false>
struct PlainRing
{
    using Base = PlainProd<TIn, typename AccOf<TIn>::type, VEC, CPT>;
    using Prod = std::conditional_t<WIN, Windowed<Base>, Base>;
    static constexpr int kDepth = WIN ? kWinDepth : Ring<Base>::depth(PlainCfg<CPT>::kWarpBytes);
    static constexpr int kRows = WIN ? kWinRows : 2 * kDepth;
    static constexpr int kSmem = kWarps * kRows * Ring<Base>::kRowBytes;
};
size_t plain_smem_bytes(int in_dtype, int cpt, bool win = false);

// Columns per lane of the plain box strip: 8 only for windows wider than a
// 4-column warp tile holds (wH > 125).  The single-image launch and the
// batch planner both decide by plain_cpt (batch_types.h), so an image's
// float sums do not depend on which of them ran.  (Eight columns per lane
// for large images was measured and lost: 198 vs 126 us for 15x15 f16 means
// at 6480x11520, 160 vs 119 us for u8 sums.)


// Geometry and task grid of one image.
struct Geo
{
    int wV, wH;
    int orows, ocols;  // output extent (valid coords)
    TaskGrid tg;
};

// Arguments of the single-image kernel (the same for every instantiation).
struct BoxArgs
{
    const void* src;
    size_t src_pitch;
    int rows, cols;
    void* dst;
    size_t dst_pitch;
    int out_dtype, oy, ox, normalize;
    float inv_n;
    int cls;  // store_class of dst, dst_pitch, ox
};

// Band height and warp tasks of an image for kernels with ctas_per_sm
// resident CTAs and cpt columns per lane (strip_rows when given, rounded to
// 16 rows): the multiple of the restart period that minimises whole rounds
// of warp tasks x (band + wV), over `copies` images of the same size (the
// disparities of the stereo costs), split below the restart period for
// images too small to occupy the GPU (exact: integer sums, whose bands
// replay nothing and may shrink further).
TaskGrid plan_tasks(int orows, int ocols, int wV, int wH, int strip_rows, int ctas_per_sm,
                    int restart = kRestart, int copies = 1, int cpt = kCPT, bool exact = false);

// Runs this warp's tasks of the image: f(C, xw, y0, nrows) for each, with C
// = (wH-1) mod CPT as a compile-time constant (the task loop is compiled
// once per value).
template <int CPT = kCPT, class F>
__device__ __forceinline__ void for_each_task(const Geo& G, F&& f)
{
    with_c<CPT>(G.wH, [&](auto cc) {
        const int tw = out_cols_per_warp(G.wH, CPT);
        const int nw = gridDim.x * kWarps;
        for (int t = blockIdx.x * kWarps + (threadIdx.x >> 5); t < G.tg.ntask; t += nw) {
            const int b = t / G.tg.nwc, c = t - b * G.tg.nwc;
            const int y0 = b * G.tg.strip_rows;
            f(cc, c * tw, y0, min(G.tg.strip_rows, G.orows - y0));
        }
    });
}

// Raises kernel FN's dynamic shared memory limit to smem bytes where that
// exceeds the 48 KB default (once per device).
template <auto FN>
cudaError_t smem_opt_in(size_t smem)
{
    if (smem <= 48 * 1024)
        return cudaSuccess;
    static DeviceOnce once;
    return once.run([&] {
        return cudaFuncSetAttribute((const void*)FN, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    });
}

// This warp's ring in the kernel's dynamic shared memory.
__device__ __forceinline__ char* warp_ring(int bytes_per_warp)
{
    extern __shared__ __align__(16) char box_smem[];
    return box_smem + (threadIdx.x >> 5) * bytes_per_warp;
}

template <class TIn, bool VEC, class TOut, int CPT = kCPT, bool WIN = false>
__global__ void __launch_bounds__(kThreads, PlainCfg<CPT>::kCtas)
    box_kernel(const __grid_constant__ Geo G, const __grid_constant__ BoxArgs A)
{
    using Acc = typename AccOf<TIn>::type;
    using R = PlainRing<TIn, VEC, CPT, WIN>;
    typename R::Prod prod;
    prod.src = A.src;
    prod.pitch = A.src_pitch;
    prod.rows = A.rows;
    prod.cols = A.cols;
    const PlainEpi<Acc, TOut> epi{A.dst, A.dst_pitch, A.out_dtype, A.oy, A.ox, A.normalize, A.inv_n, A.cls};
    char* ring = warp_ring(R::kSmem / kWarps);
    for_each_task<CPT>(G, [&](auto cc, int xw, int y0, int nrows) {
        strip_body<decltype(cc)::value, 1, Acc, R::kDepth>(prod, epi, G.wV, G.wH, xw, y0, nrows, G.ocols,
                                                             ring, A.cols, G.tg.restart, R::kRows);
    });
}

// Eight warp items of a box batch class per CTA: warp w of CTA b runs item
// 8b + w (a warp column at a multiple of out_cols_per_warp(wH, CPT) and a
// row band); padding items (job < 0) do nothing.
template <class TIn, bool VEC, class TOut, int CPT = kCPT, bool WIN = false>
__global__ void __launch_bounds__(kThreads, PlainCfg<CPT>::kCtas)
    box_batch_kernel(const batch::BoxJobD* __restrict__ jobs, const batch::Item* __restrict__ items)
{
    using Acc = typename AccOf<TIn>::type;
    using R = PlainRing<TIn, VEC, CPT, WIN>;
    const batch::Item it = items[blockIdx.x * kWarps + (threadIdx.x >> 5)];
    if (it.job < 0)
        return;  // no barrier in the strip: the other warps go on alone
    const batch::BoxJobD& J = jobs[it.job];
    const PlainEpi<Acc, TOut> epi{J.dst, J.dst_pitch, J.out_dtype, J.oy, J.ox, J.normalize,
                                  1.0f / (float)(J.wV * J.wH), J.cls};
    typename R::Prod prod;
    prod.src = J.src;
    prod.pitch = J.src_pitch;
    prod.rows = J.rows;
    prod.cols = J.cols;
    char* ring = warp_ring(R::kSmem / kWarps);
    with_c<CPT>(J.wH, [&](auto cc) {
        strip_body<decltype(cc)::value, 1, Acc, R::kDepth>(prod, epi, J.wV, J.wH, it.x0, it.y0, it.nrows,
                                                             J.ocols, ring, J.cols, kRestart, R::kRows);
    });
}

// Kernel pointers: single-image (Geo, BoxArgs) or batch (jobs, items), with
// cpt (4 or 8) columns per lane.  The generic kernels (one translation unit
// per input type) cover every input type; the typed ones only the pairs
// they were compiled for (nullptr otherwise).
template <class TIn, int CPT>
const void* generic_kernel_cpt(bool vec, bool batch)
{
    // Wide windows (8 columns per lane) run the synchronous loads only.
    if constexpr (CPT == kCPT) {
        if (vec)
            return batch ? (const void*)box_batch_kernel<TIn, true, void, CPT>
                         : (const void*)box_kernel<TIn, true, void, CPT>;
    }
    return batch ? (const void*)box_batch_kernel<TIn, false, void, CPT> : (const void*)box_kernel<TIn, false, void, CPT>;
}
template <class TIn>
const void* generic_kernel_of(bool vec, bool batch, int cpt)
{
    return cpt == 8 ? generic_kernel_cpt<TIn, 8>(vec, batch) : generic_kernel_cpt<TIn, 4>(vec, batch);
}
const void* generic_kernel_u8(bool vec, bool batch, int cpt);
const void* generic_kernel_i32(bool vec, bool batch, int cpt);
const void* generic_kernel_f16(bool vec, bool batch, int cpt);
const void* generic_kernel_bf16(bool vec, bool batch, int cpt);
const void* generic_kernel_f32(bool vec, bool batch, int cpt);

inline const void* generic_kernel(int in_dtype, bool vec, bool batch, int cpt)
{
    switch (in_dtype) {
    case U8: return generic_kernel_u8(vec, batch, cpt);
    case I32: return generic_kernel_i32(vec, batch, cpt);
    case F16: return generic_kernel_f16(vec, batch, cpt);
    case BF16: return generic_kernel_bf16(vec, batch, cpt);
    case F32: return generic_kernel_f32(vec, batch, cpt);
    default: return nullptr;
    }
}
// win: the window-ring kernels (1- and 2-byte input, wV <= kWinMaxV).
const void* typed_kernel(int in_dtype, int out_dtype, bool batch, int cpt, bool win = false);

}  // namespace box
}  // namespace tucu
