// box_plain.cuh -- the plain box filter kernels (single image and batch
// class) on the window-sum strip, compiled per input type, vector-load
// flag and output type (TOut = void: output dtype read at run time).  The
// instantiations live in box_generic.cu and box_typed.cu.
#pragma once
#include "batch_types.h"
#include "box_ops.cuh"

namespace tucu
{
namespace box
{

// CTAs per SM the plain box kernels are compiled for (registers per thread
// at most 65536 / (256 * kBoxCtas)), and the shared memory each warp gives
// its row ring (kBoxCtas * kWarps * kBoxWarpBytes per SM).
constexpr int kBoxCtas = 4;
constexpr int kBoxWarpBytes = 4096;

template <class TIn> struct AccOf { using type = float; };
template <> struct AccOf<uint8_t> { using type = int; };
template <> struct AccOf<int32_t> { using type = int; };

// Ring depth and dynamic shared memory of the plain box kernels.
template <class TIn, bool VEC>
struct PlainRing
{
    using Prod = PlainProd<TIn, typename AccOf<TIn>::type, VEC>;
    static constexpr int kDepth = Ring<Prod>::depth(kBoxWarpBytes);
    static constexpr int kSmem = kWarps * kDepth * Ring<Prod>::kStepBytes;
};
size_t plain_smem_bytes(int in_dtype);

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
// resident CTAs (strip_rows when given, rounded to 16 rows): the multiple of
// the restart period that minimises whole rounds of warp tasks x (band + wV),
// over `copies` images of the same size (the disparities of the stereo
// costs), split below the restart period for images too small to occupy the
// GPU.
TaskGrid plan_tasks(int orows, int ocols, int wV, int wH, int strip_rows, int ctas_per_sm,
                    int restart = kRestart, int copies = 1);

// Runs this warp's tasks of the image: f(C, xw, y0, nrows) for each, with C
// = (wH-1) mod 4 as a compile-time constant (the task loop is compiled once
// per value).
template <class F>
__device__ __forceinline__ void for_each_task(const Geo& G, F&& f)
{
    with_c(G.wH, [&](auto cc) {
        const int tw = out_cols_per_warp(G.wH);
        const int nw = gridDim.x * kWarps;
        for (int t = blockIdx.x * kWarps + (threadIdx.x >> 5); t < G.tg.ntask; t += nw) {
            const int b = t / G.tg.nwc, c = t - b * G.tg.nwc;
            const int y0 = b * G.tg.strip_rows;
            f(cc, c * tw, y0, min(G.tg.strip_rows, G.orows - y0));
        }
    });
}

// This warp's ring in the kernel's dynamic shared memory.
__device__ __forceinline__ char* warp_ring(int bytes_per_warp)
{
    extern __shared__ __align__(16) char box_smem[];
    return box_smem + (threadIdx.x >> 5) * bytes_per_warp;
}

template <class TIn, bool VEC, class TOut>
__global__ void __launch_bounds__(kThreads, kBoxCtas)
    box_kernel(const __grid_constant__ Geo G, const __grid_constant__ BoxArgs A)
{
    using Acc = typename AccOf<TIn>::type;
    using R = PlainRing<TIn, VEC>;
    const PlainProd<TIn, Acc, VEC> prod{A.src, A.src_pitch, A.rows, A.cols};
    const PlainEpi<Acc, TOut> epi{A.dst, A.dst_pitch, A.out_dtype, A.oy, A.ox, A.normalize, A.inv_n, A.cls};
    char* ring = warp_ring(R::kSmem / kWarps);
    for_each_task(G, [&](auto cc, int xw, int y0, int nrows) {
        strip_body<decltype(cc)::value, 1, Acc, R::kDepth>(prod, epi, G.wV, G.wH, xw, y0, nrows, G.ocols,
                                                             ring, A.cols, G.tg.restart);
    });
}

// Eight warp items of a box batch class per CTA: warp w of CTA b runs item
// 8b + w (a warp column at a multiple of out_cols_per_warp and a row band);
// padding items (job < 0) do nothing.
template <class TIn, bool VEC, class TOut>
__global__ void __launch_bounds__(kThreads, kBoxCtas)
    box_batch_kernel(const batch::BoxJobD* __restrict__ jobs, const batch::Item* __restrict__ items)
{
    using Acc = typename AccOf<TIn>::type;
    using R = PlainRing<TIn, VEC>;
    const batch::Item it = items[blockIdx.x * kWarps + (threadIdx.x >> 5)];
    if (it.job < 0)
        return;  // no barrier in the strip: the other warps go on alone
    const batch::BoxJobD& J = jobs[it.job];
    const PlainEpi<Acc, TOut> epi{J.dst, J.dst_pitch, J.out_dtype, J.oy, J.ox, J.normalize,
                                  1.0f / (float)(J.wV * J.wH), J.cls};
    const PlainProd<TIn, Acc, VEC> prod{J.src, J.src_pitch, J.rows, J.cols};
    run_strip<1, Acc, R::kDepth>(prod, epi, J.wV, J.wH, it.x0, it.y0, it.nrows, J.ocols,
                                 warp_ring(R::kSmem / kWarps), J.cols);
}

// Kernel pointers: single-image (Geo, BoxArgs) or batch (jobs, items).
// The generic kernels (one translation unit per input type) cover every
// input type; the typed ones only the pairs they were compiled for
// (nullptr otherwise).
template <class TIn>
const void* generic_kernel_of(bool vec, bool batch)
{
    if (batch)
        return vec ? (const void*)box_batch_kernel<TIn, true, void> : (const void*)box_batch_kernel<TIn, false, void>;
    return vec ? (const void*)box_kernel<TIn, true, void> : (const void*)box_kernel<TIn, false, void>;
}
const void* generic_kernel_u8(bool vec, bool batch);
const void* generic_kernel_i32(bool vec, bool batch);
const void* generic_kernel_f16(bool vec, bool batch);
const void* generic_kernel_bf16(bool vec, bool batch);
const void* generic_kernel_f32(bool vec, bool batch);

inline const void* generic_kernel(int in_dtype, bool vec, bool batch)
{
    switch (in_dtype) {
    case U8: return generic_kernel_u8(vec, batch);
    case I32: return generic_kernel_i32(vec, batch);
    case F16: return generic_kernel_f16(vec, batch);
    case BF16: return generic_kernel_bf16(vec, batch);
    case F32: return generic_kernel_f32(vec, batch);
    default: return nullptr;
    }
}
const void* typed_kernel(int in_dtype, int out_dtype, bool batch);

}  // namespace box
}  // namespace tucu
