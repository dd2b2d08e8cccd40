// batch_types.h -- device descriptors of the batched launch (batch.cu), shared
// with the translation units that hold the per-class kernels.
#pragma once
#include "fir_strip.cuh"

namespace tucu
{
namespace batch
{

// One FIR / Gaussian job of a batch.
struct alignas(64) FirJobD
{
    fir::FirJob fir;
    fir::LobeSet lobes;
    int has_tmap;
};

// One box job of a batch.
struct alignas(16) BoxJobD
{
    const void* src;
    size_t src_pitch;
    int rows, cols;
    int wV, wH, orows, ocols;
    void* dst;
    size_t dst_pitch;
    int out_dtype, oy, ox, normalize;
    int cls;  // alignment class of the output stores (box::store_class)
};

// One strip of one job.
struct Item
{
    int job;
    int x0, y0, nrows;
};

}  // namespace batch

namespace box
{
// Kernel of the box batch class for an input / output type pair and cpt
// columns per lane; arguments (const BoxJobD*, const Item*), eight warp
// items per CTA.
const void* batch_kernel(int in_dtype, int out_dtype, bool vec, int cpt, bool win);
// Dynamic shared memory of the plain box kernels for an input type.
size_t plain_smem_bytes(int in_dtype, int cpt, bool win);
// The window-ring kernels apply (results are the same either way).
bool plain_win(int in_dtype, int out_dtype, bool vec, int cpt, int wV);
// Columns per lane of the plain box strip for a window width, and whether an
// image's rows are aligned for the copies of cpt-pixel groups.
int plain_cpt(int wH);
bool plain_vec(const void* src, size_t pitch, int in_dtype, int cpt);
}  // namespace box

}  // namespace tucu
