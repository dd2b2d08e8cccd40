// box_stereo.cu -- stereo cost aggregation: BoxFilter2::convolve(rowL, rowLe,
// rowR, rowO, op, disparitySearchWidth) (TU/cu/BoxFilter.h:585-746) with the
// thresholded difference op diff<T> (TU/cu/functional.h:385-398), in the
// reference's disparity-major layout (DISPARITY_MAJOR): for every disparity
// d < D,
//
//   costs[d][y][x] = sum over the wV x wH window at (y, x) of
//                    min(|L[y'][x'] - R[y'][x' + d]|, thresh)
//
// for the (rows+1-wV) x (cols+1-wH) window origins, written at (y, x).
// Right-image pixels past the last column count as 0 (the reference reads
// them from its zero-filled row padding).
//
// The reference runs a horizontal pass (box_filterH, a running sum of the
// costs) into a cost volume and a vertical pass over it (box_filterV), with
// device-wide synchronisation between them.  Here every (disparity, warp
// column, row band) is one warp task of the one-pass window-sum strip
// (box_strip.cuh): the producer forms the costs as it expands each input row,
// so no cost volume is stored, and each output element is written once.
// The right image of disparity d starts d columns to the right of the left
// one, which breaks the 4-pixel alignment the lanes' asynchronous copies
// need; each lane copies two aligned 4-pixel groups of the right row and
// shifts them by d mod 4 pixels (the same for the whole warp).  For 1- and
// 2-byte input a warp task covers four consecutive disparities as four
// summed quantities (three right groups, one left), so the copies, ring
// reads and step bookkeeping are shared by four cost slices.  Windows wider
// than a 4-column warp tile holds (wH > 125) run 8 columns per lane, one
// disparity per task, with 8-pixel groups shifted by d mod 8.
#include <algorithm>

#include "stereo.cuh"

namespace tucu
{
namespace box
{

cudaError_t launch_stereo(const StereoLaunch& L, cudaStream_t st)
{
    if (L.wV < 1 || L.wH < 1 || L.ndisp < 1)
        return cudaErrorInvalidValue;
    Geo G;
    G.wV = L.wV;
    G.wH = L.wH;
    G.orows = L.rows + 1 - L.wV;
    G.ocols = L.cols + 1 - L.wH;
    if (G.orows <= 0 || G.ocols <= 0)
        return cudaSuccess;
    const bool integral = L.dtype == U8 || L.dtype == I32;
    const int cpt = out_cols_per_warp(L.wH, 4) > 0 ? 4 : 8;
    const int ctas = stereo_ctas(L.dtype, cpt);
    // Band height: the whole-rounds rule of the box filter over the warp
    // tasks of all disparity groups.
    const int ngroups = (L.ndisp + stereo_group(L.dtype, cpt) - 1) / stereo_group(L.dtype, cpt);
    G.tg = plan_tasks(G.orows, G.ocols, L.wV, L.wH, 0, ctas, integral ? 16 : kRestart, ngroups, cpt, integral);
    const TaskGrid& tg = G.tg;
    StereoArgs A;
    A.left = L.left;
    A.lpitch = L.left_pitch;
    A.right = L.right;
    A.rpitch = L.right_pitch;
    A.rows = L.rows;
    A.cols = L.cols;
    A.thresh = L.thresh;
    A.ndisp = L.ndisp;
    A.costs = static_cast<char*>(L.costs);
    A.cost_pitch = L.cost_pitch;
    A.slice_pitch = L.slice_pitch;
    A.out_dtype = L.cost_dtype;
    const int es = dtype_size(L.cost_dtype);
    A.cls = L.slice_pitch % (4 * (size_t)es) == 0 ? store_class(L.costs, L.cost_pitch, 0, es) : 0;
    const bool vec = plain_vec(L.left, L.left_pitch, L.dtype, cpt) && plain_vec(L.right, L.right_pitch, L.dtype, cpt);
    const long want = ((long)tg.ntask * ngroups + kWarps - 1) / kWarps;
    const long grid = std::max(1L, std::min(want, (long)ctas * sm_count()));
    return cpt == 8 ? launch_stereo_wide(G, A, L.dtype, vec, grid, st)
                    : launch_stereo_cpt<4>(G, A, L.dtype, vec, grid, st);
}

}  // namespace box
}  // namespace tucu
