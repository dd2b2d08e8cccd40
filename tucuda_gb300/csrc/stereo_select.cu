// stereo_select.cu -- DisparitySelector (TU/cu/StereoUtility.h:56-217): the
// step after stereo cost aggregation.  For each pixel of a disparity-major
// cost volume C[d][y][x] (d < D):
//
//   dL(x)  = first d minimising C[d][y][x]                 (left image)
//   dR(xr) = first d minimising C[d][y][xr - d], d <= xr   (right image: the
//            left pixel x = xr - d sees right pixel xr at disparity d)
//   out[y][x] = |dL(x) - dR(x + dL(x))| < inconsistency ? disparityMax - dL(x) : 0
//
// as select_disparity computes it (StereoUtility.h:56-107: strict "<", so the
// smallest disparity wins ties; the same output formula).  Two places where
// the reference's result is not defined are given a definite one here: its
// right-image minima live in a global row that the blocks of a row update and
// initialise without synchronising with one another, and x + dL(x) past the
// row's end reads outside the row; here dR is the exact minimum over every d
// and such pixels get 0.
//
// One CTA per (image row, tile of 256 columns), two threads per column (one
// per half of the disparities); a thread keeps the running minima of one left
// column and one right column (the tile's columns and the D - 1 columns past
// the tile, whose right minima the tile's left pixels may look up), so each
// cost is read about twice, from L1, and once from HBM.  The right minima of
// the tile and its halo sit in shared memory for the check.
#include <cfloat>
#include <climits>

#include "stereo_select.h"
#include "tucu_common.cuh"

namespace tucu
{
namespace sel
{

constexpr int kTile = 256;
constexpr int kMaxD = 256;  // disparity search widths up to 256 (shared halo)

template <class T> __device__ __forceinline__ T worst();
template <> __device__ __forceinline__ int32_t worst<int32_t>() { return INT_MAX; }
template <> __device__ __forceinline__ float worst<float>() { return FLT_MAX; }

template <class T>
__global__ void __launch_bounds__(2 * kTile) select_kernel(SelectLaunch L)
{
    // two threads per column: half 0 takes the lower disparities, half 1 the
    // upper ones; their minima are merged with half 0 winning ties (the
    // smaller d), which is the first minimum over all d
    __shared__ int dR_s[kTile + kMaxD];
    __shared__ T mval[3][kTile];
    __shared__ int mdisp[3][kTile];
    const int y = blockIdx.y, x0 = blockIdx.x * kTile;
    const int t = threadIdx.x % kTile, half = threadIdx.x / kTile;
    const char* base = static_cast<const char*>(L.costs) + (size_t)y * L.cost_pitch;
    auto cost = [&](int d, int x) -> T {
        return *reinterpret_cast<const T*>(base + (size_t)d * L.slice_pitch + (size_t)x * sizeof(T));
    };
    const int D = L.disparities, W = L.cols;
    const int span = min(kTile + D - 1, W - x0);  // columns whose right minima are needed
    // left minimum of column x0 + t and right minima of x0 + t and x0 + kTile + t
    const int x = x0 + t;
    T cl = worst<T>(), cr = worst<T>(), ch = worst<T>();
    int dl = 0, dr = 0, dh = 0;
    const bool has_l = x < W, has_h = t < D - 1 && kTile + t < span;
    const int xh = x0 + kTile + t;
    const int dh0 = (D + 1) / 2;
    const int dbeg = half ? dh0 : 0, dend = half ? D : dh0;
    // eight disparities per step: their loads are all issued before the
    // compares (in increasing d, so the first minimum wins)
    constexpr int kStep = 8;
    for (int d0 = dbeg; d0 < dend; d0 += kStep) {
        T a[kStep], b[kStep], h[kStep];
#pragma unroll
        for (int k = 0; k < kStep; ++k) {
            const int d = d0 + k;
            a[k] = has_l && d < dend ? cost(d, x) : worst<T>();
            b[k] = has_l && d < dend && d <= x ? cost(d, x - d) : worst<T>();
            h[k] = has_h && d < dend && d <= xh ? cost(d, xh - d) : worst<T>();
        }
#pragma unroll
        for (int k = 0; k < kStep; ++k) {
            if (a[k] < cl) {
                cl = a[k];
                dl = d0 + k;
            }
            if (b[k] < cr) {
                cr = b[k];
                dr = d0 + k;
            }
            if (h[k] < ch) {
                ch = h[k];
                dh = d0 + k;
            }
        }
    }
    if (half) {
        mval[0][t] = cl;
        mdisp[0][t] = dl;
        mval[1][t] = cr;
        mdisp[1][t] = dr;
        mval[2][t] = ch;
        mdisp[2][t] = dh;
    }
    __syncthreads();
    if (!half) {
        if (mval[0][t] < cl)
            dl = mdisp[0][t];
        if (mval[1][t] < cr)
            dr = mdisp[1][t];
        if (mval[2][t] < ch)
            dh = mdisp[2][t];
        if (t < span)
            dR_s[t] = dr;
        if (has_h)
            dR_s[kTile + t] = dh;
    }
    __syncthreads();
    if (half || !has_l)
        return;
    const int xr = x + dl;
    int v = 0;
    if (xr < W) {
        const int diff = dl > dR_s[xr - x0] ? dl - dR_s[xr - x0] : dR_s[xr - x0] - dl;
        v = diff < L.inconsistency ? L.disparity_max - dl : 0;
    }
    char* orow = static_cast<char*>(L.out) + (size_t)(y + L.oy) * L.out_pitch;
    store_i32(orow, x + L.ox, L.out_dtype, v);
}

cudaError_t launch_select(const SelectLaunch& L, cudaStream_t st)
{
    if (L.rows <= 0 || L.cols <= 0)
        return cudaSuccess;
    if (L.disparities < 1 || L.disparities > kMaxD)
        return cudaErrorInvalidValue;
    const dim3 grid((unsigned)((L.cols + kTile - 1) / kTile), (unsigned)L.rows);
    if (L.cost_dtype == I32)
        select_kernel<int32_t><<<grid, 2 * kTile, 0, st>>>(L);
    else if (L.cost_dtype == F32)
        select_kernel<float><<<grid, 2 * kTile, 0, st>>>(L);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

}  // namespace sel
}  // namespace tucu
