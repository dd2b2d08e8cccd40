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
// select_kernel4 (rows on 16-byte boundaries): one CTA per (image row, 1024
// columns), 4 columns per thread with 16-byte loads of the left costs.
// select_kernel (any pitch): one CTA per (image row, 256 columns), two
// threads per column (one per half of the disparities).  A thread keeps the
// running minima of its left columns and of as many right columns (the tile's
// and the D - 1 past it, whose right minima the tile's left pixels may look
// up), so each cost is read about twice, from L1, and once from HBM.  The
// right minima of the tile and its halo sit in shared memory for the check.
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

// Wider runs per slice: 4 columns per thread (16-byte loads of the left
// costs), 1024 columns per CTA; costs rows on 16-byte boundaries.
constexpr int kVTile = 1024;

template <class T, class T4>
__global__ void __launch_bounds__(256) select_kernel4(SelectLaunch L)
{
    __shared__ int dR_s[kVTile + kMaxD];
    const int y = blockIdx.y, x0 = blockIdx.x * kVTile, t = threadIdx.x;
    const char* base = static_cast<const char*>(L.costs) + (size_t)y * L.cost_pitch;
    auto cost = [&](int d, int x) -> T {
        return *reinterpret_cast<const T*>(base + (size_t)d * L.slice_pitch + (size_t)x * sizeof(T));
    };
    const int D = L.disparities, W = L.cols;
    const int span = min(kVTile + D - 1, W - x0);
    const int xb = x0 + 4 * t;         // this thread's first column
    const int xhb = x0 + kVTile + 4 * t;  // its first halo column (threads with 4t < D - 1)
    const bool full = xb + 3 < W;
    T cl[4], cr[4], ch[4];
    int dl[4], dr[4], dh[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        cl[j] = cr[j] = ch[j] = worst<T>();
        dl[j] = dr[j] = dh[j] = 0;
    }
    constexpr int kStep = 4;
    for (int d0 = 0; d0 < D; d0 += kStep) {
        T a[kStep][4], b[kStep][4], h[kStep][4];
#pragma unroll
        for (int k = 0; k < kStep; ++k) {
            const int d = d0 + k;
            if (full && d < D) {
                const T4 v = *reinterpret_cast<const T4*>(base + (size_t)d * L.slice_pitch + (size_t)xb * sizeof(T));
                a[k][0] = v.x;
                a[k][1] = v.y;
                a[k][2] = v.z;
                a[k][3] = v.w;
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    a[k][j] = d < D && xb + j < W ? cost(d, xb + j) : worst<T>();
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                b[k][j] = d < D && xb + j < W && d <= xb + j ? cost(d, xb + j - d) : worst<T>();
                const int xh = xhb + j;
                h[k][j] = d < D && 4 * t + j < D - 1 && kVTile + 4 * t + j < span && d <= xh
                              ? cost(d, xh - d)
                              : worst<T>();
            }
        }
#pragma unroll
        for (int k = 0; k < kStep; ++k)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (a[k][j] < cl[j]) {
                    cl[j] = a[k][j];
                    dl[j] = d0 + k;
                }
                if (b[k][j] < cr[j]) {
                    cr[j] = b[k][j];
                    dr[j] = d0 + k;
                }
                if (h[k][j] < ch[j]) {
                    ch[j] = h[k][j];
                    dh[j] = d0 + k;
                }
            }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (4 * t + j < span)
            dR_s[4 * t + j] = dr[j];
        if (4 * t + j < D - 1 && kVTile + 4 * t + j < span)
            dR_s[kVTile + 4 * t + j] = dh[j];
    }
    __syncthreads();
    char* orow = static_cast<char*>(L.out) + (size_t)(y + L.oy) * L.out_pitch;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int x = xb + j;
        if (x >= W)
            break;
        const int xr = x + dl[j];
        int v = 0;
        if (xr < W) {
            const int r = dR_s[xr - x0];
            const int diff = dl[j] > r ? dl[j] - r : r - dl[j];
            v = diff < L.inconsistency ? L.disparity_max - dl[j] : 0;
        }
        store_i32(orow, x + L.ox, L.out_dtype, v);
    }
}

cudaError_t launch_select(const SelectLaunch& L, cudaStream_t st)
{
    if (L.rows <= 0 || L.cols <= 0)
        return cudaSuccess;
    if (L.disparities < 1 || L.disparities > kMaxD)
        return cudaErrorInvalidValue;
    const bool vec16 = reinterpret_cast<uintptr_t>(L.costs) % 16 == 0 && L.cost_pitch % 16 == 0 &&
                       L.slice_pitch % 16 == 0;
    if (vec16) {
        const dim3 g4((unsigned)((L.cols + kVTile - 1) / kVTile), (unsigned)L.rows);
        if (L.cost_dtype == I32)
            select_kernel4<int32_t, int4><<<g4, 256, 0, st>>>(L);
        else if (L.cost_dtype == F32)
            select_kernel4<float, float4><<<g4, 256, 0, st>>>(L);
        else
            return cudaErrorInvalidValue;
        return cudaGetLastError();
    }
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
