// extrema.cu -- sliding-window minimum / maximum with the position of each
// extremum: BoxFilter2 with the extrema_finder convolver
// (TU/cu/BoxFilter.h:196-233 over the two passes of BoxFilter.h:542-583).
//
// The reference runs a monotone deque down each column (one thread per
// column, one tile row of threads busy), writes the column extrema and their
// rows to a transposed buffer and runs the deque again along the rows.  Its
// result for a window is the extremum of the column extrema, and among equal
// values the leftmost column, whose row is the topmost one among equal values
// in that column.  Here one CTA makes a 24 x 128 output tile in one pass with
// the van Herk / Gil-Werman scheme in both directions: the tile is cut into
// blocks of w rows (then w columns); each block gets running extrema from its
// start (prefix) and from its end (suffix), and a window [i, i+w-1] is the
// better of suffix[i] and prefix[i+w-1], ties going to the suffix, which holds
// the earlier element.  Prefixes keep the earlier element on ties and
// suffixes take the earlier one, so every result is the reference's element,
// at three comparisons per pixel and direction whatever the window.
//
//   input tile ........ (32 + wV - 1) x (128 + wH - 1) keys in shared
//                       memory, coalesced rows
//   vertical pass ..... one thread per tile column: prefix extrema forward,
//                       suffix extrema backward, column results (value, row)
//   horizontal pass ... one thread per (tile row, block of wH columns):
//                       prefix extrema forward into shared memory, then
//                       suffix extrema backward combined with the prefixes
//   store ............. coalesced rows of values and (x, y) positions
#include <climits>
#include <cmath>

#include "extrema.h"
#include "tucu_common.cuh"
#include "tucu_internal.h"

namespace tucu
{
namespace ext
{

constexpr int kThreads = 256;
// Output rows per tile: the row passes run one thread per (row, block of wH
// columns), and at 24 rows a 15-wide window's 24 x 10 tasks fit one round of
// the 256 threads (measured: 16, 20, 24, 32 rows -> 442, 376, 356, 415 us for
// 15x15 u8 minima at 6480x11520).
constexpr int kTH = 24;
constexpr int kTW = 128;  // output columns per tile

// Comparison keys: exact for every storage type (u8 as itself, so a tile of
// u8 keys takes a quarter of the shared memory; f16, bf16, f32 as float;
// int32 as int).
template <class T> struct KeyOf { using type = float; };
template <> struct KeyOf<int32_t> { using type = int; };
template <> struct KeyOf<uint8_t> { using type = uint8_t; };

template <class T>
__device__ __forceinline__ typename KeyOf<T>::type key_of(T v)
{
    return to_float(v);
}
template <>
__device__ __forceinline__ int key_of<int32_t>(int32_t v)
{
    return v;
}
template <>
__device__ __forceinline__ uint8_t key_of<uint8_t>(uint8_t v)
{
    return v;
}

template <class T> __device__ __forceinline__ T from_key(typename KeyOf<T>::type k);
template <> __device__ __forceinline__ uint8_t from_key<uint8_t>(uint8_t k) { return k; }
template <> __device__ __forceinline__ __half from_key<__half>(float k) { return __float2half_rn(k); }
template <> __device__ __forceinline__ __nv_bfloat16 from_key<__nv_bfloat16>(float k) { return __float2bfloat16_rn(k); }
template <> __device__ __forceinline__ float from_key<float>(float k) { return k; }
template <> __device__ __forceinline__ int32_t from_key<int32_t>(int k) { return k; }

// The key no pixel beats (fills positions outside the image; such positions
// only ever reach outputs outside the valid region).
template <class K, bool MAX> __device__ __forceinline__ K worst();
template <> __device__ __forceinline__ float worst<float, false>() { return INFINITY; }
template <> __device__ __forceinline__ float worst<float, true>() { return -INFINITY; }
template <> __device__ __forceinline__ int worst<int, false>() { return INT_MAX; }
template <> __device__ __forceinline__ int worst<int, true>() { return INT_MIN; }
template <> __device__ __forceinline__ uint8_t worst<uint8_t, false>() { return 255; }
template <> __device__ __forceinline__ uint8_t worst<uint8_t, true>() { return 0; }

// a strictly better than b (the reference's comparison functor: less for
// the minimum, greater for the maximum).
template <bool MAX, class K>
__device__ __forceinline__ bool beats(K a, K b)
{
    return MAX ? (a > b) : (a < b);
}

struct ExArgs
{
    const void* src;
    size_t src_pitch;
    int rows, cols;
    int orows, ocols;
    int wV, wH;
    void* val;
    size_t val_pitch;
    void* pos;
    size_t pos_pitch;
    int oy, ox;
};

__host__ __device__ inline int tile_cols(int wH) { return kTW + wH - 1; }

// Row strides in shared memory (elements): an odd number of 32-bit words,
// so that the 32 rows a warp walks in the row passes fall in 32 different
// banks: ks-byte keys (ks = 1: a multiple of 4 bytes, 4 mod 8; ks = 4: odd)
// and 2-byte row / column indices (2 mod 4).
__host__ __device__ inline int key_stride(int wH, int ks)
{
    const int wt = tile_cols(wH);
    return ks == 1 ? (wt + 3) / 8 * 8 + 4 : wt | 1;
}
__host__ __device__ inline int idx_stride(int wH) { return (tile_cols(wH) + 1) / 4 * 4 + 2; }

// Shared memory, for ks-byte keys: column results vkey [kTH][KS] and vrow
// [kTH][IS], and one region that first holds the input tile [HT][KS] and
// then the row results akey [kTH][KS] and their columns acol [kTH][IS] (KS,
// IS: key_stride, idx_stride).  Each array starts on a
// 16-byte boundary.  Without positions (pos false) only the key arrays
// exist.
__host__ __device__ inline size_t al16(size_t b) { return (b + 15) / 16 * 16; }
__host__ __device__ inline size_t region_bytes(int wV, int wH, int ks, bool pos)
{
    const size_t KS = (size_t)key_stride(wH, ks), IS = (size_t)idx_stride(wH), ht = (size_t)(kTH + wV - 1);
    const size_t a = al16(ht * KS * ks), b = al16((size_t)kTH * KS * ks) + (pos ? al16((size_t)kTH * IS * 2) : 0);
    return a > b ? a : b;
}
__host__ __device__ inline size_t smem_bytes(int wV, int wH, int ks, bool pos)
{
    const size_t KS = (size_t)key_stride(wH, ks), IS = (size_t)idx_stride(wH);
    return region_bytes(wV, wH, ks, pos) + al16((size_t)kTH * KS * ks) + (pos ? al16((size_t)kTH * IS * 2) : 0);
}

// POS: positions are written (else values only, and no row or column is
// tracked).
template <class T, bool MAX, bool POS>
__global__ void __launch_bounds__(kThreads) extrema_kernel(const __grid_constant__ ExArgs A)
{
    using K = typename KeyOf<T>::type;
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int ks = (int)sizeof(K);
    const int WT = tile_cols(A.wH);
    const int HT = kTH + A.wV - 1;
    const int KS = key_stride(A.wH, ks), IS = idx_stride(A.wH);
    const size_t keys = al16((size_t)kTH * KS * ks);
    K* tile = reinterpret_cast<K*>(smem);                         // [HT][KS] input keys
    K* akey = reinterpret_cast<K*>(smem);                         // [kTH][KS] row prefixes (after the tile)
    short* acol = reinterpret_cast<short*>(smem + keys);          // [kTH][IS] their tile columns
    unsigned char* rest = smem + region_bytes(A.wV, A.wH, ks, POS);
    K* vkey = reinterpret_cast<K*>(rest);                         // [kTH][KS] column extrema, then results
    short* vrow = reinterpret_cast<short*>(rest + keys);          // [kTH][IS] their tile rows
    const int x0 = blockIdx.x * kTW, y0 = blockIdx.y * kTH;
    const int tid = threadIdx.x;
    const int wV = A.wV, wH = A.wH;

    // ---- input tile as keys (positions outside the image get the worst key;
    // they only ever reach outputs outside the valid region) ----
    {
        const int rlim = min(HT, A.rows - y0);
        for (int c = tid; c < WT; c += kThreads) {
            const int x = x0 + c;
            const int rl = x < A.cols ? rlim : 0;
            const char* src = reinterpret_cast<const char*>(
                reinterpret_cast<const T*>(row_ptr(A.src, A.src_pitch, y0)) + x);
#pragma unroll 8
            for (int r = 0; r < rl; ++r)
                tile[r * KS + c] = key_of(*reinterpret_cast<const T*>(src + (size_t)r * A.src_pitch));
            for (int r = max(rl, 0); r < HT; ++r)
                tile[r * KS + c] = worst<K, MAX>();
        }
    }
    __syncthreads();

    // ---- vertical pass: one thread per tile column ----
    for (int c = tid; c < WT; c += kThreads) {
        const K* col = tile + c;
        // Prefix extrema over blocks of wV rows starting at tile row 0; the
        // prefix at row r >= wV-1 is the far end of the window starting at
        // r - wV + 1.
        K pk = worst<K, MAX>();
        int pr = 0;
        for (int r = 0, m = 0; r < HT; ++r) {  // m = r mod wV
            const K k = col[r * KS];
            if (m == 0 || beats<MAX>(k, pk)) {
                pk = k;
                pr = r;
            }
            if (++m == wV)
                m = 0;
            if (r >= wV - 1) {
                vkey[(r - wV + 1) * KS + c] = pk;
                if constexpr (POS)
                    vrow[(r - wV + 1) * IS + c] = (short)pr;
            }
        }
        // Suffix extrema from the end of the block holding tile row kTH-1,
        // each combined with the stored prefix of its window.
        const int rb = ((kTH - 1) / wV + 1) * wV - 1;  // <= HT - 1
        K sk = worst<K, MAX>();
        int sr = rb;
        for (int r = rb, m = 0; r >= 0; --r) {  // m = (rb - r) mod wV
            const K k = col[r * KS];
            if (m == 0 || !beats<MAX>(sk, k)) {
                sk = k;
                sr = r;
            }
            if (++m == wV)
                m = 0;
            if (r < kTH) {
                if (!beats<MAX>(vkey[r * KS + c], sk)) {
                    vkey[r * KS + c] = sk;
                    if constexpr (POS)
                        vrow[r * IS + c] = (short)sr;
                }
            }
        }
    }
    __syncthreads();  // the tile region now holds the row results

    // ---- row pass: thread (tile row r, block b of wH columns) forms block
    // b's suffix extrema backward (into akey/acol), then walks block b+1
    // forward with its prefix extrema and lets each replace the suffix of
    // the window that ends there when strictly better (ties stay with the
    // suffix: the earlier element).  A thread reads the column extrema and
    // writes block b's slots only, so the two halves need no barrier.
    // Consecutive threads take consecutive rows of a block (the row strides
    // put a block's rows in different banks). ----
    const int nbh = (WT + wH - 1) / wH;
    for (int t = tid; t < kTH * nbh; t += kThreads) {
        const int r = t % kTH, b = t / kTH;
        const int c0 = b * wH;
        if (c0 >= kTW)
            continue;  // no window starts in this block
        const int c1 = min(c0 + wH, WT) - 1;
        const K* vk = vkey + r * KS;
        K* ak = akey + r * KS;
        short* ac = acol + r * IS;
        K sk = vk[c1];
        int sc = c1;
        for (int c = c1; c >= c0; --c) {
            const K k = vk[c];
            if (!beats<MAX>(sk, k)) {
                sk = k;
                sc = c;
            }
            ak[c] = sk;
            if constexpr (POS)
                ac[c] = (short)sc;
        }
        // Window [c, c+wH-1], c0 < c < c0+wH: suffix at c and the prefix of
        // block b+1 at j = c+wH-1 (c < kTW keeps j inside the tile).
        const int d0 = c0 + wH, d1 = min(c0 + 2 * wH - 1, kTW + wH - 1);
        if (d0 < d1) {
            K pk = vk[d0];
            int pc = d0;
            for (int jj = d0; jj < d1; ++jj) {
                const K k = vk[jj];
                if (beats<MAX>(k, pk)) {
                    pk = k;
                    pc = jj;
                }
                const int c = jj - wH + 1;
                if (beats<MAX>(pk, ak[c])) {
                    ak[c] = pk;
                    if constexpr (POS)
                        ac[c] = (short)pc;
                }
            }
        }
    }
    __syncthreads();

    // ---- store: coalesced rows ----
    for (int i = tid; i < kTH * kTW; i += kThreads) {
        const int r = i / kTW, c = i - r * kTW;
        const int y = y0 + r, x = x0 + c;
        if (y >= A.orows || x >= A.ocols)
            continue;
        if (A.val)
            reinterpret_cast<T*>(row_ptr(A.val, A.val_pitch, y + A.oy))[x + A.ox] =
                from_key<T>(akey[r * KS + c]);
        if constexpr (POS) {
            const int cs = acol[r * IS + c];
            reinterpret_cast<int2*>(row_ptr(A.pos, A.pos_pitch, y + A.oy))[x + A.ox] =
                make_int2(x0 + cs, y0 + vrow[r * IS + cs]);
        }
    }
}

template <class T, bool MAX, bool POS>
static cudaError_t launch_t(const ExArgs& A, cudaStream_t st)
{
    auto kern = extrema_kernel<T, MAX, POS>;
    constexpr int ks = (int)sizeof(typename KeyOf<T>::type);
    static DeviceOnce attr_once;
    cudaError_t e = attr_once.run([&] {
        return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem_bytes(kWinLimit, kWinLimit, ks, POS));
    });
    if (e != cudaSuccess)
        return e;
    const dim3 grid((A.ocols + kTW - 1) / kTW, (A.orows + kTH - 1) / kTH);
    kern<<<grid, kThreads, smem_bytes(A.wV, A.wH, ks, POS), st>>>(A);
    return cudaGetLastError();
}

template <class T>
static cudaError_t launch_op(const ExArgs& A, bool is_max, cudaStream_t st)
{
    if (A.pos)
        return is_max ? launch_t<T, true, true>(A, st) : launch_t<T, false, true>(A, st);
    return is_max ? launch_t<T, true, false>(A, st) : launch_t<T, false, false>(A, st);
}

cudaError_t launch_extrema(const ExtremaLaunch& L, cudaStream_t st)
{
    if (L.wV < 1 || L.wH < 1 || L.wV > kWinLimit || L.wH > kWinLimit)
        return cudaErrorInvalidValue;
    ExArgs A;
    A.src = L.src;
    A.src_pitch = L.src_pitch;
    A.rows = L.rows;
    A.cols = L.cols;
    A.orows = L.rows + 1 - L.wV;
    A.ocols = L.cols + 1 - L.wH;
    A.wV = L.wV;
    A.wH = L.wH;
    A.val = L.val;
    A.val_pitch = L.val_pitch;
    A.pos = L.pos;
    A.pos_pitch = L.pos_pitch;
    A.oy = L.oy;
    A.ox = L.ox;
    if (A.orows <= 0 || A.ocols <= 0)
        return cudaSuccess;
    switch (L.dtype) {
    case U8: return launch_op<uint8_t>(A, L.is_max, st);
    case F16: return launch_op<__half>(A, L.is_max, st);
    case BF16: return launch_op<__nv_bfloat16>(A, L.is_max, st);
    case F32: return launch_op<float>(A, L.is_max, st);
    case I32: return launch_op<int32_t>(A, L.is_max, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace ext
}  // namespace tucu

