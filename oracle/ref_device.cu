// ref_device.cu -- test infrastructure for the oracle, never linked into the
// library: kernels that run the reference's own device code on small arrays,
// compiled from its headers where they lie.
//
//   TU/cu/FIRFilter.h:66-176  device::convolve, the tap expressions of the
//                             even (odd L) and odd (even L) lobes
//   TU/cu/BoxFilter.h:175-194 box_convolver, the running window sums down a
//                             column of a tile
//   TU/cu/BoxFilter.h:196-233 extrema_finder with extrema_value (BoxFilter.h:
//                             104-117), the sliding minima / maxima down a column,
//                             and with extrema_position (BoxFilter.h:119-159), the
//                             same with the row each one came from
//
// ref_shim_dev/ stands in for the headers these two include (declarations
// only).  `make ref_device REF=<checkout>` builds _ref/ref_device.cubin with
// nvcc's default device flags (FMA contraction on, as the reference's own build
// compiles these expressions) and _ref/ref_device_nofma.cubin with
// -fmad=false; tests/golden/make_ref_device.py runs both on a GPU and stores
// the outputs as fixtures.  Every kernel checks its sizes against the buffers
// it is given before any access.
#include <cstddef>
#include <type_traits>

#include "TU/cu/FIRFilter.h"
#include "TU/cu/BoxFilter.h"

namespace
{

template <size_t L>
__device__ __forceinline__ float tap(const float* in, const float* lobe)
{
    return TU::cu::device::convolve(in, lobe, std::integral_constant<size_t, L>());
}

// The reference's tap expression for lobe length L (its FIRFilter2 accepts
// 2, 3, 4, 5, 8, 9, 16 and 17); in[0 .. 2*(L & ~1)] are read.
__device__ float tap_any(const float* in, const float* lobe, int L)
{
    switch (L) {
    case 2: return tap<2>(in, lobe);
    case 3: return tap<3>(in, lobe);
    case 4: return tap<4>(in, lobe);
    case 5: return tap<5>(in, lobe);
    case 8: return tap<8>(in, lobe);
    case 9: return tap<9>(in, lobe);
    case 16: return tap<16>(in, lobe);
    default: return tap<17>(in, lobe);
    }
}

__device__ bool lobe_ok(int L)
{
    return L == 2 || L == 3 || L == 4 || L == 5 || L == 8 || L == 9 || L == 16 || L == 17;
}

// Column tiles: kCols columns (one thread each) of at most kRowsMax rows;
// shared rows padded by one element as the reference's kernels pad theirs.
constexpr int kCols = 32;
constexpr int kRowsMax = 64;
constexpr int kW = kCols + 1;

struct LessF
{
    using first_argument_type = float;
    __device__ bool operator()(float a, float b) const { return a < b; }
};
struct GreaterF
{
    using first_argument_type = float;
    __device__ bool operator()(float a, float b) const { return a > b; }
};

template <class T>
__device__ void load_tile(const T* in, int rows, T (*in_s)[kW])
{
    for (int y = 0; y < rows; ++y)
        in_s[y][threadIdx.x] = in[y * kCols + threadIdx.x];
}

template <class T>
__device__ void store_tile(const T (*out_s)[kW], int rows, T* out)
{
    for (int y = 0; y < rows; ++y)
        out[y * kCols + threadIdx.x] = out_s[y][threadIdx.x];
}

template <class T>
__device__ void box_cols(const T* in, int rows, int win, T* out)
{
    __shared__ T in_s[kRowsMax][kW];
    __shared__ T out_s[kRowsMax][kW];
    const int ye = rows - win + 1;  // output rows
    if (threadIdx.x >= kCols || rows > kRowsMax || win < 1 || ye < 1)
        return;
    load_tile(in, rows, in_s);
    const TU::cu::device::box_convolver<T> convolve;
    convolve(in_s, out_s, win, ye);
    store_tile(out_s, ye, out);
}

template <class COMP>
__device__ void extrema_cols(const float* in, int rows, int win, float* out)
{
    __shared__ float in_s[kRowsMax][kW];
    __shared__ float out_s[kRowsMax][kW];
    const int ye = rows - win + 1;
    // windows below the finder's deque size less one (WMAX = 23)
    if (threadIdx.x >= kCols || rows > kRowsMax || win < 2 || win > 21 || ye < 1)
        return;
    load_tile(in, rows, in_s);
    const TU::cu::device::extrema_finder<TU::cu::device::extrema_value<COMP>, 23> find;
    find(in_s, out_s, win, ye);
    store_tile(out_s, ye, out);
}

// The column pass with positions: extrema_position's tuples (value, row) in
// shared memory (raw storage: the tuple type has a constructor), then the
// values and rows written out.
template <class COMP>
__device__ void arg_extrema_cols(const float* in, int rows, int win, float* val, int* row)
{
    using Tup = cuda::std::tuple<float, int>;
    __shared__ float in_s[kRowsMax][kW];
    __shared__ alignas(8) unsigned char out_raw[kRowsMax * kW * sizeof(Tup)];
    Tup (*out_s)[kW] = reinterpret_cast<Tup (*)[kW]>(out_raw);
    const int ye = rows - win + 1;
    if (threadIdx.x >= kCols || rows > kRowsMax || win < 2 || win > 21 || ye < 1)
        return;
    load_tile(in, rows, in_s);
    const TU::cu::device::extrema_finder<TU::cu::device::extrema_position<COMP>, 23> find;
    find(in_s, out_s, win, ye);
    for (int y = 0; y < ye; ++y) {
        val[y * kCols + threadIdx.x] = cuda::std::get<0>(out_s[y][threadIdx.x]);
        row[y * kCols + threadIdx.x] = cuda::std::get<1>(out_s[y][threadIdx.x]);
    }
}

}  // namespace

// out[i] = device::convolve(in + i, lobe, L) for i + 2*(L & ~1) < n.
extern "C" __global__ void ref_fir_row(const float* in, int n, const float* lobe, int L, float* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (lobe_ok(L) && i + 2 * (L & ~1) < n)
        out[i] = tap_any(in + i, lobe, L);
}

// The same taps assigned to an unsigned char, as fir_filterV assigns them to
// u8 outputs (FIRFilter.h:207-231): the compiler's float -> u8 conversion.
extern "C" __global__ void ref_fir_row_u8(const float* in, int n, const float* lobe, int L,
                                          unsigned char* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (lobe_ok(L) && i + 2 * (L & ~1) < n)
        out[i] = tap_any(in + i, lobe, L);
}

// Window sums down the columns of a rows x 32 tile (row-major, 32 columns):
// out[y][x] for y < rows + 1 - win.  One block of 32 threads.
extern "C" __global__ void ref_box_cols_f32(const float* in, int rows, int win, float* out)
{
    box_cols<float>(in, rows, win, out);
}
extern "C" __global__ void ref_box_cols_i32(const int* in, int rows, int win, int* out)
{
    box_cols<int>(in, rows, win, out);
}

// Sliding minima / maxima down the columns of a rows x 32 tile.
extern "C" __global__ void ref_min_cols_f32(const float* in, int rows, int win, float* out)
{
    extrema_cols<LessF>(in, rows, win, out);
}
extern "C" __global__ void ref_max_cols_f32(const float* in, int rows, int win, float* out)
{
    extrema_cols<GreaterF>(in, rows, win, out);
}

// The same with the row of each extremum (blockIdx 0, so rows count from the
// tile's first row).
extern "C" __global__ void ref_argmin_cols_f32(const float* in, int rows, int win, float* val, int* row)
{
    arg_extrema_cols<LessF>(in, rows, win, val, row);
}
extern "C" __global__ void ref_argmax_cols_f32(const float* in, int rows, int win, float* val, int* row)
{
    arg_extrema_cols<GreaterF>(in, rows, win, val, row);
}
