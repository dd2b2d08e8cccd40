// extrema.h -- launcher of the sliding-window minimum / maximum kernel
// (extrema.cu), called by the C ABI in capi.cu.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace tucu
{
namespace ext
{

constexpr int kWinLimit = 64;  // largest window side the tile kernel takes

struct ExtremaLaunch
{
    const void* src;
    size_t src_pitch;
    int rows, cols;
    int dtype;       // input and value-output type
    int wV, wH;
    int is_max;      // 0: minimum, 1: maximum
    void* val;       // window extrema (input type), or nullptr
    size_t val_pitch;
    void* pos;       // int32 (x, y) input position of each extremum, or nullptr
    size_t pos_pitch;
    int oy, ox;      // placement of the valid region in the outputs
};

cudaError_t launch_extrema(const ExtremaLaunch& L, cudaStream_t stream);

}  // namespace ext
}  // namespace tucu
