// stereo_select.h -- host-side launch description of the disparity selection
// kernel (stereo_select.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace tucu
{
namespace sel
{

struct SelectLaunch
{
    const void* costs;  // C[d][y][x]: cost_pitch between rows, slice_pitch between slices
    size_t cost_pitch, slice_pitch;
    int rows, cols;     // the region of each slice that is selected over
    int cost_dtype;     // TUCU_I32 or TUCU_F32
    int disparities;    // D, 1..256
    int disparity_max, inconsistency;
    void* out;          // out[oy + y][ox + x]
    size_t out_pitch;
    int out_dtype;
    int oy, ox;
};

cudaError_t launch_select(const SelectLaunch& L, cudaStream_t st);

}  // namespace sel
}  // namespace tucu
