// box_kernels.h -- host-side launch descriptions of the box and guided
// kernels (box_kernels.cu).
#pragma once
#include <type_traits>

#include "tucu_common.cuh"
#include "tucu_internal.h"

namespace tucu
{
namespace box
{

struct BoxLaunch
{
    const void* src;
    size_t src_pitch;
    int rows, cols, in_dtype;
    int wV, wH;
    void* dst;
    size_t dst_pitch;
    int out_dtype;
    int oy, ox;       // placement of the valid region
    int normalize;    // window means instead of sums
    int strip_rows;   // <= 0 picks a default
};

struct GuidedLaunch
{
    const void* src;
    size_t src_pitch;
    const void* guide;  // nullptr = self-guided
    size_t guide_pitch;
    int rows, cols, in_dtype;
    int wV, wH;
    float e;            // squared inside, as in the reference
    void* coef;         // scratch: (rows+1-wV) x (cols+1-wH) float2
    size_t coef_pitch;
    void* dst;
    size_t dst_pitch;
    int out_dtype;
    int oy, ox;
    int strip_rows;
};

// Stereo cost aggregation (box_stereo.cu): costs[d][y][x] for d < ndisp.
struct StereoLaunch
{
    const void* left;
    size_t left_pitch;
    const void* right;
    size_t right_pitch;
    int rows, cols, dtype;
    int wV, wH;
    float thresh;
    int ndisp;
    void* costs;
    size_t cost_pitch, slice_pitch;
    int cost_dtype;
};

// Box sums of N-channel float pixels (box_vec.cu).
struct VecLaunch
{
    const void* src;  // rows of cols x channels float32, 16-byte aligned rows
    size_t src_pitch;
    int rows, cols, channels;
    int wV, wH;
    void* dst;
    size_t dst_pitch;
    int oy, ox;
    int normalize;
};

cudaError_t launch_box(const BoxLaunch& L, cudaStream_t st);
cudaError_t launch_vec(const VecLaunch& L, cudaStream_t st);
cudaError_t launch_stereo(const StereoLaunch& L, cudaStream_t st);
cudaError_t launch_guided(const GuidedLaunch& L, cudaStream_t st);
// The guided passes at 4 and at 8 columns per lane (guided_narrow.cu,
// guided_wide.cu); launch_guided picks by the window width.
cudaError_t launch_guided_narrow(const GuidedLaunch& L, cudaStream_t st);
cudaError_t launch_guided_wide(const GuidedLaunch& L, cudaStream_t st);

}  // namespace box
}  // namespace tucu
