// box_stereo_wide.cu -- the stereo cost kernel at 8 columns per lane, for
// windows wider than 125 columns (stereo.cuh).
#include "stereo.cuh"

namespace tucu
{
namespace box
{

cudaError_t launch_stereo_wide(const Geo& G, const StereoArgs& A, int dtype, bool vec, long grid,
                               cudaStream_t st)
{
    return launch_stereo_cpt<8>(G, A, dtype, vec, grid, st);
}

}  // namespace box
}  // namespace tucu
