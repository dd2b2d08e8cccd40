// guided_wide.cu -- the guided passes with 8 columns per lane (windows wider than 125 columns)
// (guided.cuh).
#include "guided.cuh"

namespace tucu
{
namespace box
{

cudaError_t launch_guided_wide(const GuidedLaunch& L, cudaStream_t st) { return launch_guided_cpt<8>(L, st); }

}  // namespace box
}  // namespace tucu
