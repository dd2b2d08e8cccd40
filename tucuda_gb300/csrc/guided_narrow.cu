// guided_narrow.cu -- the guided passes with 4 columns per lane (windows up to 125 columns)
// (guided.cuh).
#include "guided.cuh"

namespace tucu
{
namespace box
{

cudaError_t launch_guided_narrow(const GuidedLaunch& L, cudaStream_t st) { return launch_guided_cpt<4>(L, st); }

}  // namespace box
}  // namespace tucu
