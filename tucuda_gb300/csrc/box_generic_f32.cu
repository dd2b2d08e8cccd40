// box_generic_f32.cu -- plain box kernels for f32 input with the output dtype
// read at run time (box_plain.cuh).
#include "box_plain.cuh"

namespace tucu
{
namespace box
{

const void* generic_kernel_f32(bool vec, bool batch, int cpt)
{
    return generic_kernel_of<float>(vec, batch, cpt);
}

}  // namespace box
}  // namespace tucu
