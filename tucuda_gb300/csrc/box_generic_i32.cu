// box_generic_i32.cu -- plain box kernels for i32 input with the output dtype
// read at run time (box_plain.cuh).
#include "box_plain.cuh"

namespace tucu
{
namespace box
{

const void* generic_kernel_i32(bool vec, bool batch, int cpt)
{
    return generic_kernel_of<int32_t>(vec, batch, cpt);
}

}  // namespace box
}  // namespace tucu
