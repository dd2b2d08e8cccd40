// box_generic_bf16.cu -- plain box kernels for bf16 input with the output dtype
// read at run time (box_plain.cuh).
#include "box_plain.cuh"

namespace tucu
{
namespace box
{

const void* generic_kernel_bf16(bool vec, bool batch, int cpt)
{
    return generic_kernel_of<__nv_bfloat16>(vec, batch, cpt);
}

}  // namespace box
}  // namespace tucu
