// box_generic_f16.cu -- plain box kernels for f16 input with the output dtype
// read at run time (box_plain.cuh).
#include "box_plain.cuh"

namespace tucu
{
namespace box
{

const void* generic_kernel_f16(bool vec, bool batch, int cpt)
{
    return generic_kernel_of<__half>(vec, batch, cpt);
}

}  // namespace box
}  // namespace tucu
