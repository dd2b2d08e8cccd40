// box_generic_u8.cu -- plain box kernels for u8 input with the output dtype
// read at run time (box_plain.cuh).
#include "box_plain.cuh"

namespace tucu
{
namespace box
{

const void* generic_kernel_u8(bool vec, bool batch, int cpt)
{
    return generic_kernel_of<uint8_t>(vec, batch, cpt);
}

}  // namespace box
}  // namespace tucu
