// box_typed.cu -- plain box kernels compiled for the common (input, output)
// type pairs, aligned input rows only (box_plain.cuh): u8 -> int32 sums,
// u8 -> u8 / f16 means, and every other type onto itself; 4 columns per
// lane (wide windows take the generic 8-column kernels).
#include "box_plain.cuh"

namespace tucu
{
namespace box
{

const void* typed_kernel(int in_dtype, int out_dtype, bool batch, int cpt, bool win)
{
    if (cpt != kCPT)
        return nullptr;
    auto pick = [&](auto tin, auto tout) -> const void* {
        using TIn = decltype(tin);
        using TOut = decltype(tout);
        if constexpr (sizeof(TIn) <= 2) {
            if (win)
                return batch ? (const void*)box_batch_kernel<TIn, true, TOut, kCPT, true>
                             : (const void*)box_kernel<TIn, true, TOut, kCPT, true>;
        } else {
            if (win)
                return nullptr;
        }
        return batch ? (const void*)box_batch_kernel<TIn, true, TOut> : (const void*)box_kernel<TIn, true, TOut>;
    };
    switch (in_dtype) {
    case U8:
        if (out_dtype == I32) return pick(uint8_t(), int32_t());
        if (out_dtype == U8) return pick(uint8_t(), uint8_t());
        if (out_dtype == F16) return pick(uint8_t(), __half());
        return nullptr;
    case I32: return out_dtype == I32 ? pick(int32_t(), int32_t()) : nullptr;
    case F16: return out_dtype == F16 ? pick(__half(), __half()) : nullptr;
    case BF16: return out_dtype == BF16 ? pick(__nv_bfloat16(), __nv_bfloat16()) : nullptr;
    case F32: return out_dtype == F32 ? pick(float(), float()) : nullptr;
    default: return nullptr;
    }
}

}  // namespace box
}  // namespace tucu
