// fir3_bf16_u8.cu -- warp-specialised FIR strips, __nv_bfloat16 in, uint8_t out (fir3_kernels.cuh).
#include "fir3_kernels.cuh"
TUCU_FIR3_INSTANTIATE(bf16, __nv_bfloat16, u8, uint8_t)
