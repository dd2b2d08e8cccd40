// fir3_u8_bf16.cu -- warp-specialised FIR strips, uint8_t in, __nv_bfloat16 out (fir3_kernels.cuh).
#include "fir3_kernels.cuh"
TUCU_FIR3_INSTANTIATE(u8, uint8_t, bf16, __nv_bfloat16)
