// fir3_bf16_i32.cu -- warp-specialised FIR strips, __nv_bfloat16 in, int32_t out (fir3_kernels.cuh).
#include "fir3_kernels.cuh"
TUCU_FIR3_INSTANTIATE(bf16, __nv_bfloat16, i32, int32_t)
