// fir3_bf16_bf16.cu -- warp-specialised FIR strips, __nv_bfloat16 in, __nv_bfloat16 out (fir3_kernels.cuh).
#include "fir3_kernels.cuh"
TUCU_FIR3_INSTANTIATE(bf16, __nv_bfloat16, bf16, __nv_bfloat16)
