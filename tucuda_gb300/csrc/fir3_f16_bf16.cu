// fir3_f16_bf16.cu -- warp-specialised FIR strips, __half in, __nv_bfloat16 out (fir3_kernels.cuh).
#include "fir3_kernels.cuh"
TUCU_FIR3_INSTANTIATE(f16, __half, bf16, __nv_bfloat16)
