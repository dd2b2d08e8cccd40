// fir3_bf16_f16.cu -- warp-specialised FIR strips, __nv_bfloat16 in, __half out (fir3_kernels.cuh).
#include "fir3_kernels.cuh"
TUCU_FIR3_INSTANTIATE(bf16, __nv_bfloat16, f16, __half)
