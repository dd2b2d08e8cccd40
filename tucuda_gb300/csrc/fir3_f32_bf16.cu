// fir3_f32_bf16.cu -- warp-specialised FIR strips, float in, __nv_bfloat16 out (fir3_kernels.cuh).
#include "fir3_kernels.cuh"
TUCU_FIR3_INSTANTIATE(f32, float, bf16, __nv_bfloat16)
