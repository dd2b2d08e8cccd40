// fir3_bf16_f32.cu -- warp-specialised FIR strips, __nv_bfloat16 in, float out (fir3_kernels.cuh).
#include "fir3_kernels.cuh"
TUCU_FIR3_INSTANTIATE(bf16, __nv_bfloat16, f32, float)
