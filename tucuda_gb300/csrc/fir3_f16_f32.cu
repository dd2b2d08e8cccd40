// fir3_f16_f32.cu -- warp-specialised FIR strips, __half in, float out (fir3_kernels.cuh).
#include "fir3_kernels.cuh"
TUCU_FIR3_INSTANTIATE(f16, __half, f32, float)
