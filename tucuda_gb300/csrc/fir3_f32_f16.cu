// fir3_f32_f16.cu -- warp-specialised FIR strips, float in, __half out (fir3_kernels.cuh).
#include "fir3_kernels.cuh"
TUCU_FIR3_INSTANTIATE(f32, float, f16, __half)
