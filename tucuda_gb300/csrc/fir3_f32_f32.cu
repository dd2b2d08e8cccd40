// fir3_f32_f32.cu -- warp-specialised FIR strips, float in, float out (fir3_kernels.cuh).
#include "fir3_kernels.cuh"
TUCU_FIR3_INSTANTIATE(f32, float, f32, float)
