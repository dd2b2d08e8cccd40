// fir3_f32_i32.cu -- warp-specialised FIR strips, float in, int32_t out (fir3_kernels.cuh).
#include "fir3_kernels.cuh"
TUCU_FIR3_INSTANTIATE(f32, float, i32, int32_t)
