// fir3_f16_i32.cu -- warp-specialised FIR strips, __half in, int32_t out (fir3_kernels.cuh).
#include "fir3_kernels.cuh"
TUCU_FIR3_INSTANTIATE(f16, __half, i32, int32_t)
