// fir3_u8_i32.cu -- warp-specialised FIR strips, uint8_t in, int32_t out (fir3_kernels.cuh).
#include "fir3_kernels.cuh"
TUCU_FIR3_INSTANTIATE(u8, uint8_t, i32, int32_t)
