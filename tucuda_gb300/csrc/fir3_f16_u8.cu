// fir3_f16_u8.cu -- warp-specialised FIR strips, __half in, uint8_t out (fir3_kernels.cuh).
#include "fir3_kernels.cuh"
TUCU_FIR3_INSTANTIATE(f16, __half, u8, uint8_t)
