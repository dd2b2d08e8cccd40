// fir3_u8_u8.cu -- warp-specialised FIR strips, uint8_t in, uint8_t out (fir3_kernels.cuh).
#include "fir3_kernels.cuh"
TUCU_FIR3_INSTANTIATE(u8, uint8_t, u8, uint8_t)
