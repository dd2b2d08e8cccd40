// fir3_f32_u8.cu -- warp-specialised FIR strips, float in, uint8_t out (fir3_kernels.cuh).
#include "fir3_kernels.cuh"
TUCU_FIR3_INSTANTIATE(f32, float, u8, uint8_t)
