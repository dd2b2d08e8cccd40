// fir3_u8_f32.cu -- warp-specialised FIR strips, uint8_t in, float out (fir3_kernels.cuh).
#include "fir3_kernels.cuh"
TUCU_FIR3_INSTANTIATE(u8, uint8_t, f32, float)
