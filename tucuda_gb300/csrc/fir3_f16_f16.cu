// fir3_f16_f16.cu -- warp-specialised FIR strips, __half in, __half out (fir3_kernels.cuh).
#include "fir3_kernels.cuh"
TUCU_FIR3_INSTANTIATE(f16, __half, f16, __half)
