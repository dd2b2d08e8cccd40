// fir_u8.cu -- FIR strip kernels for uint8_t input (see fir_kernels.cuh).
#include "fir_kernels.cuh"
TUCU_FIR_INSTANTIATE(u8, uint8_t)
