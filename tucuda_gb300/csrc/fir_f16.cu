// fir_f16.cu -- FIR strip kernels for __half input (see fir_kernels.cuh).
#include "fir_kernels.cuh"
TUCU_FIR_INSTANTIATE(f16, __half)
