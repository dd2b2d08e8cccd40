// fir_f32.cu -- FIR strip kernels for float input (see fir_kernels.cuh).
#include "fir_kernels.cuh"
TUCU_FIR_INSTANTIATE(f32, float)
