// fir_bf16.cu -- FIR strip kernels for __nv_bfloat16 input (see fir_kernels.cuh).
#include "fir_kernels.cuh"
TUCU_FIR_INSTANTIATE(bf16, __nv_bfloat16)
