// tucu_common.cuh -- shared device/host definitions for the sm_103a kernels of
// the TUCuda 2D-filter path: pixel types, load/store conversions, the image
// view the kernels take, and the bounded-wait error flag.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "tucu_gb300.h"

namespace tucu
{

// Pixel storage types (the values of tucu_dtype).
enum Dtype : int { U8 = TUCU_U8, F16 = TUCU_F16, BF16 = TUCU_BF16, F32 = TUCU_F32, I32 = TUCU_I32 };

inline __host__ __device__ int dtype_size(int dt)
{
    return dt == U8 ? 1 : (dt == F16 || dt == BF16) ? 2 : 4;
}

// A pitched 2D image in device memory (pitch in bytes).
struct Image
{
    const void* data;
    size_t pitch;
    int rows, cols;
    int dtype;
};

struct OutImage
{
    void* data;
    size_t pitch;
    int dtype;
};

template <class T> struct PixelOf;
template <> struct PixelOf<uint8_t> { static constexpr int dt = U8; };
template <> struct PixelOf<__half> { static constexpr int dt = F16; };
template <> struct PixelOf<__nv_bfloat16> { static constexpr int dt = BF16; };
template <> struct PixelOf<float> { static constexpr int dt = F32; };
template <> struct PixelOf<int32_t> { static constexpr int dt = I32; };

__device__ __forceinline__ float to_float(uint8_t v) { return (float)v; }
__device__ __forceinline__ float to_float(__half v) { return __half2float(v); }
__device__ __forceinline__ float to_float(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ float to_float(float v) { return v; }
__device__ __forceinline__ float to_float(int32_t v) { return (float)v; }

// float -> u8 as the reference's implicit float-to-u_char assignment runs on
// this GPU (measured with its own device code, nvcc 13.0, sm_103a): truncation
// toward zero, saturation to the unsigned 32-bit range (negative values and
// NaN give 0), then the low byte, so values from 256 on wrap modulo 256.
__device__ __forceinline__ uint8_t f2u8(float v)
{
    return (uint8_t)__float2uint_rz(v);
}

// Integer window sums -> u8 as the reference's default convolver stores them
// (float sums, then the float-to-u_char assignment of f2u8): negative sums
// give 0, the others their low byte (the sums here are exact integers).
__device__ __forceinline__ uint8_t sum2u8(int s)
{
    return s < 0 ? (uint8_t)0 : (uint8_t)s;
}

// Stores one float result into an output row in the output's dtype.
__device__ __forceinline__ void store_px(void* row, int x, int dt, float v)
{
    switch (dt) {
    case U8: static_cast<uint8_t*>(row)[x] = f2u8(v); break;
    case F16: static_cast<__half*>(row)[x] = __float2half_rn(v); break;
    case BF16: static_cast<__nv_bfloat16*>(row)[x] = __float2bfloat16_rn(v); break;
    case I32: static_cast<int32_t*>(row)[x] = __float2int_rz(v); break;
    default: static_cast<float*>(row)[x] = v; break;
    }
}

// Stores two horizontally adjacent results (x even-aligned when possible).
__device__ __forceinline__ void store_px2(void* row, int x, int dt, float a, float b, bool both)
{
    if (!both) {
        store_px(row, x, dt, a);
        return;
    }
    const uintptr_t addr = reinterpret_cast<uintptr_t>(row) + (uintptr_t)x * dtype_size(dt);
    switch (dt) {
    case U8:
        if ((addr & 1) == 0) {
            const uint16_t v = (uint16_t)f2u8(a) | ((uint16_t)f2u8(b) << 8);
            *reinterpret_cast<uint16_t*>(addr) = v;
            return;
        }
        break;
    case F16:
        if ((addr & 3) == 0) {
            *reinterpret_cast<__half2*>(addr) = __floats2half2_rn(a, b);
            return;
        }
        break;
    case BF16:
        if ((addr & 3) == 0) {
            *reinterpret_cast<__nv_bfloat162*>(addr) = __floats2bfloat162_rn(a, b);
            return;
        }
        break;
    case F32:
        if ((addr & 7) == 0) {
            *reinterpret_cast<float2*>(addr) = make_float2(a, b);
            return;
        }
        break;
    default: break;
    }
    store_px(row, x, dt, a);
    store_px(row, x + 1, dt, b);
}

__device__ __forceinline__ void store_i32(void* row, int x, int dt, int32_t v)
{
    switch (dt) {
    case I32: static_cast<int32_t*>(row)[x] = v; break;
    case U8: static_cast<uint8_t*>(row)[x] = (uint8_t)v; break;  // C++ int -> u_char: the low byte
    default: store_px(row, x, dt, (float)v); break;
    }
}

template <class T>
__device__ __forceinline__ float load_px(const void* row, int x)
{
    return to_float(static_cast<const T*>(row)[x]);
}

__device__ __forceinline__ const char* row_ptr(const void* base, size_t pitch, int y)
{
    return static_cast<const char*>(base) + (size_t)y * pitch;
}
__device__ __forceinline__ char* row_ptr(void* base, size_t pitch, int y)
{
    return static_cast<char*>(base) + (size_t)y * pitch;
}

// Device-side error word, set by a kernel whose bounded wait ran out.  Each
// translation unit has its own copy (no relocatable device code);
// TUCU_DEFINE_ERROR_ACCESSOR gives each one a host reader, and
// tucu_device_error() polls all of them.
static __device__ int g_tucu_device_error;

constexpr int kErrWaitTimeout = 1;  // an mbarrier wait gave up
constexpr int kErrRange = 2;        // a tensor-core intermediate left the f16 range
constexpr int kErrAlign = 3;        // shared memory not aligned as a kernel needs (nothing done)

__device__ __forceinline__ void raise_device_error(int code)
{
    atomicCAS(&g_tucu_device_error, 0, code);
}

}  // namespace tucu

#define TUCU_DEFINE_ERROR_ACCESSOR(fn)                                              \
    int fn(bool clear)                                                              \
    {                                                                               \
        int v = 0;                                                                  \
        if (cudaMemcpyFromSymbol(&v, tucu::g_tucu_device_error, sizeof(int)) !=     \
            cudaSuccess)                                                            \
            return -1;                                                              \
        if (clear && v) {                                                           \
            const int z = 0;                                                        \
            cudaMemcpyToSymbol(tucu::g_tucu_device_error, &z, sizeof(int));          \
        }                                                                           \
        return v;                                                                   \
    }
