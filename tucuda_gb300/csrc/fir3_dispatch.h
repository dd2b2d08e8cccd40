// fir3_dispatch.h -- lookup of the warp-specialised FIR launchers by
// (input type, output type); the launchers live in fir3_<in>_<out>.cu.
#pragma once
#include "fir_strip.cuh"

namespace tucu
{
namespace fir
{
cudaError_t launch3_u8_u8(const FirLaunch& L, cudaStream_t stream);
const void* batch3_u8_u8(int r, size_t* smem);
cudaError_t launch3_u8_f16(const FirLaunch& L, cudaStream_t stream);
const void* batch3_u8_f16(int r, size_t* smem);
cudaError_t launch3_u8_bf16(const FirLaunch& L, cudaStream_t stream);
const void* batch3_u8_bf16(int r, size_t* smem);
cudaError_t launch3_u8_f32(const FirLaunch& L, cudaStream_t stream);
const void* batch3_u8_f32(int r, size_t* smem);
cudaError_t launch3_u8_i32(const FirLaunch& L, cudaStream_t stream);
const void* batch3_u8_i32(int r, size_t* smem);
cudaError_t launch3_f16_u8(const FirLaunch& L, cudaStream_t stream);
const void* batch3_f16_u8(int r, size_t* smem);
cudaError_t launch3_f16_f16(const FirLaunch& L, cudaStream_t stream);
const void* batch3_f16_f16(int r, size_t* smem);
cudaError_t launch3_f16_bf16(const FirLaunch& L, cudaStream_t stream);
const void* batch3_f16_bf16(int r, size_t* smem);
cudaError_t launch3_f16_f32(const FirLaunch& L, cudaStream_t stream);
const void* batch3_f16_f32(int r, size_t* smem);
cudaError_t launch3_f16_i32(const FirLaunch& L, cudaStream_t stream);
const void* batch3_f16_i32(int r, size_t* smem);
cudaError_t launch3_bf16_u8(const FirLaunch& L, cudaStream_t stream);
const void* batch3_bf16_u8(int r, size_t* smem);
cudaError_t launch3_bf16_f16(const FirLaunch& L, cudaStream_t stream);
const void* batch3_bf16_f16(int r, size_t* smem);
cudaError_t launch3_bf16_bf16(const FirLaunch& L, cudaStream_t stream);
const void* batch3_bf16_bf16(int r, size_t* smem);
cudaError_t launch3_bf16_f32(const FirLaunch& L, cudaStream_t stream);
const void* batch3_bf16_f32(int r, size_t* smem);
cudaError_t launch3_bf16_i32(const FirLaunch& L, cudaStream_t stream);
const void* batch3_bf16_i32(int r, size_t* smem);
cudaError_t launch3_f32_u8(const FirLaunch& L, cudaStream_t stream);
const void* batch3_f32_u8(int r, size_t* smem);
cudaError_t launch3_f32_f16(const FirLaunch& L, cudaStream_t stream);
const void* batch3_f32_f16(int r, size_t* smem);
cudaError_t launch3_f32_bf16(const FirLaunch& L, cudaStream_t stream);
const void* batch3_f32_bf16(int r, size_t* smem);
cudaError_t launch3_f32_f32(const FirLaunch& L, cudaStream_t stream);
const void* batch3_f32_f32(int r, size_t* smem);
cudaError_t launch3_f32_i32(const FirLaunch& L, cudaStream_t stream);
const void* batch3_f32_i32(int r, size_t* smem);

typedef cudaError_t (*Launch3Fn)(const FirLaunch&, cudaStream_t);
typedef const void* (*Batch3Fn)(int, size_t*);

// Index of an input type (u8, f16, bf16, f32) and of an output type
// (u8, f16, bf16, f32, i32) in the tables; -1 if unsupported.
inline int in_index(int dt) { return dt == U8 ? 0 : dt == F16 ? 1 : dt == BF16 ? 2 : dt == F32 ? 3 : -1; }
inline int out_index(int dt) { return dt >= U8 && dt <= I32 ? dt : -1; }

inline Launch3Fn launch3_fn(int in_dt, int out_dt)
{
    static const Launch3Fn t[4][5] = {
        {launch3_u8_u8, launch3_u8_f16, launch3_u8_bf16, launch3_u8_f32, launch3_u8_i32},
        {launch3_f16_u8, launch3_f16_f16, launch3_f16_bf16, launch3_f16_f32, launch3_f16_i32},
        {launch3_bf16_u8, launch3_bf16_f16, launch3_bf16_bf16, launch3_bf16_f32, launch3_bf16_i32},
        {launch3_f32_u8, launch3_f32_f16, launch3_f32_bf16, launch3_f32_f32, launch3_f32_i32},
    };
    const int i = in_index(in_dt), o = out_index(out_dt);
    return i < 0 || o < 0 ? nullptr : t[i][o];
}

inline Batch3Fn batch3_fn(int in_dt, int out_dt)
{
    static const Batch3Fn t[4][5] = {
        {batch3_u8_u8, batch3_u8_f16, batch3_u8_bf16, batch3_u8_f32, batch3_u8_i32},
        {batch3_f16_u8, batch3_f16_f16, batch3_f16_bf16, batch3_f16_f32, batch3_f16_i32},
        {batch3_bf16_u8, batch3_bf16_f16, batch3_bf16_bf16, batch3_bf16_f32, batch3_bf16_i32},
        {batch3_f32_u8, batch3_f32_f16, batch3_f32_bf16, batch3_f32_f32, batch3_f32_i32},
    };
    const int i = in_index(in_dt), o = out_index(out_dt);
    return i < 0 || o < 0 ? nullptr : t[i][o];
}

}  // namespace fir
}  // namespace tucu

int tucu_fir3_u8_u8_tu_error(bool clear);
int tucu_fir3_u8_f16_tu_error(bool clear);
int tucu_fir3_u8_bf16_tu_error(bool clear);
int tucu_fir3_u8_f32_tu_error(bool clear);
int tucu_fir3_u8_i32_tu_error(bool clear);
int tucu_fir3_f16_u8_tu_error(bool clear);
int tucu_fir3_f16_f16_tu_error(bool clear);
int tucu_fir3_f16_bf16_tu_error(bool clear);
int tucu_fir3_f16_f32_tu_error(bool clear);
int tucu_fir3_f16_i32_tu_error(bool clear);
int tucu_fir3_bf16_u8_tu_error(bool clear);
int tucu_fir3_bf16_f16_tu_error(bool clear);
int tucu_fir3_bf16_bf16_tu_error(bool clear);
int tucu_fir3_bf16_f32_tu_error(bool clear);
int tucu_fir3_bf16_i32_tu_error(bool clear);
int tucu_fir3_f32_u8_tu_error(bool clear);
int tucu_fir3_f32_f16_tu_error(bool clear);
int tucu_fir3_f32_bf16_tu_error(bool clear);
int tucu_fir3_f32_f32_tu_error(bool clear);
int tucu_fir3_f32_i32_tu_error(bool clear);
