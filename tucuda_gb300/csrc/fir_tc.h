// fir_tc.h -- host-side description of the tensor-core FIR / box kernel
// (fir_tc.cu): one job per image, one CTA per strip of 128 output columns
// x a band of rows (batch::Item).
#pragma once
#include <cuda.h>

#include "batch_types.h"

namespace tucu
{
namespace tcf
{

constexpr int kTW = 128;      // output columns per strip (the MMA's M)
constexpr int kCH = 32;       // output rows per V chunk (the V MMAs' N; H chunks are 64)
constexpr int kMaxTaps = 33;  // taps per direction
constexpr int kK1Max = 160;   // staged input columns: round_up(128 + taps - 1, 16)
constexpr int kK2Max = 64;    // input rows per 32 output rows: round_up(32 + taps - 1, 16)

// One image: out[oy + r][ox + c] = post * sum_{i<tv, j<th} cv[i] ch[j] in[r + i][c + j]
// for r < orows, c < ocols (the valid correlation, as FIRFilter2 and BoxFilter2).
struct TcJob
{
    CUtensorMap tmap;  // f16 input, boxes of 64 columns x 64 rows, 128-byte swizzle
    void* dst;
    size_t dst_pitch;
    int out_dtype;
    int orows, ocols, oy, ox;
    int th, tv;
    int split_h, split_v;  // some tap is not exact in f16: add the low-part products
    float post;
    float ch[kMaxTaps], cv[kMaxTaps];
    unsigned long long wait_ns;  // limit of every barrier wait (1 s outside tests)
    unsigned tx_pad;             // extra bytes each input stage expects (0 outside tests)
};

// Kernel for an output type (f16 or f32), arguments (const TcJob*, const
// batch::Item*), kThreads threads per CTA; nullptr when unsupported.
const void* kernel_for(int out_dtype);
constexpr int kThreads = 352;
size_t smem_bytes();

// Runs one job as a single launch (the job travels as a kernel parameter;
// row bands planned for two CTAs per SM); the caller filled it with fill_job.
cudaError_t launch_single(const TcJob& job, cudaStream_t stream);

// The full taps v[0 .. 2*LS] of a lobe of length L stored outermost first
// (LS = L & ~1): symmetric lobes (odd L) mirror, antisymmetric ones mirror with
// the sign flipped and have a zero centre tap (FIRFilter.h:66-176).  Returns
// the tap count 2*LS + 1.
int full_taps(const float* lobe, int L, float* taps);

// True when a job of these types and tap counts can run here.
bool eligible(int in_dtype, int out_dtype, int taps_h, int taps_v);

// Fills a job (wait limit and stage padding as set by tucu_debug_tc_wait);
// false when the input cannot be described by a TMA map
// (base not 16-byte aligned or pitch not a multiple of 16 bytes).
bool fill_job(TcJob* job, const void* src, size_t src_pitch, int rows, int cols, void* dst,
              size_t dst_pitch, int out_dtype, int oy, int ox, const float* taps_h, int th,
              const float* taps_v, int tv, float post);

}  // namespace tcf
}  // namespace tucu
