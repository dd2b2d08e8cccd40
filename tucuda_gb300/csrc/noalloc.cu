// noalloc.cu -- a guided-filter entry point that allocates nothing.
//
// tucu_guided_convolve keeps its coefficient image (the scratch between the
// two window-sum passes) in device memory that the handle allocates with
// cudaMalloc on first use.  Some callers cannot allocate: applications whose
// memory manager owns every byte of the GPU and forbids cudaMalloc after
// start-up, or real-time loops that cannot afford the device-wide
// synchronisation cudaMalloc/cudaFree imply.  For them,
// tucu_guided_convolve_noalloc runs the same two kernels with the scratch in
// a file-scope device array of fixed size.  The array comes with the
// library's device code, which CUDA loads on a device at the first call that
// needs it (here: the first call of this entry point), and stays until the
// process exits.  It creates no handle and calls no allocating routine (no
// cudaMalloc, cudaFree or library allocator).
#include <cmath>
#include <cstring>
#include <mutex>

#include "box_kernels.h"
#include "tucu_internal.h"

namespace
{

// Largest coefficient image: (rows+1-wV) x (cols+1-wH) float2 values with rows
// padded to 16 bytes must fit in 16 MiB (2^21 float2, enough for a 1920x1080
// image at any window).
constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;

static __device__ __align__(256) float2 g_noalloc_coef[kNoAllocScratchBytes / sizeof(float2)];

// Device address of g_noalloc_coef per device, looked up once per device at
// its first call.  In host code the array's name is only a host-side
// stand-in; the address a kernel needs comes from cudaGetSymbolAddress with
// that device current.  The address is kept for the life of the process: a
// cudaDeviceReset between calls would leave it stale, which the header
// documents as unsupported.
std::mutex g_mu;
void* g_addr[64] = {nullptr};

int scratch_address(void** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return tucu::cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= 64)
        return tucu::fail(TUCU_ERR_ARG, "device index out of range");
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_coef);
        if (e != cudaSuccess || !p)
            return tucu::cuda_fail(e, "cudaGetSymbolAddress of the guided scratch");
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return TUCU_OK;
}

}  // namespace

extern "C" int tucu_guided_convolve_noalloc(int winV, int winH, float e, const void* in,
                                            size_t in_pitch, const void* guide,
                                            size_t guide_pitch, int rows, int cols,
                                            int in_dtype, void* out, size_t out_pitch,
                                            int out_dtype, int shift, void* stream)
{
    using namespace tucu;
    if (winV < 1 || winH < 1 || winV > TUCU_WIN_LIMIT || winH > TUCU_WIN_LIMIT)
        return fail(TUCU_ERR_WINDOW, "window size out of range");
    if (!std::isfinite(e))
        return fail(TUCU_ERR_ARG, "epsilon must be finite");
    if (!in || !out || rows < 0 || cols < 0)
        return fail(TUCU_ERR_ARG, "null image or negative size");
    if (in_dtype != U8 && in_dtype != F16 && in_dtype != BF16 && in_dtype != F32)
        return fail(TUCU_ERR_DTYPE, "guided input must be u8, f16, bf16 or f32");
    if (out_dtype < U8 || out_dtype > I32)
        return fail(TUCU_ERR_DTYPE, "unknown output dtype");
    const int es = dtype_size(in_dtype);
    if (rows > 0 && (in_pitch < (size_t)cols * es ||
                     (guide && guide_pitch < (size_t)cols * es) ||
                     out_pitch < (size_t)cols * dtype_size(out_dtype)))
        return fail(TUCU_ERR_ARG, "pitch smaller than a row");
    if (rows == 0 || rows < 2 * winV - 1 || cols < 2 * winH - 1)
        return TUCU_NOOP;
    const int cr = rows + 1 - winV, cc = cols + 1 - winH;
    const size_t cpitch = ((size_t)cc * sizeof(float2) + 15) / 16 * 16;
    if (cpitch * (size_t)cr > kNoAllocScratchBytes)
        return fail(TUCU_ERR_ARG,
                    "image too large for tucu_guided_convolve_noalloc: the coefficient image "
                    "(rows+1-winV) x (cols+1-winH) x 8 bytes must fit in 16 MiB; use "
                    "tucu_guided_convolve");
    void* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc != TUCU_OK)
        return rc;
    // Pass A writes every coefficient pass B reads, so nothing has to be cleared.
    box::GuidedLaunch L;
    std::memset(&L, 0, sizeof(L));
    L.src = in;
    L.src_pitch = in_pitch;
    L.guide = guide;
    L.guide_pitch = guide_pitch;
    L.rows = rows;
    L.cols = cols;
    L.in_dtype = in_dtype;
    L.wV = winV;
    L.wH = winH;
    L.e = e;
    L.coef = scratch;
    L.coef_pitch = cpitch;
    L.dst = out;
    L.dst_pitch = out_pitch;
    L.out_dtype = out_dtype;
    L.oy = shift ? winV - 1 : 0;
    L.ox = shift ? winH - 1 : 0;
    const cudaError_t ce = box::launch_guided(L, static_cast<cudaStream_t>(stream));
    return ce == cudaSuccess ? TUCU_OK : cuda_fail(ce, "guided launch (no-alloc)");
}
