// npp_gauss_time.cpp -- the timing reference of the reference's nppGauss test
// program (Testprog/nppGauss/main.cu:29-41 through TU/cu/npp.h:101-160):
// NPP's 15x15 Gaussian (nppiFilterGauss_8u_C1R with NPP_MASK_SIZE_15_X_15) on
// a rows x cols u8 image, over the valid region (the source pointer offset by
// the mask radius, as NPP reads outside the ROI), timed with CUDA events.
// Prints one JSON line.  NPP is a library timing reference only; its output
// is not compared (its coefficients are its own).
//   npp_gauss_time ROWS COLS REPS
#include <cuda_runtime.h>
#include <npp.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

int main(int argc, char** argv)
{
    const int rows = argc > 1 ? std::atoi(argv[1]) : 1080;
    const int cols = argc > 2 ? std::atoi(argv[2]) : 1920;
    const int reps = argc > 3 ? std::atoi(argv[3]) : 100;
    const int r = 7;  // 15 x 15 mask
    if (rows <= 2 * r || cols <= 2 * r || reps < 1) {
        std::fprintf(stderr, "bad size\n");
        return 2;
    }
    size_t pitch = 0, opitch = 0;
    Npp8u *in = nullptr, *out = nullptr;
    if (cudaMallocPitch((void**)&in, &pitch, cols, rows) != cudaSuccess ||
        cudaMallocPitch((void**)&out, &opitch, cols, rows) != cudaSuccess) {
        std::fprintf(stderr, "allocation failed\n");
        return 1;
    }
    std::vector<Npp8u> host((size_t)rows * cols);
    for (size_t i = 0; i < host.size(); ++i)
        host[i] = (Npp8u)((i * 2654435761u >> 11) % 256u);
    cudaMemcpy2D(in, pitch, host.data(), cols, cols, rows, cudaMemcpyHostToDevice);
    cudaStream_t st;
    cudaStreamCreate(&st);
    NppStreamContext ctx = {};
    cudaDeviceProp prop;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaGetDeviceProperties(&prop, dev);
    ctx.hStream = st;
    ctx.nCudaDeviceId = dev;
    ctx.nMultiProcessorCount = prop.multiProcessorCount;
    ctx.nMaxThreadsPerMultiProcessor = prop.maxThreadsPerMultiProcessor;
    ctx.nMaxThreadsPerBlock = prop.maxThreadsPerBlock;
    ctx.nSharedMemPerBlock = prop.sharedMemPerBlock;
    cudaDeviceGetAttribute(&ctx.nCudaDevAttrComputeCapabilityMajor, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&ctx.nCudaDevAttrComputeCapabilityMinor, cudaDevAttrComputeCapabilityMinor, dev);
    cudaStreamGetFlags(st, &ctx.nStreamFlags);
    const NppiSize roi = {cols - 2 * r, rows - 2 * r};
    const Npp8u* src = in + (size_t)r * pitch + r;
    Npp8u* dst = out + (size_t)r * opitch + r;
    auto run = [&] {
        return nppiFilterGauss_8u_C1R_Ctx(src, (int)pitch, dst, (int)opitch, roi, NPP_MASK_SIZE_15_X_15, ctx);
    };
    for (int i = 0; i < 3; ++i)
        if (run() != NPP_SUCCESS) {
            std::fprintf(stderr, "nppiFilterGauss failed\n");
            return 1;
        }
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, st);
    for (int i = 0; i < reps; ++i)
        run();
    cudaEventRecord(b, st);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    ms /= reps;
    const cudaError_t e = cudaGetLastError();
    std::printf("{\"npp\": \"nppiFilterGauss_8u_C1R 15x15\", \"rows\": %d, \"cols\": %d, \"ms\": %.5f, "
                "\"gpix_per_s\": %.3f, \"cuda\": \"%s\"}\n",
                rows, cols, ms, (double)rows * cols / (ms * 1e-3) / 1e9, cudaGetErrorString(e));
    return e == cudaSuccess ? 0 : 1;
}
