// peak.cu -- the FP64 pipe's issue rate on this GPU, measured, for the FP64
// form's roofline: a grid of warps that each run independent chains of fused
// multiply-adds (no memory traffic), timed with CUDA events.
#include <cuda_runtime.h>

#include "solver2d.h"

namespace hydro {

// 8 independent chains per thread, `iters` rounds of 8 dependent-chain steps:
// 64 DFMA per thread per round.  The result is written so nothing is dropped.
static __global__ void k_dfma_loop(double* out, int iters, double a, double b)
{
    double x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k)
        x[k] = threadIdx.x * 1e-3 + k;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int k = 0; k < 8; ++k)
                x[k] = fma(x[k], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        s += x[k];
    if (s == 1234.5678)  // never true for these inputs; keeps the chains live
        out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace hydro

extern "C" int hydro_fp64_peak(double* dfma_per_s)
{
    using namespace hydro;
    int dev = 0, sms = 0;
    if (!cuda_ok(cudaGetDevice(&dev), "device") ||
        !cuda_ok(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count"))
        return -1;
    double* out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (!cuda_ok(cudaMalloc(&out, sizeof(double) * 256 * 8 * (size_t)sms), "peak buffer") ||
        !cuda_ok(cudaEventCreate(&e0), "event") || !cuda_ok(cudaEventCreate(&e1), "event")) {
        cudaFree(out);
        return -1;
    }
    const int blocks = 8 * sms, threads = 256, iters = 2000;
    k_dfma_loop<<<blocks, threads>>>(out, 200, 0.999999, 1e-7);  // warm-up
    cudaEventRecord(e0);
    k_dfma_loop<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    count_launch(2);
    const bool ok = cuda_ok(cudaEventSynchronize(e1), "peak run");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (!ok || ms <= 0.f)
        return -1;
    *dfma_per_s = (double)blocks * threads * iters * 64.0 / (ms * 1e-3);
    return 0;
}
