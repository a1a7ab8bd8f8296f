// diag.cu -- throughput probes used to state roofline denominators.
//
// hlanc_diag_fp64_tflops: dense FP64 FMA throughput of the device (eight
// independent FMA chains per thread, 8 CTAs of 256 threads per SM).  An
// all-FP64 CGS kernel issues one FP64 FMA per 8-byte element, so on GB300
// its ceiling is min(HBM bandwidth, this rate x 8 bytes / 2 flops); the
// hybrid kernels put part of the columns on the integer pipes to pass it.
// (hlanc_diag_cgs, the CGS kernels alone, lives in engine.cu beside the
// engine it sets up.)
#include <cuda_runtime.h>

#include "internal.cuh"

namespace {
__global__ void k_dfma_probe(double *out, int iters, double a, double b) {
    double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
}  // namespace

extern "C" int hlanc_diag_fp64_tflops(int dev, double *tflops) {
    if (!tflops) return HLANC_ERR_INVALID;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(dev);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8, threads = 256, iters = 4096;
    double *out = nullptr;
    cudaEvent_t e0, e1;
    if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) { cudaSetDevice(prev); return HLANC_ERR_CUDA; }
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        k_dfma_probe<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    hlanc::launch_counter() += 4;
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    cudaSetDevice(prev);
    if (e != cudaSuccess) return HLANC_ERR_CUDA;
    *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
    return HLANC_OK;
}
