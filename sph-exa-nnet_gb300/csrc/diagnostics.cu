// Diagnostics of the C ABI: solver operation counts for roofline accounting, and a
// measurement of the device's FP64 fused-multiply-add throughput (the pipe the burn
// kernels are bound by on GB300, whose FP64 rate is a small fraction of its FP32 rate).
#include <cuda_runtime.h>

#include "../../include/nnet_gb300.h"

namespace
{
// 8 independent FMA chains per thread keep the FP64 pipe fed; values stay finite.
__global__ void fp64FmaProbe(double* out, int iters)
{
    double a[8];
    for (int k = 0; k < 8; ++k)
        a[k] = 1.0 + 1e-3 * (threadIdx.x + k);
    const double m = 0.999999, c = 1e-7;
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int k = 0; k < 8; ++k)
            a[k] = fma(a[k], m, c);
    double s = 0;
    for (int k = 0; k < 8; ++k)
        s += a[k];
    if (s == 12345.0) out[0] = s; // never true; keeps the chains live
}
} // namespace

extern "C" int nnet_measure_fp64_peak(int device, double* tflops)
{
    if (!tflops) return NNET_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return NNET_ERR_CUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return NNET_ERR_CUDA;
    const int   threads = 256, blocks = sms * 8, iters = 4096;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0), cudaEventCreate(&e1);
    fp64FmaProbe<<<blocks, threads>>>(out, 64); // warm-up
    cudaEventRecord(e0);
    fp64FmaProbe<<<blocks, threads>>>(out, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0), cudaEventDestroy(e1);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess || ms <= 0) return NNET_ERR_CUDA;
    *tflops = 2.0 * 8.0 * iters * (double)threads * blocks / (ms * 1e-3) / 1e12;
    return NNET_SUCCESS;
}
