// FP32 throughput probe: the denominator for the Biot-Savart roofline.
//
// The sweep kernels run on the FP32 pipes (not tensor cores), so their roofline is the
// FP32 FMA rate of this GPU at its current clocks. Each thread advances 8 independent FMA
// chains; the grid covers every SM with several CTAs. FLOPs = 2 per FMA.
#include <cuda_runtime.h>

#include "sb_kernels.h"

namespace sbgpu {

__global__ void __launch_bounds__(256) k_fma_probe(float* out, int iters, float a, float b) {
    float x0 = threadIdx.x * 1e-7f, x1 = x0 + 1e-3f, x2 = x0 + 2e-3f, x3 = x0 + 3e-3f;
    float x4 = x0 + 4e-3f, x5 = x0 + 5e-3f, x6 = x0 + 6e-3f, x7 = x0 + 7e-3f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
            x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
        }
    }
    float s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == 12345.678f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

// Returns FP32 TFLOP/s (best of `reps` launches) or a negative value on error.
double measure_fp32_peak(int device, int reps) {
    if (cudaSetDevice(device) != cudaSuccess) return -1.0;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = sms * 8, threads = 256, iters = 4096;
    float* out = nullptr;
    if (cudaMalloc(&out, static_cast<size_t>(blocks) * threads * sizeof(float)) != cudaSuccess) return -1.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 0.0;
    k_fma_probe<<<blocks, threads>>>(out, iters / 8, 0.9999f, 1e-4f);  // warm-up
    for (int r = 0; r < reps; ++r) {
        cudaEventRecord(e0);
        k_fma_probe<<<blocks, threads>>>(out, iters, 0.9999f, 1e-4f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        double flops = 2.0 * 8.0 * 16.0 * iters * static_cast<double>(blocks) * threads;
        if (ms > 0.f) best = fmax(best, flops / (ms * 1e-3) / 1e12);
    }
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    return err == cudaSuccess ? best : -1.0;
}

}  // namespace sbgpu
