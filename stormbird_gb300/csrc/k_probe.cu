// FP32 / FP64 throughput probes: the denominators for the Biot-Savart roofline.
//
// The sweep kernels run on the FP32 pipes (not tensor cores), so their roofline is the
// FP32 FMA rate of this GPU at its current clocks; the FP64 sweep of the precision study is
// set against the FP64 FMA rate. Each thread advances 8 independent FMA chains; the grid
// covers every SM with several CTAs. FLOPs = 2 per FMA.
#include <cuda_runtime.h>

#include "sb_kernels.h"
#include "sb_ptx.cuh"

namespace sbgpu {

template <class T>
__global__ void __launch_bounds__(256) k_fma_probe(T* out, int iters, T a, T b) {
    T x0 = threadIdx.x * T(1e-7), x1 = x0 + T(1e-3), x2 = x0 + T(2e-3), x3 = x0 + T(3e-3);
    T x4 = x0 + T(4e-3), x5 = x0 + T(5e-3), x6 = x0 + T(6e-3), x7 = x0 + T(7e-3);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
            x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
        }
    }
    T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == T(12345.678)) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

// Returns TFLOP/s of type T (best of `reps` launches) or a negative value on error.
template <class T>
static double measure_peak(int device, int reps, int iters) {
    if (cudaSetDevice(device) != cudaSuccess) return -1.0;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = sms * 8, threads = 256;
    T* out = nullptr;
    if (cudaMalloc(&out, static_cast<size_t>(blocks) * threads * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();  // leave no error behind for later launch checks
        return -1.0;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 0.0;
    k_fma_probe<T><<<blocks, threads>>>(out, iters / 8, T(0.9999), T(1e-4));  // warm-up
    for (int r = 0; r < reps; ++r) {
        cudaEventRecord(e0);
        k_fma_probe<T><<<blocks, threads>>>(out, iters, T(0.9999), T(1e-4));
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

// Failure path of the bounded waits: thread 0 arms an mbarrier for 16 bytes of a copy that is
// never issued, so its phase cannot complete; every thread's bounded wait runs out after
// `polls` polls and records kDevTimeout, and the kernel returns. Nothing is in flight into
// shared memory when the CTA exits.
__global__ void __launch_bounds__(128) k_wait_probe(int polls, int* err) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
        mbar_expect_tx(&bar, 16);  // the single arrival, with 16 bytes still expected
    }
    __syncthreads();
    mbar_wait_bounded(&bar, 0, err, polls);
}

cudaError_t launch_wait_probe(int polls, int* err, cudaStream_t s) {
    k_wait_probe<<<1, 128, 0, s>>>(polls, err);
    return cudaGetLastError();
}

double measure_fp32_peak(int device, int reps) { return measure_peak<float>(device, reps, 4096); }
double measure_fp64_peak(int device, int reps) { return measure_peak<double>(device, reps, 256); }

}  // namespace sbgpu
