// FP32 FMA throughput of the device, measured with independent FMA chains on
// every SM.  It is the denominator of the force kernels' roofline:
// MEASURED_PEAKS-style copy/GEMM figures say nothing about the FP32 pipe.

#include <cuda_runtime.h>
#include <stdint.h>

#define TG_EXPORT extern "C" __attribute__((visibility("default")))

namespace {

constexpr int CHAINS = 16;

__global__ void __launch_bounds__(256) fma_chains(float *sink, int iters)
{
    float a[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) a[c] = 1e-3f * (threadIdx.x + c);
    const float b = 0.9999f, d = 1e-6f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < CHAINS; ++c) a[c] = __fmaf_rn(a[c], b, d);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) s += a[c];
    if (s == 12345.f) sink[threadIdx.x] = s;   // keeps the chains alive
}

}  // namespace

// Launches one FMA-chain sweep on `stream` (for timing by the caller) and
// returns the number of floating-point operations it performs (2 per FMA).
TG_EXPORT double tupan_gb300_fma_sweep(int iters, void *stream)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    static float *sink = nullptr;
    if (!sink && cudaMalloc(&sink, 256 * sizeof(float)) != cudaSuccess)
        return -1.0;
    const int blocks = sms * 8;
    fma_chains<<<blocks, 256, 0, (cudaStream_t)stream>>>(sink, iters);
    if (cudaGetLastError() != cudaSuccess) return -1.0;
    return 2.0 * CHAINS * (double)iters * 256.0 * blocks;
}

// Measured FP32 FMA throughput in TFLOP/s (best of `reps` timed sweeps).
TG_EXPORT double tupan_gb300_fp32_peak_tflops(int iters, int reps)
{
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess) return -1.0;
    cudaEventCreate(&b);
    double best = 0.0;
    tupan_gb300_fma_sweep(iters / 4 + 1, nullptr);   // warm-up
    for (int r = 0; r < reps; ++r) {
        cudaEventRecord(a, nullptr);
        double flops = tupan_gb300_fma_sweep(iters, nullptr);
        cudaEventRecord(b, nullptr);
        if (cudaEventSynchronize(b) != cudaSuccess || flops < 0) {
            best = -1.0;
            break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        double tf = flops / (ms * 1e-3) / 1e12;
        if (tf > best) best = tf;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return best;
}
