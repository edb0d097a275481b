// Measured FP64 issue rate of this GPU, the second ceiling of the FP64 method.
//
// GB300 runs FP64 arithmetic at a small fraction of its FP32 rate, so the FP64
// kernels of this library (the plain step, the self-gravity transforms) can be
// bound by FP64 issue before HBM bandwidth.  Their roofline against this
// ceiling needs the rate the hardware actually sustains, measured here rather
// than taken from a datasheet: every thread runs eight independent chains of
// dependent FMAs (enough to cover the FP64 pipe's latency), 2 CTAs of 256
// threads per SM, about ten milliseconds per launch, timed with CUDA
// events after a warm-up launch (best of three).
#include "../../include/odis_gpu.h"

#include <cuda_runtime.h>

namespace {

constexpr int kProbeThreads = 256;
constexpr int kChains = 8;

__global__ void __launch_bounds__(kProbeThreads) k_fp64_fma(int iters, double seed, double* out)
{
    double x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = seed + 1e-3 * (threadIdx.x + c);
    const double a = 0.999999999, b = 1e-9;
    for (int k = 0; k < iters; k++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) x[c] = fma(x[c], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += x[c];
    if (s == 12345.678) out[blockIdx.x] = s;      // never true; keeps the chains live
}

}  // namespace

extern "C" odis_status odis_measure_fp64_rate(double* tflops)
{
    if (!tflops) return ODIS_ERR_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return ODIS_ERR_CUDA;
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * 2 * sms) != cudaSuccess) return ODIS_ERR_NOMEM;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int blocks = 2 * sms, iters = 1 << 13;
    k_fp64_fma<<<blocks, kProbeThreads>>>(iters, 1.0, out);          // warm-up
    float best = 1e30f;
    for (int r = 0; r < 3; r++) {
        cudaEventRecord(a);
        k_fp64_fma<<<blocks, kProbeThreads>>>(iters, 1.0 + r, out);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        if (ms < best) best = ms;
    }
    const cudaError_t e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    if (e != cudaSuccess || !(best > 0.f)) return ODIS_ERR_CUDA;
    const double flops = 2.0 * kChains * (double)iters * blocks * kProbeThreads;
    *tflops = flops / (best * 1e-3) / 1e12;
    return ODIS_OK;
}
