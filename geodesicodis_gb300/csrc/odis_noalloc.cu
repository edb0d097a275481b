// Area-mean tidal dissipation (the reference's updateEnergy, LINEAR branch,
// src/energy.cpp:13-61) for callers that cannot allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is not allowed or not safe --
// inside a host callback or a host node of someone else's CUDA graph, in a
// real-time loop with a fixed memory budget, in a plugin that only receives
// device buffers from its host application, or after the caller's allocator
// has been locked down.  odis_update_energy needs an odis_ctx, and creating
// one allocates; this entry point needs nothing but the caller's buffers.
//
// The block partial sums of the reduction live in a file-scope __device__
// array of kNoAllocMaxBlocks doubles (64 KiB, 256-byte aligned), so every GPU
// that loads libodis_gpu.so holds these 64 KiB until the process exits.  Host
// code cannot use the array's name as a device address: the first call on
// each device, with that device current, looks the address up with
// cudaGetSymbolAddress and caches it (make that first call before any stream
// capture).  All calls share the array: two calls that overlap on the GPU
// (different streams, or threads racing) race on it and may return wrong sums;
// serialise them.  Nothing in the array has to start at zero: each call writes
// every partial it later reads.  The cached address belongs to the device's
// primary context: after a cudaDeviceReset in this process it is stale, and
// this entry point must not be called again.  QUADRATIC friction is not
// computed here; odis_update_energy covers it.
#include "../../include/odis_gpu.h"

#include <cuda_runtime.h>

#include <mutex>

namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocMaxBlocks = 8192;          // faces <= 8192 * 256 = 2,097,152
constexpr int kMaxDevices = 64;

__device__ __align__(256) double g_energy_scratch[kNoAllocMaxBlocks];

std::mutex g_setup_mutex;
double* g_scratch_addr[kMaxDevices] = {};

__device__ __forceinline__ double warp_sum_na(double x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    return x;
}

__global__ void __launch_bounds__(kNoAllocThreads) k_energy_partial_na(const double* __restrict__ uv,
                                                                       const double* __restrict__ area, int n, double coef,
                                                                       double* __restrict__ e_out, double* __restrict__ partial)
{
    __shared__ double red[kNoAllocThreads / 32];
    const int i = blockIdx.x * kNoAllocThreads + threadIdx.x;
    double x = 0.0;
    if (i < n) {
        const double u = uv[2 * i], w = uv[2 * i + 1];
        const double ei = coef * (u * u + w * w);
        if (e_out) e_out[i] = ei;
        x = ei * area[i];
    }
    x = warp_sum_na(x);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
        double s = threadIdx.x < kNoAllocThreads / 32 ? red[threadIdx.x] : 0.0;
        s = warp_sum_na(s);
        if (threadIdx.x == 0) partial[blockIdx.x] = s;
    }
}

__global__ void k_energy_fold_na(const double* __restrict__ partial, int nb, double divisor, double* __restrict__ out)
{
    double s = 0.0;
    for (int k = threadIdx.x; k < nb; k += 32) s += partial[k];
    s = warp_sum_na(s);
    if (threadIdx.x == 0) *out = s / divisor;
}

// Device address of the scratch array on the current device (looked up once per device).
odis_status scratch_for_current_device(double** out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return ODIS_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_energy_scratch) != cudaSuccess || !p) return ODIS_ERR_CUDA;
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[dev];
    return ODIS_OK;
}

}  // namespace

extern "C" odis_status odis_update_energy_noalloc(const double* uv, const double* area, int n_faces, double alpha,
                                                  double h, double radius, double* e_out, double* avg_out,
                                                  void* stream)
{
    if (!uv || !area || !avg_out || n_faces <= 0 || !(radius > 0.0)) return ODIS_ERR_ARG;
    const int nb = (n_faces + kNoAllocThreads - 1) / kNoAllocThreads;
    if (nb > kNoAllocMaxBlocks) return ODIS_ERR_ARG;     // more faces than the fixed scratch can reduce
    double* scratch = nullptr;
    const odis_status st = scratch_for_current_device(&scratch);
    if (st != ODIS_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const double pi = 3.1415926535897932384626433832795028841971693993751058;
    k_energy_partial_na<<<nb, kNoAllocThreads, 0, s>>>(uv, area, n_faces, alpha * 1000.0 * h, e_out, scratch);
    k_energy_fold_na<<<1, 32, 0, s>>>(scratch, nb, (4 * pi) * (radius * radius), avg_out);
    return cudaGetLastError() == cudaSuccess ? ODIS_OK : ODIS_ERR_CUDA;
}
