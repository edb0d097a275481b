// Grid generation and mesh build on the GPU: the steps of odis_grid_gen.cuh and
// odis_mesh_build.cuh, one kernel per step over the elements (lattice points,
// leaves, nodes, faces, vertices), with the scans between them on the host.
//
// Compiled with -fmad=false: the host steps evaluate every product and sum
// unfused, in the reference's order, and so do these kernels.  The integer
// outputs (numbering, friends, TRiSK stencils) are the host's exactly; the
// positions and circumcentres of the generator too (sums, products, square
// roots and quotients round the same on both sides).  Where CUDA's sin, cos,
// acos, asin and atan2 round differently from the C library's in the last bit,
// the geometry differs from the host build's by that much.
//
// Every index a kernel forms is checked on the host first (input ranges) or in
// the step itself (ids looked up from earlier steps), which sets the error flag
// and skips the access.
#include "../../include/odis_gpu.h"
#include "odis_exec.cuh"
#include "odis_grid_gen.cuh"
#include "odis_internal.h"
#include "odis_mesh_build.cuh"

#include <cuda_runtime.h>

#include <vector>

namespace odis {

namespace {

constexpr int kSetupThreads = 128;

template <class T>
__global__ void k_fill(T* p, long long n, T v)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

template <class F>
__global__ void __launch_bounds__(kSetupThreads) k_each(long long n, F f)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) f(i);
}

// executor of the setup steps on the current device (see odis_exec.cuh)
struct DevExec {
    cudaStream_t s = nullptr;
    int st = ODIS_OK;
    std::vector<void*> mem;
    struct Out { void* d; void* h; size_t bytes; };
    std::vector<Out> outs;
    template <class T> struct Buf { T* ptr; };

    DevExec()
    {
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) { s = nullptr; st = ODIS_ERR_CUDA; }
    }
    ~DevExec()
    {
        if (s) cudaStreamSynchronize(s);
        for (void* p : mem) cudaFree(p);
        if (s) cudaStreamDestroy(s);
    }
    void check()
    {
        if (cudaGetLastError() != cudaSuccess && st == ODIS_OK) st = ODIS_ERR_CUDA;
    }
    static unsigned blocks(long long n) { return (unsigned)((n + kSetupThreads - 1) / kSetupThreads); }
    template <class T> T* alloc(size_t n)
    {
        if (st) return nullptr;
        void* p = nullptr;
        if (cudaMalloc(&p, sizeof(T) * (n ? n : 1)) != cudaSuccess) {
            (void)cudaGetLastError();
            st = ODIS_ERR_NOMEM;
            return nullptr;
        }
        mem.push_back(p);
        return (T*)p;
    }
    template <class T> void fill(T* p, size_t n, T v)
    {
        if (st || !p || !n) return;
        k_fill<T><<<blocks((long long)n), kSetupThreads, 0, s>>>(p, (long long)n, v);
        check();
    }
    template <class T> T* out(std::vector<T>& v, size_t n, T init)
    {
        T* p = alloc<T>(n);
        fill(p, n, init);
        v.assign(n, init);
        if (p) outs.push_back({p, v.data(), sizeof(T) * n});
        return p;
    }
    template <class T> Buf<T> tmp(size_t n, T init)
    {
        T* p = alloc<T>(n);
        fill(p, n, init);
        return {p};
    }
    template <class T> const T* in(const T* h, size_t n)
    {
        T* p = alloc<T>(n);
        if (p && cudaMemcpyAsync(p, h, sizeof(T) * n, cudaMemcpyHostToDevice, s) != cudaSuccess) {
            (void)cudaGetLastError();
            if (st == ODIS_OK) st = ODIS_ERR_CUDA;
        }
        return p;
    }
    template <class F> void run(long long n, const F& f)
    {
        if (st || n <= 0) return;
        k_each<F><<<blocks(n), kSetupThreads, 0, s>>>(n, f);
        check();
    }
    template <class T> void to_host(T* dst, const T* src, size_t n)
    {
        if (st) return;
        if (cudaMemcpyAsync(dst, src, sizeof(T) * n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            st = ODIS_ERR_CUDA;
    }
    template <class T> void to_dev(T* dst, const T* src, size_t n)
    {
        if (st) return;
        if (cudaMemcpyAsync(dst, src, sizeof(T) * n, cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            st = ODIS_ERR_CUDA;
    }
    long long scan(int* p, long long n)
    {
        std::vector<int> h((size_t)n);
        to_host(h.data(), p, (size_t)n);
        if (st) return -1;
        long long sum = 0;
        for (long long i = 0; i < n; i++) {
            const int c = h[i];
            h[i] = (int)sum;
            sum += c;
        }
        to_dev(p, h.data(), (size_t)n);
        return st ? -1 : sum;
    }
    bool failed(const int* err)
    {
        int h = 0;
        to_host(&h, err, 1);
        return st != ODIS_OK || h != 0;
    }
    int status() const { return st; }
    int finish()
    {
        for (const Out& o : outs) {
            if (st) break;
            if (cudaMemcpyAsync(o.h, o.d, o.bytes, cudaMemcpyDeviceToHost, s) != cudaSuccess) st = ODIS_ERR_CUDA;
        }
        if (!st && cudaStreamSynchronize(s) != cudaSuccess) st = ODIS_ERR_CUDA;
        return st;
    }
};

}  // namespace

int generate_grid_device(int level, GridArrays& g)
{
    DevExec x;
    if (x.status()) return x.status();
    return generate_grid_steps(x, level, g);
}

int build_mesh_device(int N, const double* node_sph, const int* friends, const double* cent_sph, double radius,
                      Mesh& m)
{
    DevExec x;
    if (x.status()) return x.status();
    return build_mesh_steps(x, N, node_sph, friends, cent_sph, radius, m);
}

}  // namespace odis
