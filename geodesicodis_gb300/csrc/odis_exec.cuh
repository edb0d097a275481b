// Executors of the setup steps (mesh build, grid generation): the same
// per-element steps run as OpenMP loops on the host (HostExec, here) or as one
// kernel per step on the device (DevExec, odis_mesh_dev.cu).
//
// An executor X provides
//   X::Buf<T>          handle of an array, with .ptr
//   x.out(vec, n, v)   array of n elements set to v, delivered into vec by x.finish()
//   x.tmp<T>(n, v)     scratch array of n elements set to v
//   x.in(p, n)         an input array
//   x.run(n, step)     step(i) for every i < n, in any order
//   x.scan(p, n)       exclusive prefix sum of p[0..n) in place; returns the total
//   x.to_host / x.to_dev   copies between the executor's arrays and host memory
//   x.failed(err)      the steps' error flag (waits for them)
//   x.status()         the executor's own failure (allocation, launch), else 0
//   x.finish()         delivers the out arrays
#pragma once

#include "../../include/odis_gpu.h"

#include <cstring>
#include <vector>

#ifndef ODIS_HD
#ifdef __CUDACC__
#define ODIS_HD __host__ __device__
#else
#define ODIS_HD
#endif
#endif

namespace odis {

ODIS_HD inline int exec_atomic_add(int* p, int v)
{
#ifdef __CUDA_ARCH__
    return atomicAdd(p, v);
#else
    return __atomic_fetch_add(p, v, __ATOMIC_RELAXED);
#endif
}

ODIS_HD inline void exec_atomic_min(int* p, int v)
{
#ifdef __CUDA_ARCH__
    atomicMin(p, v);
#else
    int cur = __atomic_load_n(p, __ATOMIC_RELAXED);
    while (v < cur && !__atomic_compare_exchange_n(p, &cur, v, true, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
    }
#endif
}

ODIS_HD inline void exec_flag(int* err)
{
#ifdef __CUDA_ARCH__
    atomicOr(err, 1);
#else
    __atomic_store_n(err, 1, __ATOMIC_RELAXED);
#endif
}

struct HostExec {
    template <class T> struct Buf { T* ptr; std::vector<T> own; };
    template <class T> T* out(std::vector<T>& v, size_t n, T init) { v.assign(n, init); return v.data(); }
    template <class T> Buf<T> tmp(size_t n, T init)
    {
        Buf<T> b{nullptr, std::vector<T>(n, init)};
        b.ptr = b.own.data();
        return b;
    }
    template <class T> const T* in(const T* p, size_t) { return p; }
    template <class F> void run(long long n, const F& f)
    {
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < n; i++) f(i);
    }
    long long scan(int* p, long long n)
    {
        long long s = 0;
        for (long long i = 0; i < n; i++) {
            const int c = p[i];
            p[i] = (int)s;
            s += c;
        }
        return s;
    }
    template <class T> void to_host(T* dst, const T* src, size_t n) { std::memcpy(dst, src, sizeof(T) * n); }
    template <class T> void to_dev(T* dst, const T* src, size_t n) { std::memcpy(dst, src, sizeof(T) * n); }
    bool failed(const int* err) { return *err != 0; }
    int status() const { return ODIS_OK; }
    int finish() { return ODIS_OK; }
};

}  // namespace odis
