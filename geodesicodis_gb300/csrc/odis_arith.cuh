// Arithmetic policies shared by kernels templated on the method's number type:
// double (FP64 method), float2 = df64 (double-float method), float (FP32 state).
#pragma once

#include <cuda_runtime.h>

#include "odis_df64.cuh"

namespace odis {

template <class T> struct Ar;
template <> struct Ar<double> {
    using V = double;
    __device__ static V zero() { return 0.0; }
    __device__ static V fma(V a, V b, V c) { return ::fma(a, b, c); }
    __device__ static V fma_acc(V a, V b, V c) { return ::fma(a, b, c); }   // running sums (see Ar<df64>)
    __device__ static V norm(V a) { return a; }
    __device__ static V mul(V a, V b) { return a * b; }
    __device__ static V add(V a, V b) { return a + b; }
    __device__ static V sub(V a, V b) { return a - b; }
    __device__ static V neg(V a) { return -a; }
    __device__ static V div(V a, V b) { return a / b; }
    __device__ static V abs(V a) { return ::fabs(a); }
    __device__ static V half(V a) { return a * 0.5; }
    __device__ static V from(double x) { return x; }
    __device__ static double to(V a) { return a; }
    __device__ static V shfl(V a, int o) { return __shfl_down_sync(0xffffffffu, a, o); }
    __device__ static bool finite(V a) { return (__double2hiint(a) & 0x7ff00000) != 0x7ff00000; }
    __device__ static V ldcg(const V* p) { return __ldcg(p); }
    __device__ static void stcg(V* p, V v) { __stcg(p, v); }
    // two adjacent values in one aligned vector load (p[0] and p[1], p 16-byte aligned)
    __device__ static void ld2(const V* p, V& a, V& b) { const double2 v = *reinterpret_cast<const double2*>(p); a = v.x; b = v.y; }
};
template <> struct Ar<float> {
    using V = float;
    __device__ static V zero() { return 0.f; }
    __device__ static V fma(V a, V b, V c) { return fmaf(a, b, c); }
    __device__ static V fma_acc(V a, V b, V c) { return fmaf(a, b, c); }
    __device__ static V norm(V a) { return a; }
    __device__ static V mul(V a, V b) { return a * b; }
    __device__ static V add(V a, V b) { return a + b; }
    __device__ static V sub(V a, V b) { return a - b; }
    __device__ static V neg(V a) { return -a; }
    __device__ static V div(V a, V b) { return a / b; }
    __device__ static V abs(V a) { return fabsf(a); }
    __device__ static V half(V a) { return a * 0.5f; }
    __device__ static V from(double x) { return (float)x; }
    __device__ static double to(V a) { return (double)a; }
    __device__ static V shfl(V a, int o) { return __shfl_down_sync(0xffffffffu, a, o); }
    __device__ static bool finite(V a) { return (__float_as_int(a) & 0x7f800000) != 0x7f800000; }
    __device__ static V ldcg(const V* p) { return __ldcg(p); }
    __device__ static void stcg(V* p, V v) { __stcg(p, v); }
    __device__ static void ld2(const V* p, V& a, V& b) { const float2 v = *reinterpret_cast<const float2*>(p); a = v.x; b = v.y; }
};
template <> struct Ar<df64> {
    using V = df64;
    __device__ static V zero() { return df_make(0.f, 0.f); }
    __device__ static V fma(V a, V b, V c) { return df_fma(a, b, c); }
    // running sums: no renormalisation per term; norm() before the sum is used
    __device__ static V fma_acc(V a, V b, V c) { return df_fma_acc(a, b, c); }
    __device__ static V norm(V a) { return df_norm(a); }
    __device__ static V mul(V a, V b) { return df_mul(a, b); }
    __device__ static V add(V a, V b) { return df_add(a, b); }
    __device__ static V sub(V a, V b) { return df_sub(a, b); }
    __device__ static V neg(V a) { return df_neg(a); }
    __device__ static V div(V a, V b) { return df_div(a, b); }
    __device__ static V abs(V a) { return df_abs(a); }
    __device__ static V half(V a) { return df_scale2(a, 0.5f); }
    __device__ static V from(double x) { return df_from_double(x); }
    __device__ static double to(V a) { return df_to_double(a); }
    __device__ static V shfl(V a, int o) { return df_shfl_down(a, o); }
    __device__ static bool finite(V a) { return df_finite(a); }
    __device__ static V ldcg(const V* p) { return __ldcg(p); }
    __device__ static void stcg(V* p, V v) { __stcg(p, v); }
    __device__ static void ld2(const V* p, V& a, V& b)
    {
        const float4 v = *reinterpret_cast<const float4*>(p);
        a = make_float2(v.x, v.y);
        b = make_float2(v.z, v.w);
    }
};

}  // namespace odis
