// Double-float ("df64") arithmetic: a value is an unevaluated sum hi + lo of
// two FP32 numbers (|lo| <= ulp(hi)/2), a 48-bit significand.  GB300 runs FP64
// at 1/74 of its FP32 rate (measured 1.0 vs 74 TFLOP/s), so the ODIS_DF64
// method evaluates the FP64 step on the FP32 pipes with these error-free
// transformations (Dekker 1971; Knuth TAOCP vol. 2, 4.2.2; the FMA form of
// the exact product):
//   two_sum(a, b):       s = a + b exactly as s + e           (6 flops)
//   quick_two_sum(a, b): same for |a| >= |b|                   (3 flops)
//   exact product:       p = a*b, e = fma(a, b, -p)            (2 flops)
// Additions are the "sloppy" form (one two_sum on the high parts), which keeps
// an absolute error of ~2^-48 of the larger operand -- enough for the 1e-10
// parity of the time loop, which is verified against the FP64 oracle.
// The compiler must not reassociate: these files are built without fast-math.
#pragma once

#include <cuda_runtime.h>

namespace odis {

using df64 = float2;      // .x = hi, .y = lo

__host__ __device__ __forceinline__ df64 df_make(float hi, float lo) { return make_float2(hi, lo); }

// exact split of a double into a df64 (host, or device on cold paths)
__host__ __device__ __forceinline__ df64 df_from_double(double x)
{
    const float hi = (float)x;
    const float lo = (float)(x - (double)hi);
    return make_float2(hi, lo);
}

__host__ __device__ __forceinline__ double df_to_double(df64 a) { return (double)a.x + (double)a.y; }

__device__ __forceinline__ df64 df_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return make_float2(s, e);
}

__device__ __forceinline__ df64 df_quick_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float e = __fsub_rn(b, __fsub_rn(s, a));
    return make_float2(s, e);
}

__device__ __forceinline__ df64 df_add(df64 a, df64 b)
{
    const df64 s = df_two_sum(a.x, b.x);
    const float e = __fadd_rn(s.y, __fadd_rn(a.y, b.y));
    return df_quick_two_sum(s.x, e);
}

__device__ __forceinline__ df64 df_neg(df64 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ df64 df_sub(df64 a, df64 b) { return df_add(a, df_neg(b)); }

__device__ __forceinline__ df64 df_mul(df64 a, df64 b)
{
    const float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    return df_quick_two_sum(p, e);
}

// a*b + c
__device__ __forceinline__ df64 df_fma(df64 a, df64 b, df64 c)
{
    const float p = __fmul_rn(a.x, b.x);
    float pe = __fmaf_rn(a.x, b.x, -p);
    pe = __fmaf_rn(a.x, b.y, pe);
    pe = __fmaf_rn(a.y, b.x, pe);
    const df64 s = df_two_sum(p, c.x);
    const float e = __fadd_rn(s.y, __fadd_rn(pe, c.y));
    return df_quick_two_sum(s.x, e);
}

// a*b + c for a running sum: the low words collect the rounding errors without
// a renormalisation per term (12 instead of 15 FP32 operations).  The result is
// a valid pair after df_norm; short sums (tens of terms) keep the 2^-48 bound.
__device__ __forceinline__ df64 df_fma_acc(df64 a, df64 b, df64 c)
{
    const float p = __fmul_rn(a.x, b.x);
    float pe = __fmaf_rn(a.x, b.x, -p);
    pe = __fmaf_rn(a.x, b.y, pe);
    pe = __fmaf_rn(a.y, b.x, pe);
    const df64 s = df_two_sum(p, c.x);
    return make_float2(s.x, __fadd_rn(c.y, __fadd_rn(s.y, pe)));
}

__device__ __forceinline__ df64 df_norm(df64 a) { return df_quick_two_sum(a.x, a.y); }

// a / b (Dekker's long division in double-float): an FP32 quotient q1, the
// remainder a - q1 b in double-float, one FP32 correction q2; about 2^-47 relative
__device__ __forceinline__ df64 df_div(df64 a, df64 b)
{
    const float q1 = __fdiv_rn(a.x, b.x);
    const df64 r = df_sub(a, df_mul(b, make_float2(q1, 0.f)));
    const float q2 = __fdiv_rn(r.x, b.x);
    return df_quick_two_sum(q1, q2);
}

__device__ __forceinline__ df64 df_abs(df64 a) { return a.x < 0.f ? df_neg(a) : a; }

// a * 2^k for a power-of-two factor: exact on both words
__device__ __forceinline__ df64 df_scale2(df64 a, float s) { return make_float2(a.x * s, a.y * s); }

__device__ __forceinline__ df64 df_shfl_down(df64 a, int o)
{
    return make_float2(__shfl_down_sync(0xffffffffu, a.x, o), __shfl_down_sync(0xffffffffu, a.y, o));
}

__device__ __forceinline__ bool df_finite(df64 a) { return (__float_as_int(a.x) & 0x7f800000) != 0x7f800000; }

// Square root of a non-negative double-float: the FP32 root s of the high part,
// refined by one Newton step on the residual a - s^2, whose s^2 is formed
// exactly (Karp and Markstein, "High-precision division and square root", ACM
// TOMS 23, 1997): relative error about 2^-46.  Zero for a <= 0.
__device__ __forceinline__ df64 df_sqrt(df64 a)
{
    if (!(a.x > 0.f)) return df_make(0.f, 0.f);
    const float s = sqrtf(a.x);
    const float p = s * s, pe = fmaf(s, s, -p);      // s^2 = p + pe exactly
    const float r = ((a.x - p) - pe) + a.y;
    return df_two_sum(s, r * (0.5f / s));
}

// Dissipation of one face from q = u^2 + v^2 and the face's coefficient d
// (updateEnergy, src/energy.cpp:30-53, times A_e / (4 pi r^2)): d q for LINEAR
// friction and d q sqrt(q) for QUADRATIC.
__device__ __forceinline__ double face_diss(double d, double q, int quad)
{
    const double x = d * q;
    return quad ? x * sqrt(q) : x;
}
__device__ __forceinline__ float face_diss(float d, float q, int quad)
{
    const float x = d * q;
    return quad ? x * sqrtf(q) : x;
}
__device__ __forceinline__ df64 face_diss(df64 d, df64 q, int quad)
{
    const df64 x = df_mul(d, q);
    return quad ? df_mul(x, df_sqrt(q)) : x;
}

}  // namespace odis
