// sm_103a kernels of the LTE timestep (src/timeIntegrator.cpp:205-272 of the
// reference, linear branch).
//
// One step is two launches:
//   k_edge_step : per face e (one thread each)
//       T_e   = sum_k w_ek v_nbr(e,k)                  TRiSK tangential velocity of v^n
//       P^{n-1} partial: diss_e (v_e^2 + T_e^2)         (dissipation of v^n, block partial)
//       f_e   = -g (G eta^n)_e - 2 Omega sin(phi_e) T_e  (updateMomentum, linear branch)
//       v^{n+1} = v^n + dt AB3(f) + dt (-alpha v^n + (G U(t^{n+1}))_e)
//   k_cell_step : per cell i
//       q_i   = h (D v^{n+1})_i                         (updateEta, linear branch)
//       eta^{n+1} = eta^n + dt AB3(q)
//       block 0 also folds the face kernel's block partials into P^{n-1}
// The tangential reconstruction of v^{n+1} is needed twice in the reference
// (Coriolis of step n+1 and the dissipation of step n); it is computed once,
// in the next step's face kernel, so the dissipation of the last step of a
// run is finished by k_power_tail.
//
// Reductions are deterministic: fixed-shape warp shuffles inside a block,
// then one warp summing the per-block partials in block order.
#include "../../include/odis_gpu.h"
#include "odis_device.cuh"
#include "odis_df64.cuh"
#include "odis_kernels.cuh"
#include "odis_pdl.cuh"
#include "odis_forcing.cuh"

#include <type_traits>

#include <cmath>

namespace odis {

namespace {

template <class T> __device__ __forceinline__ T fmaT(T a, T b, T c);
template <> __device__ __forceinline__ double fmaT<double>(double a, double b, double c) { return fma(a, b, c); }
template <> __device__ __forceinline__ float fmaT<float>(float a, float b, float c) { return fmaf(a, b, c); }

__device__ __forceinline__ double warp_sum(double x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    return x;
}

// Sum of one double per thread over the block; the result is valid in thread 0.
template <int kThreads>
__device__ __forceinline__ double block_sum(double x, double* smem)
{
    x = warp_sum(x);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) smem[wid] = x;
    __syncthreads();
    double s = 0.0;
    if (wid == 0) {
        s = lane < kThreads / 32 ? smem[lane] : 0.0;
        s = warp_sum(s);
    }
    return s;
}

// One warp sums n partials in a fixed order; result in lane 0.
__device__ __forceinline__ double fold_partials(const double* p, int n)
{
    const int lane = threadIdx.x & 31;
    double s = 0.0;
    for (int k = lane; k < n; k += 32) s += p[k];
    return warp_sum(s);
}

// step constants in the kernel's type: the double itself, or its FP32 copy
template <class T> __device__ __forceinline__ T kc(double d, float f);
template <> __device__ __forceinline__ double kc<double>(double d, float) { return d; }
template <> __device__ __forceinline__ float kc<float>(double, float f) { return f; }

// (hi, lo) += x exactly to double-float precision: Knuth two-sum, then renormalise
// (explicit round-to-nearest adds, so no contraction can break the error terms)
__device__ __forceinline__ void df_accumulate(float& hi, float& lo, float x)
{
    const float s = __fadd_rn(hi, x);
    const float bb = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
    const float t = __fadd_rn(lo, err);
    const float h2 = __fadd_rn(s, t);
    lo = __fsub_rn(t, __fsub_rn(h2, s));
    hi = h2;
}

// finiteness from the exponent bits (integer pipe, no FP64 compare)
__device__ __forceinline__ bool finite_bits(double x) { return (__double2hiint(x) & 0x7ff00000) != 0x7ff00000; }

// Block sum of the per-thread dissipation, valid in thread 0.  FP64 method:
// every thread parks its term in shared memory (smem: kStepThreads doubles) and
// warp 0 adds them, eight per lane then a shuffle tree -- 12 FP64 additions a
// block instead of a 5-step shuffle tree in every warp (the FP64 pipe is the
// face kernel's bound).  FP32 variant: FP32 within a warp (32 terms) and FP64
// across warps.
template <class T>
__device__ __forceinline__ double block_power(T pw, double* smem)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if constexpr (std::is_same<T, double>::value) {
        smem[threadIdx.x] = pw;
        __syncthreads();
        double s = 0.0;
        if (wid == 0) {
            s = smem[lane];
#pragma unroll
            for (int r = 1; r < kStepThreads / 32; r++) s += smem[lane + 32 * r];
            s = warp_sum(s);
        }
        return s;
    } else {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) pw += __shfl_down_sync(0xffffffffu, pw, o);
        if (lane == 0) smem[wid] = (double)pw;
        __syncthreads();
        double s = 0.0;
        if (wid == 0) {
            s = lane < kStepThreads / 32 ? smem[lane] : 0.0;
            s = warp_sum(s);
        }
        return s;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// fused step, face part
// ---------------------------------------------------------------------------
// kQuad: QUADRATIC friction.  A compile-time switch here because the FP64 square
// root's code, even untaken, raised the FP64 kernel from 32 to 38 registers and
// cost occupancy (FP64 plain step 3.3 -> 2.7 G cell-steps/s at level 6).
template <class T, bool kMaster, bool kQuad>
__global__ void __launch_bounds__(kStepThreads) k_edge_step(FaceCoef<T> fc, State<T> st, StepConst sc, int offset)
{
    pdl_wait();
    __shared__ double s_red[kStepThreads];
    const long long it = *st.iter + offset;
    // forcing phase at t^{n+1} (precomputed per run by k_phase)
    const long long kstep = it - *st.run_first;
    const T cosM = st.phase[2 * kstep], sinM = st.phase[2 * kstep + 1];
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const int Ep = sc.Ep;
    const T* __restrict__ vin = ((it & 1) ? st.v[1] : st.v[0]);
    T pw = T(0);
    if (e < sc.E) {
        T tsum = T(0);
#pragma unroll
        for (int k = 0; k < kTrisk; k++) tsum = fmaT<T>(__ldg(&fc.w[k * Ep + e]), vin[__ldg(&fc.nbr[k * Ep + e])], tsum);
        const T ve = vin[e];
        const int i0 = __ldg(&fc.n0[e]), i1 = __ldg(&fc.n1[e]);
        pw = face_diss(__ldg(&fc.diss[e]), fmaT<T>(ve, ve, tsum * tsum), kQuad);
        // updateMomentum: -g G eta + C v
        const T g0 = __ldg(&fc.gg0[e]), g1 = __ldg(&fc.gg1[e]);
        const T f0 = fmaT<T>(__ldg(&fc.cor[e]), tsum, fmaT<T>(g0, st.eta[i0], g1 * st.eta[i1]));
        // forcing gradient G U(t^{n+1}) (+ self-gravity), then linear drag
        T gu = fmaT<T>(cosM, __ldg(&fc.fP[e]), sinM * __ldg(&fc.fQ[e]));
        if (sc.use_sg) gu -= fmaT<T>(g0, st.usg[i0], g1 * st.usg[i1]);
        const T kdt = kc<T>(sc.dt, sc.f_dt);
        const T drag = fmaT<T>(kc<T>(-sc.alpha, sc.f_malpha), ve, gu);
        T* hcur = ((it & 1) ? st.hv[1] : st.hv[0]);
        T inc = f0;
        if (sc.init_load || it > 1) {
            const T f1 = ((it & 1) ? st.hv[0] : st.hv[1])[e];
            const T f2 = hcur[e];
            inc = fmaT<T>(kc<T>(sc.ab3c, sc.f_c), f2, fmaT<T>(kc<T>(sc.ab3b, sc.f_b), f1, kc<T>(sc.ab3a, sc.f_a) * f0));
        }
        hcur[e] = f0;
        if constexpr (kMaster) {
            // FP32 increment, double-float accumulation into (v, vlo)
            float hi = ve, lo = st.vlo[e];
            df_accumulate(hi, lo, kdt * (inc + drag));
            st.vlo[e] = lo;
            ((it & 1) ? st.v[0] : st.v[1])[e] = hi;
            if (!isfinite(hi)) atomicOr(st.status, 1 << ODIS_ERR_NONFINITE);
        } else {
            T vn = fmaT<T>(inc, kdt, ve);
            vn = fmaT<T>(kdt, drag, vn);
            ((it & 1) ? st.v[0] : st.v[1])[e] = vn;
            if (!finite_bits((double)vn)) atomicOr(st.status, 1 << ODIS_ERR_NONFINITE);
        }
    }
    const double bs = block_power<T>(pw, s_red);
    // row kstep of the run's partial table: the dissipation of v^it, the power after step it-1
    if (threadIdx.x == 0) st.partial[kstep * gridDim.x + blockIdx.x] = bs;
}

// ---------------------------------------------------------------------------
// FP32-state variant, face part: two neighbouring faces per thread
// ---------------------------------------------------------------------------
// Same arithmetic per face as k_edge_step<float, true>, but each thread owns the
// face pair (2p, 2p+1) and moves their coefficients and state with 8-byte
// (float2 / int2) loads and stores.  With 4-byte values one face per thread
// keeps only half the bytes in flight of the 8-byte methods, and the kernel is
// latency bound well below the HBM rate once the working set leaves L2.  The
// pad faces past E (Ep is a multiple of 128) have zero coefficients and point
// at face 0, so the second face of an odd tail computes and stores zeros.
template <bool kQuad>   // QUADRATIC friction, a compile-time switch as in k_edge_step
__global__ void __launch_bounds__(kStepThreads) k_edge_step_f32x2(FaceCoef<float> fc, State<float> st, StepConst sc,
                                                                     int offset)
{
    pdl_wait();
    __shared__ double s_red[kStepThreads];
    const long long it = *st.iter + offset;
    const long long kstep = it - *st.run_first;
    const float cosM = st.phase[2 * kstep], sinM = st.phase[2 * kstep + 1];
    const int e = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int Ep = sc.Ep;
    const float* __restrict__ vin = ((it & 1) ? st.v[1] : st.v[0]);
    float pw = 0.f;
    if (e < sc.E) {
        float tx = 0.f, ty = 0.f;
#pragma unroll
        for (int k = 0; k < kTrisk; k++) {
            const float2 w = __ldg(reinterpret_cast<const float2*>(&fc.w[k * Ep + e]));
            const int2 nb = __ldg(reinterpret_cast<const int2*>(&fc.nbr[k * Ep + e]));
            tx = fmaf(w.x, vin[nb.x], tx);
            ty = fmaf(w.y, vin[nb.y], ty);
        }
        const float2 ve = *reinterpret_cast<const float2*>(&vin[e]);
        const float2 diss = __ldg(reinterpret_cast<const float2*>(&fc.diss[e]));
        pw = face_diss(diss.x, fmaf(ve.x, ve.x, tx * tx), kQuad) + face_diss(diss.y, fmaf(ve.y, ve.y, ty * ty), kQuad);
        const int2 n0 = __ldg(reinterpret_cast<const int2*>(&fc.n0[e]));
        const int2 n1 = __ldg(reinterpret_cast<const int2*>(&fc.n1[e]));
        const float2 g0 = __ldg(reinterpret_cast<const float2*>(&fc.gg0[e]));
        const float2 g1 = __ldg(reinterpret_cast<const float2*>(&fc.gg1[e]));
        const float2 cor = __ldg(reinterpret_cast<const float2*>(&fc.cor[e]));
        const float2 fP = __ldg(reinterpret_cast<const float2*>(&fc.fP[e]));
        const float2 fQ = __ldg(reinterpret_cast<const float2*>(&fc.fQ[e]));
        float2 f0;
        f0.x = fmaf(cor.x, tx, fmaf(g0.x, st.eta[n0.x], g1.x * st.eta[n1.x]));
        f0.y = fmaf(cor.y, ty, fmaf(g0.y, st.eta[n0.y], g1.y * st.eta[n1.y]));
        float2 gu = make_float2(fmaf(cosM, fP.x, sinM * fQ.x), fmaf(cosM, fP.y, sinM * fQ.y));
        if (sc.use_sg) {
            gu.x -= fmaf(g0.x, st.usg[n0.x], g1.x * st.usg[n1.x]);
            gu.y -= fmaf(g0.y, st.usg[n0.y], g1.y * st.usg[n1.y]);
        }
        const float2 drag = make_float2(fmaf(sc.f_malpha, ve.x, gu.x), fmaf(sc.f_malpha, ve.y, gu.y));
        float* hcur = ((it & 1) ? st.hv[1] : st.hv[0]);
        float2 inc = f0;
        if (sc.init_load || it > 1) {
            const float2 f1 = *reinterpret_cast<const float2*>(&((it & 1) ? st.hv[0] : st.hv[1])[e]);
            const float2 f2 = *reinterpret_cast<const float2*>(&hcur[e]);
            inc.x = fmaf(sc.f_c, f2.x, fmaf(sc.f_b, f1.x, sc.f_a * f0.x));
            inc.y = fmaf(sc.f_c, f2.y, fmaf(sc.f_b, f1.y, sc.f_a * f0.y));
        }
        *reinterpret_cast<float2*>(&hcur[e]) = f0;
        float2 lo = *reinterpret_cast<const float2*>(&st.vlo[e]);
        float2 hi = ve;
        df_accumulate(hi.x, lo.x, sc.f_dt * (inc.x + drag.x));
        df_accumulate(hi.y, lo.y, sc.f_dt * (inc.y + drag.y));
        *reinterpret_cast<float2*>(&st.vlo[e]) = lo;
        *reinterpret_cast<float2*>(&((it & 1) ? st.v[0] : st.v[1])[e]) = hi;
        if (!isfinite(hi.x) || !isfinite(hi.y)) atomicOr(st.status, 1 << ODIS_ERR_NONFINITE);
    }
    const double bs = block_power<float>(pw, s_red);
    if (threadIdx.x == 0) st.partial[kstep * gridDim.x + blockIdx.x] = bs;
}

// Dissipation of the current v after the last step of a run, in the pair layout of k_edge_step_f32x2.
__global__ void __launch_bounds__(kStepThreads) k_power_partial_f32x2(FaceCoef<float> fc, State<float> st,
                                                                      StepConst sc)
{
    __shared__ double s_red[kStepThreads];
    const long long it = *st.iter;
    const int e = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int Ep = sc.Ep;
    const float* __restrict__ vin = ((it & 1) ? st.v[1] : st.v[0]);
    float pw = 0.f;
    for (int c = 0; c < 2; c++) {
        const int f = e + c;
        if (f >= sc.E) break;
        float tsum = 0.f;
#pragma unroll
        for (int k = 0; k < kTrisk; k++) tsum = fmaf(__ldg(&fc.w[k * Ep + f]), vin[__ldg(&fc.nbr[k * Ep + f])], tsum);
        const float ve = vin[f];
        pw += face_diss(__ldg(&fc.diss[f]), fmaf(ve, ve, tsum * tsum), sc.quad);
    }
    const double bs = block_power<float>(pw, s_red);
    if (threadIdx.x == 0) st.partial[(it - *st.run_first) * gridDim.x + blockIdx.x] = bs;
}

// ---------------------------------------------------------------------------
// fused step, cell part
// ---------------------------------------------------------------------------
template <class T, bool kMaster>
__global__ void __launch_bounds__(kStepThreads) k_cell_step(CellCoef<T> cc, State<T> st, StepConst sc, int offset)
{
    pdl_wait();
    const long long it = *st.iter + offset;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int Np = sc.Np;
    const T* __restrict__ vn = ((it & 1) ? st.v[0] : st.v[1]);
    if (i < sc.N) {
        T q = T(0);
#pragma unroll
        for (int k = 0; k < kCellFaces; k++) q = fmaT<T>(__ldg(&cc.hw[k * Np + i]), vn[__ldg(&cc.edge[k * Np + i])], q);
        T* hcur = ((it & 1) ? st.he[1] : st.he[0]);
        const T kdt = kc<T>(sc.dt, sc.f_dt);
        T inc = q;
        if (sc.init_load || it > 1) {
            const T f1 = ((it & 1) ? st.he[0] : st.he[1])[i];
            const T f2 = hcur[i];
            inc = fmaT<T>(kc<T>(sc.ab3c, sc.f_c), f2, fmaT<T>(kc<T>(sc.ab3b, sc.f_b), f1, kc<T>(sc.ab3a, sc.f_a) * q));
        }
        hcur[i] = q;
        if constexpr (kMaster) {
            float hi = st.eta[i], lo = st.etalo[i];
            df_accumulate(hi, lo, kdt * inc);
            st.etalo[i] = lo;
            st.eta[i] = hi;
        } else {
            st.eta[i] = fmaT<T>(inc, kdt, st.eta[i]);
        }
    }
}

// Dissipation of the current v (after the last step of a run).
template <class T>
__global__ void __launch_bounds__(kStepThreads) k_power_partial(FaceCoef<T> fc, State<T> st, StepConst sc)
{
    __shared__ double s_red[kStepThreads];
    const long long it = *st.iter;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const int Ep = sc.Ep;
    const T* __restrict__ vin = ((it & 1) ? st.v[1] : st.v[0]);
    T pw = T(0);
    if (e < sc.E) {
        T tsum = T(0);
#pragma unroll
        for (int k = 0; k < kTrisk; k++) tsum = fmaT<T>(__ldg(&fc.w[k * Ep + e]), vin[__ldg(&fc.nbr[k * Ep + e])], tsum);
        const T ve = vin[e];
        pw = face_diss(__ldg(&fc.diss[e]), fmaT<T>(ve, ve, tsum * tsum), sc.quad);
    }
    // the face kernel's block reduction, so that a run's last power value has the
    // bits it would have inside a longer run
    const double bs = block_power<T>(pw, s_red);
    if (threadIdx.x == 0) st.partial[(it - *st.run_first) * gridDim.x + blockIdx.x] = bs;
}

// power[k] = sum of row k+1 of the run's partial table (k < n), one warp per step,
// the partials of a row in a fixed order
__global__ void k_power_fold(const double* __restrict__ part, int nb, int n, double* __restrict__ power)
{
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (k >= n) return;
    const double s = fold_partials(part + (size_t)(k + 1) * nb, nb);
    if ((threadIdx.x & 31) == 0) power[k] = s;
}

__global__ void k_bump_iter(long long* iter, int n)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) *iter += n;
}

template <class T> __device__ __forceinline__ T from_double_dev(double x) { return (T)x; }
template <> __device__ __forceinline__ float2 from_double_dev<float2>(double x) { return df_from_double(x); }
__device__ __forceinline__ double to_double_dev(double x) { return x; }
__device__ __forceinline__ double to_double_dev(float x) { return (double)x; }
__device__ __forceinline__ double to_double_dev(float2 x) { return df_to_double(x); }

// cos, sin of the forcing phase Omega * t^{n+1}, t^{n+1} = dt*n + dt
// (src/timeIntegrator.cpp:218), for the steps first .. first+n-1, stored in
// the method's own number type; one thread per step, so no step's critical
// path carries a serial FP64 sincos.
template <class T>
__global__ void k_phase(T* out, long long first, int n, double dt, double angvel)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double t = dt * (double)(first + k) + dt;
    double s, c;
    sincos(angvel * t, &s, &c);
    out[2 * k] = from_double_dev<T>(c);
    out[2 * k + 1] = from_double_dev<T>(s);
}

void launch_phase(void* out, int precision, long long first, int n, double dt, double angvel, cudaStream_t s)
{
    const int nb = (n + 255) / 256;
    if (precision == ODIS_FP64) k_phase<double><<<nb, 256, 0, s>>>((double*)out, first, n, dt, angvel);
    else if (precision == ODIS_FP32) k_phase<float><<<nb, 256, 0, s>>>((float*)out, first, n, dt, angvel);
    else k_phase<float2><<<nb, 256, 0, s>>>((float2*)out, first, n, dt, angvel);
}

// ---------------------------------------------------------------------------
// per-operator kernels (the reference's free functions)
// ---------------------------------------------------------------------------
// updateMomentum (linear): dvdt = -g G eta + C v
__global__ void k_momentum(FaceCoef<double> fc, int E, int Ep, double* dvdt, const double* v, const double* eta)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    double t = 0.0;
#pragma unroll
    for (int k = 0; k < kTrisk; k++) t = fma(fc.w[k * Ep + e], v[fc.nbr[k * Ep + e]], t);
    dvdt[e] = fma(fc.cor[e], t, fma(fc.gg0[e], eta[fc.n0[e]], fc.gg1[e] * eta[fc.n1[e]]));
}

// updateEta (linear): detadt = h D v
__global__ void k_divergence(CellCoef<double> cc, int N, int Np, double* q, const double* v)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kCellFaces; k++) s = fma(cc.hw[k * Np + i], v[cc.edge[k * Np + i]], s);
    q[i] = s;
}

// forcing (src/tidalPotentials.cpp:29-334) at one time, from the node table
// trig[kNodeTrig][Np] and the time terms computed on the host
__global__ void k_forcing(const double* __restrict__ trig, int N, int Np, double* __restrict__ U, ForcingConst k,
                          ForcingTerms f)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    double tr[kNodeTrig];
#pragma unroll
    for (int q = 0; q < kNodeTrig; q++) tr[q] = trig[(size_t)q * Np + i];
    U[i] = forcing_node(k, f, tr);
}

// time terms of every step of a run: row k at t = dt (first + k) + dt
__global__ void k_forcing_terms(double* __restrict__ terms, ForcingConst k, long long first, int n, double dt)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const ForcingTerms f = forcing_terms(k, dt * (double)(first + q) + dt);
    const double* src = reinterpret_cast<const double*>(&f);
#pragma unroll
    for (int j = 0; j < kForcingTerms; j++) terms[(size_t)q * kForcingTerms + j] = src[j];
}

// the fused loop's nodal forcing (FULL2, PLANET, GENERAL): the potential at
// t^{n+1} over g, written (or added, after the self-gravity synthesis) into the
// node buffer whose gradient the face kernel adds to the momentum forcing
template <class T>
__global__ void __launch_bounds__(256) k_node_forcing(const double* __restrict__ trig, int N, int Np, T* __restrict__ usg,
                                                      int add, double inv_g, ForcingConst k,
                                                      const double* __restrict__ terms, const long long* iter,
                                                      const long long* run_first, int offset)
{
    pdl_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const long long kstep = *iter + offset - *run_first;
    ForcingTerms f;
    double* dst = reinterpret_cast<double*>(&f);
#pragma unroll
    for (int j = 0; j < kForcingTerms; j++) dst[j] = __ldg(&terms[(size_t)kstep * kForcingTerms + j]);
    double tr[kNodeTrig];
#pragma unroll
    for (int q = 0; q < kNodeTrig; q++) tr[q] = __ldg(&trig[(size_t)q * Np + i]);
    double u = forcing_node(k, f, tr) * inv_g;
    if (add) u += to_double_dev(usg[i]);
    usg[i] = from_double_dev<T>(u);
}

// integrateAB3scalar with the reference's [num][3] history layout
__global__ void k_ab3_ref(double* s, double* h, int iter, int num, double dt, int init_load)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= num) return;
    const double a = 23. / 12., b = -16. / 12., c = 5. / 12.;
    double* hi = h + (size_t)i * 3;
    if (iter > 1 || init_load) {
        s[i] += (a * hi[0] + b * hi[1] + c * hi[2]) * dt;
        hi[2] = hi[1];
        hi[1] = hi[0];
    } else if (iter == 0) {
        s[i] += hi[0] * dt;
        hi[2] = hi[0];
    } else if (iter == 1) {
        s[i] += hi[0] * dt;
        hi[1] = hi[0];
    }
}

// interpolateVelocity: uv[e] = n v_e + t v_t,e with t = (n_y, -n_x)
__global__ void k_interp(FaceCoef<double> fc, const double* nrm, int E, int Ep, double* uv, const double* v)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    double t = 0.0;
#pragma unroll
    for (int k = 0; k < kTrisk; k++) t = fma(fc.w[k * Ep + e], v[fc.nbr[k * Ep + e]], t);
    const double nx = nrm[e], ny = nrm[Ep + e];
    uv[2 * e] = nx * v[e] + ny * t;
    uv[2 * e + 1] = ny * v[e] + (-nx) * t;
}

// updateEnergy (LINEAR): e_i = alpha 1000 h |uv_i|^2, block partials of e_i * A_i
__global__ void __launch_bounds__(kStepThreads) k_energy_partial(const double* area, int E, double coef, int quad,
                                                                 const double* uv, double* e_out, double* partial)
{
    __shared__ double s_red[kStepThreads];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double x = 0.0;
    if (i < E) {
        const double u = uv[2 * i], w = uv[2 * i + 1];
        const double q = u * u + w * w;
        // src/energy.cpp:34 (LINEAR) and :48-49 (QUADRATIC, coef sqrt(q) q in the reference's order)
        const double ei = quad ? coef * sqrt(q) * q : coef * q;
        if (e_out) e_out[i] = ei;
        x = ei * area[i];
    }
    const double bs = block_sum<kStepThreads>(x, s_red);
    if (threadIdx.x == 0) partial[blockIdx.x] = bs;
}

// Cartesian velocity at the nodes from the face-normal velocities (RBF operator,
// per node a 3 x 6 block over its faces; missing pentagon entries are zero).
__global__ void k_rbf(const double* __restrict__ rbf, const int* __restrict__ edge, int N, int Np,
                      const double* __restrict__ v, double* __restrict__ uxyz)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    double vf[kCellFaces];
#pragma unroll
    for (int j = 0; j < kCellFaces; j++) vf[j] = v[__ldg(&edge[j * Np + i])];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        double u = 0.0;
#pragma unroll
        for (int j = 0; j < kCellFaces; j++) u = fma(__ldg(&rbf[(c * kCellFaces + j) * Np + i]), vf[j], u);
        uxyz[3 * i + c] = u;
    }
}

void launch_rbf(const double* rbf, const int* edge, int N, int Np, const double* v, double* uxyz, cudaStream_t s)
{
    k_rbf<<<(N + 255) / 256, 256, 0, s>>>(rbf, edge, N, Np, v, uxyz);
}

__global__ void k_fold(const double* partial, int n, double divisor, double* out)
{
    const double s = fold_partials(partial, n);
    if (threadIdx.x == 0) *out = s / divisor;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <class T, bool kMaster>
void launch_edge(const FaceCoef<T>& fc, const State<T>& st, const StepConst& sc, int offset, cudaStream_t s)
{
    if constexpr (kMaster) {
        if (sc.quad) pdl_launch(k_edge_step_f32x2<true>, face_blocks(sc, true), kStepThreads, 0, s, fc, st, sc, offset);
        else pdl_launch(k_edge_step_f32x2<false>, face_blocks(sc, true), kStepThreads, 0, s, fc, st, sc, offset);
    } else {
        if (sc.quad) pdl_launch(k_edge_step<T, kMaster, true>, face_blocks(sc, false), kStepThreads, 0, s, fc, st, sc, offset);
        else pdl_launch(k_edge_step<T, kMaster, false>, face_blocks(sc, false), kStepThreads, 0, s, fc, st, sc, offset);
    }
}

int face_blocks(const StepConst& sc, bool pairs)
{
    const int n = pairs ? (sc.E + 1) / 2 : sc.E;
    return (n + kStepThreads - 1) / kStepThreads;
}

template <class T, bool kMaster>
void launch_cell(const CellCoef<T>& cc, const State<T>& st, const StepConst& sc, int offset, cudaStream_t s)
{
    const int cb = (sc.N + kStepThreads - 1) / kStepThreads;
    pdl_launch(k_cell_step<T, kMaster>, cb, kStepThreads, 0, s, cc, st, sc, offset);
}

template <class T, bool kMaster>
void launch_step(const FaceCoef<T>& fc, const CellCoef<T>& cc, const State<T>& st, const StepConst& sc,
                 int offset, cudaStream_t s)
{
    launch_edge<T, kMaster>(fc, st, sc, offset, s);
    launch_cell<T, kMaster>(cc, st, sc, offset, s);
}

template <class T>
void launch_power_tail(const FaceCoef<T>& fc, const State<T>& st, const StepConst& sc, int n, cudaStream_t s)
{
    constexpr bool pairs = std::is_same<T, float>::value;
    const int eb = face_blocks(sc, pairs);
    if constexpr (pairs) k_power_partial_f32x2<<<eb, kStepThreads, 0, s>>>(fc, st, sc);
    else k_power_partial<T><<<eb, kStepThreads, 0, s>>>(fc, st, sc);
    launch_power_fold(st.partial, eb, n, st.power, s);
}

void launch_power_fold(const double* part, int nb, int n, double* power, cudaStream_t s)
{
    if (!power || n <= 0) return;
    k_power_fold<<<(n * 32 + 255) / 256, 256, 0, s>>>(part, nb, n, power);
}

void launch_bump(long long* iter, int n, cudaStream_t s) { k_bump_iter<<<1, 32, 0, s>>>(iter, n); }

template void launch_edge<double, false>(const FaceCoef<double>&, const State<double>&, const StepConst&, int, cudaStream_t);
template void launch_edge<float, true>(const FaceCoef<float>&, const State<float>&, const StepConst&, int, cudaStream_t);
template void launch_cell<double, false>(const CellCoef<double>&, const State<double>&, const StepConst&, int, cudaStream_t);
template void launch_cell<float, true>(const CellCoef<float>&, const State<float>&, const StepConst&, int, cudaStream_t);
template void launch_step<double, false>(const FaceCoef<double>&, const CellCoef<double>&, const State<double>&,
                                         const StepConst&, int, cudaStream_t);
template void launch_step<float, true>(const FaceCoef<float>&, const CellCoef<float>&, const State<float>&,
                                       const StepConst&, int, cudaStream_t);
template void launch_power_tail<double>(const FaceCoef<double>&, const State<double>&, const StepConst&, int, cudaStream_t);
template void launch_power_tail<float>(const FaceCoef<float>&, const State<float>&, const StepConst&, int, cudaStream_t);

static inline int blocks(int n, int t) { return (n + t - 1) / t; }

void launch_momentum(const FaceCoef<double>& fc, int E, int Ep, double* dvdt, const double* v, const double* eta, cudaStream_t s)
{ k_momentum<<<blocks(E, 256), 256, 0, s>>>(fc, E, Ep, dvdt, v, eta); }

void launch_divergence(const CellCoef<double>& cc, int N, int Np, double* q, const double* v, cudaStream_t s)
{ k_divergence<<<blocks(N, 256), 256, 0, s>>>(cc, N, Np, q, v); }

void launch_forcing(const double* trig, int N, int Np, double* U, const ForcingConst& k, const ForcingTerms& f,
                    cudaStream_t s)
{ k_forcing<<<blocks(N, 256), 256, 0, s>>>(trig, N, Np, U, k, f); }

void launch_forcing_terms(double* terms, const ForcingConst& k, long long first, int n, double dt, cudaStream_t s)
{ k_forcing_terms<<<blocks(n, 128), 128, 0, s>>>(terms, k, first, n, dt); }

void launch_node_forcing(int precision, const double* trig, int N, int Np, void* usg, int add, double inv_g,
                         const ForcingConst& k, const double* terms, const long long* iter, const long long* run_first,
                         int offset, cudaStream_t s)
{
    const int nb = blocks(N, 256);
    if (precision == ODIS_FP64)
        pdl_launch(k_node_forcing<double>, nb, 256, 0, s, trig, N, Np, (double*)usg, add, inv_g, k, terms, iter, run_first, offset);
    else if (precision == ODIS_FP32)
        pdl_launch(k_node_forcing<float>, nb, 256, 0, s, trig, N, Np, (float*)usg, add, inv_g, k, terms, iter, run_first, offset);
    else
        pdl_launch(k_node_forcing<float2>, nb, 256, 0, s, trig, N, Np, (float2*)usg, add, inv_g, k, terms, iter, run_first, offset);
}

void launch_ab3_ref(double* x, double* h, int iter, int num, double dt, int init_load, cudaStream_t s)
{ k_ab3_ref<<<blocks(num, 256), 256, 0, s>>>(x, h, iter, num, dt, init_load); }

void launch_interp(const FaceCoef<double>& fc, const double* nrm, int E, int Ep, double* uv, const double* v, cudaStream_t s)
{ k_interp<<<blocks(E, 256), 256, 0, s>>>(fc, nrm, E, Ep, uv, v); }

int energy_blocks(int E) { return blocks(E, kStepThreads); }

void launch_energy(const double* area, int E, double coef, int quad, double divisor, const double* uv, double* e_out,
                   double* partial, double* out, cudaStream_t s)
{
    const int nb = energy_blocks(E);
    k_energy_partial<<<nb, kStepThreads, 0, s>>>(area, E, coef, quad, uv, e_out, partial);
    k_fold<<<1, 32, 0, s>>>(partial, nb, divisor, out);
}

}  // namespace odis
