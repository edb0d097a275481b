// Step kernels of the ODIS_DF64 method: the FP64 time loop of
// src/timeIntegrator.cpp:205-272 (linear branch) evaluated in double-float
// arithmetic on the FP32 pipes (odis_df64.cuh).  Same data flow as the FP64
// kernels of odis_kernels.cu -- face kernel (TRiSK tangential velocity,
// dissipation of v^n, -g G eta + C v, forcing gradient, drag, AB3) then cell
// kernel (h D v^{n+1}, AB3) -- with every coefficient and state value stored as
// a float2 (hi, lo) pair: one 8-byte load per value, as for FP64.
#include "../../include/odis_gpu.h"
#include "odis_device.cuh"
#include "odis_df64.cuh"
#include "odis_kernels.cuh"
#include "odis_pdl.cuh"

namespace odis {

namespace {

// block sum of a df64 per thread; the result (as FP64) is valid in thread 0.
// Every thread parks its term in shared memory (smem: kStepThreads values) and
// warp 0 adds them, eight per lane then a shuffle tree: 12 double-float
// additions a block instead of a 5-step shuffle tree in every warp.
__device__ __forceinline__ double block_sum_df(df64 x, df64* smem)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    smem[threadIdx.x] = x;
    __syncthreads();
    df64 s = df_make(0.f, 0.f);
    if (wid == 0) {
        s = smem[lane];
#pragma unroll
        for (int r = 1; r < kStepThreads / 32; r++) s = df_add(s, smem[lane + 32 * r]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s = df_add(s, df_shfl_down(s, o));
    }
    return df_to_double(s);
}

__device__ __forceinline__ df64 ldg2(const df64* p) { return __ldg(p); }

}  // namespace

template <bool kQuad>   // QUADRATIC friction, a compile-time switch as in k_edge_step
__global__ void __launch_bounds__(kStepThreads) k_edge_step_df(FaceCoef<df64> fc, State<df64> st, StepConst sc, int offset)
{
    pdl_wait();
    __shared__ df64 s_red[kStepThreads];
    const long long it = *st.iter + offset;
    const long long kstep = it - *st.run_first;        // forcing phase at t^{n+1}, precomputed per run
    const df64 cosM = st.phase[2 * kstep], sinM = st.phase[2 * kstep + 1];
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const int Ep = sc.Ep;
    const df64* __restrict__ vin = ((it & 1) ? st.v[1] : st.v[0]);
    df64 pw = df_make(0.f, 0.f);
    if (e < sc.E) {
        df64 tsum = df_make(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < kTrisk; k++) tsum = df_fma(ldg2(&fc.w[k * Ep + e]), vin[__ldg(&fc.nbr[k * Ep + e])], tsum);
        const df64 ve = vin[e];
        const int i0 = __ldg(&fc.n0[e]), i1 = __ldg(&fc.n1[e]);
        pw = face_diss(ldg2(&fc.diss[e]), df_fma(ve, ve, df_mul(tsum, tsum)), kQuad);
        const df64 g0 = ldg2(&fc.gg0[e]), g1 = ldg2(&fc.gg1[e]);
        const df64 f0 = df_fma(ldg2(&fc.cor[e]), tsum, df_fma(g0, st.eta[i0], df_mul(g1, st.eta[i1])));
        df64 gu = df_fma(cosM, ldg2(&fc.fP[e]), df_mul(sinM, ldg2(&fc.fQ[e])));
        if (sc.use_sg) gu = df_sub(gu, df_fma(g0, st.usg[i0], df_mul(g1, st.usg[i1])));
        const df64 drag = df_fma(sc.df_malpha, ve, gu);
        df64* hcur = ((it & 1) ? st.hv[1] : st.hv[0]);
        df64 inc = f0;
        if (sc.init_load || it > 1) {
            const df64 f1 = ((it & 1) ? st.hv[0] : st.hv[1])[e];
            const df64 f2 = hcur[e];
            inc = df_fma(sc.df_c, f2, df_fma(sc.df_b, f1, df_mul(sc.df_a, f0)));
        }
        hcur[e] = f0;
        df64 vn = df_fma(inc, sc.df_dt, ve);
        vn = df_fma(sc.df_dt, drag, vn);
        ((it & 1) ? st.v[0] : st.v[1])[e] = vn;
        if (!df_finite(vn)) atomicOr(st.status, 1 << ODIS_ERR_NONFINITE);
    }
    const double bs = block_sum_df(pw, s_red);
    // row kstep of the run's partial table: the dissipation of v^it, the power after step it-1
    if (threadIdx.x == 0) st.partial[kstep * gridDim.x + blockIdx.x] = bs;
}

__global__ void __launch_bounds__(kStepThreads) k_cell_step_df(CellCoef<df64> cc, State<df64> st, StepConst sc, int offset)
{
    pdl_wait();
    const long long it = *st.iter + offset;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int Np = sc.Np;
    const df64* __restrict__ vn = ((it & 1) ? st.v[0] : st.v[1]);
    if (i < sc.N) {
        df64 q = df_make(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < kCellFaces; k++) q = df_fma(ldg2(&cc.hw[k * Np + i]), vn[__ldg(&cc.edge[k * Np + i])], q);
        df64* hcur = ((it & 1) ? st.he[1] : st.he[0]);
        df64 inc = q;
        if (sc.init_load || it > 1) {
            const df64 f1 = ((it & 1) ? st.he[0] : st.he[1])[i];
            const df64 f2 = hcur[i];
            inc = df_fma(sc.df_c, f2, df_fma(sc.df_b, f1, df_mul(sc.df_a, q)));
        }
        hcur[i] = q;
        st.eta[i] = df_fma(inc, sc.df_dt, st.eta[i]);
    }
}

__global__ void __launch_bounds__(kStepThreads) k_power_partial_df(FaceCoef<df64> fc, State<df64> st, StepConst sc)
{
    __shared__ df64 s_red[kStepThreads];
    const long long it = *st.iter;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const int Ep = sc.Ep;
    const df64* __restrict__ vin = ((it & 1) ? st.v[1] : st.v[0]);
    df64 pw = df_make(0.f, 0.f);
    if (e < sc.E) {
        df64 tsum = df_make(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < kTrisk; k++) tsum = df_fma(ldg2(&fc.w[k * Ep + e]), vin[__ldg(&fc.nbr[k * Ep + e])], tsum);
        const df64 ve = vin[e];
        pw = face_diss(ldg2(&fc.diss[e]), df_fma(ve, ve, df_mul(tsum, tsum)), sc.quad);
    }
    const double bs = block_sum_df(pw, s_red);
    if (threadIdx.x == 0) st.partial[(it - *st.run_first) * gridDim.x + blockIdx.x] = bs;
}

void launch_edge_df(const FaceCoef<df64>& fc, const State<df64>& st, const StepConst& sc, int offset, cudaStream_t s)
{
    const int eb = (sc.E + kStepThreads - 1) / kStepThreads;
    if (sc.quad) pdl_launch(k_edge_step_df<true>, eb, kStepThreads, 0, s, fc, st, sc, offset);
    else pdl_launch(k_edge_step_df<false>, eb, kStepThreads, 0, s, fc, st, sc, offset);
}

void launch_cell_df(const CellCoef<df64>& cc, const State<df64>& st, const StepConst& sc, int offset, cudaStream_t s)
{
    const int cb = (sc.N + kStepThreads - 1) / kStepThreads;
    pdl_launch(k_cell_step_df, cb, kStepThreads, 0, s, cc, st, sc, offset);
}

void launch_power_tail_df(const FaceCoef<df64>& fc, const State<df64>& st, const StepConst& sc, int n, cudaStream_t s)
{
    const int eb = (sc.E + kStepThreads - 1) / kStepThreads;
    k_power_partial_df<<<eb, kStepThreads, 0, s>>>(fc, st, sc);
    launch_power_fold(st.partial, eb, n, st.power, s);
}

}  // namespace odis
