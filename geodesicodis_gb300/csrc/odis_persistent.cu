// Persistent time loop: a whole run of n LTE steps in one cooperative launch.
//
// One CTA per SM owns a contiguous range of faces and of cells (the mesh is
// numbered along a space-filling walk, so a range is a compact patch of the
// sphere).  For the whole run the CTA keeps in shared memory the
// coefficients of its faces and cells, their AB3 histories, and its own v
// (both time levels) and eta.  Gathers of values the CTA owns are served from
// shared memory; only values owned by other CTAs go through L2.
//
// Each CTA orders its faces and cells interior first: an interior face reads
// only faces and cells of its own CTA (and, by the symmetry of the TRiSK and
// face-cell relations, is read by no other CTA), so it is computed without
// waiting for anyone and is written to global memory only at the end of the
// run.  Boundary faces and cells wait for their producers:
//   * after its face phase of step s a CTA publishes flag_e = s+1, after its
//     cell phase flag_c = s+1 (CTA barrier, then one thread fences and stores
//     with release semantics, as a grid barrier does);
//   * before its boundary faces of step s a CTA waits for flag_c >= s of the
//     CTAs in set A (owners of the faces and cells its faces read), before its
//     boundary cells for flag_e >= s+1 of set C (owners of its cells' faces).
// The same sets cover the write-after-read hazards on the double-buffered v
// and the in-place eta, because the read relations are symmetric.  Every wait
// is bounded: after kSpinLimitDefault polls (or the plan's spin_limit) the CTA records ODIS_ERR_TIMEOUT and
// leaves the loop, so no CTA waits forever.  Values other CTAs write during the
// run are read with ld.global.cg (L2, never a stale L1 line).
#include "../../include/odis_gpu.h"
#include "odis_arith.cuh"
#include "odis_device.cuh"
#include "odis_kernels.cuh"
#include "odis_persistent.cuh"

namespace odis {

namespace {

constexpr unsigned kSpinLimitDefault = 1u << 22;   // polls of one wait (about a second with the back-off)

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Wait until flags[dep[q]] >= target for every dependency q; false on timeout.
__device__ bool wait_deps(const unsigned* flags, const int* dep, int nd, unsigned target, int* status,
                          unsigned limit)
{
    const unsigned lim = limit ? limit : kSpinLimitDefault;
    bool ok = true;
    for (int q = threadIdx.x; q < nd; q += blockDim.x) {
        const unsigned* f = flags + dep[q];
        unsigned spins = 0;
        while (ld_acquire_u32(f) < target) {
            if (++spins > lim) {
                atomicOr(status, 1 << ODIS_ERR_TIMEOUT);
                ok = false;
                break;
            }
            if (spins > 32) __nanosleep(32);
        }
    }
    return __syncthreads_and(ok) != 0;
}

// CTA barrier, then one thread publishes v with a GPU-scope release: the barrier
// orders the CTA's writes before it, and the release is cumulative over them.
// A withheld CTA (test hook) skips the store, so the waits on it run out.
__device__ __forceinline__ void signal(unsigned* flag, unsigned v, bool withheld)
{
    __syncthreads();
    if (threadIdx.x == 0 && !withheld) st_release_u32(flag, v);
}

template <class T>
__device__ T block_sum_t(T x, T* red)
{
    using A = Ar<T>;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = A::add(x, A::shfl(x, o));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) red[wid] = x;
    __syncthreads();
    T s = A::zero();
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s = A::add(s, red[w]);
    return s;
}


// one face of step s: TRiSK tangential velocity, dissipation partial, momentum
// tendency, forcing gradient, drag and the AB3 update (the same arithmetic, in
// the same order, as k_edge_step)
template <class T>
struct FaceCtx {
    const T *sw, *sgg0, *sgg1, *scor, *sfp, *sfq, *sdiss, *svi, *seta;
    const int *snbr, *sn0, *sn1, *sface;
    T *hcur, *svo;
    const T *hold;
    const T* vin;
    T* vout;
    const T* eta;
    T cosM, sinM, malpha, ca, cb, cc3, dt;
    int NF, nfi;
    int quad;           // QUADRATIC friction
    bool ab3;
    int* status;
};

template <class T>
__device__ __forceinline__ void face_update(const FaceCtx<T> f, int lf, T& pw)
{
    using A = Ar<T>;
    const int NF = f.NF;
    T tsum = A::zero();
#pragma unroll
    for (int k = 0; k < kTrisk; k++) {
        const int c = f.snbr[k * NF + lf];
        tsum = A::fma(f.sw[k * NF + lf], c >= 0 ? f.svi[c] : A::ldcg(&f.vin[-1 - c]), tsum);
    }
    const T ve = f.svi[lf];
    pw = A::add(pw, face_diss(f.sdiss[lf], A::fma(ve, ve, A::mul(tsum, tsum)), f.quad));
    const int c0 = f.sn0[lf], c1 = f.sn1[lf];
    const T e0 = c0 >= 0 ? f.seta[c0] : A::ldcg(&f.eta[-1 - c0]);
    const T e1 = c1 >= 0 ? f.seta[c1] : A::ldcg(&f.eta[-1 - c1]);
    const T f0 = A::fma(f.scor[lf], tsum, A::fma(f.sgg0[lf], e0, A::mul(f.sgg1[lf], e1)));
    const T gu = A::fma(f.cosM, f.sfp[lf], A::mul(f.sinM, f.sfq[lf]));
    const T drag = A::fma(f.malpha, ve, gu);
    T inc = f0;
    if (f.ab3) inc = A::fma(f.cc3, f.hcur[lf], A::fma(f.cb, f.hold[lf], A::mul(f.ca, f0)));
    f.hcur[lf] = f0;
    T vn = A::fma(inc, f.dt, ve);
    vn = A::fma(f.dt, drag, vn);
    f.svo[lf] = vn;
    if (lf >= f.nfi) A::stcg(&f.vout[f.sface[lf]], vn);     // boundary faces are read by other CTAs
    if (!A::finite(vn)) atomicOr(f.status, 1 << ODIS_ERR_NONFINITE);
}

// one cell of step s: h D v^{n+1} and the AB3 update of eta
template <class T>
struct CellCtx {
    const T *shw, *svo, *ho;
    T *hc, *seta;
    const int *sedge, *scell;
    const T* vout;
    T* eta;
    T ca, cb, cc3, dt;
    int NC, nci;
    bool ab3;
};

template <class T>
__device__ __forceinline__ void cell_update(const CellCtx<T> c, int lc)
{
    using A = Ar<T>;
    const int NC = c.NC;
    T q = A::zero();
#pragma unroll
    for (int k = 0; k < kCellFaces; k++) {
        const int x = c.sedge[k * NC + lc];
        q = A::fma(c.shw[k * NC + lc], x >= 0 ? c.svo[x] : A::ldcg(&c.vout[-1 - x]), q);
    }
    T inc = q;
    if (c.ab3) inc = A::fma(c.cc3, c.hc[lc], A::fma(c.cb, c.ho[lc], A::mul(c.ca, q)));
    c.hc[lc] = q;
    const T en = A::fma(inc, c.dt, c.seta[lc]);
    c.seta[lc] = en;
    if (lc >= c.nci) A::stcg(&c.eta[c.scell[lc]], en);
}

template <class T>
__global__ void __launch_bounds__(kPersistThreads) k_persistent(FaceCoef<T> fc, CellCoef<T> cc, State<T> st, StepConst sc,
                                                                PersistPlan pl, int n, long long first)
{
    using A = Ar<T>;
    extern __shared__ __align__(16) unsigned char smem[];
    const int b = blockIdx.x, P = gridDim.x;
    const int fs = pl.fstart[b], nf = pl.fstart[b + 1] - fs, nfi = pl.fint[b];
    const int cs = pl.cstart[b], nc = pl.cstart[b + 1] - cs, nci = pl.cint[b];
    const int NF = pl.nf_max, NC = pl.nc_max;
    // shared layout: T arrays first, then int arrays
    T* sw = reinterpret_cast<T*>(smem);                 // [10][NF]
    T* sgg0 = sw + kTrisk * NF;
    T* sgg1 = sgg0 + NF;
    T* scor = sgg1 + NF;
    T* sfp = scor + NF;
    T* sfq = sfp + NF;
    T* sdiss = sfq + NF;
    T* shv = sdiss + NF;                                // [2][NF] AB3 history of v
    T* sv = shv + 2 * NF;                               // [2][NF] own v, both time levels
    T* shw = sv + 2 * NF;                               // [6][NC]
    T* she = shw + kCellFaces * NC;                     // [2][NC] AB3 history of eta
    T* seta = she + 2 * NC;                             // [NC] own eta
    T* red = seta + NC;                                 // [warps]
    int* snbr = reinterpret_cast<int*>(red + kPersistThreads / 32);   // [10][NF] codes
    int* sn0 = snbr + kTrisk * NF;                      // codes of the end cells
    int* sn1 = sn0 + NF;
    int* sface = sn1 + NF;                              // global face id
    int* sedge = sface + NF;                            // [6][NC] codes of the cell faces
    int* scell = sedge + kCellFaces * NC;               // global cell id
    // a code c >= 0 is a position in this CTA's shared arrays, c < 0 the global index -1-c

    const int Ep = sc.Ep, Np = sc.Np;
    for (int lf = threadIdx.x; lf < nf; lf += blockDim.x) {
        const int e = pl.forder[fs + lf];
        sface[lf] = e;
        for (int k = 0; k < kTrisk; k++) {
            sw[k * NF + lf] = fc.w[k * Ep + e];
            const int f = fc.nbr[k * Ep + e];
            snbr[k * NF + lf] = pl.fowner[f] == b ? pl.fpos[f] : -1 - f;
        }
        sgg0[lf] = fc.gg0[e]; sgg1[lf] = fc.gg1[e]; scor[lf] = fc.cor[e];
        sfp[lf] = fc.fP[e]; sfq[lf] = fc.fQ[e]; sdiss[lf] = fc.diss[e];
        const int i0 = fc.n0[e], i1 = fc.n1[e];
        sn0[lf] = pl.cowner[i0] == b ? pl.cpos[i0] : -1 - i0;
        sn1[lf] = pl.cowner[i1] == b ? pl.cpos[i1] : -1 - i1;
        shv[lf] = st.hv[0][e];
        shv[NF + lf] = st.hv[1][e];
        sv[lf] = st.v[0][e];
        sv[NF + lf] = st.v[1][e];
    }
    for (int lc = threadIdx.x; lc < nc; lc += blockDim.x) {
        const int i = pl.corder[cs + lc];
        scell[lc] = i;
        for (int k = 0; k < kCellFaces; k++) {
            shw[k * NC + lc] = cc.hw[k * Np + i];
            const int f = cc.edge[k * Np + i];
            sedge[k * NC + lc] = pl.fowner[f] == b ? pl.fpos[f] : -1 - f;
        }
        she[lc] = st.he[0][i];
        she[NC + lc] = st.he[1][i];
        seta[lc] = st.eta[i];
    }
    __syncthreads();

    const int* depA = pl.depA + pl.depA_ptr[b];
    const int ndA = pl.depA_ptr[b + 1] - pl.depA_ptr[b];
    const int* depC = pl.depC + pl.depC_ptr[b];
    const int ndC = pl.depC_ptr[b + 1] - pl.depC_ptr[b];
    const T dt = A::from(sc.dt);
    const T malpha = A::from(-sc.alpha);
    const T ca = A::from(sc.ab3a), cb = A::from(sc.ab3b), cc3 = A::from(sc.ab3c);
    T* part = reinterpret_cast<T*>(pl.part);
    bool ok = true;
    for (int s = 0; s < n; s++) {
        const long long it = first + s;
        const int bi = (int)(it & 1), bo = (int)((it + 1) & 1);
        const T* vin = (bi ? st.v[1] : st.v[0]);
        T* vout = (bo ? st.v[1] : st.v[0]);
        const T* svi = sv + bi * NF;
        T* svo = sv + bo * NF;
        const T cosM = st.phase[2 * s], sinM = st.phase[2 * s + 1];
        const bool ab3 = sc.init_load || it > 1;
        T* hcur = shv + bi * NF;
        const T* hold = shv + bo * NF;
        T pw = A::zero();
        FaceCtx<T> fx;
        fx.sw = sw; fx.sgg0 = sgg0; fx.sgg1 = sgg1; fx.scor = scor; fx.sfp = sfp; fx.sfq = sfq; fx.sdiss = sdiss;
        fx.svi = svi; fx.seta = seta; fx.snbr = snbr; fx.sn0 = sn0; fx.sn1 = sn1; fx.sface = sface;
        fx.hcur = hcur; fx.svo = svo; fx.hold = hold; fx.vin = vin; fx.vout = vout; fx.eta = st.eta;
        fx.cosM = cosM; fx.sinM = sinM; fx.malpha = malpha; fx.ca = ca; fx.cb = cb; fx.cc3 = cc3; fx.dt = dt;
        fx.NF = NF; fx.nfi = nfi; fx.quad = sc.quad; fx.ab3 = ab3; fx.status = st.status;
        for (int lf = threadIdx.x; lf < nfi; lf += blockDim.x) face_update<T>(fx, lf, pw);
        if (s > 0 && !wait_deps(pl.flag_c, depA, ndA, (unsigned)s, st.status, pl.spin_limit)) { ok = false; break; }
        for (int lf = nfi + threadIdx.x; lf < nf; lf += blockDim.x) face_update<T>(fx, lf, pw);
        const T bs = block_sum_t<T>(pw, red);
        if (threadIdx.x == 0) part[(size_t)s * P + b] = bs;
        signal(&pl.flag_e[b], (unsigned)(s + 1), b == pl.withhold);

        CellCtx<T> cx;
        cx.shw = shw; cx.svo = svo; cx.ho = she + bo * NC; cx.hc = she + bi * NC; cx.seta = seta;
        cx.sedge = sedge; cx.scell = scell; cx.vout = vout; cx.eta = st.eta;
        cx.ca = ca; cx.cb = cb; cx.cc3 = cc3; cx.dt = dt; cx.NC = NC; cx.nci = nci; cx.ab3 = ab3;
        for (int lc = threadIdx.x; lc < nci; lc += blockDim.x) cell_update<T>(cx, lc);
        if (!wait_deps(pl.flag_e, depC, ndC, (unsigned)(s + 1), st.status, pl.spin_limit)) { ok = false; break; }
        for (int lc = nci + threadIdx.x; lc < nc; lc += blockDim.x) cell_update<T>(cx, lc);
        signal(&pl.flag_c[b], (unsigned)(s + 1), b == pl.withhold);
    }
    // dissipation of the final state (power of the run's last step)
    if (ok && wait_deps(pl.flag_e, depA, ndA, (unsigned)n, st.status, pl.spin_limit)) {
        const int bf = (int)((first + n) & 1);
        const T* vin = (bf ? st.v[1] : st.v[0]);
        const T* svi = sv + bf * NF;
        T pw = A::zero();
        for (int lf = threadIdx.x; lf < nf; lf += blockDim.x) {
            T tsum = A::zero();
#pragma unroll
            for (int k = 0; k < kTrisk; k++) {
                const int c = snbr[k * NF + lf];
                tsum = A::fma(sw[k * NF + lf], c >= 0 ? svi[c] : A::ldcg(&vin[-1 - c]), tsum);
            }
            const T ve = svi[lf];
            pw = A::add(pw, face_diss(sdiss[lf], A::fma(ve, ve, A::mul(tsum, tsum)), sc.quad));
        }
        const T bs = block_sum_t<T>(pw, red);
        if (threadIdx.x == 0) part[(size_t)n * P + b] = bs;
    }
    // own state back to global memory (the next launch or odis_get_state reads it)
    __syncthreads();
    for (int lf = threadIdx.x; lf < nf; lf += blockDim.x) {
        const int e = sface[lf];
        st.hv[0][e] = shv[lf];
        st.hv[1][e] = shv[NF + lf];
        st.v[0][e] = sv[lf];
        st.v[1][e] = sv[NF + lf];
    }
    for (int lc = threadIdx.x; lc < nc; lc += blockDim.x) {
        const int i = scell[lc];
        st.he[0][i] = she[lc];
        st.he[1][i] = she[NC + lc];
        st.eta[i] = seta[lc];
    }
}

// power[k] = sum over CTAs of the dissipation partials of the state after step k
template <class T>
__global__ void k_persist_fold(const T* __restrict__ part, int P, int n, double* __restrict__ power)
{
    using A = Ar<T>;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || !power) return;
    const T* row = part + (size_t)(k + 1) * P;
    T s = A::zero();
    for (int b = 0; b < P; b++) s = A::add(s, row[b]);
    power[k] = A::to(s);
}

}  // namespace

size_t persist_smem_bytes(int value_bytes, int nf_max, int nc_max)
{
    const size_t t = (size_t)value_bytes * ((size_t)(kTrisk + 6 + 4) * nf_max + (size_t)(kCellFaces + 3) * nc_max +
                                            kPersistThreads / 32);
    const size_t ints = sizeof(int) * ((size_t)(kTrisk + 3) * nf_max + (size_t)(kCellFaces + 1) * nc_max);
    return t + ints;
}

template <class T>
static int launch_persistent_t(const FaceCoef<T>& fc, const CellCoef<T>& cc, const State<T>& st, const StepConst& sc,
                               const PersistPlan& pl, int n, long long first, double* power, cudaStream_t s)
{
    const size_t smem = persist_smem_bytes((int)sizeof(T), pl.nf_max, pl.nc_max);
    if (cudaFuncSetAttribute(k_persistent<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return ODIS_ERR_CUDA;
    FaceCoef<T> a0 = fc;
    CellCoef<T> a1 = cc;
    State<T> a2 = st;
    StepConst a3 = sc;
    PersistPlan a4 = pl;
    int a5 = n;
    long long a6 = first;
    void* args[] = {&a0, &a1, &a2, &a3, &a4, &a5, &a6};
    if (cudaMemsetAsync(pl.flag_e, 0, sizeof(unsigned) * pl.P, s) != cudaSuccess) return ODIS_ERR_CUDA;
    if (cudaMemsetAsync(pl.flag_c, 0, sizeof(unsigned) * pl.P, s) != cudaSuccess) return ODIS_ERR_CUDA;
    if (cudaLaunchCooperativeKernel((const void*)k_persistent<T>, dim3(pl.P), dim3(kPersistThreads), args, smem, s) !=
        cudaSuccess)
        return ODIS_ERR_CUDA;
    k_persist_fold<T><<<(n + 127) / 128, 128, 0, s>>>((const T*)pl.part, pl.P, n, power);
    return cudaGetLastError() == cudaSuccess ? ODIS_OK : ODIS_ERR_CUDA;
}

int launch_persistent(int precision, const void* fc, const void* cc, const void* st, const StepConst& sc,
                      const PersistPlan& pl, int n, long long first, double* power, cudaStream_t s)
{
    if (precision == ODIS_FP64)
        return launch_persistent_t<double>(*(const FaceCoef<double>*)fc, *(const CellCoef<double>*)cc,
                                           *(const State<double>*)st, sc, pl, n, first, power, s);
    if (precision == ODIS_DF64)
        return launch_persistent_t<df64>(*(const FaceCoef<df64>*)fc, *(const CellCoef<df64>*)cc,
                                         *(const State<df64>*)st, sc, pl, n, first, power, s);
    return ODIS_ERR_ARG;
}

int persistent_fits(int precision, const PersistPlan& pl, int* max_blocks_per_sm)
{
    const int vb = precision == ODIS_FP64 ? (int)sizeof(double) : (int)sizeof(df64);
    const size_t smem = persist_smem_bytes(vb, pl.nf_max, pl.nc_max);
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (smem > (size_t)optin) return 0;
    int nb = 0;
    if (precision == ODIS_FP64) {
        cudaFuncSetAttribute(k_persistent<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_persistent<double>, kPersistThreads, smem);
    } else {
        cudaFuncSetAttribute(k_persistent<df64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_persistent<df64>, kPersistThreads, smem);
    }
    if (max_blocks_per_sm) *max_blocks_per_sm = nb;
    return nb >= 1 ? 1 : 0;
}

}  // namespace odis
