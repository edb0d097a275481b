// Nonlinear momentum advection (calculateMomentumAdvection, src/momAdvection.cpp:11-267)
// and the advective time step on the device.  The kernels are templated on the
// method's number type through the Ar<T> policies: double (ODIS_FP64, and every
// per-operator call) or the double-float pair df64 (ODIS_DF64: the same
// arithmetic on the FP32 pipes, whose issue rate on GB300 is about 64 times the
// FP64 one).
//
// Per momentum-advection call (odis_momentum_advection):
//   k_adv_pv     per vertex: relative vorticity from the curl of v (three faces,
//                ascending face order), thickness at the vertex from the three
//                nodes' thicknesses weighted by control-volume area x kite
//                fraction over the vertex area (Ringler et al. 2010 eq. 25, the
//                weights premultiplied per vertex), potential vorticity q = (zeta + f) / h
//   k_adv_edge   per face: q averaged from the face's two vertices, the thickness
//                flux h_e v_e with h_e averaged from its two nodes, and h_e v_e q_e
//   k_adv_node   per node: kinetic energy from the RBF Cartesian velocity
//   k_adv_flux   per face: dvdt -= -sum_j w_j l_j / d_e (h_j v_j) (q_e + q_j) / 2
//                (eq. 49), as (q_e sum_j c_j (h v)_j + sum_j c_j (h v q)_j) / 2 with
//                c_j = w_j l_j / d_e (the TRiSK table), then dvdt += -(G KE)_e
// Products are fused into the sums (in FP64 the loop is bound by GB300's FP64
// issue rate), so the results match the FP64 restatement to rounding, not bit
// for bit.  The AB3 histories are slot-outermost on the device ([3][n]);
// adv_get_state / adv_set_state convert to and from the reference's [n][3].
//
// One step of the advective loop (src/timeIntegrator.cpp:205-269) is seven kernels:
//   k_adv_pv, k_adv_edge
//   k_adv_node         also the forcing U at the nodes for this step's phase
//   k_adv_flux<true>   dvdt starts from -g (G eta)_e
//   k_adv_vstep        drag, G U, AB3 of v
//   k_adv_lsq_power    interpolateLSQFlux of h + eta, then updateEnergy of the new
//                      v (tangential velocity, e_i A_i block partials); the last
//                      block to finish folds the partials in a fixed order
//   k_adv_estep        D flux, AB3 of eta, h + eta for the next step; one extra
//                      block advances the step counter and the next forcing phase
#include "odis_advection.cuh"
#include "odis_arith.cuh"
#include "odis_kernels.cuh"
#include "odis_pdl.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <type_traits>
#include <vector>

namespace odis {

namespace {

constexpr int kAdvThreads = 256;        // largest block; k_adv_lsq_power's reduction is sized for it
constexpr int kAdvGraphSteps = 64;      // steps per captured graph of the advective loop

__device__ __forceinline__ double adv_warp_sum(double x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    return x;
}



// vwt[j][i] = A_n R_j / A_v: the node's control-volume area times the kite
// fraction over the vertex area, so that h_v = sum_j vwt_j h_n
template <class T>
__global__ void k_adv_pv(const int* __restrict__ vface, const T* __restrict__ vcoef, const int* __restrict__ vnode,
                         const T* __restrict__ vwt, const T* __restrict__ vf, int V, int Vp, const T* __restrict__ v,
                         const T* __restrict__ h, T* __restrict__ q)
{
    using A = Ar<T>;
    pdl_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    T zeta = A::zero(), th = A::zero();
#pragma unroll
    for (int j = 0; j < 3; j++) {
        zeta = A::fma(vcoef[j * Vp + i], v[vface[j * Vp + i]], zeta);
        th = A::fma(h[vnode[j * Vp + i]], vwt[j * Vp + i], th);
    }
    q[i] = A::div(A::add(zeta, vf[i]), th);
}

// per face: q_e, the thickness flux h_e v_e and its product with q_e
template <class T>
__global__ void k_adv_edge(const int* __restrict__ fvert, const int* __restrict__ fnode, int E, int Ep,
                           const T* __restrict__ q, const T* __restrict__ h, const T* __restrict__ v,
                           T* __restrict__ qe, T* __restrict__ hve, T* __restrict__ hvq)
{
    using A = Ar<T>;
    pdl_wait();
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const T qv = A::half(A::add(q[fvert[e]], q[fvert[Ep + e]]));
    const T hv = A::mul(A::half(A::add(h[fnode[e]], h[fnode[Ep + e]])), v[e]);
    qe[e] = qv;
    hve[e] = hv;
    hvq[e] = A::mul(hv, qv);
}

// kinetic energy 0.5 |u|^2 at the nodes, u from the RBF Cartesian reconstruction
// (3 x 6 block per node, missing pentagon entries zero; the sums of k_rbf); with
// U given, also the forcing U_i = cos(M) Ua_i + sin(M) Ub_i of the step's phase
template <class T>
__global__ void k_adv_node(const T* __restrict__ rbf, const int* __restrict__ edge, int N, int Np,
                           const T* __restrict__ v, T* __restrict__ ek, const T* __restrict__ phase,
                           const T* __restrict__ Ua, const T* __restrict__ Ub, T* __restrict__ U)
{
    using A = Ar<T>;
    pdl_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    T vf[kCellFaces];
#pragma unroll
    for (int j = 0; j < kCellFaces; j++) vf[j] = v[__ldg(&edge[j * Np + i])];
    T u[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        T t = A::zero();
#pragma unroll
        for (int j = 0; j < kCellFaces; j++) t = A::fma(rbf[(c * kCellFaces + j) * Np + i], vf[j], t);
        u[c] = t;
    }
    ek[i] = A::half(A::fma(u[2], u[2], A::fma(u[1], u[1], A::mul(u[0], u[0]))));
    if (U) U[i] = A::fma(phase[1], Ub[i], A::mul(phase[0], Ua[i]));
}

// kGrad: dvdt_e = ga (G eta)_e (gradient row in ascending node order), else
// dvdt_e as given; then the PV flux and -(G KE)_e.  The flux
// sum_j w_j (h v)_j (q_e + q_j) / 2 is formed as (q_e sum_j w_j (h v)_j + sum_j w_j (h v q)_j) / 2
// over the context's TRiSK table (w_j = w_ee' l_e' / d_e, zero in unused slots), the
// same table the power kernel reads for the tangential velocity.
template <class T, bool kGrad>
__global__ void k_adv_flux(const int* __restrict__ nbr, const T* __restrict__ tw,
                           const int* __restrict__ gcol, const T* __restrict__ gval, int E, int Ep,
                           const T* __restrict__ qe, const T* __restrict__ hve, const T* __restrict__ hvq,
                           const T* __restrict__ ek, T ga, const T* __restrict__ eta, T* __restrict__ dvdt)
{
    using A = Ar<T>;
    pdl_wait();
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const int g0 = gcol[e], g1 = gcol[Ep + e];
    const T w0 = gval[e], w1 = gval[Ep + e];
    T d;
    if constexpr (kGrad) d = A::mul(ga, A::fma(w1, eta[g1], A::mul(w0, eta[g0])));
    else d = dvdt[e];
    T s1 = A::zero(), s2 = A::zero();
#pragma unroll
    for (int j = 0; j < kTrisk; j++) {
        const int f = nbr[j * Ep + e];
        const T c = tw[j * Ep + e];
        s1 = A::fma(c, hve[f], s1);
        s2 = A::fma(c, hvq[f], s2);
    }
    d = A::add(d, A::half(A::fma(qe[e], s1, s2)));
    d = A::sub(d, A::fma(w1, ek[g1], A::mul(w0, ek[g0])));
    dvdt[e] = d;
}

// interpolateLSQFlux (src/interpolation.cpp:311-356), beta = 1, at face e: the
// directional second derivatives at the face's two nodes (7-term rows, ascending
// node order, fused multiply-adds), then the third-order upwind-biased thickness
// flux (u/2 (h_i + h_o) - dx^2/12 (d2_o + d2_i) u + dx^2/12 |u| (d2_o - d2_i)).
// dx2: d_e^2 / 12 per face, rounded on the host as the reference rounds it.
template <class T>
__device__ __forceinline__ T lsq_flux_at(int e, int Ep, const int* __restrict__ col, const T* __restrict__ val,
                                         const T* __restrict__ dx2v, const int* __restrict__ fnode, T vel,
                                         const T* __restrict__ h)
{
    using A = Ar<T>;
    const size_t R = (size_t)2 * Ep;
    T d2i = A::zero(), d2o = A::zero();
#pragma unroll
    for (int j = 0; j < 7; j++) {
        // the inner and outer rows' j-th terms are adjacent: one 16-byte load of each pair
        T vi, vo;
        A::ld2(val + j * R + 2 * e, vi, vo);
        const int2 c = *reinterpret_cast<const int2*>(col + j * R + 2 * e);
        d2i = A::fma(vi, h[c.x], d2i);
        d2o = A::fma(vo, h[c.y], d2o);
    }
    const T dx2 = dx2v[e];
    const T a = A::mul(A::half(vel), A::add(h[fnode[e]], h[fnode[Ep + e]]));
    const T b = A::mul(A::mul(dx2, A::add(d2o, d2i)), vel);
    return A::fma(A::mul(dx2, A::abs(vel)), A::sub(d2o, d2i), A::sub(a, b));
}

__global__ void k_lsq_flux(const int* __restrict__ col, const double* __restrict__ val, const double* __restrict__ dx2,
                           const int* __restrict__ fnode, int E, int Ep, const double* __restrict__ v,
                           const double* __restrict__ h, double* __restrict__ flux)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    flux[e] = lsq_flux_at<double>(e, Ep, col, val, dx2, fnode, v[e], h);
}

// ---- the advective time step (src/timeIntegrator.cpp:205-269, advection true) ----

// step constants in the method's number type
template <class T>
struct AdvK {
    T a, b, c;          // AB3: 23/12, -16/12, 5/12
    T dt, malpha, ga;   // dt, -alpha, -g (gradient of eta)
    T h0, coef;         // mean thickness; alpha 1000 h (LINEAR) or alpha / h (QUADRATIC) dissipation
    int quad;
};

// integrateAB3scalar (src/temporalOperators.cpp:17-68) for one unknown; h = its [3] history
template <class T>
__device__ __forceinline__ void ab3_step(T& s, T* h, int iter, const AdvK<T>& k, int init_load)
{
    using A = Ar<T>;
    if (iter > 1 || init_load) {
        s = A::fma(A::fma(k.c, h[2], A::fma(k.b, h[1], A::mul(k.a, h[0]))), k.dt, s);
        h[2] = h[1];
        h[1] = h[0];
    } else if (iter == 0) {
        s = A::fma(h[0], k.dt, s);
        h[2] = h[0];
    } else {
        s = A::fma(h[0], k.dt, s);
        h[1] = h[0];
    }
}

// AB3 of unknown i with the new tendency f: the history is slot-outermost
// ([3][P]: slot 0 the latest tendency, as the reference's [n][3] columns), so the
// three slot accesses of a warp are each one contiguous run
template <class T>
__device__ __forceinline__ void ab3_slots(T& s, T f, T* __restrict__ hist, int i, int P, int iter, const AdvK<T>& k,
                                          int init_load)
{
    T h[3] = {f, hist[P + i], hist[2 * P + i]};
    ab3_step<T>(s, h, iter, k, init_load);
    hist[i] = h[0];
    hist[P + i] = h[1];
    hist[2 * P + i] = h[2];
}

// momentum update: drag_e = -alpha v_e + (G U)_e from the velocity before the
// step, history slot 0 = dvdt, AB3, then v += dt drag (src/timeIntegrator.cpp:213-242).
// U: the forcing at the nodes at t + dt (k_adv_node).
template <class T>
__global__ void k_adv_vstep(const int* __restrict__ gcol, const T* __restrict__ gval, int E, int Ep, AdvK<T> k,
                            int iter, int init_load, const T* __restrict__ dv0, const T* __restrict__ U,
                            T* __restrict__ v, T* __restrict__ hist)
{
    using A = Ar<T>;
    pdl_wait();
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const T gu = A::fma(gval[Ep + e], U[gcol[Ep + e]], A::mul(gval[e], U[gcol[e]]));
    T ve = v[e];
    const T drag = A::fma(k.malpha, ve, gu);
    ab3_slots<T>(ve, dv0[e], hist, e, Ep, iter, k, init_load);
    v[e] = A::fma(k.dt, drag, ve);
}

template <class T>
struct PowerArgs {
    const int* nbr;       // [10][Ep] TRiSK neighbour faces (zero weight in unused slots)
    const T* w;           // [10][Ep] TRiSK weights
    const T* nrm;         // [2][Ep] face normal (east, north)
    const T* area;        // [Ep] face area
    double divisor;       // 4 pi r^2
    double* part;         // [blocks] partial sums
    unsigned* count;      // finished blocks of the launch (0 between launches)
    double* out;          // the step's power
    int quad;             // QUADRATIC friction
};

// LSQ thickness flux of the step, then updateEnergy (LINEAR or QUADRATIC) of the updated v:
// tangential velocity t_e = sum_k w_k v_k, (u, w) = (nx v + ny t, ny v - nx t),
// e_i = alpha 1000 h |(u, w)|^2, and the FP64 block sum of e_i A_i.  The last
// block to finish sums the block partials in a fixed order (lane-strided, then
// the warp tree), so the power does not depend on which block finishes last.
template <class T>
__global__ void __launch_bounds__(kAdvThreads)
k_adv_lsq_power(const int* __restrict__ col, const T* __restrict__ val, const T* __restrict__ dx2,
                const int* __restrict__ fnode, int E, int Ep, const T* __restrict__ v, const T* __restrict__ h,
                T* __restrict__ flux, T coef, PowerArgs<T> pa)
{
    using A = Ar<T>;
    pdl_wait();
    __shared__ double s_red[kAdvThreads / 32];
    __shared__ bool s_last;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    double x = 0.0;
    if (e < E) {
        const T ve = v[e];
        flux[e] = lsq_flux_at<T>(e, Ep, col, val, dx2, fnode, ve, h);
        T t = A::zero();
#pragma unroll
        for (int k = 0; k < kTrisk; k++) t = A::fma(pa.w[k * Ep + e], v[pa.nbr[k * Ep + e]], t);
        const T nx = pa.nrm[e], ny = pa.nrm[Ep + e];
        const T u = A::fma(nx, ve, A::mul(ny, t));
        const T w = A::fma(ny, ve, A::mul(A::neg(nx), t));
        x = A::to(A::mul(face_diss(coef, A::fma(u, u, A::mul(w, w)), pa.quad), pa.area[e]));
    }
    x = adv_warp_sum(x);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) s_red[wid] = x;
    __syncthreads();
    if (wid == 0) {
        double s = lane < (int)(blockDim.x >> 5) ? s_red[lane] : 0.0;
        s = adv_warp_sum(s);
        if (lane == 0) {
            pa.part[blockIdx.x] = s;
            __threadfence();
            s_last = atomicAdd(pa.count, 1u) == gridDim.x - 1;
        }
        __syncwarp();
    }
    __syncthreads();
    if (!s_last || wid != 0) return;
    __threadfence();
    double s = 0.0;
    for (int k = lane; k < (int)gridDim.x; k += 32) s += __ldcg(pa.part + k);
    s = adv_warp_sum(s);
    if (lane == 0) {
        *pa.out = s / pa.divisor;
        *pa.count = 0u;
    }
}

// forcing phase (cos, sin) of M = Omega t, t = dt step + dt (src/timeIntegrator.cpp:218)
template <class T>
__device__ __forceinline__ void adv_phase(long long step, double dt, double angvel, T* phase)
{
    const double t = dt * (double)step + dt;
    double sn, c;
    sincos(angvel * t, &sn, &c);
    phase[0] = Ar<T>::from(c);
    phase[1] = Ar<T>::from(sn);
}

// continuity update: detadt = D flux (cell's faces in ascending face order),
// history slot 0, AB3 (src/timeIntegrator.cpp:249-253), and the column thickness
// h + eta of the next step.  The launch has one block more than the cells need:
// its first thread advances the step counter and computes the next step's phase,
// alongside the cell blocks.
template <class T>
__global__ void k_adv_estep(const int* __restrict__ dcol, const T* __restrict__ dval, int N, int Np, AdvK<T> k,
                            int iter, int init_load, const T* __restrict__ flux, T* __restrict__ eta,
                            T* __restrict__ hist, T* __restrict__ ht, long long* __restrict__ step, double dt,
                            double angvel, T* __restrict__ phase)
{
    using A = Ar<T>;
    pdl_wait();
    if (blockIdx.x == gridDim.x - 1) {
        if (threadIdx.x == 0) {
            const long long s = *step + 1;
            *step = s;
            adv_phase<T>(s, dt, angvel, phase);
        }
        return;
    }
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    T t = A::zero();
#pragma unroll
    for (int j = 0; j < 6; j++) t = A::fma(dval[j * Np + i], flux[dcol[j * Np + i]], t);
    T s = eta[i];
    ab3_slots<T>(s, t, hist, i, Np, iter, k, init_load);
    eta[i] = s;
    ht[i] = A::add(k.h0, s);
}

// column thickness h + eta (after a state is loaded)
template <class T>
__global__ void k_adv_thickness(int N, T h0, const T* __restrict__ eta, T* __restrict__ ht)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) ht[i] = Ar<T>::add(h0, eta[i]);
}

template <class T>
__global__ void k_adv_set_step(long long* step, long long v, double dt, double angvel, T* phase)
{
    *step = v;
    adv_phase<T>(v, dt, angvel, phase);
}

// host-side conversion of the FP64 tables to the method's number type
template <class T> T host_cvt(double x);
template <> double host_cvt<double>(double x) { return x; }
template <> df64 host_cvt<df64>(double x) { return df_from_double(x); }

template <class T>
T* upload_as(const std::vector<double>& h)
{
    std::vector<T> c(h.size());
    for (size_t i = 0; i < h.size(); i++) c[i] = host_cvt<T>(h[i]);
    T* d = nullptr;
    if (cudaMalloc(&d, sizeof(T) * std::max<size_t>(1, c.size())) != cudaSuccess) return nullptr;
    if (!c.empty() && cudaMemcpy(d, c.data(), sizeof(T) * c.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        return nullptr;
    }
    return d;
}

int* upload_int(const std::vector<int>& h)
{
    int* d = nullptr;
    if (cudaMalloc(&d, sizeof(int) * std::max<size_t>(1, h.size())) != cudaSuccess) return nullptr;
    if (!h.empty() && cudaMemcpy(d, h.data(), sizeof(int) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        return nullptr;
    }
    return d;
}

template <class T>
T* dalloc(size_t n, bool zero = true)
{
    T* d = nullptr;
    if (cudaMalloc(&d, sizeof(T) * std::max<size_t>(1, n)) != cudaSuccess) return nullptr;
    if (zero) cudaMemset(d, 0, sizeof(T) * std::max<size_t>(1, n));
    return d;
}

}  // namespace

// coefficient tables in the method's number type
template <class T>
struct AdvTab {
    T *vcoef = nullptr, *vwt = nullptr, *vf = nullptr;   // [3][Vp] curl, vertex-thickness weights; [Vp] f
    T *gval = nullptr;                                   // [2][Ep] gradient row, ascending node order
    T *lval = nullptr, *dx2 = nullptr;                   // [7][2 Ep] second-derivative rows; [Ep] d_e^2 / 12
    T *dval = nullptr;                                   // [6][Np] divergence rows
    void release()
    {
        for (T* p : {vcoef, vwt, vf, gval, lval, dx2, dval}) cudaFree(p);
    }
    bool ok() const { return vcoef && vwt && vf && gval && lval && dx2 && dval; }
};

// work arrays and the state of a run, in the method's number type
template <class T>
struct AdvWork {
    T *q = nullptr, *qe = nullptr, *hve = nullptr, *hvq = nullptr, *ek = nullptr;
    T *v = nullptr, *eta = nullptr, *hv = nullptr, *hp = nullptr, *ht = nullptr, *U = nullptr, *dv0 = nullptr,
      *flux = nullptr, *Ua = nullptr, *Ub = nullptr, *phase = nullptr;
    void release()
    {
        for (T* p : {q, qe, hve, hvq, ek, v, eta, hv, hp, ht, U, dv0, flux, Ua, Ub, phase}) cudaFree(p);
    }
};

struct AdvDev {
    int V = 0, Vp = 0, E = 0, Ep = 0, N = 0, Np = 0;
    int *vface = nullptr, *vnode = nullptr, *fvert = nullptr, *fnode = nullptr, *gcol = nullptr;
    int* lcol = nullptr;         // [7][2 Ep] operatorDirectionalSecondDeriv rows
    int* dcol = nullptr;         // [6][Np] divergence rows, ascending face order (padded with zero weights)
    AdvTab<double> t64;          // FP64 tables: per-operator calls and ODIS_FP64 runs
    AdvTab<df64> tdf;            // double-float tables of an ODIS_DF64 run
    AdvWork<double> w64;         // FP64 work arrays (per-operator calls) and the ODIS_FP64 run state
    AdvWork<df64> wdf;           // the ODIS_DF64 run state
    std::vector<double> host[7]; // FP64 tables (vcoef, vwt, vf, gval, lval, dx2, dval) for a DF64 run's copies
    int prec = -1;               // precision of the run state, once allocated
    double angvel = 0.0;
    long long* step = nullptr;   // device step counter (forcing phase)
    double* part = nullptr;      // [faces / 32] power partial sums
    unsigned* count = nullptr;   // finished blocks of k_adv_lsq_power
    double* pbuf = nullptr;      // [kAdvGraphSteps] power of a graph chunk
    // threads per block for the node/vertex, face, and LSQ + power kernels.  FP64: small
    // blocks spread the FP64-issue-bound one-wave grids evenly over the SMs (level 6:
    // 45.7 us/step against 49.4 us with 256 threads); DF64 is fastest with 256 (42.4
    // against 44.8 us).  ODIS_ADV_BLOCKS="n,f,p[,v,e]" overrides both.
    int bn = 64, bf = 64, bp = 128, bv = 64, be = 64;   // + AB3 kernels: vstep, estep
    bool blocks_fixed = false;
    cudaGraphExec_t graph = nullptr;
};

void adv_destroy(AdvDev* a)
{
    if (!a) return;
    for (void* p : {(void*)a->vface, (void*)a->vnode, (void*)a->fvert, (void*)a->fnode, (void*)a->gcol, (void*)a->lcol, (void*)a->dcol, (void*)a->step, (void*)a->part, (void*)a->count,
                    (void*)a->pbuf})
        cudaFree(p);
    a->t64.release();
    a->tdf.release();
    a->w64.release();
    a->wdf.release();
    if (a->graph) cudaGraphExecDestroy(a->graph);
    delete a;
}

// the host copies of the FP64 tables are needed only for a double-float run's tables
static void release_host(AdvDev* a)
{
    for (std::vector<double>& h : a->host) std::vector<double>().swap(h);
}

template <class T>
static bool upload_tables(AdvDev* a, AdvTab<T>& t)
{
    t.vcoef = upload_as<T>(a->host[0]);
    t.vwt = upload_as<T>(a->host[1]);
    t.vf = upload_as<T>(a->host[2]);
    t.gval = upload_as<T>(a->host[3]);
    t.lval = upload_as<T>(a->host[4]);
    t.dx2 = upload_as<T>(a->host[5]);
    t.dval = upload_as<T>(a->host[6]);
    return t.ok();
}

int adv_create(AdvDev** out, const Mesh& m, double angvel, int Ep, int Np, bool df64_run)
{
    *out = nullptr;
    if (m.vert_area.empty()) return ODIS_ERR_MESH;
    AdvDev* a = new AdvDev;
    if (const char* env = std::getenv("ODIS_ADV_BLOCKS")) {
        int b[5] = {0, 0, 0, 0, 0};
        const int got = std::sscanf(env, "%d,%d,%d,%d,%d", &b[0], &b[1], &b[2], &b[3], &b[4]);
        bool ok = got == 3 || got == 5;
        for (int k = 0; k < got && ok; k++) ok = b[k] >= 32 && b[k] <= 256 && b[k] % 32 == 0;
        if (ok) {
            a->bn = b[0]; a->bf = b[1]; a->bp = b[2];
            a->bv = got == 5 ? b[3] : b[1];
            a->be = got == 5 ? b[4] : b[0];
            a->blocks_fixed = true;
        }
    }
    a->V = m.V; a->Vp = (m.V + 127) / 128 * 128; a->E = m.E; a->Ep = Ep; a->N = m.N; a->Np = Np;
    a->angvel = angvel;
    const int V = m.V, Vp = a->Vp, E = m.E;
    std::vector<int> vface((size_t)3 * Vp, 0), vnode((size_t)3 * Vp, 0);
    std::vector<double> vcoef((size_t)3 * Vp, 0.0), vwt((size_t)3 * Vp, 0.0), vf(Vp, 0.0);
    for (int v = 0; v < V; v++) {
        // operatorCurl row (src/mesh.cpp:3122-3175): ascending face order
        int idx[3] = {0, 1, 2};
        std::sort(idx, idx + 3, [&](int x, int y) { return m.vert_faces[v * 3 + x] < m.vert_faces[v * 3 + y]; });
        for (int j = 0; j < 3; j++) {
            const int s = idx[j], f = m.vert_faces[v * 3 + s];
            vface[(size_t)j * Vp + v] = f;
            vcoef[(size_t)j * Vp + v] = m.face_dist[f] * m.vert_face_dir[v * 3 + s] / m.vert_area[v];
            const int n = m.vert_nodes[v * 3 + j];
            vnode[(size_t)j * Vp + v] = n;
            // thickness at the vertex (Ringler et al. 2010 eq. 25): kite-weighted node thicknesses
            vwt[(size_t)j * Vp + v] = m.cv_area[n] * m.vert_R[v * 3 + j] / m.vert_area[v];
        }
        vf[v] = -2 * angvel * std::sin(m.vert_sph[v * 2]);
    }
    std::vector<int> fvert((size_t)2 * Ep, 0), fnode((size_t)2 * Ep, 0), gcol((size_t)2 * Ep, 0);
    std::vector<double> gval((size_t)2 * Ep, 0.0);
    for (int e = 0; e < E; e++) {
        fvert[e] = m.face_verts[e * 2];
        fvert[(size_t)Ep + e] = m.face_verts[e * 2 + 1];
        fnode[e] = m.face_nodes[e * 2];
        fnode[(size_t)Ep + e] = m.face_nodes[e * 2 + 1];
        // operatorGradient row (src/mesh.cpp:3005-3120), ascending node order
        const int n0 = m.face_nodes[e * 2], n1 = m.face_nodes[e * 2 + 1];
        const double d = m.face_dist[e];
        const double g0 = (-m.face_m[e * 2]) / d, g1 = (m.face_m[e * 2 + 1]) / d;
        const bool sw = n1 < n0;
        gcol[e] = sw ? n1 : n0;
        gval[e] = sw ? g1 : g0;
        gcol[(size_t)Ep + e] = sw ? n0 : n1;
        gval[(size_t)Ep + e] = sw ? g0 : g1;
    }
    std::vector<int> lc((size_t)7 * 2 * Ep, 0);
    std::vector<double> lv((size_t)7 * 2 * Ep, 0.0), dx2(Ep, 1.0);
    {
        std::vector<int> rc;
        std::vector<double> rv;
        const int st = build_lsq_rows(m, kRbfEps, rc, rv);
        if (st != ODIS_OK) { adv_destroy(a); return st; }
        for (int row = 0; row < 2 * E; row++)
            for (int j = 0; j < 7; j++) {
                lc[(size_t)j * 2 * Ep + row] = rc[(size_t)row * 7 + j];
                lv[(size_t)j * 2 * Ep + row] = rv[(size_t)row * 7 + j];
            }
        for (int e = 0; e < E; e++) dx2[e] = (m.face_dist[e] * m.face_dist[e]) * (1. / 12.0);
    }
    // operatorDivergence rows (src/mesh.cpp:3177-3288), ascending face order
    std::vector<int> dc((size_t)6 * Np, 0);
    std::vector<double> dvv((size_t)6 * Np, 0.0);
    for (int i = 0; i < m.N; i++) {
        const int k = m.nfriends(i);
        int idx[6] = {0, 1, 2, 3, 4, 5};
        std::sort(idx, idx + k, [&](int x, int y) { return m.faces[i * 6 + x] < m.faces[i * 6 + y]; });
        for (int j = 0; j < 6; j++) {
            const int s = idx[j < k ? j : k - 1];
            const int f = m.faces[i * 6 + s];
            dc[(size_t)j * Np + i] = f;
            dvv[(size_t)j * Np + i] = j < k ? -m.node_face_dir[i * 6 + s] * m.face_len[f] / m.cv_area[i] : 0.0;
        }
    }
    a->host[0] = std::move(vcoef); a->host[1] = std::move(vwt); a->host[2] = std::move(vf);
    a->host[3] = std::move(gval); a->host[4] = std::move(lv);
    a->host[5] = std::move(dx2); a->host[6] = std::move(dvv);
    a->vface = upload_int(vface); a->vnode = upload_int(vnode); a->fvert = upload_int(fvert);
    a->fnode = upload_int(fnode); a->gcol = upload_int(gcol);
    a->lcol = upload_int(lc); a->dcol = upload_int(dc);
    bool ok = a->vface && a->vnode && a->fvert && a->fnode && a->gcol && a->lcol && a->dcol &&
              upload_tables<double>(a, a->t64);
    AdvWork<double>& w = a->w64;
    ok = ok && (w.q = dalloc<double>(Vp)) && (w.qe = dalloc<double>(Ep)) && (w.hve = dalloc<double>(Ep)) &&
         (w.hvq = dalloc<double>(Ep)) && (w.ek = dalloc<double>(Np));
    if (!ok) { adv_destroy(a); return ODIS_ERR_NOMEM; }
    if (!df64_run) release_host(a);
    *out = a;
    return ODIS_OK;
}

double* adv_ekin_scratch(AdvDev* a) { return a->w64.ek; }

template <class T>
static void momentum_head(AdvDev* a, const AdvTab<T>& t, AdvWork<T>& w, const T* rbf, const int* cell_face,
                          const T* v, const T* h_total, T* ekin, T* U, cudaStream_t s)
{
    pdl_launch(k_adv_pv<T>, (a->V + a->bn - 1) / a->bn, a->bn, 0, s, a->vface, t.vcoef, a->vnode, t.vwt, t.vf, a->V,
               a->Vp, v, h_total, w.q);
    pdl_launch(k_adv_edge<T>, (a->E + a->bf - 1) / a->bf, a->bf, 0, s, a->fvert, a->fnode, a->E, a->Ep, w.q, h_total, v,
               w.qe, w.hve, w.hvq);
    pdl_launch(k_adv_node<T>, (a->N + a->bn - 1) / a->bn, a->bn, 0, s, rbf, cell_face, a->N, a->Np, v, ekin, w.phase,
               w.Ua, w.Ub, U);
}

void adv_momentum(AdvDev* a, const double* rbf, const int* cell_face, const int* nbr, const double* tw, double* dvdt,
                  const double* v, const double* h_total, double* ekin, cudaStream_t s)
{
    momentum_head<double>(a, a->t64, a->w64, rbf, cell_face, v, h_total, ekin, nullptr, s);
    k_adv_flux<double, false><<<(a->E + a->bf - 1) / a->bf, a->bf, 0, s>>>(
        nbr, tw, a->gcol, a->t64.gval, a->E, a->Ep, a->w64.qe, a->w64.hve, a->w64.hvq, ekin, 0.0, nullptr, dvdt);
}

int adv_kernels_per_call() { return 4; }

template <class T>
static int alloc_run(AdvDev* a, AdvWork<T>& w, double h0, const std::vector<double>& Ua, const std::vector<double>& Ub)
{
    const size_t E = a->Ep, N = a->Np;
    std::vector<double> ua(N, 0.0), ub(N, 0.0);
    for (int i = 0; i < a->N; i++) { ua[i] = Ua[i]; ub[i] = Ub[i]; }
    w.Ua = upload_as<T>(ua);
    w.Ub = upload_as<T>(ub);
    const bool ok = w.Ua && w.Ub && (w.q || (w.q = dalloc<T>(a->Vp))) && (w.qe || (w.qe = dalloc<T>(E))) &&
                    (w.hve || (w.hve = dalloc<T>(E))) && (w.hvq || (w.hvq = dalloc<T>(E))) &&
                    (w.ek || (w.ek = dalloc<T>(N))) && (w.v = dalloc<T>(E)) && (w.eta = dalloc<T>(N)) &&
                    (w.hv = dalloc<T>(3 * E)) && (w.hp = dalloc<T>(3 * N)) && (w.ht = dalloc<T>(N)) &&
                    (w.U = dalloc<T>(N)) && (w.dv0 = dalloc<T>(E)) && (w.flux = dalloc<T>(E)) &&
                    (w.phase = dalloc<T>(2));
    if (!ok) return ODIS_ERR_NOMEM;
    k_adv_thickness<T><<<(a->N + kAdvThreads - 1) / kAdvThreads, kAdvThreads>>>(a->N, host_cvt<T>(h0), w.eta, w.ht);
    return ODIS_OK;
}

int adv_state_alloc(AdvDev* a, int precision, double h0, const std::vector<double>& Ua, const std::vector<double>& Ub)
{
    if (a->prec >= 0) return a->prec == precision ? ODIS_OK : ODIS_ERR_ARG;
    if (precision != ODIS_FP64 && precision != ODIS_DF64) return ODIS_ERR_ARG;
    const int eb = (a->E + 31) / 32;      // enough partials for any block size
    if (!(a->step = dalloc<long long>(1)) || !(a->part = dalloc<double>(eb)) || !(a->count = dalloc<unsigned>(1)) ||
        !(a->pbuf = dalloc<double>(kAdvGraphSteps)))
        return ODIS_ERR_NOMEM;
    int st = ODIS_OK;
    if (precision == ODIS_DF64) {
        if (!a->blocks_fixed) a->bn = a->bf = a->bp = a->bv = a->be = 256;
        if (a->host[0].empty() || !upload_tables<df64>(a, a->tdf)) return ODIS_ERR_NOMEM;
        st = alloc_run<df64>(a, a->wdf, h0, Ua, Ub);
    } else {
        st = alloc_run<double>(a, a->w64, h0, Ua, Ub);
    }
    if (st != ODIS_OK) return st;
    release_host(a);
    a->prec = precision;
    // the allocations' zero fills and k_adv_thickness ran on the legacy default stream;
    // this wait orders them before the caller's first use of the context's own stream
    return cudaDeviceSynchronize() == cudaSuccess ? ODIS_OK : ODIS_ERR_CUDA;
}

void adv_set_step(AdvDev* a, long long step, double dt, cudaStream_t s)
{
    if (a->prec == ODIS_DF64) k_adv_set_step<df64><<<1, 1, 0, s>>>(a->step, step, dt, a->angvel, a->wdf.phase);
    else k_adv_set_step<double><<<1, 1, 0, s>>>(a->step, step, dt, a->angvel, a->w64.phase);
}

template <class T>
static void step_t(AdvDev* a, const AdvTab<T>& t, AdvWork<T>& w, const AdvStepArgs& x, const T* rbf, const T* tw,
                   const T* nrm, const T* area, int iter, double* power, cudaStream_t s)
{
    const int fb = (a->E + a->bf - 1) / a->bf, pb = (a->E + a->bp - 1) / a->bp;
    const int vb = (a->E + a->bv - 1) / a->bv, nb = (a->N + a->be - 1) / a->be;
    AdvK<T> k;
    k.a = host_cvt<T>(23. / 12.);
    k.b = host_cvt<T>(-16. / 12.);
    k.c = host_cvt<T>(5. / 12.);
    k.dt = host_cvt<T>(x.dt);
    k.malpha = host_cvt<T>(-x.alpha);
    k.ga = host_cvt<T>(-x.g * (1 - 0.5 * 0.0));
    k.h0 = host_cvt<T>(x.h0);
    k.coef = host_cvt<T>(x.quad ? x.alpha / x.h0 : x.alpha * 1000.0 * x.h0);
    k.quad = x.quad;
    // updateMomentum, advection branch: -g G eta + PV flux - G KE
    momentum_head<T>(a, t, w, rbf, x.cell_face, w.v, w.ht, w.ek, w.U, s);
    pdl_launch(k_adv_flux<T, true>, fb, a->bf, 0, s, x.nbr, tw, a->gcol, t.gval, a->E, a->Ep, w.qe, w.hve, w.hvq, w.ek,
               k.ga, w.eta, w.dv0);
    pdl_launch(k_adv_vstep<T>, vb, a->bv, 0, s, a->gcol, t.gval, a->E, a->Ep, k, iter, x.init_load, w.dv0, w.U, w.v,
               w.hv);
    // updateEta, advection branch: D (LSQ flux of h + eta); updateEnergy of the new v
    const PowerArgs<T> pa{x.nbr, tw, nrm, area, x.divisor, a->part, a->count, power, x.quad};
    pdl_launch(k_adv_lsq_power<T>, pb, a->bp, 0, s, a->lcol, t.lval, t.dx2, a->fnode, a->E, a->Ep, w.v, w.ht, w.flux,
               k.coef, pa);
    pdl_launch(k_adv_estep<T>, nb + 1, a->be, 0, s, a->dcol, t.dval, a->N, a->Np, k, iter, x.init_load, w.flux, w.eta,
               w.hp, w.ht, a->step, x.dt, a->angvel, w.phase);
}

void adv_step(AdvDev* a, const AdvStepArgs& x, int iter, double* power, cudaStream_t s)
{
    if (a->prec == ODIS_DF64)
        step_t<df64>(a, a->tdf, a->wdf, x, static_cast<const df64*>(x.rbf), static_cast<const df64*>(x.w),
                     static_cast<const df64*>(x.nrm), static_cast<const df64*>(x.area), iter, power, s);
    else
        step_t<double>(a, a->t64, a->w64, x, static_cast<const double*>(x.rbf), static_cast<const double*>(x.w),
                       static_cast<const double*>(x.nrm), static_cast<const double*>(x.area), iter, power, s);
}

void adv_thickness(AdvDev* a, double h0, cudaStream_t s)
{
    const int nb = (a->N + kAdvThreads - 1) / kAdvThreads;
    if (a->prec == ODIS_DF64)
        k_adv_thickness<df64><<<nb, kAdvThreads, 0, s>>>(a->N, host_cvt<df64>(h0), a->wdf.eta, a->wdf.ht);
    else
        k_adv_thickness<double><<<nb, kAdvThreads, 0, s>>>(a->N, h0, a->w64.eta, a->w64.ht);
}

template <class T>
static double to_host_double(T x)
{
    if constexpr (std::is_same<T, df64>::value) return df_to_double(x);
    else return x;
}

// device values -> host doubles; with stride P: the [3][P] history -> the reference's [n][3]
template <class T>
static int get_t(const T* d, size_t n, double* out, size_t P = 0)
{
    if (!out) return ODIS_OK;
    const size_t m = P ? 3 * P : n;
    std::vector<T> h(m);
    if (cudaMemcpy(h.data(), d, sizeof(T) * m, cudaMemcpyDeviceToHost) != cudaSuccess) return ODIS_ERR_CUDA;
    if (!P) {
        for (size_t i = 0; i < n; i++) out[i] = to_host_double(h[i]);
    } else {
        for (size_t i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) out[3 * i + k] = to_host_double(h[(size_t)k * P + i]);
    }
    return ODIS_OK;
}

template <class T>
static int set_t(T* d, size_t n, const double* in, size_t P = 0)
{
    if (!in) return ODIS_OK;
    const size_t m = P ? 3 * P : n;
    std::vector<T> h(m, host_cvt<T>(0.0));
    if (!P) {
        for (size_t i = 0; i < n; i++) h[i] = host_cvt<T>(in[i]);
    } else {
        for (size_t i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) h[(size_t)k * P + i] = host_cvt<T>(in[3 * i + k]);
    }
    return cudaMemcpy(d, h.data(), sizeof(T) * m, cudaMemcpyHostToDevice) == cudaSuccess ? ODIS_OK : ODIS_ERR_CUDA;
}

template <class T>
static int get_state_t(AdvDev* a, const AdvWork<T>& w, double* v, double* eta, double* dvdt, double* detadt)
{
    int st = get_t(w.v, a->E, v);
    if (st == ODIS_OK) st = get_t(w.eta, a->N, eta);
    if (st == ODIS_OK) st = get_t(w.hv, a->E, dvdt, a->Ep);
    if (st == ODIS_OK) st = get_t(w.hp, a->N, detadt, a->Np);
    return st;
}

template <class T>
static int set_state_t(AdvDev* a, AdvWork<T>& w, const double* v, const double* eta, const double* dvdt,
                       const double* detadt)
{
    int st = set_t(w.v, a->E, v);
    if (st == ODIS_OK) st = set_t(w.eta, a->N, eta);
    if (st == ODIS_OK) st = set_t(w.hv, a->E, dvdt, a->Ep);
    if (st == ODIS_OK) st = set_t(w.hp, a->N, detadt, a->Np);
    return st;
}

int adv_get_state(AdvDev* a, double* v, double* eta, double* dvdt, double* detadt)
{
    return a->prec == ODIS_DF64 ? get_state_t(a, a->wdf, v, eta, dvdt, detadt)
                                : get_state_t(a, a->w64, v, eta, dvdt, detadt);
}

int adv_set_state(AdvDev* a, const double* v, const double* eta, const double* dvdt, const double* detadt)
{
    return a->prec == ODIS_DF64 ? set_state_t(a, a->wdf, v, eta, dvdt, detadt)
                                : set_state_t(a, a->w64, v, eta, dvdt, detadt);
}

double* adv_graph_power(AdvDev* a) { return a->pbuf; }
cudaGraphExec_t* adv_graph(AdvDev* a) { return &a->graph; }

int adv_kernels_per_step() { return 7; }
int adv_graph_steps() { return kAdvGraphSteps; }

void adv_lsq_flux(AdvDev* a, double* flux, const double* v, const double* h_total, cudaStream_t s)
{
    k_lsq_flux<<<(a->E + kAdvThreads - 1) / kAdvThreads, kAdvThreads, 0, s>>>(a->lcol, a->t64.lval, a->t64.dx2,
                                                                             a->fnode, a->E, a->Ep, v, h_total, flux);
}

}  // namespace odis
