// Nonlinear momentum advection (calculateMomentumAdvection, src/momAdvection.cpp:11-267)
// and the advective time step on the device, FP64.
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
//                (eq. 49), as q_e sum_j c_j (h v)_j + sum_j c_j (h v q)_j with
//                c_j = w_j l_j / (2 d_e), then dvdt += -(G KE)_e
// Products are fused into the sums (the nonlinear loop is bound by GB300's FP64
// issue rate), so the results match the FP64 restatement to rounding, not bit
// for bit.
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
#include "odis_kernels.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

namespace odis {

namespace {

constexpr int kAdvThreads = 256;       // largest block; k_adv_lsq_power's reduction is sized for it
constexpr int kAdvGraphSteps = 64;      // steps per captured graph of the advective loop

__device__ __forceinline__ double adv_warp_sum(double x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    return x;
}

// vwt[j][i] = A_n R_j / A_v: the node's control-volume area times the kite
// fraction over the vertex area, so that h_v = sum_j vwt_j h_n
__global__ void k_adv_pv(const int* __restrict__ vface, const double* __restrict__ vcoef, const int* __restrict__ vnode,
                         const double* __restrict__ vwt, const double* __restrict__ vf, int V, int Vp,
                         const double* __restrict__ v, const double* __restrict__ h, double* __restrict__ q)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    double zeta = 0.0, th = 0.0;
#pragma unroll
    for (int j = 0; j < 3; j++) {
        zeta = fma(vcoef[j * Vp + i], v[vface[j * Vp + i]], zeta);
        th = fma(h[vnode[j * Vp + i]], vwt[j * Vp + i], th);
    }
    q[i] = (zeta + vf[i]) / th;
}

// per face: q_e, the thickness flux h_e v_e and its product with q_e
__global__ void k_adv_edge(const int* __restrict__ fvert, const int* __restrict__ fnode, int E, int Ep,
                           const double* __restrict__ q, const double* __restrict__ h, const double* __restrict__ v,
                           double* __restrict__ qe, double* __restrict__ hve, double* __restrict__ hvq)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const double qv = 0.5 * (q[fvert[e]] + q[fvert[Ep + e]]);
    const double hv = (0.5 * (h[fnode[e]] + h[fnode[Ep + e]])) * v[e];
    qe[e] = qv;
    hve[e] = hv;
    hvq[e] = hv * qv;
}

// kinetic energy 0.5 |u|^2 at the nodes, u from the RBF Cartesian reconstruction
// (3 x 6 block per node, missing pentagon entries zero; same sums as k_rbf); with
// U given, also the forcing U_i = cos(M) Ua_i + sin(M) Ub_i of the step's phase
__global__ void k_adv_node(const double* __restrict__ rbf, const int* __restrict__ edge, int N, int Np,
                           const double* __restrict__ v, double* __restrict__ ek, const double* __restrict__ phase,
                           const double* __restrict__ Ua, const double* __restrict__ Ub, double* __restrict__ U)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    double vf[kCellFaces];
#pragma unroll
    for (int j = 0; j < kCellFaces; j++) vf[j] = v[__ldg(&edge[j * Np + i])];
    double u[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        double t = 0.0;
#pragma unroll
        for (int j = 0; j < kCellFaces; j++) t = fma(__ldg(&rbf[(c * kCellFaces + j) * Np + i]), vf[j], t);
        u[c] = t;
    }
    ek[i] = 0.5 * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    if (U) U[i] = fma(phase[1], Ub[i], phase[0] * Ua[i]);
}

// kGrad: dvdt_e = alpha (G eta)_e (gradient row in ascending node order), else
// dvdt_e as given; then the PV flux and -(G KE)_e.  The flux
// sum_j c_j (h v)_j (q_e + q_j) is formed as q_e sum_j c_j (h v)_j + sum_j c_j (h v q)_j.
template <bool kGrad>
__global__ void k_adv_flux(const int* __restrict__ fr, const double* __restrict__ cwh, const int* __restrict__ nfr,
                           const int* __restrict__ gcol, const double* __restrict__ gval, int E, int Ep,
                           const double* __restrict__ qe, const double* __restrict__ hve, const double* __restrict__ hvq,
                           const double* __restrict__ ek, double alpha, const double* __restrict__ eta,
                           double* __restrict__ dvdt)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const int g0 = gcol[e], g1 = gcol[Ep + e];
    const double w0 = gval[e], w1 = gval[Ep + e];
    double d;
    if constexpr (kGrad) {
        d = alpha * fma(w1, eta[g1], w0 * eta[g0]);
    } else {
        d = dvdt[e];
    }
    double s1 = 0.0, s2 = 0.0;
    const int n = nfr[e];
    for (int j = 0; j < n; j++) {
        const int f = fr[j * Ep + e];
        const double c = cwh[j * Ep + e];
        s1 = fma(c, hve[f], s1);
        s2 = fma(c, hvq[f], s2);
    }
    d += fma(qe[e], s1, s2);
    double gk = 0.0;
    gk += w0 * ek[g0];
    gk += w1 * ek[g1];
    d += -gk;
    dvdt[e] = d;
}

// interpolateLSQFlux (src/interpolation.cpp:311-356), beta = 1, at face e: the
// directional second derivatives at the face's two nodes (7-term rows, ascending
// node order, fused multiply-adds), then the third-order upwind-biased thickness
// flux (u/2 (h_i + h_o) - dx^2/12 (d2_o + d2_i) u + dx^2/12 |u| (d2_o - d2_i)).
// dx2: d_e^2 / 12 per face, rounded on the host as the reference rounds it.
__device__ __forceinline__ double lsq_flux_at(int e, int Ep, const int* __restrict__ col,
                                              const double* __restrict__ val, const double* __restrict__ dx2v,
                                              const int* __restrict__ fnode, double vel, const double* __restrict__ h)
{
    const size_t R = (size_t)2 * Ep;
    double d2i = 0.0, d2o = 0.0;
#pragma unroll
    for (int j = 0; j < 7; j++) {
        d2i = fma(val[j * R + 2 * e], h[col[j * R + 2 * e]], d2i);
        d2o = fma(val[j * R + 2 * e + 1], h[col[j * R + 2 * e + 1]], d2o);
    }
    const double dx2 = dx2v[e];
    const double a = (vel * 0.5) * (h[fnode[e]] + h[fnode[Ep + e]]);
    const double b = (dx2 * (d2o + d2i)) * vel;
    return fma(dx2 * fabs(vel), d2o - d2i, a - b);
}

__global__ void k_lsq_flux(const int* __restrict__ col, const double* __restrict__ val, const double* __restrict__ dx2,
                           const int* __restrict__ fnode, int E, int Ep, const double* __restrict__ v,
                           const double* __restrict__ h, double* __restrict__ flux)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    flux[e] = lsq_flux_at(e, Ep, col, val, dx2, fnode, v[e], h);
}

// ---- the advective time step (src/timeIntegrator.cpp:205-269, advection true) ----

// integrateAB3scalar (src/temporalOperators.cpp:17-68) for one unknown; h = its [3] history
__device__ __forceinline__ void ab3_step(double& s, double* h, int iter, double dt, int init_load)
{
    const double a = 23. / 12., b = -16. / 12., c = 5. / 12.;
    if (iter > 1 || init_load) {
        s = fma(fma(c, h[2], fma(b, h[1], a * h[0])), dt, s);
        h[2] = h[1];
        h[1] = h[0];
    } else if (iter == 0) {
        s = fma(h[0], dt, s);
        h[2] = h[0];
    } else {
        s = fma(h[0], dt, s);
        h[1] = h[0];
    }
}

// momentum update: drag_e = -alpha v_e + (G U)_e from the velocity before the
// step, history slot 0 = dvdt, AB3, then v += dt drag (src/timeIntegrator.cpp:213-242).
// U: the forcing at the nodes at t + dt (k_adv_node).
__global__ void k_adv_vstep(const int* __restrict__ gcol, const double* __restrict__ gval, int E, int Ep, double alpha,
                            double dt, int iter, int init_load, const double* __restrict__ dv0,
                            const double* __restrict__ U, double* __restrict__ v, double* __restrict__ hist)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const double gu = fma(gval[Ep + e], U[gcol[Ep + e]], gval[e] * U[gcol[e]]);
    double ve = v[e];
    const double drag = fma(-alpha, ve, gu);
    double* h = hist + (size_t)e * 3;
    h[0] = dv0[e];
    ab3_step(ve, h, iter, dt, init_load);
    v[e] = fma(dt, drag, ve);
}

struct PowerArgs {
    const int* nbr;       // [10][Ep] TRiSK neighbour faces (zero weight in unused slots)
    const double* w;      // [10][Ep] TRiSK weights
    const double* nrm;    // [2][Ep] face normal (east, north)
    const double* area;   // [Ep] face area
    double coef;          // alpha 1000 h
    double divisor;       // 4 pi r^2
    double* part;         // [blocks] partial sums
    unsigned* count;      // finished blocks of the launch (0 between launches)
    double* out;          // the step's power
};

// LSQ thickness flux of the step, then updateEnergy (LINEAR) of the updated v:
// tangential velocity t_e = sum_k w_k v_k, (u, w) = (nx v + ny t, ny v - nx t),
// e_i = alpha 1000 h |(u, w)|^2, and the block sum of e_i A_i.  The last block to
// finish sums the block partials in a fixed order (lane-strided, then the warp
// tree), so the power does not depend on which block finishes last.
__global__ void __launch_bounds__(kAdvThreads)
k_adv_lsq_power(const int* __restrict__ col, const double* __restrict__ val, const double* __restrict__ dx2,
                const int* __restrict__ fnode, int E, int Ep, const double* __restrict__ v, const double* __restrict__ h,
                double* __restrict__ flux, PowerArgs pa)
{
    __shared__ double s_red[kAdvThreads / 32];
    __shared__ bool s_last;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    double x = 0.0;
    if (e < E) {
        const double ve = v[e];
        flux[e] = lsq_flux_at(e, Ep, col, val, dx2, fnode, ve, h);
        double t = 0.0;
#pragma unroll
        for (int k = 0; k < kTrisk; k++) t = fma(pa.w[k * Ep + e], v[pa.nbr[k * Ep + e]], t);
        const double nx = pa.nrm[e], ny = pa.nrm[Ep + e];
        const double u = nx * ve + ny * t;
        const double w = ny * ve + (-nx) * t;
        const double ei = pa.coef * (u * u + w * w);
        x = ei * pa.area[e];
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
__device__ __forceinline__ void adv_phase(long long step, double dt, double angvel, double* phase)
{
    const double t = dt * (double)step + dt;
    double sn, c;
    sincos(angvel * t, &sn, &c);
    phase[0] = c;
    phase[1] = sn;
}

// continuity update: detadt = D flux (cell's faces in ascending face order),
// history slot 0, AB3 (src/timeIntegrator.cpp:249-253), and the column thickness
// h + eta of the next step.  The launch has one block more than the cells need:
// its first thread advances the step counter and computes the next step's phase,
// alongside the cell blocks.
__global__ void k_adv_estep(const int* __restrict__ dcol, const double* __restrict__ dval, int N, int Np, double dt,
                            int iter, int init_load, double h0, const double* __restrict__ flux,
                            double* __restrict__ eta, double* __restrict__ hist, double* __restrict__ ht,
                            long long* __restrict__ step, double angvel, double* __restrict__ phase)
{
    if (blockIdx.x == gridDim.x - 1) {
        if (threadIdx.x == 0) {
            const long long s = *step + 1;
            *step = s;
            adv_phase(s, dt, angvel, phase);
        }
        return;
    }
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    double t = 0.0;
#pragma unroll
    for (int j = 0; j < 6; j++) t = fma(dval[j * Np + i], flux[dcol[j * Np + i]], t);
    double* h = hist + (size_t)i * 3;
    h[0] = t;
    double s = eta[i];
    ab3_step(s, h, iter, dt, init_load);
    eta[i] = s;
    ht[i] = h0 + s;
}

// column thickness h + eta (after a state is loaded)
__global__ void k_adv_thickness(int N, double h0, const double* __restrict__ eta, double* __restrict__ ht)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) ht[i] = h0 + eta[i];
}

__global__ void k_adv_set_step(long long* step, long long v, double dt, double angvel, double* phase)
{
    *step = v;
    adv_phase(v, dt, angvel, phase);
}

template <class T>
T* upload(const std::vector<T>& h)
{
    T* d = nullptr;
    if (cudaMalloc(&d, sizeof(T) * std::max<size_t>(1, h.size())) != cudaSuccess) return nullptr;
    if (!h.empty() && cudaMemcpy(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        return nullptr;
    }
    return d;
}

}  // namespace

struct AdvDev {
    int V = 0, Vp = 0, E = 0, Ep = 0, N = 0, Np = 0;
    int *vface = nullptr, *vnode = nullptr, *fvert = nullptr, *fnode = nullptr, *fr = nullptr, *nfr = nullptr,
        *gcol = nullptr;
    double *vcoef = nullptr, *vwt = nullptr, *vf = nullptr, *cwh = nullptr,
           *gval = nullptr;
    double *q = nullptr, *qe = nullptr, *hve = nullptr, *hvq = nullptr, *ek = nullptr;
    int* lcol = nullptr;         // [7][2 Ep] operatorDirectionalSecondDeriv rows
    double *lval = nullptr, *dx2 = nullptr;     // rows' weights; d_e^2 / 12 per face
    int* dcol = nullptr;         // [6][Np] divergence rows, ascending face order (padded with zero weights)
    double* dval = nullptr;
    // state of an advective run, in the reference's layout
    double *v = nullptr, *eta = nullptr, *hv = nullptr, *hp = nullptr, *ht = nullptr;
    double *U = nullptr, *dv0 = nullptr, *flux = nullptr;
    double *Ua = nullptr, *Ub = nullptr;    // forcing U = cos(M) Ua + sin(M) Ub at the nodes
    double angvel = 0.0;
    long long* step = nullptr;              // device step counter (forcing phase)
    double* phase = nullptr;                // [2] cos, sin of the counter's forcing phase
    double* part = nullptr;                 // [face blocks] power partial sums
    unsigned* count = nullptr;              // finished blocks of k_adv_lsq_power
    double* pbuf = nullptr;                 // [kAdvGraphSteps] power of a graph chunk
    // threads per block for the node/vertex, face, and LSQ + power kernels: small blocks
    // spread these one-wave grids evenly over the SMs (level 6: 46 us/step against 49 us
    // with 256 threads everywhere); ODIS_ADV_BLOCKS="n,f,p" overrides them
    int bn = 64, bf = 64, bp = 128;
    cudaGraphExec_t graph = nullptr;
};

void adv_destroy(AdvDev* a)
{
    if (!a) return;
    for (void* p : {(void*)a->vface, (void*)a->vnode, (void*)a->fvert, (void*)a->fnode, (void*)a->fr, (void*)a->nfr,
                    (void*)a->gcol, (void*)a->vcoef, (void*)a->vwt, (void*)a->vf,
                    (void*)a->cwh, (void*)a->gval, (void*)a->q, (void*)a->qe, (void*)a->hve, (void*)a->hvq, (void*)a->ek,
                    (void*)a->lcol, (void*)a->lval, (void*)a->dx2, (void*)a->dcol, (void*)a->dval, (void*)a->v,
                    (void*)a->eta, (void*)a->hv, (void*)a->hp, (void*)a->ht, (void*)a->U, (void*)a->dv0,
                    (void*)a->flux, (void*)a->Ua, (void*)a->Ub, (void*)a->step, (void*)a->phase, (void*)a->part,
                    (void*)a->count, (void*)a->pbuf})
        cudaFree(p);
    if (a->graph) cudaGraphExecDestroy(a->graph);
    delete a;
}

int adv_create(AdvDev** out, const Mesh& m, double angvel, int Ep, int Np)
{
    *out = nullptr;
    if (m.vert_area.empty()) return ODIS_ERR_MESH;
    AdvDev* a = new AdvDev;
    if (const char* env = std::getenv("ODIS_ADV_BLOCKS")) {
        int x = 0, y = 0, z = 0;
        if (std::sscanf(env, "%d,%d,%d", &x, &y, &z) == 3 && x >= 32 && y >= 32 && z >= 32 && x <= 256 && y <= 256 &&
            z <= 256 && x % 32 == 0 && y % 32 == 0 && z % 32 == 0) {
            a->bn = x; a->bf = y; a->bp = z;
        }
    }
    a->V = m.V; a->Vp = (m.V + 127) / 128 * 128; a->E = m.E; a->Ep = Ep; a->N = m.N; a->Np = Np;
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
    std::vector<int> fvert((size_t)2 * Ep, 0), fnode((size_t)2 * Ep, 0), fr((size_t)10 * Ep, 0), nfr(Ep, 0),
        gcol((size_t)2 * Ep, 0);
    std::vector<double> cwh((size_t)10 * Ep, 0.0), gval((size_t)2 * Ep, 0.0);
    for (int e = 0; e < E; e++) {
        fvert[e] = m.face_verts[e * 2];
        fvert[(size_t)Ep + e] = m.face_verts[e * 2 + 1];
        fnode[e] = m.face_nodes[e * 2];
        fnode[(size_t)Ep + e] = m.face_nodes[e * 2 + 1];
        nfr[e] = m.interp_n[e];
        const double dr = 1.0 / m.face_dist[e];
        for (int j = 0; j < m.interp_n[e]; j++) {
            const int f = m.interp_friends[e * 10 + j];
            fr[(size_t)j * Ep + e] = f;
            cwh[(size_t)j * Ep + e] = m.interp_w[e * 10 + j] * m.face_len[f] * dr * 0.5;
        }
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
    {
        std::vector<int> rc;
        std::vector<double> rv;
        const int st = build_lsq_rows(m, kRbfEps, rc, rv);
        if (st != ODIS_OK) { adv_destroy(a); return st; }
        std::vector<int> lc((size_t)7 * 2 * Ep, 0);
        std::vector<double> lv((size_t)7 * 2 * Ep, 0.0), dx2(Ep, 1.0);
        for (int row = 0; row < 2 * E; row++)
            for (int j = 0; j < 7; j++) {
                lc[(size_t)j * 2 * Ep + row] = rc[(size_t)row * 7 + j];
                lv[(size_t)j * 2 * Ep + row] = rv[(size_t)row * 7 + j];
            }
        for (int e = 0; e < E; e++) dx2[e] = (m.face_dist[e] * m.face_dist[e]) * (1. / 12.0);
        a->lcol = upload(lc);
        a->lval = upload(lv);
        a->dx2 = upload(dx2);
        if (!a->lcol || !a->lval || !a->dx2) { adv_destroy(a); return ODIS_ERR_NOMEM; }
    }
    {   // operatorDivergence rows (src/mesh.cpp:3177-3288), ascending face order
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
        a->dcol = upload(dc);
        a->dval = upload(dvv);
        if (!a->dcol || !a->dval) { adv_destroy(a); return ODIS_ERR_NOMEM; }
    }
    a->vface = upload(vface); a->vnode = upload(vnode); a->vcoef = upload(vcoef); a->vwt = upload(vwt);
    a->vf = upload(vf);
    a->fvert = upload(fvert); a->fnode = upload(fnode); a->fr = upload(fr); a->nfr = upload(nfr);
    a->cwh = upload(cwh); a->gcol = upload(gcol); a->gval = upload(gval);
    bool ok = a->vface && a->vnode && a->vcoef && a->vwt && a->vf && a->fvert && a->fnode &&
              a->fr && a->nfr && a->cwh && a->gcol && a->gval;
    ok = ok && cudaMalloc(&a->q, sizeof(double) * Vp) == cudaSuccess &&
         cudaMalloc(&a->qe, sizeof(double) * Ep) == cudaSuccess && cudaMalloc(&a->hve, sizeof(double) * Ep) == cudaSuccess &&
         cudaMalloc(&a->hvq, sizeof(double) * Ep) == cudaSuccess &&
         cudaMalloc(&a->ek, sizeof(double) * Np) == cudaSuccess;
    if (!ok) { adv_destroy(a); return ODIS_ERR_NOMEM; }
    *out = a;
    return ODIS_OK;
}

double* adv_ekin_scratch(AdvDev* a) { return a->ek; }

static void momentum_head(AdvDev* a, const double* rbf, const int* cell_face, const double* v, const double* h_total,
                          double* ekin, double* U, cudaStream_t s)
{
    k_adv_pv<<<(a->V + a->bn - 1) / a->bn, a->bn, 0, s>>>(a->vface, a->vcoef, a->vnode, a->vwt, a->vf, a->V, a->Vp, v,
                                                         h_total, a->q);
    k_adv_edge<<<(a->E + a->bf - 1) / a->bf, a->bf, 0, s>>>(a->fvert, a->fnode, a->E, a->Ep, a->q,
                                                                             h_total, v, a->qe, a->hve, a->hvq);
    k_adv_node<<<(a->N + a->bn - 1) / a->bn, a->bn, 0, s>>>(rbf, cell_face, a->N, a->Np, v, ekin,
                                                                             a->phase, a->Ua, a->Ub, U);
}

void adv_momentum(AdvDev* a, const double* rbf, const int* cell_face, double* dvdt, const double* v,
                  const double* h_total, double* ekin, cudaStream_t s)
{
    momentum_head(a, rbf, cell_face, v, h_total, ekin, nullptr, s);
    k_adv_flux<false><<<(a->E + a->bf - 1) / a->bf, a->bf, 0, s>>>(
        a->fr, a->cwh, a->nfr, a->gcol, a->gval, a->E, a->Ep, a->qe, a->hve, a->hvq, ekin, 0.0, nullptr, dvdt);
}

int adv_kernels_per_call() { return 4; }

int adv_state_alloc(AdvDev* a, double h0, const std::vector<double>& Ua, const std::vector<double>& Ub, double angvel)
{
    if (a->v) return ODIS_OK;
    {
        std::vector<double> ua(a->Np, 0.0), ub(a->Np, 0.0);
        for (int i = 0; i < a->N; i++) { ua[i] = Ua[i]; ub[i] = Ub[i]; }
        a->Ua = upload(ua);
        a->Ub = upload(ub);
        a->angvel = angvel;
        const int eb = (a->E + 31) / 32;      // enough partials for any block size
        if (!a->Ua || !a->Ub || cudaMalloc(&a->step, sizeof(long long)) != cudaSuccess ||
            cudaMalloc(&a->phase, sizeof(double) * 2) != cudaSuccess ||
            cudaMalloc(&a->part, sizeof(double) * eb) != cudaSuccess ||
            cudaMalloc(&a->count, sizeof(unsigned)) != cudaSuccess ||
            cudaMalloc(&a->pbuf, sizeof(double) * kAdvGraphSteps) != cudaSuccess)
            return ODIS_ERR_NOMEM;
        cudaMemset(a->step, 0, sizeof(long long));
        cudaMemset(a->phase, 0, sizeof(double) * 2);
        cudaMemset(a->count, 0, sizeof(unsigned));
    }
    const size_t E = a->Ep, N = a->Np;
    if (cudaMalloc(&a->v, sizeof(double) * E) != cudaSuccess || cudaMalloc(&a->eta, sizeof(double) * N) != cudaSuccess ||
        cudaMalloc(&a->hv, sizeof(double) * 3 * E) != cudaSuccess || cudaMalloc(&a->hp, sizeof(double) * 3 * N) != cudaSuccess ||
        cudaMalloc(&a->ht, sizeof(double) * N) != cudaSuccess || cudaMalloc(&a->U, sizeof(double) * N) != cudaSuccess ||
        cudaMalloc(&a->dv0, sizeof(double) * E) != cudaSuccess || cudaMalloc(&a->flux, sizeof(double) * E) != cudaSuccess)
        return ODIS_ERR_NOMEM;
    cudaMemset(a->v, 0, sizeof(double) * E);
    cudaMemset(a->eta, 0, sizeof(double) * N);
    cudaMemset(a->hv, 0, sizeof(double) * 3 * E);
    cudaMemset(a->hp, 0, sizeof(double) * 3 * N);
    cudaMemset(a->U, 0, sizeof(double) * N);
    k_adv_thickness<<<(a->N + kAdvThreads - 1) / kAdvThreads, kAdvThreads>>>(a->N, h0, a->eta, a->ht);
    return cudaDeviceSynchronize() == cudaSuccess ? ODIS_OK : ODIS_ERR_CUDA;
}

AdvState adv_state(AdvDev* a) { return AdvState{a->v, a->eta, a->hv, a->hp, a->ht, a->U}; }

void adv_set_step(AdvDev* a, long long step, double dt, cudaStream_t s)
{
    k_adv_set_step<<<1, 1, 0, s>>>(a->step, step, dt, a->angvel, a->phase);
}

void adv_step(AdvDev* a, const AdvStepArgs& x, int iter, double* power, cudaStream_t s)
{
    const int fb = (a->E + a->bf - 1) / a->bf, pb = (a->E + a->bp - 1) / a->bp, nb = (a->N + a->bn - 1) / a->bn;
    // updateMomentum, advection branch: -g G eta + PV flux - G KE
    momentum_head(a, x.rbf, x.cell_face, a->v, a->ht, a->ek, a->U, s);
    k_adv_flux<true><<<fb, a->bf, 0, s>>>(a->fr, a->cwh, a->nfr, a->gcol, a->gval, a->E, a->Ep, a->qe, a->hve,
                                                a->hvq, a->ek, -x.g * (1 - 0.5 * 0.0), a->eta, a->dv0);
    k_adv_vstep<<<fb, a->bf, 0, s>>>(a->gcol, a->gval, a->E, a->Ep, x.alpha, x.dt, iter, x.init_load, a->dv0,
                                          a->U, a->v, a->hv);
    // updateEta, advection branch: D (LSQ flux of h + eta); updateEnergy of the new v
    const PowerArgs pa{x.nbr, x.w, x.nrm, x.area, x.alpha * 1000.0 * x.h0, x.divisor, a->part, a->count, power};
    k_adv_lsq_power<<<pb, a->bp, 0, s>>>(a->lcol, a->lval, a->dx2, a->fnode, a->E, a->Ep, a->v, a->ht, a->flux,
                                              pa);
    k_adv_estep<<<nb + 1, a->bn, 0, s>>>(a->dcol, a->dval, a->N, a->Np, x.dt, iter, x.init_load, x.h0, a->flux,
                                              a->eta, a->hp, a->ht, a->step, a->angvel, a->phase);
}

void adv_thickness(AdvDev* a, double h0, cudaStream_t s)
{
    k_adv_thickness<<<(a->N + kAdvThreads - 1) / kAdvThreads, kAdvThreads, 0, s>>>(a->N, h0, a->eta, a->ht);
}

double* adv_graph_power(AdvDev* a) { return a->pbuf; }
cudaGraphExec_t* adv_graph(AdvDev* a) { return &a->graph; }

int adv_kernels_per_step() { return 7; }
int adv_graph_steps() { return kAdvGraphSteps; }

void adv_lsq_flux(AdvDev* a, double* flux, const double* v, const double* h_total, cudaStream_t s)
{
    k_lsq_flux<<<(a->E + kAdvThreads - 1) / kAdvThreads, kAdvThreads, 0, s>>>(a->lcol, a->lval, a->dx2, a->fnode, a->E,
                                                                             a->Ep, v, h_total, flux);
}

}  // namespace odis
