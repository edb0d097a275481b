// Nonlinear momentum advection (calculateMomentumAdvection, src/momAdvection.cpp:11-267)
// on the device, FP64.
//
// Per call:
//   k_adv_pv     per vertex: relative vorticity from the curl of v (three faces,
//                ascending face order), thickness at the vertex from the three
//                nodes' thicknesses weighted by control-volume area x kite
//                fraction over the vertex area (Ringler et al. 2010 eq. 25),
//                potential vorticity q = (zeta + f) / h
//   k_adv_edge   per face: q and h averaged from the face's two vertices / nodes
//   k_rbf + k_adv_ke  kinetic energy at the nodes from the RBF Cartesian velocity
//   k_adv_flux   per face: dvdt -= -sum_j w_j l_j / d_e (h_j v_j) (q_e + q_j) / 2
//                (eq. 49), then dvdt += -(G KE)_e with the gradient's two terms in
//                ascending node order
// Every sum and product is evaluated in the reference's order, so the results
// match the FP64 restatement to rounding.
#include "odis_advection.cuh"
#include "odis_kernels.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace odis {

namespace {

constexpr int kAdvThreads = 256;

__global__ void k_adv_pv(const int* __restrict__ vface, const double* __restrict__ vcoef, const int* __restrict__ vnode,
                         const double* __restrict__ vR, const double* __restrict__ vinv, const double* __restrict__ vf,
                         const double* __restrict__ cvA, int V, int Vp, const double* __restrict__ v,
                         const double* __restrict__ h, double* __restrict__ q)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    double zeta = 0.0;
#pragma unroll
    for (int j = 0; j < 3; j++) zeta += vcoef[j * Vp + i] * v[vface[j * Vp + i]];
    double th = 0.0;
#pragma unroll
    for (int j = 0; j < 3; j++) {
        const int n = vnode[j * Vp + i];
        th += h[n] * cvA[n] * vR[j * Vp + i];
    }
    th *= vinv[i];
    q[i] = (zeta + vf[i]) / th;
}

__global__ void k_adv_edge(const int* __restrict__ fvert, const int* __restrict__ fnode, int E, int Ep,
                           const double* __restrict__ q, const double* __restrict__ h, double* __restrict__ qe,
                           double* __restrict__ he)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    qe[e] = 0.5 * (q[fvert[e]] + q[fvert[Ep + e]]);
    he[e] = 0.5 * (h[fnode[e]] + h[fnode[Ep + e]]);
}

__global__ void k_adv_ke(const double* __restrict__ uxyz, int N, double* __restrict__ ek)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const double x = uxyz[3 * i], y = uxyz[3 * i + 1], z = uxyz[3 * i + 2];
    ek[i] = 0.5 * (x * x + y * y + z * z);
}

__global__ void k_adv_flux(const int* __restrict__ fr, const double* __restrict__ cw, const int* __restrict__ nfr,
                           const int* __restrict__ gcol, const double* __restrict__ gval, int E, int Ep,
                           const double* __restrict__ v, const double* __restrict__ qe, const double* __restrict__ he,
                           const double* __restrict__ ek, double* __restrict__ dvdt)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const double q0 = qe[e];
    double F = 0.0;
    const int n = nfr[e];
    for (int j = 0; j < n; j++) {
        const int f = fr[j * Ep + e];
        F += cw[j * Ep + e] * (he[f] * v[f]) * (q0 + qe[f]) * 0.5;
    }
    double d = dvdt[e];
    d -= -F;
    double gk = 0.0;
    gk += gval[e] * ek[gcol[e]];
    gk += gval[Ep + e] * ek[gcol[Ep + e]];
    d += -gk;
    dvdt[e] = d;
}

// interpolateLSQFlux (src/interpolation.cpp:311-356), beta = 1: the directional
// second derivatives at the face's two nodes (7-term rows, ascending node
// order), then the third-order upwind-biased thickness flux.  Products and sums
// are rounded separately, as in the unfused FP64 restatement.
__global__ void k_lsq_flux(const int* __restrict__ col, const double* __restrict__ val, const double* __restrict__ dist,
                           const int* __restrict__ fnode, int E, int Ep, const double* __restrict__ v,
                           const double* __restrict__ h, double* __restrict__ flux)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const size_t R = (size_t)2 * Ep;
    double d2i = 0.0, d2o = 0.0;
#pragma unroll
    for (int j = 0; j < 7; j++) {
        d2i = __dadd_rn(d2i, __dmul_rn(val[j * R + 2 * e], h[col[j * R + 2 * e]]));
        d2o = __dadd_rn(d2o, __dmul_rn(val[j * R + 2 * e + 1], h[col[j * R + 2 * e + 1]]));
    }
    const double dx = dist[e];
    const double dx2 = __dmul_rn(__dmul_rn(dx, dx), 1. / 12.0);
    const double vel = v[e];
    const double a = __dmul_rn(__dmul_rn(vel, 0.5), __dadd_rn(h[fnode[e]], h[fnode[Ep + e]]));
    const double b = __dmul_rn(__dmul_rn(dx2, __dadd_rn(d2o, d2i)), vel);
    const double c = __dmul_rn(__dmul_rn(__dmul_rn(dx2, 1.0), fabs(vel)), __dsub_rn(d2o, d2i));
    flux[e] = __dadd_rn(__dsub_rn(a, b), c);
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
    double *vcoef = nullptr, *vR = nullptr, *vinv = nullptr, *vf = nullptr, *cvA = nullptr, *cw = nullptr,
           *gval = nullptr;
    double *q = nullptr, *qe = nullptr, *he = nullptr, *uxyz = nullptr, *ek = nullptr;
    int* lcol = nullptr;         // [7][2 Ep] operatorDirectionalSecondDeriv rows
    double *lval = nullptr, *dist = nullptr;
};

void adv_destroy(AdvDev* a)
{
    if (!a) return;
    for (void* p : {(void*)a->vface, (void*)a->vnode, (void*)a->fvert, (void*)a->fnode, (void*)a->fr, (void*)a->nfr,
                    (void*)a->gcol, (void*)a->vcoef, (void*)a->vR, (void*)a->vinv, (void*)a->vf, (void*)a->cvA,
                    (void*)a->cw, (void*)a->gval, (void*)a->q, (void*)a->qe, (void*)a->he, (void*)a->uxyz,
                    (void*)a->ek, (void*)a->lcol, (void*)a->lval, (void*)a->dist})
        cudaFree(p);
    delete a;
}

int adv_create(AdvDev** out, const Mesh& m, double angvel, int Ep, int Np)
{
    *out = nullptr;
    if (m.vert_area.empty()) return ODIS_ERR_MESH;
    AdvDev* a = new AdvDev;
    a->V = m.V; a->Vp = (m.V + 127) / 128 * 128; a->E = m.E; a->Ep = Ep; a->N = m.N; a->Np = Np;
    const int V = m.V, Vp = a->Vp, E = m.E;
    std::vector<int> vface((size_t)3 * Vp, 0), vnode((size_t)3 * Vp, 0);
    std::vector<double> vcoef((size_t)3 * Vp, 0.0), vR((size_t)3 * Vp, 0.0), vinv(Vp, 1.0), vf(Vp, 0.0);
    for (int v = 0; v < V; v++) {
        // operatorCurl row (src/mesh.cpp:3122-3175): ascending face order
        int idx[3] = {0, 1, 2};
        std::sort(idx, idx + 3, [&](int x, int y) { return m.vert_faces[v * 3 + x] < m.vert_faces[v * 3 + y]; });
        for (int j = 0; j < 3; j++) {
            const int s = idx[j], f = m.vert_faces[v * 3 + s];
            vface[(size_t)j * Vp + v] = f;
            vcoef[(size_t)j * Vp + v] = m.face_dist[f] * m.vert_face_dir[v * 3 + s] / m.vert_area[v];
            vnode[(size_t)j * Vp + v] = m.vert_nodes[v * 3 + j];
            vR[(size_t)j * Vp + v] = m.vert_R[v * 3 + j];
        }
        vinv[v] = 1.0 / m.vert_area[v];
        vf[v] = -2 * angvel * std::sin(m.vert_sph[v * 2]);
    }
    std::vector<double> cvA(Np, 0.0);
    for (int i = 0; i < m.N; i++) cvA[i] = m.cv_area[i];
    std::vector<int> fvert((size_t)2 * Ep, 0), fnode((size_t)2 * Ep, 0), fr((size_t)10 * Ep, 0), nfr(Ep, 0),
        gcol((size_t)2 * Ep, 0);
    std::vector<double> cw((size_t)10 * Ep, 0.0), gval((size_t)2 * Ep, 0.0);
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
            cw[(size_t)j * Ep + e] = m.interp_w[e * 10 + j] * m.face_len[f] * dr;
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
        std::vector<double> lv((size_t)7 * 2 * Ep, 0.0), dist(Ep, 1.0);
        for (int row = 0; row < 2 * E; row++)
            for (int j = 0; j < 7; j++) {
                lc[(size_t)j * 2 * Ep + row] = rc[(size_t)row * 7 + j];
                lv[(size_t)j * 2 * Ep + row] = rv[(size_t)row * 7 + j];
            }
        for (int e = 0; e < E; e++) dist[e] = m.face_dist[e];
        a->lcol = upload(lc);
        a->lval = upload(lv);
        a->dist = upload(dist);
        if (!a->lcol || !a->lval || !a->dist) { adv_destroy(a); return ODIS_ERR_NOMEM; }
    }
    a->vface = upload(vface); a->vnode = upload(vnode); a->vcoef = upload(vcoef); a->vR = upload(vR);
    a->vinv = upload(vinv); a->vf = upload(vf); a->cvA = upload(cvA);
    a->fvert = upload(fvert); a->fnode = upload(fnode); a->fr = upload(fr); a->nfr = upload(nfr);
    a->cw = upload(cw); a->gcol = upload(gcol); a->gval = upload(gval);
    bool ok = a->vface && a->vnode && a->vcoef && a->vR && a->vinv && a->vf && a->cvA && a->fvert && a->fnode &&
              a->fr && a->nfr && a->cw && a->gcol && a->gval;
    ok = ok && cudaMalloc(&a->q, sizeof(double) * Vp) == cudaSuccess &&
         cudaMalloc(&a->qe, sizeof(double) * Ep) == cudaSuccess && cudaMalloc(&a->he, sizeof(double) * Ep) == cudaSuccess &&
         cudaMalloc(&a->uxyz, sizeof(double) * 3 * (size_t)Np) == cudaSuccess &&
         cudaMalloc(&a->ek, sizeof(double) * Np) == cudaSuccess;
    if (!ok) { adv_destroy(a); return ODIS_ERR_NOMEM; }
    *out = a;
    return ODIS_OK;
}

double* adv_ekin_scratch(AdvDev* a) { return a->ek; }

void adv_momentum(AdvDev* a, const double* rbf, const int* cell_face, double* dvdt, const double* v,
                  const double* h_total, double* ekin, cudaStream_t s)
{
    k_adv_pv<<<(a->V + kAdvThreads - 1) / kAdvThreads, kAdvThreads, 0, s>>>(a->vface, a->vcoef, a->vnode, a->vR, a->vinv,
                                                                           a->vf, a->cvA, a->V, a->Vp, v, h_total, a->q);
    k_adv_edge<<<(a->E + kAdvThreads - 1) / kAdvThreads, kAdvThreads, 0, s>>>(a->fvert, a->fnode, a->E, a->Ep, a->q,
                                                                             h_total, a->qe, a->he);
    launch_rbf(rbf, cell_face, a->N, a->Np, v, a->uxyz, s);
    k_adv_ke<<<(a->N + kAdvThreads - 1) / kAdvThreads, kAdvThreads, 0, s>>>(a->uxyz, a->N, ekin);
    k_adv_flux<<<(a->E + kAdvThreads - 1) / kAdvThreads, kAdvThreads, 0, s>>>(a->fr, a->cw, a->nfr, a->gcol, a->gval,
                                                                             a->E, a->Ep, v, a->qe, a->he, ekin, dvdt);
}

int adv_kernels_per_call() { return 5; }

void adv_lsq_flux(AdvDev* a, double* flux, const double* v, const double* h_total, cudaStream_t s)
{
    k_lsq_flux<<<(a->E + kAdvThreads - 1) / kAdvThreads, kAdvThreads, 0, s>>>(a->lcol, a->lval, a->dist, a->fnode, a->E,
                                                                             a->Ep, v, h_total, flux);
}

}  // namespace odis
