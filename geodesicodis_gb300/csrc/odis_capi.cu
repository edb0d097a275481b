// C ABI of libodis_gpu.so (declared in include/odis_gpu.h).
//
// A context owns: the device copy of the mesh operators in the layout of
// odis_device.cuh (FP64, or FP32 for the FP32-state variant), the state of
// one ocean instance, a stream, and a CUDA graph of kGraphSteps fused steps
// that odis_run_steps replays.  The per-step kernels read the step index
// from a device counter, so one instantiated graph serves every chunk of
// every run.
#include "odis_internal.h"
#include "odis_device.cuh"
#include "odis_kernels.cuh"
#include "odis_sh.cuh"
#include "odis_advection.cuh"
#include "odis_df64.cuh"
#include "odis_persistent.cuh"
#include "odis_text_round.cuh"

#include <algorithm>
#include <chrono>

#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

using namespace odis;

namespace {

constexpr double kPi = 3.1415926535897932384626433832795028841971693993751058;
constexpr int kGraphSteps = 64;

int pad128(int n) { return (n + 127) / 128 * 128; }

#define ODIS_CK(call)                                  \
    do {                                               \
        cudaError_t _e = (call);                       \
        if (_e != cudaSuccess) return ODIS_ERR_CUDA;   \
    } while (0)

// device allocation list freed with the context
struct DevArena {
    std::vector<void*> ptrs;
    template <class T>
    T* alloc(size_t n) {
        void* p = nullptr;
        if (cudaMalloc(&p, n * sizeof(T) + 16) != cudaSuccess) return nullptr;
        cudaMemset(p, 0, n * sizeof(T) + 16);
        ptrs.push_back(p);
        return (T*)p;
    }
    template <class T>
    T* upload(const std::vector<T>& h) {
        T* d = alloc<T>(h.size());
        if (d && !h.empty()) cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
        return d;
    }
    ~DevArena() { for (void* p : ptrs) cudaFree(p); }
};

// value conversions between the host's FP64 and each method's storage type
template <class T> T cvt(double x) { return (T)x; }
template <> float2 cvt<float2>(double x) { return df_from_double(x); }
inline double to_d(double x) { return x; }
inline double to_d(float x) { return (double)x; }
inline double to_d(float2 x) { return df_to_double(x); }

template <class T>
struct Operators {
    FaceCoef<T> fc{};
    CellCoef<T> cc{};
};

}  // namespace

struct odis_ctx {
    odis_params p{};
    std::vector<double> sh_factors;
    int E = 0, N = 0, Ep = 0, Np = 0, eb = 0;
    double r = 0.0;
    DevArena mem;
    Operators<double> op64;      // always present: per-operator calls are FP64
    Operators<float> op32;       // FP32-state variant
    Operators<float2> opdf;      // double-float method
    double* nrm = nullptr;       // [2][Ep]
    double* area = nullptr;      // [Ep]
    double* trig = nullptr;      // [kNodeTrig][Np] node trig table and Pbar_20, Pbar_22 (forcing)
    ForcingConst fk{};           // the run's forcing type and constants
    bool nodal = false;          // forcing evaluated at the nodes every step (FULL2, PLANET, GENERAL)
    double* d_fterms = nullptr;  // [fterms_cap][kForcingTerms] time terms of the current run (nodal forcing)
    int fterms_cap = 0;
    void* ufr = nullptr;         // [Np] nodal forcing / g in the method's type when there is no self-gravity
    double* rbf = nullptr;       // [3][6][Np] Cartesian reconstruction blocks
    // double-float copies of rbf, nrm and area for an ODIS_DF64 nonlinear run
    float2 *rbf_df = nullptr, *nrm_df = nullptr, *area_df = nullptr;
    State<double> s64{};
    State<float> s32{};
    State<float2> sdf{};
    long long* d_iter = nullptr;
    long long* d_run_first = nullptr;
    int* d_status = nullptr;
    double* d_partial = nullptr;
    double* d_power = nullptr;
    int power_cap = 0;
    void* d_phase = nullptr;     // forcing-phase table of the current run (method type)
    int phase_cap = 0;
    long long iter = 0;
    std::vector<double> slot0_saved;    // reference history slot 0 before the first step
    StepConst sc{};
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaGraphExec_t graph = nullptr;
    double* stage[4] = {nullptr, nullptr, nullptr, nullptr};
    size_t stage_n = 0;
    ShLoading* sh = nullptr;
    AdvDev* adv = nullptr;           // nonlinear advection operators (built on first use)
    PersistPlan plan{};          // persistent single-launch loop (FP64 / DF64 without self-gravity)
    bool persist_ok = false;     // the plan fits one CTA per SM and cooperative launch is available
    bool persist_on = true;      // odis_set_persistent
    bool persist_auto = true;    // the faster path as timed by choose_exec_path at creation
    double exec_ms[2] = {0, 0};  // those timings: graph-replayed pair, persistent loop (ms per step)
    int part_cap = 0;            // steps the plan's partial buffer holds
    double persist_frac = 0.0;   // fraction of faces interior to their CTA
    int fold_rows = 0;           // steps per run chunk (rows of the partial table minus one)
    long long launches = 0;      // kernels of this library launched by this context
    ~odis_ctx() {
        if (graph) cudaGraphExecDestroy(graph);
        if (sh) sh_destroy(sh);
        if (adv) adv_destroy(adv);
        if (d_power) cudaFree(d_power);
        if (d_phase) cudaFree(d_phase);
        if (d_fterms) cudaFree(d_fterms);
        if (plan.part) cudaFree(plan.part);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }
};

// ---------------------------------------------------------------------------
// grid / mesh
// ---------------------------------------------------------------------------
extern "C" odis_status odis_grid_generate_file(int level, const char* path)
{
    if (!path) return ODIS_ERR_ARG;
    GridArrays g;
    int st = generate_grid(level, g);
    if (st != ODIS_OK) return st;
    return write_grid(g, path);
}

static odis_status mesh_from_grid(const GridArrays& g, double radius, odis_mesh** out, bool device = false)
{
    const double rc = kPi / 180.0;
    std::vector<double> ns(g.node_deg.size()), cs(g.cent_deg.size());
    for (size_t k = 0; k < ns.size(); k++) ns[k] = g.node_deg[k] * rc;
    for (size_t k = 0; k < cs.size(); k++) cs[k] = g.cent_deg[k] * rc;
    return device ? odis_mesh_from_arrays_device(g.N, ns.data(), g.friends.data(), cs.data(), radius, out)
                  : odis_mesh_from_arrays(g.N, ns.data(), g.friends.data(), cs.data(), radius, out);
}

extern "C" odis_status odis_grid_generate_arrays(int level, int on_device, double* node_deg, int* friends,
                                                 double* cent_deg)
{
    if (!node_deg || !friends || !cent_deg) return ODIS_ERR_ARG;
    GridArrays g;
    const int st = on_device ? generate_grid_device(level, g) : generate_grid(level, g);
    if (st != ODIS_OK) return st;
    std::memcpy(node_deg, g.node_deg.data(), sizeof(double) * g.node_deg.size());
    std::memcpy(friends, g.friends.data(), sizeof(int) * g.friends.size());
    std::memcpy(cent_deg, g.cent_deg.data(), sizeof(double) * g.cent_deg.size());
    return ODIS_OK;
}

extern "C" odis_status odis_text_round16(const double* in, double* out, long long n)
{
    if (n < 0 || (n > 0 && (!in || !out))) return ODIS_ERR_ARG;
    for (long long i = 0; i < n; i++) out[i] = text_round16(in[i]);
    return ODIS_OK;
}

extern "C" odis_status odis_mesh_from_arrays_device(int n_nodes, const double* node_sph, const int* friends,
                                                    const double* cent_sph, double radius, odis_mesh** out)
{
    if (!out) return ODIS_ERR_ARG;
    *out = nullptr;
    odis_mesh* m = new (std::nothrow) odis_mesh;
    if (!m) return ODIS_ERR_NOMEM;
    int st = build_mesh_device(n_nodes, node_sph, friends, cent_sph, radius, m->m);
    if (st != ODIS_OK) { delete m; return st; }
    *out = m;
    return ODIS_OK;
}

extern "C" odis_status odis_mesh_from_file_device(const char* path, double radius, odis_mesh** out)
{
    if (!path || !out) return ODIS_ERR_ARG;
    GridArrays g;
    int st = read_grid(path, g);
    if (st != ODIS_OK) return st;
    return mesh_from_grid(g, radius, out, true);
}

extern "C" odis_status odis_mesh_generate_device(int level, double radius, odis_mesh** out)
{
    if (!out) return ODIS_ERR_ARG;
    GridArrays g;
    int st = generate_grid_device(level, g);
    if (st != ODIS_OK) return st;
    return mesh_from_grid(g, radius, out, true);
}

// largest |a - b| of one array over its largest |b|, and integer mismatches;
// lonlat: (lat, lon) pairs, longitudes compared modulo 2 pi (a point at lon 0
// may come out at 2 pi)
template <class T>
static void cmp_array(const std::vector<T>& a, const std::vector<T>& b, double* rel, long long* bad,
                      bool lonlat = false)
{
    if (a.size() != b.size()) { *bad += (long long)std::max(a.size(), b.size()) + 1; return; }
    if constexpr (std::is_integral<T>::value) {
        for (size_t k = 0; k < a.size(); k++) *bad += a[k] != b[k];
    } else {
        double d = 0.0, s = 0.0;
        for (size_t k = 0; k < a.size(); k++) {
            double dk = std::fabs(a[k] - b[k]);
            if (lonlat && (k & 1)) dk = std::min(dk, std::fabs(dk - 2 * kPi));
            d = std::max(d, dk);
            s = std::max(s, std::fabs(b[k]));
        }
        if (d > 0.0) *rel = std::max(*rel, s > 0.0 ? d / s : INFINITY);
    }
}

extern "C" odis_status odis_mesh_compare(const odis_mesh* ap, const odis_mesh* bp, double* max_rel, long long* int_mismatches)
{
    if (!ap || !bp || !max_rel || !int_mismatches) return ODIS_ERR_ARG;
    const Mesh &a = ap->m, &b = bp->m;
    double rel = 0.0;
    long long bad = (a.N != b.N) + (a.E != b.E) + (a.V != b.V);
    if (!bad) {
        for (auto pr : {std::make_pair(&a.friends, &b.friends), std::make_pair(&a.vertexes, &b.vertexes),
                        std::make_pair(&a.faces, &b.faces), std::make_pair(&a.node_face_dir, &b.node_face_dir),
                        std::make_pair(&a.face_nodes, &b.face_nodes), std::make_pair(&a.interp_friends, &b.interp_friends),
                        std::make_pair(&a.interp_n, &b.interp_n), std::make_pair(&a.vert_nodes, &b.vert_nodes),
                        std::make_pair(&a.face_verts, &b.face_verts), std::make_pair(&a.vert_faces, &b.vert_faces),
                        std::make_pair(&a.vert_face_dir, &b.vert_face_dir)})
            cmp_array(*pr.first, *pr.second, &rel, &bad);
        for (auto pr : {std::make_pair(&a.node_sph, &b.node_sph), std::make_pair(&a.cent_sph, &b.cent_sph),
                        std::make_pair(&a.vert_sph, &b.vert_sph), std::make_pair(&a.face_centre, &b.face_centre),
                        std::make_pair(&a.face_int, &b.face_int)})
            cmp_array(*pr.first, *pr.second, &rel, &bad, true);
        for (auto pr : {std::make_pair(&a.cv_area, &b.cv_area), std::make_pair(&a.face_len, &b.face_len),
                        std::make_pair(&a.face_dist, &b.face_dist), std::make_pair(&a.face_area, &b.face_area),
                        std::make_pair(&a.face_m, &b.face_m), std::make_pair(&a.face_normal, &b.face_normal),
                        std::make_pair(&a.face_nxyz, &b.face_nxyz), std::make_pair(&a.interp_w, &b.interp_w),
                        std::make_pair(&a.vert_R, &b.vert_R), std::make_pair(&a.vert_area, &b.vert_area)})
            cmp_array(*pr.first, *pr.second, &rel, &bad);
    }
    *max_rel = rel;
    *int_mismatches = bad;
    return ODIS_OK;
}

extern "C" odis_status odis_mesh_from_arrays(int n_nodes, const double* node_sph, const int* friends,
                                             const double* cent_sph, double radius, odis_mesh** out)
{
    if (!out) return ODIS_ERR_ARG;
    *out = nullptr;
    odis_mesh* m = new (std::nothrow) odis_mesh;
    if (!m) return ODIS_ERR_NOMEM;
    int st = build_mesh(n_nodes, node_sph, friends, cent_sph, radius, m->m);
    if (st != ODIS_OK) { delete m; return st; }
    *out = m;
    return ODIS_OK;
}

extern "C" odis_status odis_mesh_from_file(const char* path, double radius, odis_mesh** out)
{
    if (!path || !out) return ODIS_ERR_ARG;
    GridArrays g;
    int st = read_grid(path, g);
    if (st != ODIS_OK) return st;
    return mesh_from_grid(g, radius, out);
}

extern "C" odis_status odis_mesh_generate(int level, double radius, odis_mesh** out)
{
    if (!out) return ODIS_ERR_ARG;
    GridArrays g;
    int st = generate_grid(level, g);
    if (st != ODIS_OK) return st;
    return mesh_from_grid(g, radius, out);
}

extern "C" odis_status odis_mesh_sizes(const odis_mesh* m, int* n_cells, int* n_edges, int* n_vertices)
{
    if (!m) return ODIS_ERR_ARG;
    if (n_cells) *n_cells = m->m.N;
    if (n_edges) *n_edges = m->m.E;
    if (n_vertices) *n_vertices = m->m.V;
    return ODIS_OK;
}

extern "C" odis_status odis_mesh_field(const odis_mesh* mp, int which, double* out)
{
    if (!mp || !out) return ODIS_ERR_ARG;
    const Mesh& m = mp->m;
    const int E = m.E;
    auto col = [&](const std::vector<double>& v, int c) { for (int i = 0; i < E; i++) out[i] = v[(size_t)i * 2 + c]; };
    switch (which) {
    case 0: std::memcpy(out, m.face_len.data(), sizeof(double) * E); break;
    case 1: std::memcpy(out, m.face_dist.data(), sizeof(double) * E); break;
    case 2: std::memcpy(out, m.face_area.data(), sizeof(double) * E); break;
    case 3: std::memcpy(out, m.cv_area.data(), sizeof(double) * m.N); break;
    case 4: col(m.face_centre, 0); break;
    case 5: col(m.face_centre, 1); break;
    case 6: col(m.face_m, 0); break;
    case 7: col(m.face_m, 1); break;
    case 8: col(m.face_normal, 0); break;
    case 9: col(m.face_normal, 1); break;
    case 10: col(m.face_int, 0); break;
    case 11: col(m.face_int, 1); break;
    case 12: for (int i = 0; i < m.N; i++) out[i] = m.node_sph[(size_t)i * 2]; break;
    case 13: for (int i = 0; i < m.N; i++) out[i] = m.node_sph[(size_t)i * 2 + 1]; break;
    default: return ODIS_ERR_ARG;
    }
    return ODIS_OK;
}

extern "C" odis_status odis_mesh_topology(const odis_mesh* mp, int* face_nodes, int* faces, int* node_face_dir,
                                          int* interp_friends, double* interp_w, int* interp_n)
{
    if (!mp) return ODIS_ERR_ARG;
    const Mesh& m = mp->m;
    if (face_nodes) std::memcpy(face_nodes, m.face_nodes.data(), sizeof(int) * m.E * 2);
    if (faces) std::memcpy(faces, m.faces.data(), sizeof(int) * m.N * 6);
    if (node_face_dir) std::memcpy(node_face_dir, m.node_face_dir.data(), sizeof(int) * m.N * 6);
    if (interp_friends) std::memcpy(interp_friends, m.interp_friends.data(), sizeof(int) * m.E * 10);
    if (interp_w) std::memcpy(interp_w, m.interp_w.data(), sizeof(double) * m.E * 10);
    if (interp_n) std::memcpy(interp_n, m.interp_n.data(), sizeof(int) * m.E);
    return ODIS_OK;
}

extern "C" odis_status odis_mesh_vertex_field(const odis_mesh* mp, int which, double* out)
{
    if (!mp || !out) return ODIS_ERR_ARG;
    const Mesh& m = mp->m;
    for (int v = 0; v < m.V; v++) {
        if (which == 0) out[v] = m.vert_area[v];
        else if (which >= 1 && which <= 3) out[v] = m.vert_R[(size_t)v * 3 + which - 1];
        else if (which == 4) out[v] = std::sin(m.vert_sph[(size_t)v * 2]);
        else return ODIS_ERR_ARG;
    }
    return ODIS_OK;
}

extern "C" odis_status odis_mesh_vertex_topology(const odis_mesh* mp, int* vert_nodes, int* vert_faces,
                                                 int* vert_face_dir, int* face_verts)
{
    if (!mp) return ODIS_ERR_ARG;
    const Mesh& m = mp->m;
    if (vert_nodes) std::memcpy(vert_nodes, m.vert_nodes.data(), sizeof(int) * m.V * 3);
    if (vert_faces) std::memcpy(vert_faces, m.vert_faces.data(), sizeof(int) * m.V * 3);
    if (vert_face_dir) std::memcpy(vert_face_dir, m.vert_face_dir.data(), sizeof(int) * m.V * 3);
    if (face_verts) std::memcpy(face_verts, m.face_verts.data(), sizeof(int) * m.E * 2);
    return ODIS_OK;
}

extern "C" void odis_mesh_destroy(odis_mesh* m) { delete m; }

extern "C" odis_status odis_mesh_gravity_wave_omega(const odis_mesh* m, double g, double h, int iters, double* omega)
{
    if (!m || !omega || !(g > 0.0) || !(h > 0.0) || iters <= 0) return ODIS_ERR_ARG;
    *omega = gravity_wave_omega(m->m, g, h, iters);
    return ODIS_OK;
}

// FREE_LOADING degree factors of src/boundaryConditions.cpp:29-76: loading
// Love numbers from a uniform elastic body (rigidity 40 GPa, bulk density
// 1609.22 kg/m^3, ocean 1000 kg/m^3) and gamma_l = (1 + k_l - h_l) 3 rho_o / ((2l+1) rho_b).
extern "C" odis_status odis_loading_factors(double g, double radius, int lmax, double* out)
{
    if (!out || lmax < 0 || !(g > 0.0) || !(radius > 0.0)) return ODIS_ERR_ARG;
    const double ocean_den = 1000.0, bulk_den = 1609.22, rig = 40e9;
    out[0] = 0.0;
    for (int l = 1; l <= lmax; l++) {
        double eff_rig = (double)(2 * l * l + 4 * l + 3);
        eff_rig /= (double)l;
        eff_rig *= rig / (bulk_den * g * radius);
        const double k_l = -(1.0 / (1.0 + eff_rig));
        const double h_l = -(1.0 / (1.0 + eff_rig)) * (2.0 * (double)l + 1.0) / 3.0;
        double f = (1.0 + k_l - h_l);
        f *= 3. * ocean_den / ((2. * (double)l + 1.0) * bulk_den);
        out[l] = f;
    }
    return ODIS_OK;
}

extern "C" odis_status odis_stable_steps_per_orbit(double period, double omega_max, double margin, int* steps)
{
    if (!steps || !(period > 0.0) || !(omega_max >= 0.0) || !(margin > 0.0 && margin <= 1.0)) return ODIS_ERR_ARG;
    // omega*dt <= margin * 6/11 with dt = period/n, n a multiple of 100 (src/mesh.cpp:1601-1618)
    const double nmin = period * omega_max / (margin * 6.0 / 11.0);
    long long n = ((long long)std::ceil(nmin / 100.0)) * 100;
    if (n < 100) n = 100;
    if (n > 2000000000LL) return ODIS_ERR_ARG;
    *steps = (int)n;
    return ODIS_OK;
}

// ---------------------------------------------------------------------------
// parameters
// ---------------------------------------------------------------------------
extern "C" odis_status odis_derive_time(double angvel_in, double dt_target, double* angvel, double* period,
                                        double* dt, int* steps_per_orbit)
{
    if (!(angvel_in > 0.0) || !(dt_target > 0.0) || !angvel || !period || !dt || !steps_per_orbit) return ODIS_ERR_ARG;
    double P = 2. * kPi / angvel_in;
    int it = (int)std::round(P / 2) * 2;
    *period = (double)it;
    *angvel = 2 * kPi / (double)it;
    double d = *period;
    int n = 100;
    while (d > dt_target) { d = *period / n; n += 100; }
    n -= 100;
    *dt = d;
    *steps_per_orbit = n;
    return ODIS_OK;
}

extern "C" odis_status odis_params_from_input(const char* path, odis_input* out)
{
    if (!path || !out) return ODIS_ERR_ARG;
    return parse_input(path, *out);
}

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
template <class T>
static int build_operators(odis_ctx* c, const Mesh& m, const std::vector<double>& Ua, const std::vector<double>& Ub,
                           Operators<T>& op)
{
    const int E = c->E, N = c->N, Ep = c->Ep, Np = c->Np;
    const odis_params& p = c->p;
    std::vector<int> nbr((size_t)kTrisk * Ep), n0(Ep), n1(Ep), edge((size_t)kCellFaces * Np);
    const T zero = cvt<T>(0.0);
    std::vector<T> w((size_t)kTrisk * Ep, zero), gg0(Ep, zero), gg1(Ep, zero), cor(Ep, zero);
    std::vector<T> fP(Ep, zero), fQ(Ep, zero), diss(Ep, zero), hw((size_t)kCellFaces * Np, zero);
    const double four_pi_r2 = 4 * kPi * std::pow(m.r, 2.0);
    for (int e = 0; e < Ep; e++) {
        const int ee = e < E ? e : 0;
        for (int k = 0; k < kTrisk; k++) {
            const bool ok = e < E && k < m.interp_n[ee];
            const int f = ok ? m.interp_friends[(size_t)ee * 10 + k] : ee;
            nbr[(size_t)k * Ep + e] = f;
            w[(size_t)k * Ep + e] = ok ? cvt<T>(m.interp_w[(size_t)ee * 10 + k] * m.face_len[f] / m.face_dist[ee]) : zero;
        }
        const int a = m.face_nodes[(size_t)ee * 2], b = m.face_nodes[(size_t)ee * 2 + 1];
        n0[e] = a;
        n1[e] = b;
        if (e >= E) continue;
        const double d = m.face_dist[e];
        const double g0 = (-m.face_m[(size_t)e * 2]) / d, g1 = (m.face_m[(size_t)e * 2 + 1]) / d;
        gg0[e] = cvt<T>(-p.g * g0);
        gg1[e] = cvt<T>(-p.g * g1);
        cor[e] = cvt<T>(-2.0 * p.angvel * std::sin(m.face_centre[(size_t)e * 2]));
        fP[e] = cvt<T>(g0 * Ua[a] + g1 * Ua[b]);
        fQ[e] = cvt<T>(g0 * Ub[a] + g1 * Ub[b]);
        diss[e] = cvt<T>(energy_coef(p) * m.face_area[e] / four_pi_r2);
    }
    for (int i = 0; i < Np; i++) {
        const int ii = i < N ? i : 0;
        const int k5 = i < N ? m.nfriends(ii) : 0;
        for (int k = 0; k < kCellFaces; k++) {
            const bool ok = k < k5;
            const int f = ok ? m.faces[(size_t)ii * 6 + k] : m.faces[(size_t)ii * 6];
            edge[(size_t)k * Np + i] = f;
            if (ok) {
                const double dv = -m.node_face_dir[(size_t)ii * 6 + k] * m.face_len[f] / m.cv_area[ii];
                hw[(size_t)k * Np + i] = cvt<T>(p.h * dv);
            }
        }
    }
    // host-side range check of every index the kernels gather through
    for (int x : nbr) if (x < 0 || x >= E) return ODIS_ERR_MESH;
    for (int x : n0) if (x < 0 || x >= N) return ODIS_ERR_MESH;
    for (int x : n1) if (x < 0 || x >= N) return ODIS_ERR_MESH;
    for (int x : edge) if (x < 0 || x >= E) return ODIS_ERR_MESH;
    DevArena& A = c->mem;
    op.fc.nbr = A.upload(nbr);
    op.fc.w = A.upload(w);
    op.fc.n0 = A.upload(n0);
    op.fc.n1 = A.upload(n1);
    op.fc.gg0 = A.upload(gg0);
    op.fc.gg1 = A.upload(gg1);
    op.fc.cor = A.upload(cor);
    op.fc.fP = A.upload(fP);
    op.fc.fQ = A.upload(fQ);
    op.fc.diss = A.upload(diss);
    op.cc.edge = A.upload(edge);
    op.cc.hw = A.upload(hw);
    if (!op.fc.nbr || !op.fc.w || !op.fc.n0 || !op.fc.n1 || !op.fc.gg0 || !op.fc.gg1 || !op.fc.cor || !op.fc.fP ||
        !op.fc.fQ || !op.fc.diss || !op.cc.edge || !op.cc.hw)
        return ODIS_ERR_NOMEM;
    return ODIS_OK;
}

template <class T>
static int alloc_state(odis_ctx* c, State<T>& s, bool split)
{
    DevArena& A = c->mem;
    for (int k = 0; k < 2; k++) {
        s.v[k] = A.alloc<T>(c->Ep);
        s.hv[k] = A.alloc<T>(c->Ep);
        s.he[k] = A.alloc<T>(c->Np);
        if (!s.v[k] || !s.hv[k] || !s.he[k]) return ODIS_ERR_NOMEM;
    }
    s.vlo = split ? A.alloc<float>(c->Ep) : nullptr;
    s.eta = A.alloc<T>(c->Np);
    s.etalo = split ? A.alloc<float>(c->Np) : nullptr;
    if (!s.eta || (split && (!s.vlo || !s.etalo))) return ODIS_ERR_NOMEM;
    s.usg = nullptr;
    s.iter = c->d_iter;
    s.run_first = c->d_run_first;
    s.partial = c->d_partial;
    s.power = nullptr;
    s.status = c->d_status;
    return ODIS_OK;
}

// Partition of faces and cells over one CTA per SM for the persistent loop,
// with each CTA's producer sets (see odis_persistent.cu).  If the partition's
// coefficients do not fit one CTA's shared memory, or the device cannot do a
// cooperative launch, the context keeps to the graph-replayed two-kernel step.
static int build_persist_plan(odis_ctx* c, const Mesh& m)
{
    int dev = 0, sms = 0, coop = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return ODIS_ERR_CUDA;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (!coop || sms <= 0) return ODIS_OK;
    const int P = sms, E = m.E, N = m.N;
    if (E < 4 * P || N < 4 * P) return ODIS_OK;          // too small to partition usefully
    std::vector<int> fstart(P + 1), cstart(P + 1), fown(E), cown(N);
    for (int b = 0; b <= P; b++) {
        fstart[b] = (int)((long long)E * b / P);
        cstart[b] = (int)((long long)N * b / P);
    }
    int nf_max = 0, nc_max = 0;
    for (int b = 0; b < P; b++) {
        for (int e = fstart[b]; e < fstart[b + 1]; e++) fown[e] = b;
        for (int i = cstart[b]; i < cstart[b + 1]; i++) cown[i] = b;
        nf_max = std::max(nf_max, fstart[b + 1] - fstart[b]);
        nc_max = std::max(nc_max, cstart[b + 1] - cstart[b]);
    }
    std::vector<int> aptr(P + 1, 0), cptr(P + 1, 0), alist, clist;
    std::vector<int> mark(P, -1);
    for (int b = 0; b < P; b++) {
        auto add = [&](int q, std::vector<int>& lst) {
            if (q != b && mark[q] != b) { mark[q] = b; lst.push_back(q); }
        };
        for (int e = fstart[b]; e < fstart[b + 1]; e++) {
            for (int k = 0; k < m.interp_n[e]; k++) add(fown[m.interp_friends[(size_t)e * 10 + k]], alist);
            add(cown[m.face_nodes[(size_t)e * 2]], alist);
            add(cown[m.face_nodes[(size_t)e * 2 + 1]], alist);
        }
        aptr[b + 1] = (int)alist.size();
        std::fill(mark.begin(), mark.end(), -1);
        for (int i = cstart[b]; i < cstart[b + 1]; i++)
            for (int k = 0; k < m.nfriends(i); k++) add(fown[m.faces[(size_t)i * 6 + k]], clist);
        cptr[b + 1] = (int)clist.size();
        std::fill(mark.begin(), mark.end(), -1);
    }
    // interior-first order inside each CTA: a face is interior when its TRiSK
    // neighbours and both end cells are owned by its CTA, a cell when all its
    // faces are
    std::vector<int> forder(E), fpos(E), corder(N), cpos(N), fint(P), cint(P);
    for (int b = 0; b < P; b++) {
        int lo = fstart[b], hi = fstart[b + 1];
        std::vector<int> in, bd;
        for (int e = lo; e < hi; e++) {
            bool interior = cown[m.face_nodes[(size_t)e * 2]] == b && cown[m.face_nodes[(size_t)e * 2 + 1]] == b;
            for (int k = 0; k < m.interp_n[e] && interior; k++) interior = fown[m.interp_friends[(size_t)e * 10 + k]] == b;
            (interior ? in : bd).push_back(e);
        }
        fint[b] = (int)in.size();
        in.insert(in.end(), bd.begin(), bd.end());
        for (int q = 0; q < (int)in.size(); q++) { forder[lo + q] = in[q]; fpos[in[q]] = q; }
        lo = cstart[b]; hi = cstart[b + 1];
        in.clear(); bd.clear();
        for (int i = lo; i < hi; i++) {
            bool interior = true;
            for (int k = 0; k < m.nfriends(i) && interior; k++) interior = fown[m.faces[(size_t)i * 6 + k]] == b;
            (interior ? in : bd).push_back(i);
        }
        cint[b] = (int)in.size();
        in.insert(in.end(), bd.begin(), bd.end());
        for (int q = 0; q < (int)in.size(); q++) { corder[lo + q] = in[q]; cpos[in[q]] = q; }
    }
    PersistPlan pl;
    pl.P = P;
    pl.nf_max = nf_max;
    pl.nc_max = nc_max;
    if (!persistent_fits(c->p.precision, pl, nullptr)) return ODIS_OK;
    DevArena& A = c->mem;
    if (alist.empty()) alist.push_back(0);
    if (clist.empty()) clist.push_back(0);
    pl.fstart = A.upload(fstart);
    pl.cstart = A.upload(cstart);
    pl.fint = A.upload(fint);
    pl.cint = A.upload(cint);
    pl.forder = A.upload(forder);
    pl.corder = A.upload(corder);
    pl.fpos = A.upload(fpos);
    pl.cpos = A.upload(cpos);
    pl.fowner = A.upload(fown);
    pl.cowner = A.upload(cown);
    pl.depA_ptr = A.upload(aptr);
    pl.depA = A.upload(alist);
    pl.depC_ptr = A.upload(cptr);
    pl.depC = A.upload(clist);
    pl.flag_e = A.alloc<unsigned>(P);
    pl.flag_c = A.alloc<unsigned>(P);
    if (!pl.fstart || !pl.cstart || !pl.fint || !pl.cint || !pl.forder || !pl.corder || !pl.fpos || !pl.cpos ||
        !pl.fowner || !pl.cowner || !pl.depA_ptr || !pl.depA || !pl.depC_ptr || !pl.depC || !pl.flag_e || !pl.flag_c)
        return ODIS_ERR_NOMEM;
    c->persist_frac = 0.0;
    for (int b = 0; b < P; b++) c->persist_frac += (double)fint[b] / E;
    c->plan = pl;
    c->persist_ok = true;
    return ODIS_OK;
}

static int choose_exec_path(odis_ctx* c);
static int choose_sh_synthesis(odis_ctx* c);

extern "C" odis_status odis_create(const odis_params* p, const odis_mesh* mp, odis_ctx** out)
{
    if (!p || !mp || !out) return ODIS_ERR_ARG;
    *out = nullptr;
    if (p->precision != ODIS_FP64 && p->precision != ODIS_FP32 && p->precision != ODIS_DF64) return ODIS_ERR_ARG;
    if (!pot_valid(p->potential)) return ODIS_ERR_ARG;
    if (p->advection && pot_nodal(p->potential)) return ODIS_ERR_ARG;
    if (!(p->dt > 0.0) || !(p->g > 0.0) || !(p->h > 0.0) || !(p->radius > 0.0) || p->alpha < 0.0) return ODIS_ERR_ARG;
    if (p->sh_lmax < 0 || p->sh_lmax > 64 || (p->sh_lmax > 0 && !p->sh_factors)) return ODIS_ERR_ARG;
    if (p->friction != ODIS_FRIC_LINEAR && p->friction != ODIS_FRIC_QUADRATIC) return ODIS_ERR_ARG;
    if (p->advection && ((p->precision != ODIS_FP64 && p->precision != ODIS_DF64) || p->sh_lmax > 0))
        return ODIS_ERR_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return ODIS_ERR_CUDA;
    std::unique_ptr<odis_ctx> c(new (std::nothrow) odis_ctx);
    if (!c) return ODIS_ERR_NOMEM;
    const Mesh& m = mp->m;
    c->p = *p;
    if (p->sh_lmax > 0) c->sh_factors.assign(p->sh_factors, p->sh_factors + p->sh_lmax + 1);
    c->p.sh_factors = c->sh_factors.empty() ? nullptr : c->sh_factors.data();
    c->E = m.E;
    c->N = m.N;
    c->Ep = pad128(m.E);
    c->Np = pad128(m.N);
    c->r = m.r;
    c->eb = (m.E + kStepThreads - 1) / kStepThreads;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return ODIS_ERR_CUDA;
    c->own_stream = true;
    DevArena& A = c->mem;
    c->d_iter = A.alloc<long long>(1);
    c->d_run_first = A.alloc<long long>(1);
    c->d_status = A.alloc<int>(1);
    // per-run table of the face kernels' dissipation partials, one row per step, folded once per run chunk
    c->fold_rows = std::max(kGraphSteps, std::min(4096, (int)((64ll << 20) / (8ll * c->eb)) / kGraphSteps * kGraphSteps));
    c->d_partial = A.alloc<double>((size_t)(c->fold_rows + 1) * c->eb + 32);
    if (!c->d_iter || !c->d_run_first || !c->d_status || !c->d_partial) return ODIS_ERR_NOMEM;

    std::vector<double> Ua, Ub;
    int st = forcing_basis(m, c->p, Ua, Ub);
    if (st != ODIS_OK) return st;
    st = build_operators<double>(c.get(), m, Ua, Ub, c->op64);
    if (st != ODIS_OK) return st;
    if (p->precision == ODIS_FP32) {
        st = build_operators<float>(c.get(), m, Ua, Ub, c->op32);
        if (st != ODIS_OK) return st;
    }
    if (p->precision == ODIS_DF64) {
        st = build_operators<float2>(c.get(), m, Ua, Ub, c->opdf);
        if (st != ODIS_OK) return st;
    }
    // geometry needed by the per-operator calls
    std::vector<double> nrm((size_t)2 * c->Ep, 0.0), area(c->Ep, 0.0), trig((size_t)kNodeTrig * c->Np, 0.0);
    for (int e = 0; e < m.E; e++) {
        nrm[e] = m.face_normal[(size_t)e * 2];
        nrm[(size_t)c->Ep + e] = m.face_normal[(size_t)e * 2 + 1];
        area[e] = m.face_area[e];
    }
    for (int i = 0; i < m.N; i++) {
        const double lat = m.node_sph[(size_t)i * 2], lon = m.node_sph[(size_t)i * 2 + 1];
        // Pbar_20, Pbar_22 (4pi-normalised, Condon-Shortley phase) of z = sin(lat) by the
        // recurrences of the fully normalised functions, as the self-gravity basis
        const double z = std::cos(kPi * 0.5 - lat), sz = std::sqrt(std::fmax(0.0, 1.0 - z * z));
        const double p10 = std::sqrt(3.0) * z, p11 = -std::sqrt(3.0) * sz;
        const double p20 = std::sqrt(15.0 / 4.0) * z * p10 - std::sqrt(5.0 / 4.0) * 1.0;
        const double p22 = -std::sqrt(5.0 / 4.0) * sz * p11;
        const double t[kNodeTrig] = {std::cos(lat), std::sin(lat), std::cos(lon), std::sin(lon), std::cos(2.0 * lat),
                                     std::sin(2.0 * lat), std::cos(2.0 * lon), std::sin(2.0 * lon),
                                     std::pow(std::cos(lat), 2.0), std::pow(std::sin(lat), 2.0), p20, p22};
        for (int k = 0; k < kNodeTrig; k++) trig[(size_t)k * c->Np + i] = t[k];
    }
    c->nrm = A.upload(nrm);
    c->area = A.upload(area);
    c->trig = A.upload(trig);
    {
        std::vector<double> blk, soa((size_t)18 * c->Np, 0.0);
        build_rbf(m, blk);
        for (int i = 0; i < m.N; i++)
            for (int q = 0; q < 18; q++) soa[(size_t)q * c->Np + i] = blk[(size_t)i * 18 + q];
        c->rbf = A.upload(soa);
        if (p->advection && p->precision == ODIS_DF64) {
            auto df = [](const std::vector<double>& x) {
                std::vector<float2> y(x.size());
                for (size_t i = 0; i < x.size(); i++) y[i] = df_from_double(x[i]);
                return y;
            };
            c->rbf_df = A.upload(df(soa));
            c->nrm_df = A.upload(df(nrm));
            c->area_df = A.upload(df(area));
            if (!c->rbf_df || !c->nrm_df || !c->area_df) return ODIS_ERR_NOMEM;
        }
    }
    if (!c->nrm || !c->area || !c->trig || !c->rbf) return ODIS_ERR_NOMEM;

    st = alloc_state<double>(c.get(), c->s64, false);
    if (st != ODIS_OK) return st;
    if (p->precision == ODIS_FP32) {
        st = alloc_state<float>(c.get(), c->s32, true);
        if (st != ODIS_OK) return st;
    }
    if (p->precision == ODIS_DF64) {
        st = alloc_state<float2>(c.get(), c->sdf, false);
        if (st != ODIS_OK) return st;
    }
    if (p->sh_lmax > 0) {
        st = sh_create(&c->sh, m, p->sh_lmax, c->p.sh_factors, p->precision, c->Np, c->d_status);
        if (st != ODIS_OK) return st;
        c->s64.usg = sh_usg64(c->sh);
        c->s32.usg = sh_usg32(c->sh);
        c->sdf.usg = sh_usgdf(c->sh);
    }
    c->fk = ForcingConst{p->potential, p->angvel, p->radius, p->love_reduct, p->ecc, p->obliq, p->semimajor_axis,
                         (double)p->fourier_freq};
    c->nodal = pot_nodal(p->potential);
    if (c->nodal && !c->sh) {      // a node buffer of its own; with self-gravity the synthesis buffer takes the sum
        const size_t esz = p->precision == ODIS_FP32 ? sizeof(float) : sizeof(double);
        c->ufr = A.alloc<double>(((size_t)c->Np * esz + 7) / 8);
        if (!c->ufr) return ODIS_ERR_NOMEM;
        c->s64.usg = p->precision == ODIS_FP64 ? (const double*)c->ufr : nullptr;
        c->s32.usg = p->precision == ODIS_FP32 ? (const float*)c->ufr : nullptr;
        c->sdf.usg = p->precision == ODIS_DF64 ? (const float2*)c->ufr : nullptr;
    }
    StepConst& sc = c->sc;
    sc.E = m.E;
    sc.N = m.N;
    sc.Ep = c->Ep;
    sc.Np = c->Np;
    sc.dt = p->dt;
    sc.alpha = p->alpha;
    sc.angvel = p->angvel;
    sc.ab3a = 23. / 12.;
    sc.ab3b = -16. / 12.;
    sc.ab3c = 5. / 12.;
    sc.init_load = p->init_load ? 1 : 0;
    sc.quad = p->friction == ODIS_FRIC_QUADRATIC ? 1 : 0;
    sc.use_sg = (p->sh_lmax > 0 || c->nodal) ? 1 : 0;
    sc.df_dt = df_from_double(p->dt);
    sc.df_malpha = df_from_double(-p->alpha);
    sc.df_a = df_from_double(sc.ab3a);
    sc.df_b = df_from_double(sc.ab3b);
    sc.df_c = df_from_double(sc.ab3c);
    sc.f_dt = (float)p->dt;
    sc.f_malpha = (float)(-p->alpha);
    sc.f_a = (float)sc.ab3a;
    sc.f_b = (float)sc.ab3b;
    sc.f_c = (float)sc.ab3c;
    if ((p->precision == ODIS_FP64 || p->precision == ODIS_DF64) && p->sh_lmax == 0 && !c->nodal) {
        st = build_persist_plan(c.get(), m);
        if (st != ODIS_OK) return st;
    }
    c->stage_n = (size_t)3 * std::max(c->Ep, c->Np);
    for (int k = 0; k < 4; k++) {
        c->stage[k] = A.alloc<double>(c->stage_n);
        if (!c->stage[k]) return ODIS_ERR_NOMEM;
    }
    c->slot0_saved.assign((size_t)(m.E + m.N), 0.0);
    if (cudaDeviceSynchronize() != cudaSuccess) return ODIS_ERR_CUDA;
    if (p->advection) {            // the nonlinear loop has its own operators and reference-layout state
        c->persist_ok = false;
        st = adv_create(&c->adv, m, p->angvel, c->Ep, c->Np, p->precision == ODIS_DF64);
        if (st == ODIS_OK) st = adv_state_alloc(c->adv, p->precision, p->h, Ua, Ub);
        if (st != ODIS_OK) return st;
    } else {
        st = choose_sh_synthesis(c.get());
        if (st == ODIS_OK) st = choose_exec_path(c.get());
        if (st != ODIS_OK) return st;
    }
    *out = c.release();
    return ODIS_OK;
}

extern "C" void odis_destroy(odis_ctx* c)
{
    if (!c) return;
    cudaStreamSynchronize(c->stream);
    delete c;
}

extern "C" odis_status odis_set_stream(odis_ctx* c, void* s)
{
    if (!c) return ODIS_ERR_ARG;
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return ODIS_ERR_CUDA;
    if (c->own_stream) cudaStreamDestroy(c->stream);
    c->own_stream = false;
    c->stream = (cudaStream_t)s;
    return ODIS_OK;
}

extern "C" odis_status odis_synchronize(odis_ctx* c)
{
    if (!c) return ODIS_ERR_ARG;
    return cudaStreamSynchronize(c->stream) == cudaSuccess ? ODIS_OK : ODIS_ERR_CUDA;
}

extern "C" odis_status odis_device_status(odis_ctx* c)
{
    if (!c) return ODIS_ERR_ARG;
    int h = 0;
    ODIS_CK(cudaMemcpyAsync(&h, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    ODIS_CK(cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream));
    ODIS_CK(cudaStreamSynchronize(c->stream));
    for (int b = 1; b < 16; b++)
        if (h & (1 << b)) return b;
    return ODIS_OK;
}

// ---------------------------------------------------------------------------
// per-operator calls
// ---------------------------------------------------------------------------
namespace {

struct Io {
    odis_ctx* c;
    int mem;
    int slot = 0;
    // device view of a caller buffer of n doubles (copied in if `in`)
    double* in(const double* p, size_t n) {
        if (mem == ODIS_MEM_DEVICE) return const_cast<double*>(p);
        double* d = c->stage[slot++];
        if (n && cudaMemcpyAsync(d, p, n * sizeof(double), cudaMemcpyHostToDevice, c->stream) != cudaSuccess) return nullptr;
        return d;
    }
    double* out(double* p) { return mem == ODIS_MEM_DEVICE ? p : c->stage[slot++]; }
    int back(double* host, const double* dev, size_t n) {
        if (mem == ODIS_MEM_DEVICE || !host) return ODIS_OK;
        ODIS_CK(cudaMemcpyAsync(host, dev, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        return ODIS_OK;
    }
    int done() {
        ODIS_CK(cudaGetLastError());
        ODIS_CK(cudaStreamSynchronize(c->stream));
        return ODIS_OK;
    }
};

bool mem_ok(int mem) { return mem == ODIS_MEM_HOST || mem == ODIS_MEM_DEVICE; }

}  // namespace

extern "C" odis_status odis_update_momentum(odis_ctx* c, double* dvdt, const double* v, const double* eta, int mem)
{
    if (!c || !dvdt || !v || !eta || !mem_ok(mem)) return ODIS_ERR_ARG;
    Io io{c, mem};
    const double* dv = io.in(v, c->E);
    const double* de = io.in(eta, c->N);
    double* dout = io.out(dvdt);
    if (!dv || !de) return ODIS_ERR_CUDA;
    launch_momentum(c->op64.fc, c->E, c->Ep, dout, dv, de, c->stream);
    int st = io.back(dvdt, dout, c->E);
    return st != ODIS_OK ? st : io.done();
}

extern "C" odis_status odis_interpolate_cartesian(odis_ctx* c, double* uxyz, const double* v, int mem)
{
    if (!c || !uxyz || !v || !mem_ok(mem)) return ODIS_ERR_ARG;
    Io io{c, mem};
    const double* dv = io.in(v, c->E);
    double* dout = io.out(uxyz);
    if (!dv) return ODIS_ERR_CUDA;
    launch_rbf(c->rbf, c->op64.cc.edge, c->N, c->Np, dv, dout, c->stream);
    int st = io.back(uxyz, dout, (size_t)3 * c->N);
    return st != ODIS_OK ? st : io.done();
}

extern "C" odis_status odis_momentum_advection(odis_ctx* c, const odis_mesh* mesh, double* dvdt, const double* v,
                                               const double* h_total, double* ekin, int mem)
{
    if (!c || !dvdt || !v || !h_total || !mem_ok(mem)) return ODIS_ERR_ARG;
    if (!c->adv) {
        if (!mesh || mesh->m.N != c->N || mesh->m.E != c->E) return ODIS_ERR_ARG;
        const int st = adv_create(&c->adv, mesh->m, c->p.angvel, c->Ep, c->Np);
        if (st != ODIS_OK) return st;
    }
    Io io{c, mem};
    const double* dv = io.in(v, c->E);
    const double* dh = io.in(h_total, c->N);
    double* dd = io.in(dvdt, c->E);
    double* dk = (mem == ODIS_MEM_DEVICE && ekin) ? ekin : (mem == ODIS_MEM_DEVICE ? adv_ekin_scratch(c->adv) : io.out(ekin));
    if (!dv || !dh || !dd) return ODIS_ERR_CUDA;
    adv_momentum(c->adv, c->rbf, c->op64.cc.edge, c->op64.fc.nbr, c->op64.fc.w, dd, dv, dh, dk, c->stream);
    c->launches += adv_kernels_per_call();
    int st = io.back(dvdt, dd, c->E);
    if (st == ODIS_OK && ekin) st = io.back(ekin, dk, c->N);
    return st != ODIS_OK ? st : io.done();
}

extern "C" odis_status odis_lsq_flux(odis_ctx* c, const odis_mesh* mesh, double* flux, const double* v,
                                     const double* h_total, int mem)
{
    if (!c || !flux || !v || !h_total || !mem_ok(mem)) return ODIS_ERR_ARG;
    if (!c->adv) {
        if (!mesh || mesh->m.N != c->N || mesh->m.E != c->E) return ODIS_ERR_ARG;
        const int st = adv_create(&c->adv, mesh->m, c->p.angvel, c->Ep, c->Np);
        if (st != ODIS_OK) return st;
    }
    Io io{c, mem};
    const double* dv = io.in(v, c->E);
    const double* dh = io.in(h_total, c->N);
    double* dout = io.out(flux);
    if (!dv || !dh) return ODIS_ERR_CUDA;
    adv_lsq_flux(c->adv, dout, dv, dh, c->stream);
    c->launches += 1;
    int st = io.back(flux, dout, c->E);
    return st != ODIS_OK ? st : io.done();
}

extern "C" odis_status odis_update_eta(odis_ctx* c, double* detadt, const double* v, int mem)
{
    if (!c || !detadt || !v || !mem_ok(mem)) return ODIS_ERR_ARG;
    Io io{c, mem};
    const double* dv = io.in(v, c->E);
    double* dout = io.out(detadt);
    if (!dv) return ODIS_ERR_CUDA;
    launch_divergence(c->op64.cc, c->N, c->Np, dout, dv, c->stream);
    int st = io.back(detadt, dout, c->N);
    return st != ODIS_OK ? st : io.done();
}

extern "C" odis_status odis_forcing(odis_ctx* c, double* U, int type, double t, double ecc, double obl, int mem)
{
    if (!c || !U || !mem_ok(mem) || !pot_valid(type)) return ODIS_ERR_ARG;
    if (!pot_has_case(type)) return ODIS_OK;       // the reference's switch leaves U as it is
    Io io{c, mem};
    double* dout = io.out(U);
    const ForcingConst k{type, c->p.angvel, c->p.radius, c->p.love_reduct, ecc, obl, c->p.semimajor_axis,
                         (double)c->p.fourier_freq};
    launch_forcing(c->trig, c->N, c->Np, dout, k, forcing_terms(k, t), c->stream);
    int st = io.back(U, dout, c->N);
    return st != ODIS_OK ? st : io.done();
}

extern "C" odis_status odis_ab3(odis_ctx* c, double* s, double* hist, int iter, int num, int mem)
{
    if (!c || !s || !hist || num < 0 || iter < 0 || !mem_ok(mem)) return ODIS_ERR_ARG;
    if ((size_t)num * 3 > c->stage_n) return ODIS_ERR_ARG;
    Io io{c, mem};
    double* ds = io.in(s, num);
    double* dh = io.in(hist, (size_t)num * 3);
    if (!ds || !dh) return ODIS_ERR_CUDA;
    launch_ab3_ref(ds, dh, iter, num, c->p.dt, c->p.init_load, c->stream);
    int st = io.back(s, ds, num);
    if (st == ODIS_OK) st = io.back(hist, dh, (size_t)num * 3);
    return st != ODIS_OK ? st : io.done();
}

extern "C" odis_status odis_interpolate_velocity(odis_ctx* c, double* uv, const double* v, int mem)
{
    if (!c || !uv || !v || !mem_ok(mem)) return ODIS_ERR_ARG;
    Io io{c, mem};
    const double* dv = io.in(v, c->E);
    double* dout = io.out(uv);
    if (!dv) return ODIS_ERR_CUDA;
    launch_interp(c->op64.fc, c->nrm, c->E, c->Ep, dout, dv, c->stream);
    int st = io.back(uv, dout, (size_t)c->E * 2);
    return st != ODIS_OK ? st : io.done();
}

extern "C" odis_status odis_update_energy(odis_ctx* c, double* avg, double* e, const double* uv, int mem)
{
    if (!c || !avg || !uv || !mem_ok(mem)) return ODIS_ERR_ARG;
    Io io{c, mem};
    const double* duv = io.in(uv, (size_t)c->E * 2);
    double* de = e ? io.out(e) : nullptr;
    double* davg = mem == ODIS_MEM_DEVICE ? avg : c->stage[3];
    if (!duv) return ODIS_ERR_CUDA;
    launch_energy(c->area, c->E, energy_coef(c->p), c->p.friction == ODIS_FRIC_QUADRATIC, 4 * kPi * std::pow(c->r, 2.0),
                  duv, de, c->d_partial, davg, c->stream);
    int st = e ? io.back(e, de, c->E) : ODIS_OK;
    if (st == ODIS_OK) st = io.back(avg, davg, 1);
    return st != ODIS_OK ? st : io.done();
}

// ---------------------------------------------------------------------------
// fused time loop
// ---------------------------------------------------------------------------
static const void* state_eta(const odis_ctx* c)
{
    return c->p.precision == ODIS_FP32 ? (const void*)c->s32.eta
         : c->p.precision == ODIS_DF64 ? (const void*)c->sdf.eta : (const void*)c->s64.eta;
}

static int kernels_per_step(const odis_ctx* c)
{
    return 2 + (c->sh ? sh_kernels_per_step(c->sh) : 0) + (c->nodal ? 1 : 0);
}

static void* usg_buffer(odis_ctx* c)
{
    return c->p.precision == ODIS_FP32 ? (void*)c->s32.usg : c->p.precision == ODIS_DF64 ? (void*)c->sdf.usg
                                                                                         : (void*)c->s64.usg;
}

static void enqueue_steps(odis_ctx* c, int n)
{
    c->launches += (long long)n * kernels_per_step(c) + 1;
    for (int k = 0; k < n; k++) {
        if (c->sh) sh_enqueue(c->sh, state_eta(c), c->stream);
        if (c->nodal)
            launch_node_forcing(c->p.precision, c->trig, c->N, c->Np, usg_buffer(c), c->sh ? 1 : 0, 1.0 / c->p.g, c->fk,
                                c->d_fterms, c->d_iter, c->d_run_first, k, c->stream);
        if (c->p.precision == ODIS_FP64) launch_step<double, false>(c->op64.fc, c->op64.cc, c->s64, c->sc, k, c->stream);
        else if (c->p.precision == ODIS_FP32) launch_step<float, true>(c->op32.fc, c->op32.cc, c->s32, c->sc, k, c->stream);
        else {
            launch_edge_df(c->opdf.fc, c->sdf, c->sc, k, c->stream);
            launch_cell_df(c->opdf.cc, c->sdf, c->sc, k, c->stream);
        }
    }
    launch_bump(c->d_iter, n, c->stream);
}

static int ensure_graph(odis_ctx* c)
{
    if (c->graph) return ODIS_OK;
    cudaGraph_t g = nullptr;
    const long long before = c->launches;
    ODIS_CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    enqueue_steps(c, kGraphSteps);
    c->launches = before;     // capture launches nothing; replays are counted
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (e != cudaSuccess) { if (g) cudaGraphDestroy(g); return ODIS_ERR_CUDA; }
    e = cudaGraphInstantiate(&c->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { c->graph = nullptr; return ODIS_ERR_CUDA; }
    return ODIS_OK;
}

// Forcing-phase table for steps first .. first+n-1 (grown as needed; a new
// buffer invalidates the instantiated graph, which bakes in the pointer).
static int prepare_phase(odis_ctx* c, long long first, int n)
{
    const size_t esz = c->p.precision == ODIS_FP32 ? sizeof(float) : c->p.precision == ODIS_DF64 ? sizeof(float2)
                                                                                              : sizeof(double);
    if (n > c->phase_cap) {
        if (c->d_phase) cudaFree(c->d_phase);
        c->d_phase = nullptr;
        c->phase_cap = 0;
        const int cap = std::max(n, 4096);
        ODIS_CK(cudaMalloc(&c->d_phase, esz * 2 * (size_t)cap));
        c->phase_cap = cap;
        c->s64.phase = (const double*)c->d_phase;
        c->s32.phase = (const float*)c->d_phase;
        c->sdf.phase = (const float2*)c->d_phase;
        if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
    }
    if (c->nodal) {
        if (n > c->fterms_cap) {
            if (c->d_fterms) cudaFree(c->d_fterms);
            c->d_fterms = nullptr;
            c->fterms_cap = 0;
            const int cap = std::max(n, 4096);
            ODIS_CK(cudaMalloc(&c->d_fterms, sizeof(double) * kForcingTerms * (size_t)cap));
            c->fterms_cap = cap;
            if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
        }
        launch_forcing_terms(c->d_fterms, c->fk, first, n, c->p.dt, c->stream);
        c->launches += 1;
    }
    launch_phase(c->d_phase, c->p.precision, first, n, c->p.dt, c->p.angvel, c->stream);
    c->launches += 1;
    return cudaGetLastError() == cudaSuccess ? ODIS_OK : ODIS_ERR_CUDA;
}

// One chunk of at most fold_rows steps; dpow (device, nullable) receives its power series.
static int run_chunk(odis_ctx* c, int n, double* dpow)
{
    const long long first = c->iter;
    ODIS_CK(cudaMemcpyAsync(c->d_run_first, &first, sizeof(long long), cudaMemcpyHostToDevice, c->stream));
    ODIS_CK(cudaMemcpyAsync(c->d_iter, &first, sizeof(long long), cudaMemcpyHostToDevice, c->stream));
    {
        const int st = prepare_phase(c, first, n);
        if (st != ODIS_OK) return st;
    }
    // only the end-of-chunk fold writes the power series (the step kernels write
    // partials), so the instantiated graph does not depend on dpow
    c->s64.power = dpow;
    c->s32.power = dpow;
    c->sdf.power = dpow;
    bool persisted = false;
    if (c->persist_ok && c->persist_on) {
        // one cooperative launch for the whole chunk
        if (n + 1 > c->part_cap) {
            if (c->plan.part) cudaFree(c->plan.part);
            c->plan.part = nullptr;
            c->part_cap = 0;
            const int cap = std::max(n + 1, 4097);
            ODIS_CK(cudaMalloc(&c->plan.part, sizeof(double) * (size_t)cap * c->plan.P));
            c->part_cap = cap;
        }
        const void* fc = c->p.precision == ODIS_FP64 ? (const void*)&c->op64.fc : (const void*)&c->opdf.fc;
        const void* cc = c->p.precision == ODIS_FP64 ? (const void*)&c->op64.cc : (const void*)&c->opdf.cc;
        const void* stp = c->p.precision == ODIS_FP64 ? (const void*)&c->s64 : (const void*)&c->sdf;
        const int st = launch_persistent(c->p.precision, fc, cc, stp, c->sc, c->plan, n, first, dpow, c->stream);
        if (st == ODIS_OK) {
            persisted = true;
            c->launches += 2;
        } else {
            // the device refused the cooperative launch (e.g. SMs taken by other
            // work): nothing ran, keep to the graph-replayed step from now on
            cudaGetLastError();
            c->persist_ok = false;
        }
    }
    if (!persisted) {
        int done = 0;
        if (n >= kGraphSteps) {
            int st = ensure_graph(c);
            if (st != ODIS_OK) return st;
            for (; done + kGraphSteps <= n; done += kGraphSteps) {
                ODIS_CK(cudaGraphLaunch(c->graph, c->stream));
                c->launches += (long long)kGraphSteps * kernels_per_step(c) + 1;
            }
        }
        if (done < n) enqueue_steps(c, n - done);
        if (c->p.precision == ODIS_FP64) launch_power_tail<double>(c->op64.fc, c->s64, c->sc, n, c->stream);
        else if (c->p.precision == ODIS_FP32) launch_power_tail<float>(c->op32.fc, c->s32, c->sc, n, c->stream);
        else launch_power_tail_df(c->opdf.fc, c->sdf, c->sc, n, c->stream);
        c->launches += dpow ? 2 : 1;
    }
    ODIS_CK(cudaGetLastError());
    c->iter += n;
    return ODIS_OK;
}

// ab3Explicit with advection true (src/timeIntegrator.cpp:205-269): per step the
// momentum tendency with the advection term, forcing at t + dt, AB3 with drag
// and forcing outside it, the continuity equation with the LSQ thickness flux,
// the dissipated power from the new velocity, then the column thickness.
static odis_status run_advective(odis_ctx* c, int n, double* dpow)
{
    const odis_params& p = c->p;
    const int G = adv_graph_steps();
    const int per_step = adv_kernels_per_step();
    const bool df = p.precision == ODIS_DF64;
    const AdvStepArgs x{df ? (const void*)c->rbf_df : (const void*)c->rbf, c->op64.cc.edge,
                        df ? c->opdf.fc.nbr : c->op64.fc.nbr, df ? (const void*)c->opdf.fc.w : (const void*)c->op64.fc.w,
                        df ? (const void*)c->nrm_df : (const void*)c->nrm,
                        df ? (const void*)c->area_df : (const void*)c->area, p.g, p.alpha, p.h,
                        p.dt, 4 * kPi * std::pow(c->r, 2.0), p.init_load, p.friction == ODIS_FRIC_QUADRATIC};
    auto step = [&](int it, double* out) { adv_step(c->adv, x, it, out, c->stream); };
    adv_set_step(c->adv, c->iter, p.dt, c->stream);
    c->launches += 1;
    for (int done = 0; done < n;) {
        const int it = (int)c->iter;
        if ((it > 1 || p.init_load) && n - done >= G) {
            // AB3 steps in whole chunks: one graph of G steps, captured once (AB3 mode
            // fixed, forcing phase from the device step counter, power into the chunk buffer)
            cudaGraphExec_t* ge = adv_graph(c->adv);
            if (!*ge) {
                cudaGraph_t gr = nullptr;
                ODIS_CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
                for (int k = 0; k < G; k++) step(2, adv_graph_power(c->adv) + k);
                ODIS_CK(cudaStreamEndCapture(c->stream, &gr));
                const cudaError_t e = cudaGraphInstantiate(ge, gr, 0);
                cudaGraphDestroy(gr);
                if (e != cudaSuccess) { *ge = nullptr; return ODIS_ERR_CUDA; }
            }
            ODIS_CK(cudaGraphLaunch(*ge, c->stream));
            if (dpow)
                ODIS_CK(cudaMemcpyAsync(dpow + done, adv_graph_power(c->adv), sizeof(double) * G,
                                        cudaMemcpyDeviceToDevice, c->stream));
            c->iter += G;
            done += G;
            c->launches += (long long)G * per_step;
        } else {
            step(it, dpow + done);
            c->iter++;
            done++;
            c->launches += per_step;
        }
    }
    ODIS_CK(cudaGetLastError());
    return ODIS_OK;
}

extern "C" odis_status odis_run_steps(odis_ctx* c, int n, double* power, int mem)
{
    if (!c || n < 0 || !mem_ok(mem)) return ODIS_ERR_ARG;
    if (n == 0) return ODIS_OK;
    if (c->p.advection) {
        double* dpow = nullptr;
        if (power && mem == ODIS_MEM_DEVICE) dpow = power;
        else {
            if (n > c->power_cap) {
                if (c->d_power) cudaFree(c->d_power);
                c->d_power = nullptr;
                c->power_cap = 0;
                ODIS_CK(cudaMalloc(&c->d_power, sizeof(double) * n));
                c->power_cap = n;
            }
            dpow = c->d_power;
        }
        const int st = run_advective(c, n, dpow);
        if (st != ODIS_OK) return st;
        double last = 0.0;
        ODIS_CK(cudaMemcpyAsync(&last, dpow + n - 1, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        if (power && mem == ODIS_MEM_HOST)
            ODIS_CK(cudaMemcpyAsync(power, dpow, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
        ODIS_CK(cudaStreamSynchronize(c->stream));
        return std::isfinite(last) ? ODIS_OK : ODIS_ERR_NONFINITE;
    }
    double* dpow = nullptr;
    if (power) {
        if (mem == ODIS_MEM_DEVICE) dpow = power;
        else {
            if (n > c->power_cap) {
                if (c->d_power) cudaFree(c->d_power);
                c->d_power = nullptr;
                c->power_cap = 0;
                ODIS_CK(cudaMalloc(&c->d_power, sizeof(double) * n));
                c->power_cap = n;
            }
            dpow = c->d_power;
        }
    }
    for (int done = 0; done < n;) {
        const int k = std::min(n - done, c->fold_rows);
        const int st = run_chunk(c, k, dpow ? dpow + done : nullptr);
        if (st != ODIS_OK) return st;
        done += k;
    }
    if (power && mem == ODIS_MEM_HOST)
        ODIS_CK(cudaMemcpyAsync(power, dpow, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    ODIS_CK(cudaStreamSynchronize(c->stream));
    int h = 0;
    ODIS_CK(cudaMemcpy(&h, c->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) ODIS_CK(cudaMemset(c->d_status, 0, sizeof(int)));
    if (h & (1 << ODIS_ERR_TIMEOUT)) return ODIS_ERR_TIMEOUT;
    if (h & (1 << ODIS_ERR_NONFINITE)) return ODIS_ERR_NONFINITE;
    return ODIS_OK;
}

// ---------------------------------------------------------------------------
// state in the reference's layout
// ---------------------------------------------------------------------------
// device vector (or its FP64 master, when present) -> host doubles
template <class T>
static int get_vec(odis_ctx* c, const T* v, const float* lo, size_t n, double* out)
{
    (void)c;
    std::vector<T> a(n);
    ODIS_CK(cudaMemcpy(a.data(), v, n * sizeof(T), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; i++) out[i] = to_d(a[i]);
    if (lo) {
        std::vector<float> b(n);
        ODIS_CK(cudaMemcpy(b.data(), lo, n * sizeof(float), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < n; i++) out[i] += (double)b[i];
    }
    return ODIS_OK;
}

// host doubles -> device vector (rounded to T) and, when present, the rounding residual
template <class T>
static int set_vec(T* v, float* lo, size_t n, const double* in)
{
    std::vector<T> a(n);
    for (size_t i = 0; i < n; i++) a[i] = cvt<T>(in[i]);
    ODIS_CK(cudaMemcpy(v, a.data(), n * sizeof(T), cudaMemcpyHostToDevice));
    if (lo) {
        std::vector<float> b(n);
        for (size_t i = 0; i < n; i++) b[i] = (float)(in[i] - to_d(a[i]));
        ODIS_CK(cudaMemcpy(lo, b.data(), n * sizeof(float), cudaMemcpyHostToDevice));
    }
    return ODIS_OK;
}

template <class T>
static int get_state_t(odis_ctx* c, State<T>& s, double* v, double* eta, double* dvdt, double* detadt)
{
    const long long k = c->iter;
    const size_t E = c->E, N = c->N;
    int st = ODIS_OK;
    if (v) st = get_vec<T>(c, s.v[k & 1], s.vlo, E, v);
    if (st == ODIS_OK && eta) st = get_vec<T>(c, s.eta, s.etalo, N, eta);
    for (int which = 0; which < 2 && st == ODIS_OK; which++) {
        double* out = which == 0 ? dvdt : detadt;
        if (!out) continue;
        const size_t n = which == 0 ? E : N;
        T* const* h = which == 0 ? s.hv : s.he;
        std::vector<double> a(n), b(n);
        st = get_vec<T>(c, h[0], nullptr, n, a.data());
        if (st == ODIS_OK) st = get_vec<T>(c, h[1], nullptr, n, b.data());
        const std::vector<double>& h0 = a;    // hv[0]
        const std::vector<double>& h1 = b;    // hv[1]
        const double* saved = c->slot0_saved.data() + (which == 0 ? 0 : E);
        for (size_t i = 0; i < n; i++) {
            double s0, s1, s2;
            if (k == 0) { s0 = saved[i]; s1 = h1[i]; s2 = h0[i]; }
            else if (k == 1 && !c->p.init_load) { s0 = h0[i]; s1 = h1[i]; s2 = h0[i]; }
            else {
                const double fl = ((k + 1) & 1) ? h1[i] : h0[i];
                const double fo = (k & 1) ? h1[i] : h0[i];
                s0 = fl; s1 = fl; s2 = fo;
            }
            out[i * 3] = s0; out[i * 3 + 1] = s1; out[i * 3 + 2] = s2;
        }
    }
    return st;
}

template <class T>
static int set_state_t(odis_ctx* c, State<T>& s, long long k, const double* v, const double* eta, const double* dvdt,
                       const double* detadt)
{
    const size_t E = c->E, N = c->N;
    int st = ODIS_OK;
    for (int q = 0; q < 2; q++) ODIS_CK(cudaMemset(s.v[q], 0, sizeof(T) * c->Ep));
    if (s.vlo) ODIS_CK(cudaMemset(s.vlo, 0, sizeof(float) * c->Ep));
    if (v) st = set_vec<T>(s.v[k & 1], s.vlo, E, v);
    ODIS_CK(cudaMemset(s.eta, 0, sizeof(T) * c->Np));
    if (s.etalo) ODIS_CK(cudaMemset(s.etalo, 0, sizeof(float) * c->Np));
    if (st == ODIS_OK && eta) st = set_vec<T>(s.eta, s.etalo, N, eta);
    for (int which = 0; which < 2 && st == ODIS_OK; which++) {
        const double* in = which == 0 ? dvdt : detadt;
        const size_t n = which == 0 ? E : N;
        T* const* h = which == 0 ? s.hv : s.he;
        std::vector<double> h0(n, 0.0), h1(n, 0.0);
        double* saved = c->slot0_saved.data() + (which == 0 ? 0 : E);
        for (size_t i = 0; i < n; i++) {
            const double s0 = in ? in[i * 3] : 0.0, s1 = in ? in[i * 3 + 1] : 0.0, s2 = in ? in[i * 3 + 2] : 0.0;
            saved[i] = s0;
            if (k == 1 && !c->p.init_load) { h0[i] = s2; h1[i] = s1; }
            else if ((k + 1) & 1) { h1[i] = s1; h0[i] = s2; }
            else { h0[i] = s1; h1[i] = s2; }
        }
        st = set_vec<T>(h[0], nullptr, n, h0.data());
        if (st == ODIS_OK) st = set_vec<T>(h[1], nullptr, n, h1.data());
    }
    return st;
}

extern "C" odis_status odis_get_state(odis_ctx* c, int* iter, double* v, double* eta, double* dvdt, double* detadt)
{
    if (!c) return ODIS_ERR_ARG;
    ODIS_CK(cudaStreamSynchronize(c->stream));
    if (iter) *iter = (int)c->iter;
    if (c->p.advection) return adv_get_state(c->adv, v, eta, dvdt, detadt);
    if (c->p.precision == ODIS_DF64) return get_state_t<float2>(c, c->sdf, v, eta, dvdt, detadt);
    return c->p.precision == ODIS_FP64 ? get_state_t<double>(c, c->s64, v, eta, dvdt, detadt)
                                       : get_state_t<float>(c, c->s32, v, eta, dvdt, detadt);
}

extern "C" odis_status odis_set_state(odis_ctx* c, int iter, const double* v, const double* eta, const double* dvdt,
                                      const double* detadt)
{
    if (!c || iter < 0) return ODIS_ERR_ARG;
    ODIS_CK(cudaStreamSynchronize(c->stream));
    c->iter = iter;
    if (c->p.advection) {
        const int st = adv_set_state(c->adv, v, eta, dvdt, detadt);
        if (st != ODIS_OK) return st;
        adv_thickness(c->adv, c->p.h, c->stream);   // src/timeIntegrator.cpp:203
        ODIS_CK(cudaStreamSynchronize(c->stream));
        return ODIS_OK;
    }
    if (c->p.precision == ODIS_DF64) return set_state_t<float2>(c, c->sdf, iter, v, eta, dvdt, detadt);
    return c->p.precision == ODIS_FP64 ? set_state_t<double>(c, c->s64, iter, v, eta, dvdt, detadt)
                                       : set_state_t<float>(c, c->s32, iter, v, eta, dvdt, detadt);
}

// Times the persistent loop against the graph-replayed kernel pair (best of two
// runs of 3 graph chunks each, after one warm-up run of each, host clock around
// the synchronising run call), keeps the faster one as the default and puts the
// context back in its freshly created state (zero state, step 0, no launches).
static int choose_exec_path(odis_ctx* c)
{
    if (!c->persist_ok) return ODIS_OK;
    const int n = 3 * kGraphSteps;
    double best[2] = {1e300, 1e300};
    for (int rep = 0; rep < 3; rep++) {
        for (int mode = 0; mode < 2 && c->persist_ok; mode++) {
            c->persist_on = mode == 1;
            const auto t0 = std::chrono::steady_clock::now();
            const int st = odis_run_steps(c, n, nullptr, ODIS_MEM_DEVICE);
            const auto t1 = std::chrono::steady_clock::now();
            // a NaN from an unstable dt is the caller's to find on a real run
            if (st == ODIS_ERR_TIMEOUT && mode == 1) { c->persist_ok = false; break; }
            if (st != ODIS_OK && st != ODIS_ERR_NONFINITE) return st;
            if (rep > 0) best[mode] = std::min(best[mode], std::chrono::duration<double, std::milli>(t1 - t0).count() / n);
        }
    }
    c->exec_ms[0] = best[0];
    c->exec_ms[1] = best[1];
    c->persist_auto = c->persist_ok && best[1] < best[0];
    c->persist_on = c->persist_auto;
    c->launches = 0;
    return odis_set_state(c, 0, nullptr, nullptr, nullptr, nullptr);
}

// The dense self-gravity synthesis against the factored one over whole
// graph-replayed steps (its matrix competes for L2 with the step's other
// arrays, which the transforms' own timing does not see): best of two runs of
// 3 graph chunks each way after a warm-up, the graph captured again for each
// choice; keeps the faster and puts the context back in its fresh state.
static int choose_sh_synthesis(odis_ctx* c)
{
    if (!c->sh || !sh_dense_candidate(c->sh)) return ODIS_OK;
    const int n = 3 * kGraphSteps;
    double best[2] = {1e300, 1e300};
    for (int rep = 0; rep < 3; rep++) {
        for (int mode = 0; mode < 2; mode++) {
            sh_try_dense(c->sh, mode == 1);
            if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
            const auto t0 = std::chrono::steady_clock::now();
            const int st = odis_run_steps(c, n, nullptr, ODIS_MEM_DEVICE);
            const auto t1 = std::chrono::steady_clock::now();
            if (st != ODIS_OK && st != ODIS_ERR_NONFINITE) return st;
            if (rep > 0) best[mode] = std::min(best[mode], std::chrono::duration<double, std::milli>(t1 - t0).count() / n);
        }
    }
    sh_set_dense(c->sh, best[1] < best[0]);
    if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
    c->launches = 0;
    return odis_set_state(c, 0, nullptr, nullptr, nullptr, nullptr);
}

// ---------------------------------------------------------------------------
// measurement helpers
// ---------------------------------------------------------------------------
extern "C" odis_status odis_set_wait_limit(odis_ctx* c, unsigned polls, int withhold)
{
    if (!c || withhold < -1 || (c->persist_ok && withhold >= c->plan.P)) return ODIS_ERR_ARG;
    c->plan.spin_limit = polls;
    c->plan.withhold = withhold;
    return ODIS_OK;
}

extern "C" odis_status odis_launch_count(odis_ctx* c, long long* n)
{
    if (!c || !n) return ODIS_ERR_ARG;
    *n = c->launches;
    return ODIS_OK;
}

// Average device time of each kernel group, each launched `reps` times back to
// back inside one CUDA graph and timed with events on the context stream:
// ms[0] face kernel, ms[1] cell kernel, ms[2] SH analysis+solve+synthesis
// (0 without self-gravity).  Leaves the state undefined.
extern "C" odis_status odis_profile_kernels(odis_ctx* c, int reps, double* ms)
{
    if (!c || reps <= 0 || !ms) return ODIS_ERR_ARG;
    // the kernels below run at step offset 2 of a run starting at the current step
    const long long first = c->iter;
    ODIS_CK(cudaMemcpyAsync(c->d_run_first, &first, sizeof(long long), cudaMemcpyHostToDevice, c->stream));
    ODIS_CK(cudaMemcpyAsync(c->d_iter, &first, sizeof(long long), cudaMemcpyHostToDevice, c->stream));
    {
        const int pst = prepare_phase(c, first, 8);
        if (pst != ODIS_OK) return pst;
    }
    ODIS_CK(cudaStreamSynchronize(c->stream));
    cudaEvent_t a, b;
    ODIS_CK(cudaEventCreate(&a));
    ODIS_CK(cudaEventCreate(&b));
    int st = ODIS_OK;
    for (int which = 0; which < 3 && st == ODIS_OK; which++) {
        ms[which] = 0.0;
        if (which == 2 && !c->sh) continue;
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) { st = ODIS_ERR_CUDA; break; }
        for (int r = 0; r < reps; r++) {
            const bool f32 = c->p.precision == ODIS_FP32, fdf = c->p.precision == ODIS_DF64;
            if (which == 0) {
                if (fdf) launch_edge_df(c->opdf.fc, c->sdf, c->sc, 2, c->stream);
                else if (f32) launch_edge<float, true>(c->op32.fc, c->s32, c->sc, 2, c->stream);
                else launch_edge<double, false>(c->op64.fc, c->s64, c->sc, 2, c->stream);
            } else if (which == 1) {
                if (fdf) launch_cell_df(c->opdf.cc, c->sdf, c->sc, 2, c->stream);
                else if (f32) launch_cell<float, true>(c->op32.cc, c->s32, c->sc, 2, c->stream);
                else launch_cell<double, false>(c->op64.cc, c->s64, c->sc, 2, c->stream);
            } else {
                sh_enqueue(c->sh, state_eta(c), c->stream);
            }
        }
        if (cudaStreamEndCapture(c->stream, &g) != cudaSuccess || cudaGraphInstantiate(&ge, g, 0) != cudaSuccess) {
            st = ODIS_ERR_CUDA;
        } else {
            cudaGraphLaunch(ge, c->stream);                 // warm-up
            cudaEventRecord(a, c->stream);
            cudaGraphLaunch(ge, c->stream);
            cudaEventRecord(b, c->stream);
            if (cudaEventSynchronize(b) != cudaSuccess) st = ODIS_ERR_CUDA;
            float t = 0.f;
            cudaEventElapsedTime(&t, a, b);
            ms[which] = (double)t / reps;
            c->launches += 2LL * reps * (which == 2 ? sh_kernels_per_step(c->sh) : 1);
        }
        if (ge) cudaGraphExecDestroy(ge);
        if (g) cudaGraphDestroy(g);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return st;
}

extern "C" odis_status odis_sh_tiles(const odis_ctx* c, int* tile_l, int* chunks, int* lanes, int* cells, int* pre)
{
    if (!c) return ODIS_ERR_ARG;
    int a = 0, b = 0, d = 0, e = 0, f = 0;
    if (c->sh) sh_tuning(c->sh, &a, &b, &d, &e, &f);
    if (tile_l) *tile_l = a;
    if (chunks) *chunks = b;
    if (lanes) *lanes = d;
    if (cells) *cells = e;
    if (pre) *pre = f;
    return ODIS_OK;
}

extern "C" odis_status odis_sh_layout(const odis_ctx* c, int* half, int* cells, long long* basis_bytes)
{
    if (!c) return ODIS_ERR_ARG;
    int a = 0, b = 0;
    long long by = 0;
    if (c->sh) sh_layout(c->sh, &a, &b, &by);
    if (half) *half = a;
    if (cells) *cells = b;
    if (basis_bytes) *basis_bytes = by;
    return ODIS_OK;
}

extern "C" odis_status odis_set_persistent(odis_ctx* c, int enable, int* active)
{
    if (!c || enable < -1 || enable > 1) return ODIS_ERR_ARG;
    c->persist_on = enable < 0 ? c->persist_auto : enable != 0;
    if (active) *active = (c->persist_ok && c->persist_on) ? 1 : 0;
    return ODIS_OK;
}
