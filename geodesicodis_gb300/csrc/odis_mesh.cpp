// Host-side mesh geometry for the GB300 LTE solver: control-volume areas,
// faces, face geometry and the TRiSK tangential-reconstruction weights.
//
// Setup work (once per mesh).  The steps themselves live in
// odis_mesh_build.cuh, shared with the device builder (odis_mesh_dev.cu);
// here they run as OpenMP loops with the C library's math functions, which
// gives the reference's coefficients bit for bit:
//   control-volume area (map coords) .. src/mesh.cpp:1828-1866
//   vertex numbering .................. src/mesh.cpp:436-506
//   face numbering + geometry ......... src/mesh.cpp:508-670
//   TRiSK weights ..................... src/mesh.cpp:680-907
//   face area (no 1/2) ................ src/mesh.cpp:1093
// and the formulas of odis_geom.cuh (include/mathRoutines.h).
#include "odis_internal.h"
#include "odis_forcing.cuh"
#include "odis_exec.cuh"
#include "odis_mesh_build.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace odis {

namespace {

using geo::arc_atan2;
using geo::kGeoPi;
using geo::LL;
using geo::stereo;
constexpr double kPi = kGeoPi;

}  // namespace

int build_mesh(int N, const double* node_sph, const int* friends, const double* cent_sph,
               double radius, Mesh& m)
{
    HostExec x;
    return build_mesh_steps(x, N, node_sph, friends, cent_sph, radius, m);
}

// Largest gravity-wave frequency of the discrete operator: sqrt of the largest
// eigenvalue of -g h D G (G gradient, D divergence as assembled in
// src/mesh.cpp:3005-3288), by power iteration.  The time loop of the
// reference (AB3 for v with the old eta, then AB3 for eta with the new v,
// src/timeIntegrator.cpp:213-253) is stable for omega_max * dt <= 6/11.
double gravity_wave_omega(const Mesh& m, double g, double h, int iters)
{
    const int N = m.N, E = m.E;
    std::vector<double> x(N), y(N), gv(E);
    for (int i = 0; i < N; i++) x[i] = ((i * 2654435761u) % 1000u) / 1000.0 - 0.5;   // deterministic start
    double lam = 0.0;
    for (int it = 0; it < iters; it++) {
        double nx = 0.0;
        for (int i = 0; i < N; i++) nx += x[i] * x[i];
        nx = std::sqrt(nx);
        for (int i = 0; i < N; i++) x[i] /= nx;
#pragma omp parallel for schedule(static)
        for (int e = 0; e < E; e++) {
            const int a = m.face_nodes[(size_t)e * 2], b = m.face_nodes[(size_t)e * 2 + 1];
            gv[e] = (-m.face_m[(size_t)e * 2] * x[a] + m.face_m[(size_t)e * 2 + 1] * x[b]) / m.face_dist[e];
        }
#pragma omp parallel for schedule(static)
        for (int i = 0; i < N; i++) {
            double s = 0.0;
            for (int j = 0; j < m.nfriends(i); j++) {
                const int f = m.faces[(size_t)i * 6 + j];
                s += -m.node_face_dir[(size_t)i * 6 + j] * m.face_len[f] / m.cv_area[i] * gv[f];
            }
            y[i] = -g * h * s;
        }
        double r = 0.0;
        for (int i = 0; i < N; i++) r += x[i] * y[i];
        lam = r;
        x.swap(y);
    }
    return std::sqrt(std::fabs(lam));
}

// U(t) = cos(M) Ua + sin(M) Ub for the single-frequency potentials of
// src/tidalPotentials.cpp:82-174 (ECC, OBLIQ, OBLIQ_WEST, FULL), using the
// node trig tables of src/mesh.cpp:2122-2152.
// Gaussian radial basis function of an arc on the unit sphere, shape parameter 1
// (include/mathRoutines.h:431-439)
static double rbf_phi(double d)
{
    return d < 1e-8 ? 1.0 : std::exp(-std::pow(d, 2.0));
}

// Inverse of a k x k matrix (k <= 6) by Gauss-Jordan elimination with partial pivoting.
static bool invert_small(int k, double a[6][6], double inv[6][6])
{
    for (int r = 0; r < k; r++)
        for (int c = 0; c < k; c++) inv[r][c] = r == c ? 1.0 : 0.0;
    for (int c = 0; c < k; c++) {
        int piv = c;
        for (int r = c + 1; r < k; r++) if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
        if (a[piv][c] == 0.0) return false;
        if (piv != c)
            for (int q = 0; q < k; q++) { std::swap(a[c][q], a[piv][q]); std::swap(inv[c][q], inv[piv][q]); }
        const double d = a[c][c];
        for (int q = 0; q < k; q++) { a[c][q] /= d; inv[c][q] /= d; }
        for (int r = 0; r < k; r++) {
            if (r == c) continue;
            const double f = a[r][c];
            if (f == 0.0) continue;
            for (int q = 0; q < k; q++) { a[r][q] -= f * a[c][q]; inv[r][q] -= f * inv[c][q]; }
        }
    }
    return true;
}

// RBF reconstruction (src/mesh.cpp:355-430 and :2263-2362, used by
// interpolateVelocityCartRBF, src/interpolation.cpp:64-174): about node i with
// faces j = 0..k-1, A[j1][j2] = phi(arc(f_j1, f_j2)) n_j1 . n_j2 and
// w[j] = phi(arc(node i, f_j)); the Cartesian velocity is
// u_c = sum_j1 w[j1] n_j1,c sum_j2 (A^-1)[j1][j2] v(f_j2).
void build_rbf(const Mesh& m, std::vector<double>& rbf)
{
    const int N = m.N;
    rbf.assign((size_t)N * 18, 0.0);
    auto node = [&](int i) { return LL{m.node_sph[i * 2], m.node_sph[i * 2 + 1]}; };
    auto fc = [&](int e) { return LL{m.face_centre[e * 2], m.face_centre[e * 2 + 1]}; };
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++) {
        const int k = m.nfriends(i);
        double A[6][6] = {}, Ai[6][6] = {}, w[6] = {};
        for (int j1 = 0; j1 < k; j1++) {
            const int f1 = m.faces[i * 6 + j1];
            for (int j2 = 0; j2 < k; j2++) {
                const int f2 = m.faces[i * 6 + j2];
                const double dot = m.face_nxyz[f1 * 3] * m.face_nxyz[f2 * 3] + m.face_nxyz[f1 * 3 + 1] * m.face_nxyz[f2 * 3 + 1] +
                                   m.face_nxyz[f1 * 3 + 2] * m.face_nxyz[f2 * 3 + 2];
                A[j1][j2] = rbf_phi(arc_atan2(fc(f1), fc(f2))) * dot;
            }
            w[j1] = rbf_phi(arc_atan2(node(i), fc(f1)));
        }
        if (!invert_small(k, A, Ai)) continue;
        for (int c = 0; c < 3; c++)
            for (int j2 = 0; j2 < k; j2++) {
                double s = 0.0;
                for (int j1 = 0; j1 < k; j1++) s += w[j1] * m.face_nxyz[m.faces[i * 6 + j1] * 3 + c] * Ai[j1][j2];
                rbf[((size_t)i * 3 + c) * 6 + j2] = s;
            }
    }
}

int forcing_basis(const Mesh& m, const odis_params& p, std::vector<double>& Ua, std::vector<double>& Ub)
{
    Ua.assign(m.N, 0.0);
    Ub.assign(m.N, 0.0);
    const double w2r2 = std::pow(p.angvel, 2.0) * std::pow(p.radius, 2.0);
    for (int i = 0; i < m.N; i++) {
        double lat = m.node_sph[i * 2], lon = m.node_sph[i * 2 + 1];
        double cosLat = std::cos(lat), sinLat = std::sin(lat), cosLon = std::cos(lon), sinLon = std::sin(lon);
        double sin2Lat = std::sin(2.0 * lat), cos2Lon = std::cos(2.0 * lon), sin2Lon = std::sin(2.0 * lon);
        double cosSqLat = std::pow(std::cos(lat), 2.0), sinSqLat = std::pow(std::sin(lat), 2.0);
        double fe = 0.75 * p.love_reduct * w2r2 * p.ecc;
        double fo = -3. / 2. * p.love_reduct * w2r2 * p.obliq;
        switch (p.potential) {
        case ODIS_POT_ECC:
            Ua[i] = fe * ((1. - 3. * sinSqLat) + cosSqLat * 3. * cos2Lon);
            Ub[i] = fe * (cosSqLat * 4. * sin2Lon);
            break;
        case ODIS_POT_OBLIQ:
            Ua[i] = fo * sin2Lat * cosLon;
            break;
        case ODIS_POT_OBLIQ_WEST: {
            double f = 0.5 * p.love_reduct * w2r2 * p.obliq;
            Ua[i] = 3 * f * sinLat * cosLat * cosLon;
            Ub[i] = -3 * f * sinLat * cosLat * sinLon;
            break; }
        case ODIS_POT_FULL:
            Ua[i] = fe * ((1 - 3 * sinSqLat) + cosSqLat * 3 * cos2Lon) + fo * sin2Lat * cosLon;
            Ub[i] = fe * (cosSqLat * 4 * sin2Lon);
            break;
        default:            // unforced types, and the nodal ones (evaluated per step at the nodes)
            if (!pot_valid(p.potential)) return ODIS_ERR_ARG;
            break;
        }
    }
    return ODIS_OK;
}

// Gaussian RBF of include/mathRoutines.h:432-439
static double rbf_gauss(double dist, double eps)
{
    double phi = std::exp(-std::pow(eps * dist, 2.0));
    if (dist < 1e-8) phi = 1;
    return phi;
}

// In-place inverse of an n x n row-major matrix (n <= 7): Gauss-Jordan
// elimination with partial pivoting.  The oracle inverts with the same steps,
// so the two agree bit for bit.
static bool gj_inverse(int n, double* a)
{
    double b[7 * 7];
    for (int i = 0; i < n * n; i++) b[i] = 0.0;
    for (int i = 0; i < n; i++) b[i * n + i] = 1.0;
    for (int c = 0; c < n; c++) {
        int piv = c;
        for (int r = c + 1; r < n; r++)
            if (std::fabs(a[r * n + c]) > std::fabs(a[piv * n + c])) piv = r;
        if (a[piv * n + c] == 0.0) return false;
        if (piv != c)
            for (int q = 0; q < n; q++) {
                std::swap(a[c * n + q], a[piv * n + q]);
                std::swap(b[c * n + q], b[piv * n + q]);
            }
        const double d = a[c * n + c];
        for (int q = 0; q < n; q++) { a[c * n + q] /= d; b[c * n + q] /= d; }
        for (int r = 0; r < n; r++) {
            if (r == c) continue;
            const double f = a[r * n + c];
            if (f == 0.0) continue;
            for (int q = 0; q < n; q++) { a[r * n + q] -= f * a[c * n + q]; b[r * n + q] -= f * b[c * n + q]; }
        }
    }
    for (int i = 0; i < n * n; i++) a[i] = b[i];
    return true;
}

int build_lsq_rows(const Mesh& m, double eps, std::vector<int>& col, std::vector<double>& val)
{
    const int N = m.N, E = m.E;
    const double r = m.r, r_recip = 1.0 / m.r;
    std::vector<double> S((size_t)N * 3 * 7, 0.0);
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad)
    for (int i = 0; i < N; i++) {
        const int k = m.nfriends(i), K = k + 1;
        const LL c0{m.node_sph[i * 2], m.node_sph[i * 2 + 1]};
        double px[7], py[7];
        for (int j = 0; j < K; j++) {              // node-centred map coordinates (src/mesh.cpp:1384-1450)
            const int f = j == 0 ? i : m.friends[i * 6 + j - 1];
            double mm;
            stereo(c0, LL{m.node_sph[f * 2], m.node_sph[f * 2 + 1]}, r, mm, px[j], py[j]);
        }
        double A[7 * 7], nnr[7] = {0, 0, 0, 0, 0, 0, 0};
        A[0] = 1.0;
        for (int j1 = 0; j1 < k; j1++) {           // src/mesh.cpp:286-345
            const double x1 = px[j1 + 1] / r, y1 = py[j1 + 1] / r;
            const double arc = std::sqrt(x1 * x1 + y1 * y1);
            A[0 * K + j1 + 1] = rbf_gauss(arc, eps);
        }
        for (int j1 = 0; j1 < k; j1++) {
            const double x1 = px[j1 + 1] / r, y1 = py[j1 + 1] / r;
            double arc = std::sqrt(x1 * x1 + y1 * y1);
            A[(j1 + 1) * K + 0] = rbf_gauss(arc, eps);
            nnr[j1 + 1] = rbf_gauss(arc, eps);
            for (int j2 = 0; j2 < k; j2++) {
                const double x2 = px[j2 + 1] / r, y2 = py[j2 + 1] / r;
                arc = std::sqrt((x1 - x2) * (x1 - x2) + (y1 - y2) * (y1 - y2));
                A[(j1 + 1) * K + j2 + 1] = rbf_gauss(arc, eps);
            }
        }
        if (!gj_inverse(K, A)) { bad++; continue; }
        double D[3][7];                            // rbfDeriv2, src/mesh.cpp:2472-2548
        for (int c = 0; c < 3; c++)
            for (int j = 0; j < K; j++) D[c][j] = 0.0;
        D[0][0] = -2.0 * eps * eps;
        D[2][0] = -2.0 * eps * eps;
        for (int j = 0; j < k; j++) {
            const double x1 = px[j + 1] * r_recip, y1 = py[j + 1] * r_recip;
            const double arc = std::sqrt(x1 * x1 + y1 * y1);
            const double xx = x1 * x1, yy = y1 * y1, xy = x1 * y1;
            const double arc2 = 1.0 / (arc * arc), arc3 = 1.0 / (arc * arc * arc);
            const double rbf = nnr[j + 1];
            const double d2phidr2 = 2 * eps * eps * rbf * (2 * arc * arc * eps * eps - 1);
            const double dphidr = -2 * arc * eps * eps * rbf;
            D[0][j + 1] = (yy * arc3 * dphidr + xx * arc2 * d2phidr2);
            D[1][j + 1] = (-xy * arc3 * dphidr + xy * arc2 * d2phidr2);
            D[2][j + 1] = (xx * arc3 * dphidr + yy * arc2 * d2phidr2);
        }
        const double sc = r_recip * r_recip;
        for (int c = 0; c < 3; c++)
            for (int j = 0; j < K; j++) {
                double t = 0.0;
                for (int q = (c == 1 ? 1 : 0); q < K; q++) t += (sc * D[c][q]) * A[q * K + j];
                S[((size_t)i * 3 + c) * 7 + j] = t;
            }
    }
    if (bad) return ODIS_ERR_MESH;
    col.assign((size_t)2 * E * 7, 0);
    val.assign((size_t)2 * E * 7, 0.0);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < E; e++)
        for (int side = 0; side < 2; side++) {
            const int n = m.face_nodes[e * 2 + side];
            const int k = m.nfriends(n), K = k + 1;
            double ca, sa;                         // velTransform, include/mathRoutines.h:79-87
            {
                const double lat1 = m.face_int[e * 2], lon1 = m.face_int[e * 2 + 1];
                const double lat2 = m.node_sph[n * 2], lon2 = m.node_sph[n * 2 + 1];
                ca = std::cos(lat1) * std::cos(lat2);
                ca += (1.0 + std::sin(lat1) * std::sin(lat2)) * std::cos(lon2 - lon1);
                ca /= (1.0 + std::sin(lat1) * std::sin(lat2) + std::cos(lat1) * std::cos(lat2) * std::cos(lon2 - lon1));
                sa = -(std::sin(lat1) + std::sin(lat2)) * std::sin(lon2 - lon1);
                sa /= (1.0 + std::sin(lat1) * std::sin(lat2) + std::cos(lat1) * std::cos(lat2) * std::cos(lon2 - lon1));
            }
            const double R[3][3] = {{ca * ca, -2 * ca * sa, sa * sa},
                                    {ca * sa, ca * ca - sa * sa, -sa * ca},
                                    {sa * sa, 2 * ca * sa, ca * ca}};
            const double nx = m.face_normal[e * 2], ny = m.face_normal[e * 2 + 1];
            const double Nv[3] = {nx * nx, 2 * nx * ny, ny * ny};
            double NR[3];
            for (int c = 0; c < 3; c++) {
                double t = 0.0;
                for (int q = 0; q < 3; q++) t += Nv[q] * R[q][c];
                NR[c] = t;
            }
            int cc[7];
            double vv[7];
            for (int j = 0; j < K; j++) {
                double t = 0.0;
                for (int c = 0; c < 3; c++) t += NR[c] * S[((size_t)n * 3 + c) * 7 + j];
                cc[j] = j == 0 ? n : m.friends[n * 6 + j - 1];
                vv[j] = t;
            }
            int idx[7] = {0, 1, 2, 3, 4, 5, 6};
            std::sort(idx, idx + K, [&](int a, int b) { return cc[a] < cc[b]; });
            const size_t row = (size_t)(2 * e + side) * 7;
            for (int j = 0; j < 7; j++) {
                col[row + j] = j < K ? cc[idx[j]] : cc[idx[K - 1]];
                val[row + j] = j < K ? vv[idx[j]] : 0.0;
            }
        }
    return ODIS_OK;
}

}  // namespace odis

