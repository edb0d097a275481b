// Host-side mesh geometry for the GB300 LTE solver: control-volume areas,
// faces, face geometry and the TRiSK tangential-reconstruction weights.
//
// This is setup work (once per mesh), done in C++ with OpenMP over faces.
// The formulas are the reference's, in the reference's evaluation order,
// because several are ill-conditioned at fine levels (acos-based arc lengths,
// spherical excess from acos angles) and the per-step kernels must see the
// same coefficients as GeodesicODIS does to agree to 1e-10:
//   map factor / map coordinates ...... include/mathRoutines.h:29-68
//   arc lengths ....................... include/mathRoutines.h:134-163
//   spherical midpoint ................ include/mathRoutines.h:172-192
//   edge normal in map coordinates .... include/mathRoutines.h:214-248
//   great-circle intersection ......... include/mathRoutines.h:320-383
//   angle about a node ................ include/mathRoutines.h:385-410
//   planar / spherical triangle areas . include/mathRoutines.h:415-439
//   control-volume area (map coords) .. src/mesh.cpp:1828-1866
//   vertex numbering .................. src/mesh.cpp:436-506
//   face numbering + geometry ......... src/mesh.cpp:508-670
//   TRiSK weights ..................... src/mesh.cpp:680-907
//   face area (no 1/2) ................ src/mesh.cpp:1093
#include "odis_internal.h"
#include "odis_forcing.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace odis {

namespace {

constexpr double kPi = 3.1415926535897932384626433832795028841971693993751058;

struct LL { double lat, lon; };

inline double mapfac(double lat1, double lat2, double lon1, double lon2)
{
    return 2.0 / (1.0 + std::sin(lat1) * std::sin(lat2) + std::cos(lat1) * std::cos(lat2) * std::cos(lon2 - lon1));
}

// stereographic coordinates of q in the plane tangent at c (radius r)
inline void stereo(LL c, LL q, double r, double& m, double& x, double& y)
{
    m = mapfac(c.lat, q.lat, c.lon, q.lon);
    x = m * r * (std::cos(q.lat) * std::sin(q.lon - c.lon));
    y = m * r * (std::sin(q.lat) * std::cos(c.lat) - std::cos(q.lat) * std::sin(c.lat) * std::cos(q.lon - c.lon));
}

inline double arc_acos(LL a, LL b, double r)
{
    return r * std::acos(std::sin(a.lat) * std::sin(b.lat) + std::cos(a.lat) * std::cos(b.lat) * std::cos(b.lon - a.lon));
}

inline void to_xyz(LL a, double p[3])
{
    // sph2cart with colatitude pi/2 - lat, unit radius
    double colat = kPi * 0.5 - a.lat;
    p[0] = 1.0 * std::sin(colat) * std::cos(a.lon);
    p[1] = 1.0 * std::sin(colat) * std::sin(a.lon);
    p[2] = 1.0 * std::cos(colat);
}

inline double arc_atan2(LL a, LL b)
{
    double p[3], q[3];
    to_xyz(a, p);
    to_xyz(b, q);
    double c = std::pow(p[1] * q[2] - p[2] * q[1], 2.0);
    c += std::pow(-(p[0] * q[2] - p[2] * q[0]), 2.0);
    c += std::pow(p[0] * q[1] - p[1] * q[0], 2.0);
    c = std::sqrt(c);
    double d = p[0] * q[0] + p[1] * q[1] + p[2] * q[2];
    return std::atan2(c, d);
}

inline void latlon_xyz(LL a, double p[3])
{
    p[0] = std::cos(a.lat) * std::cos(a.lon);
    p[1] = std::cos(a.lat) * std::sin(a.lon);
    p[2] = std::sin(a.lat);
}

inline LL midpoint(LL a, LL b)
{
    double p[3], q[3], c[3];
    latlon_xyz(a, p);
    latlon_xyz(b, q);
    for (int k = 0; k < 3; k++) c[k] = 0.5 * (p[k] + q[k]);
    return {std::atan2(c[2], std::sqrt(std::pow(c[0], 2.0) + std::pow(c[1], 2.0))), std::atan2(c[1], c[0])};
}

inline void map_normal(LL a, LL b, double n[2])
{
    LL c = midpoint(a, b);
    double m, x1, y1, x2, y2;
    stereo(c, a, 1.0, m, x1, y1);
    stereo(c, b, 1.0, m, x2, y2);
    double tx = x2 - x1, ty = y2 - y1;
    double mag = std::sqrt(tx * tx + ty * ty);
    tx /= mag;
    ty /= mag;
    n[0] = -ty;
    n[1] = tx;
}

inline LL intersect(LL a, LL b, LL c, LL d)
{
    double pa[3], pb[3], pc[3], pd[3], n1[3], n2[3], mp[3];
    latlon_xyz(a, pa); latlon_xyz(b, pb); latlon_xyz(c, pc); latlon_xyz(d, pd);
    n1[0] = pa[1] * pb[2] - pa[2] * pb[1];
    n1[1] = -(pa[0] * pb[2] - pa[2] * pb[0]);
    n1[2] = pa[0] * pb[1] - pa[1] * pb[0];
    n2[0] = pc[1] * pd[2] - pc[2] * pd[1];
    n2[1] = -(pc[0] * pd[2] - pc[2] * pd[0]);
    n2[2] = pc[0] * pd[1] - pc[1] * pd[0];
    double m1 = std::sqrt(n1[0] * n1[0] + n1[1] * n1[1] + n1[2] * n1[2]);
    double m2 = std::sqrt(n2[0] * n2[0] + n2[1] * n2[1] + n2[2] * n2[2]);
    for (int k = 0; k < 3; k++) { n1[k] /= m1; n2[k] /= m2; }
    mp[0] = n1[1] * n2[2] - n2[1] * n1[2];
    mp[1] = n2[0] * n1[2] - n1[0] * n2[2];
    mp[2] = n1[0] * n2[1] - n2[0] * n1[1];
    m1 = std::sqrt(mp[0] * mp[0] + mp[1] * mp[1] + mp[2] * mp[2]);
    for (int k = 0; k < 3; k++) mp[k] /= m1;
    LL o{std::asin(mp[2] / 1.0), std::atan2(mp[1], mp[0])};
    if (o.lon < 0.0) o.lon += 2 * kPi;
    return o;
}

// signed angle (rad) from q2 to q1 about c in c's stereographic plane
inline double angle_about(LL q1, LL q2, LL c)
{
    double m, x1, y1, x2, y2;
    stereo(c, q1, 1.0, m, x1, y1);
    stereo(c, q2, 1.0, m, x2, y2);
    double a = std::atan2(y1 - 0.0, x1 - 0.0) - std::atan2(y2 - 0.0, x2 - 0.0);
    if (a > kPi) a -= 2 * kPi;
    else if (a < -kPi) a += 2 * kPi;
    return a;
}

inline double sph_tri_area(LL p1, LL p2, LL p3, double r)
{
    double c = std::fabs(std::acos(std::sin(p1.lat) * std::sin(p2.lat) + std::cos(p1.lat) * std::cos(p2.lat) * std::cos(std::fabs(p2.lon - p1.lon))));
    double a = std::fabs(std::acos(std::sin(p2.lat) * std::sin(p3.lat) + std::cos(p2.lat) * std::cos(p3.lat) * std::cos(std::fabs(p3.lon - p2.lon))));
    double b = std::fabs(std::acos(std::sin(p3.lat) * std::sin(p1.lat) + std::cos(p3.lat) * std::cos(p1.lat) * std::cos(std::fabs(p1.lon - p3.lon))));
    double A = std::fabs(std::acos((std::cos(a) - std::cos(b) * std::cos(c)) / (std::sin(b) * std::sin(c))));
    double B = std::fabs(std::acos((std::cos(b) - std::cos(a) * std::cos(c)) / (std::sin(a) * std::sin(c))));
    double C = std::fabs(std::acos((std::cos(c) - std::cos(b) * std::cos(a)) / (std::sin(b) * std::sin(a))));
    return std::pow(r, 2.0) * std::fabs((A + B + C) - kPi);
}

struct Ranked { int id; double deg; };

}  // namespace

int build_mesh(int N, const double* node_sph, const int* friends, const double* cent_sph,
               double radius, Mesh& m)
{
    if (N < 12 || !node_sph || !friends || !cent_sph || !(radius > 0.0)) return ODIS_ERR_ARG;
    m.N = N;
    m.r = radius;
    m.node_sph.assign(node_sph, node_sph + (size_t)N * 2);
    m.friends.assign(friends, friends + (size_t)N * 6);
    m.cent_sph.assign(cent_sph, cent_sph + (size_t)N * 12);
    for (int i = 0; i < N; i++) {
        for (int j = 0; j < 5; j++) {
            int f = m.friends[i * 6 + j];
            if (f < 0 || f >= N || f == i) return ODIS_ERR_MESH;
        }
        int f5 = m.friends[i * 6 + 5];
        if (f5 < -1 || f5 >= N || f5 == i) return ODIS_ERR_MESH;
    }
    auto node = [&](int i) { return LL{m.node_sph[i * 2], m.node_sph[i * 2 + 1]}; };
    auto cent = [&](int i, int j) { return LL{m.cent_sph[(i * 6 + j) * 2], m.cent_sph[(i * 6 + j) * 2 + 1]}; };

    // control-volume areas in node-centred map coordinates
    m.cv_area.assign(N, 0.0);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++) {
        int k = m.nfriends(i);
        double mc, xc, yc;
        stereo(node(i), node(i), radius, mc, xc, yc);
        double xy[6][2];
        for (int j = 0; j < k; j++) stereo(node(i), cent(i, j), radius, mc, xy[j][0], xy[j][1]);
        double area = 0.0;
        for (int j = 0; j < k; j++) {
            const double* p1 = xy[j];
            const double* p2 = xy[(j + 1) % k];
            area += 0.5 * std::fabs(xc * (p1[1] - p2[1]) + p1[0] * (p2[1] - yc) + p2[0] * (yc - p1[1]));
        }
        m.cv_area[i] = area;
    }

    // vertex numbering: first node (in file order) to reach a centroid names it
    m.vertexes.assign((size_t)N * 6, -1);
    m.vert_sph.clear();
    m.vert_sph.reserve((size_t)N * 4);
    m.vert_nodes.clear();
    m.vert_nodes.reserve((size_t)N * 6);
    for (int i = 0; i < N; i++) {
        int k = m.nfriends(i);
        for (int j = 0; j < k; j++) {
            if (m.vertexes[i * 6 + j] >= 0) continue;
            int vid = (int)(m.vert_sph.size() / 2);
            m.vertexes[i * 6 + j] = vid;
            LL v = cent(i, j);
            m.vert_sph.push_back(v.lat);
            m.vert_sph.push_back(v.lon);
            const int nb[2] = {m.friends[i * 6 + j % k], m.friends[i * 6 + (j + 1) % k]};
            m.vert_nodes.push_back(i);
            m.vert_nodes.push_back(nb[0]);
            m.vert_nodes.push_back(nb[1]);
            for (int f : nb) {
                int kf = m.nfriends(f);
                for (int q = 0; q < kf; q++) {
                    LL c = cent(f, q);
                    if (c.lat < v.lat + 1e-9 && c.lat > v.lat - 1e-9 && c.lon < v.lon + 1e-9 && c.lon > v.lon - 1e-9)
                        m.vertexes[f * 6 + q] = vid;
                }
            }
        }
    }
    m.V = (int)(m.vert_sph.size() / 2);
    for (int i = 0; i < N * 6; i++)
        if (m.friends[i] >= 0 && m.vertexes[i] < 0) return ODIS_ERR_MESH;

    // face numbering (AssignFaces loop order)
    const int E = 3 * N - 6;
    m.E = E;
    m.faces.assign((size_t)N * 6, -1);
    m.node_face_dir.assign((size_t)N * 6, 0);
    m.face_nodes.assign((size_t)E * 2, -1);
    int fc = 0;
    for (int i = 0; i < N; i++) {
        int k = m.nfriends(i);
        for (int j = 0; j < k; j++) {
            if (m.faces[i * 6 + j] >= 0) continue;
            if (fc >= E) return ODIS_ERR_MESH;
            int f = m.friends[i * 6 + j];
            m.faces[i * 6 + j] = fc;
            m.node_face_dir[i * 6 + j] = 1;
            m.face_nodes[fc * 2] = i;
            int kf = m.nfriends(f), hit = 0;
            for (int q = 0; q < kf; q++)
                if (m.friends[f * 6 + q] == i) {
                    m.faces[f * 6 + q] = fc;
                    m.node_face_dir[f * 6 + q] = -1;
                    m.face_nodes[fc * 2 + 1] = f;
                    hit = 1;
                }
            if (!hit) return ODIS_ERR_MESH;
            fc++;
        }
    }
    if (fc != E) return ODIS_ERR_MESH;
    // the two vertices bounding each face: centroids j-1 and j of its first node
    std::vector<int> face_slot(E, -1);
    for (int i = 0; i < N; i++)
        for (int j = 0; j < m.nfriends(i); j++)
            if (m.node_face_dir[i * 6 + j] == 1) face_slot[m.faces[i * 6 + j]] = j;

    m.face_len.assign(E, 0.0);
    m.face_dist.assign(E, 0.0);
    m.face_area.assign(E, 0.0);
    m.face_centre.assign((size_t)E * 2, 0.0);
    m.face_m.assign((size_t)E * 2, 0.0);
    m.face_normal.assign((size_t)E * 2, 0.0);
    m.face_int.assign((size_t)E * 2, 0.0);
    m.face_nxyz.assign((size_t)E * 3, 0.0);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < E; e++) {
        int i = m.face_nodes[e * 2], f = m.face_nodes[e * 2 + 1], j = face_slot[e];
        int k = m.nfriends(i);
        LL v1 = cent(i, (j + k - 1) % k), v2 = cent(i, j % k);
        m.face_len[e] = std::fabs(arc_acos(v1, v2, radius));
        LL c = midpoint(v1, v2);
        if (c.lon < 0.0) c.lon += 2 * kPi;
        m.face_centre[e * 2] = c.lat;
        m.face_centre[e * 2 + 1] = c.lon;
        double mm, x, y;
        stereo(c, node(i), radius, mm, x, y);
        m.face_m[e * 2] = mm;
        stereo(c, node(f), radius, mm, x, y);
        m.face_m[e * 2 + 1] = mm;
        m.face_dist[e] = arc_atan2(node(i), node(f)) * radius;
        double n[2];
        map_normal(v1, v2, n);
        m.face_normal[e * 2] = n[0];
        m.face_normal[e * 2 + 1] = n[1];
        {
            // Cartesian normal: the unit cross product of the vertex positions (include/mathRoutines.h:246-267)
            double p1[3], p2[3];
            to_xyz(v1, p1);
            to_xyz(v2, p2);
            double c0 = p1[1] * p2[2] - p1[2] * p2[1];
            double c1 = -(p1[0] * p2[2] - p1[2] * p2[0]);
            double c2 = p1[0] * p2[1] - p1[1] * p2[0];
            const double mag = std::sqrt(c0 * c0 + c1 * c1 + c2 * c2);
            m.face_nxyz[e * 3] = c0 / mag;
            m.face_nxyz[e * 3 + 1] = c1 / mag;
            m.face_nxyz[e * 3 + 2] = c2 / mag;
        }
        LL ip = intersect(v1, v2, node(i), node(f));
        m.face_int[e * 2] = ip.lat;
        m.face_int[e * 2 + 1] = ip.lon;
        m.face_area[e] = m.face_dist[e] * m.face_len[e];
    }

    // TRiSK weights: faces and vertices about each end node ranked
    // anticlockwise from the face itself, kite fractions R, then
    // w = (sum_{j'<j} R_j' - 1/2) * n_{e',node} * t_{e,node}
    m.interp_friends.assign((size_t)E * 10, 0);
    m.interp_w.assign((size_t)E * 10, 0.0);
    m.interp_n.assign(E, 0);
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad)
    for (int e = 0; e < E; e++) {
        LL ie{m.face_int[e * 2], m.face_int[e * 2 + 1]};
        int slot = 0;
        for (int side = 0; side < 2; side++) {
            int nd = m.face_nodes[e * 2 + side];
            int k = m.nfriends(nd);
            LL c = node(nd);
            Ranked fr[6], vr[6];
            for (int j = 0; j < k; j++) {
                int id = m.faces[nd * 6 + j];
                double a = angle_about(ie, LL{m.face_int[id * 2], m.face_int[id * 2 + 1]}, c) * 180. / kPi;
                if (a > 0.0 + 1e-8) a -= 360.0;
                fr[j] = {id, a};
                int vid = m.vertexes[nd * 6 + j];
                double b = angle_about(ie, LL{m.vert_sph[vid * 2], m.vert_sph[vid * 2 + 1]}, c) * 180. / kPi;
                if (b > 0.0 + 1e-8) b -= 360.0;
                vr[j] = {vid, b};
            }
            auto desc = [](const Ranked& a, const Ranked& b) { return a.deg > b.deg; };
            std::sort(fr, fr + k, desc);
            std::sort(vr, vr + k, desc);
            auto vpos = [&](int vid) { return LL{m.vert_sph[vid * 2], m.vert_sph[vid * 2 + 1]}; };
            auto ipos = [&](int fid) { return LL{m.face_int[fid * 2], m.face_int[fid * 2 + 1]}; };
            double area_cv = 0.0;
            for (int j = 0; j < k; j++) area_cv += sph_tri_area(c, vpos(vr[j].id), vpos(vr[(j + 1) % k].id), radius);
            double R[6];
            for (int j = 0; j < k; j++) {
                LL v = vpos(vr[j].id);
                double a1 = sph_tri_area(c, v, ipos(fr[j].id), radius);
                double a2 = sph_tri_area(c, v, ipos(fr[(j + 1) % k].id), radius);
                R[j] = (a1 + a2) / area_cv;
            }
            int tev = (m.face_nodes[e * 2] == nd) ? 1 : -1;
            for (int j = 0; j < k; j++) {
                if (fr[j].id == e) continue;
                if (slot >= 10) { bad++; break; }
                double w = 0.0;
                for (int q = 0; q < j; q++) w += R[q];
                w -= 0.5;
                for (int q = 0; q < k; q++)
                    if (fr[j].id == m.faces[nd * 6 + q]) w *= m.node_face_dir[nd * 6 + q];
                w *= tev;
                m.interp_friends[e * 10 + slot] = fr[j].id;
                m.interp_w[e * 10 + slot] = w;
                slot++;
            }
        }
        m.interp_n[e] = slot;
    }
    if (bad) return ODIS_ERR_MESH;

    // --- vertex geometry of the nonlinear terms ---------------------------
    const int V = m.V;
    m.face_verts.assign((size_t)E * 2, -1);
    for (int e = 0; e < E; e++) {
        const int i = m.face_nodes[e * 2], j = face_slot[e], k = m.nfriends(i);
        m.face_verts[e * 2] = m.vertexes[i * 6 + (j + k - 1) % k];
        m.face_verts[e * 2 + 1] = m.vertexes[i * 6 + j % k];
    }
    // kite fractions: the reference assigns vertex_R(v, node) once per face about
    // the node, and the node's highest-numbered face writes last; the same
    // ranking about that face gives the same sums, bit for bit
    m.vert_R.assign((size_t)V * 3, 0.0);
    int badv = 0;
#pragma omp parallel for schedule(static) reduction(+ : badv)
    for (int nd = 0; nd < N; nd++) {
        const int k = m.nfriends(nd);
        int e = -1;
        for (int j = 0; j < k; j++) e = std::max(e, m.faces[nd * 6 + j]);
        LL ie{m.face_int[e * 2], m.face_int[e * 2 + 1]};
        LL c = node(nd);
        Ranked fr[6], vr[6];
        for (int j = 0; j < k; j++) {
            int id = m.faces[nd * 6 + j];
            double a = angle_about(ie, LL{m.face_int[id * 2], m.face_int[id * 2 + 1]}, c) * 180. / kPi;
            if (a > 0.0 + 1e-8) a -= 360.0;
            fr[j] = {id, a};
            int vid = m.vertexes[nd * 6 + j];
            double b = angle_about(ie, LL{m.vert_sph[vid * 2], m.vert_sph[vid * 2 + 1]}, c) * 180. / kPi;
            if (b > 0.0 + 1e-8) b -= 360.0;
            vr[j] = {vid, b};
        }
        auto desc = [](const Ranked& a, const Ranked& b) { return a.deg > b.deg; };
        std::sort(fr, fr + k, desc);
        std::sort(vr, vr + k, desc);
        auto vpos = [&](int vid) { return LL{m.vert_sph[vid * 2], m.vert_sph[vid * 2 + 1]}; };
        auto ipos = [&](int fid) { return LL{m.face_int[fid * 2], m.face_int[fid * 2 + 1]}; };
        double area_cv = 0.0;
        for (int j = 0; j < k; j++) area_cv += sph_tri_area(c, vpos(vr[j].id), vpos(vr[(j + 1) % k].id), radius);
        for (int j = 0; j < k; j++) {
            LL v = vpos(vr[j].id);
            const double a1 = sph_tri_area(c, v, ipos(fr[j].id), radius);
            const double a2 = sph_tri_area(c, v, ipos(fr[(j + 1) % k].id), radius);
            int slot = -1;
            for (int q = 0; q < 3; q++)
                if (m.vert_nodes[vr[j].id * 3 + q] == nd) { slot = q; break; }
            if (slot < 0) { badv++; continue; }
            m.vert_R[vr[j].id * 3 + slot] = (a1 + a2) / area_cv;
        }
    }
    if (badv) return ODIS_ERR_MESH;
    // faces about each vertex, in face order, and their circulation signs
    m.vert_faces.assign((size_t)V * 3, -1);
    m.vert_face_dir.assign((size_t)V * 3, 0);
    for (int e = 0; e < E; e++)
        for (int q = 0; q < 2; q++) {
            const int v = m.face_verts[e * 2 + q];
            for (int j = 0; j < 3; j++) {
                if (m.vert_faces[v * 3 + j] >= 0) continue;
                m.vert_faces[v * 3 + j] = e;
                double mm, xv, yv;
                stereo(LL{m.face_centre[e * 2], m.face_centre[e * 2 + 1]}, LL{m.vert_sph[v * 2], m.vert_sph[v * 2 + 1]},
                       radius, mm, xv, yv);
                const double cross = xv * m.face_normal[e * 2 + 1] - yv * m.face_normal[e * 2];
                m.vert_face_dir[v * 3 + j] = cross > 0 ? 1 : -1;
                break;
            }
        }
    m.vert_area.assign(V, 0.0);
    for (int v = 0; v < V; v++) {
        if (m.vert_faces[v * 3 + 2] < 0) return ODIS_ERR_MESH;
        double area = 0.0;
        for (int j = 0; j < 3; j++)
            area += std::fabs(sph_tri_area(LL{m.vert_sph[v * 2], m.vert_sph[v * 2 + 1]}, node(m.vert_nodes[v * 3 + j]),
                                           node(m.vert_nodes[v * 3 + (j + 1) % 3]), radius));
        m.vert_area[v] = area;
    }
    return ODIS_OK;
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

