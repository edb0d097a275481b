// Mesh topology, geometry and TRiSK weights as independent per-element steps,
// run by the host builder (odis_mesh.cpp, OpenMP loops) and the device builder
// (odis_mesh_dev.cu, one kernel per step).
//
// The reference numbers vertices and faces in sequential loops, by the first
// node, in file order, that reaches them (src/mesh.cpp:436-506, 508-561).
// Those numberings have a closed form that every element can evaluate on its
// own:
//   * vertex (i, j), the centroid shared by node i and its friends j and j+1,
//     is created by the smallest of the three nodes; its id is the number of
//     vertices created by lower nodes plus its rank among the creating slots
//     of its creator;
//   * face (i, j) is created by the smaller of node i and friend j, with the
//     same prefix-count numbering.
// So the build is: per-node counts, an exclusive scan, then per-slot, per-face,
// per-node and per-vertex steps, each writing only its own elements.  The
// floating-point formulas are those of odis_geom.cuh, in the reference's
// order; on the host they give the reference's coefficients bit for bit, on the
// device (CUDA's math functions) the same to rounding, the integers exactly.
#pragma once

#include "odis_exec.cuh"
#include "odis_geom.cuh"

namespace odis {

struct MeshView {
    int N = 0, E = 0, V = 0;
    double r = 0.0;
    const double* node_sph = nullptr;   // [N][2]
    const int* friends = nullptr;       // [N][6]
    const double* cent_sph = nullptr;   // [N][6][2]
    int* vbase = nullptr;               // [N + 1] vertices created by lower nodes (after the scan)
    int* fbase = nullptr;               // [N + 1] faces created by lower nodes
    double* cv_area = nullptr;          // [N]
    int* vertexes = nullptr;            // [N][6]
    double* vert_sph = nullptr;         // [V][2]
    int* vert_nodes = nullptr;          // [V][3]
    int* faces = nullptr;               // [N][6]
    int* node_face_dir = nullptr;       // [N][6]
    int* face_nodes = nullptr;          // [E][2]
    int* face_slot = nullptr;           // [E] slot of the face at its first node
    double *face_len = nullptr, *face_dist = nullptr, *face_area = nullptr;   // [E]
    double *face_centre = nullptr, *face_m = nullptr, *face_normal = nullptr, *face_int = nullptr;  // [E][2]
    double* face_nxyz = nullptr;        // [E][3]
    int* interp_friends = nullptr;      // [E][10]
    double* interp_w = nullptr;         // [E][10]
    int* interp_n = nullptr;            // [E]
    int* face_verts = nullptr;          // [E][2]
    double* vert_R = nullptr;           // [V][3]
    int* vert_faces = nullptr;          // [V][3]
    int* vert_face_dir = nullptr;       // [V][3]
    double* vert_area = nullptr;        // [V]
    // per node slot: the absolute angles, about the node, of the slot's face intercept and vertex, and
    // the kite areas of the slot's vertex with its cyclic successor vertex (cv) and with the faces
    // before (a1) and after (a2) it, computed once per node for every ranking about it
    double *th_f = nullptr, *th_v = nullptr, *kcv = nullptr, *ka1 = nullptr, *ka2 = nullptr;   // [N][6]
    int* err = nullptr;                 // nonzero: the arrays do not describe a valid mesh

    ODIS_HD int nfriends(int i) const { return friends[i * 6 + 5] < 0 ? 5 : 6; }
    ODIS_HD geo::LL node(int i) const { return {node_sph[i * 2], node_sph[i * 2 + 1]}; }
    ODIS_HD geo::LL cent(int i, int j) const { return {cent_sph[(i * 6 + j) * 2], cent_sph[(i * 6 + j) * 2 + 1]}; }
    ODIS_HD geo::LL vpos(int v) const { return {vert_sph[v * 2], vert_sph[v * 2 + 1]}; }
    ODIS_HD geo::LL ipos(int e) const { return {face_int[e * 2], face_int[e * 2 + 1]}; }
    // the two nodes besides i sharing centroid j of node i
    ODIS_HD int nb0(int i, int j) const { return friends[i * 6 + j % nfriends(i)]; }
    ODIS_HD int nb1(int i, int j) const { return friends[i * 6 + (j + 1) % nfriends(i)]; }
    ODIS_HD bool creates_vertex(int i, int j) const { return i < nb0(i, j) && i < nb1(i, j); }
    ODIS_HD bool creates_face(int i, int j) const { return friends[i * 6 + j] > i; }
    ODIS_HD void fail() const { exec_flag(err); }
};

// counts of created vertices and faces per node (scanned into vbase/fbase), and
// the control-volume area in node-centred map coordinates (src/mesh.cpp:1828-1866)
struct StepCounts {
    MeshView m;
    ODIS_HD void operator()(int i) const
    {
        const int k = m.nfriends(i);
        int nv = 0, nf = 0;
        for (int j = 0; j < k; j++) {
            nv += m.creates_vertex(i, j);
            nf += m.creates_face(i, j);
        }
        m.vbase[i] = nv;
        m.fbase[i] = nf;
        const double r = m.r;
        double mc, xc, yc;
        geo::stereo(m.node(i), m.node(i), r, mc, xc, yc);
        double xy[6][2];
        for (int j = 0; j < k; j++) geo::stereo(m.node(i), m.cent(i, j), r, mc, xy[j][0], xy[j][1]);
        double area = 0.0;
        for (int j = 0; j < k; j++) {
            const double* p1 = xy[j];
            const double* p2 = xy[(j + 1) % k];
            area += 0.5 * fabs(xc * (p1[1] - p2[1]) + p1[0] * (p2[1] - yc) + p2[0] * (yc - p1[1]));
        }
        m.cv_area[i] = area;
    }
};

// every slot of node i: its vertex and face ids (the creator's prefix count plus
// rank), vertex positions and nodes, face end nodes and directions
struct StepSlots {
    MeshView m;
    // id of the vertex created at slot q of node c
    ODIS_HD int vertex_id(int c, int q) const
    {
        int rank = 0;
        for (int a = 0; a < q; a++) rank += m.creates_vertex(c, a);
        return m.vbase[c] + rank;
    }
    ODIS_HD int face_id(int c, int q) const
    {
        int rank = 0;
        for (int a = 0; a < q; a++) rank += m.creates_face(c, a);
        return m.fbase[c] + rank;
    }
    ODIS_HD void operator()(int i) const
    {
        const int k = m.nfriends(i);
        for (int j = 0; j < k; j++) {
            const int a = m.nb0(i, j), b = m.nb1(i, j);
            if (m.creates_vertex(i, j)) {
                const int vid = vertex_id(i, j);
                const geo::LL v = m.cent(i, j);
                m.vertexes[i * 6 + j] = vid;
                m.vert_sph[vid * 2] = v.lat;
                m.vert_sph[vid * 2 + 1] = v.lon;
                m.vert_nodes[vid * 3] = i;
                m.vert_nodes[vid * 3 + 1] = a;
                m.vert_nodes[vid * 3 + 2] = b;
            } else {
                // the creator's slot at the same centroid (1e-9 rad, as the reference matches them)
                const int c = a < b ? a : b;
                const geo::LL v = m.cent(i, j);
                const int kc = m.nfriends(c);
                int vid = -1;
                for (int q = 0; q < kc; q++) {
                    if (!m.creates_vertex(c, q) || (m.nb0(c, q) != i && m.nb1(c, q) != i)) continue;
                    const geo::LL w = m.cent(c, q);
                    if (w.lat < v.lat + 1e-9 && w.lat > v.lat - 1e-9 && w.lon < v.lon + 1e-9 && w.lon > v.lon - 1e-9)
                        vid = vertex_id(c, q);
                }
                if (vid < 0) m.fail();
                m.vertexes[i * 6 + j] = vid;
            }
            const int f = m.friends[i * 6 + j];
            if (m.creates_face(i, j)) {
                const int fid = face_id(i, j);
                m.faces[i * 6 + j] = fid;
                m.node_face_dir[i * 6 + j] = 1;
                m.face_nodes[fid * 2] = i;
                m.face_slot[fid] = j;
            } else {
                const int kf = m.nfriends(f);
                int fid = -1;
                for (int q = 0; q < kf; q++)
                    if (m.friends[f * 6 + q] == i) fid = face_id(f, q);
                if (fid < 0) { m.fail(); continue; }
                m.faces[i * 6 + j] = fid;
                m.node_face_dir[i * 6 + j] = -1;
                m.face_nodes[fid * 2 + 1] = i;
            }
        }
    }
};

// face geometry (src/mesh.cpp:508-670, face area :1093) and the face's two vertices
struct StepFaceGeometry {
    MeshView m;
    ODIS_HD void operator()(int e) const
    {
        const int i = m.face_nodes[e * 2], f = m.face_nodes[e * 2 + 1], j = m.face_slot[e];
        if (i < 0 || f < 0 || j < 0) { m.fail(); return; }
        const int k = m.nfriends(i);
        const double r = m.r;
        const geo::LL v1 = m.cent(i, (j + k - 1) % k), v2 = m.cent(i, j % k);
        m.face_verts[e * 2] = m.vertexes[i * 6 + (j + k - 1) % k];
        m.face_verts[e * 2 + 1] = m.vertexes[i * 6 + j % k];
        m.face_len[e] = fabs(geo::arc_acos(v1, v2, r));
        geo::LL c = geo::midpoint(v1, v2);
        if (c.lon < 0.0) c.lon += 2 * geo::kGeoPi;
        m.face_centre[e * 2] = c.lat;
        m.face_centre[e * 2 + 1] = c.lon;
        double mm, x, y;
        geo::stereo(c, m.node(i), r, mm, x, y);
        m.face_m[e * 2] = mm;
        geo::stereo(c, m.node(f), r, mm, x, y);
        m.face_m[e * 2 + 1] = mm;
        m.face_dist[e] = geo::arc_atan2(m.node(i), m.node(f)) * r;
        double n[2];
        geo::map_normal(v1, v2, n);
        m.face_normal[e * 2] = n[0];
        m.face_normal[e * 2 + 1] = n[1];
        {
            // Cartesian normal: the unit cross product of the vertex positions (include/mathRoutines.h:246-267)
            double p1[3], p2[3];
            geo::to_xyz(v1, p1);
            geo::to_xyz(v2, p2);
            const double c0 = p1[1] * p2[2] - p1[2] * p2[1];
            const double c1 = -(p1[0] * p2[2] - p1[2] * p2[0]);
            const double c2 = p1[0] * p2[1] - p1[1] * p2[0];
            const double mag = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
            m.face_nxyz[e * 3] = c0 / mag;
            m.face_nxyz[e * 3 + 1] = c1 / mag;
            m.face_nxyz[e * 3 + 2] = c2 / mag;
        }
        const geo::LL ip = geo::intersect(v1, v2, m.node(i), m.node(f));
        m.face_int[e * 2] = ip.lat;
        m.face_int[e * 2 + 1] = ip.lon;
        m.face_area[e] = m.face_dist[e] * m.face_len[e];
    }
};

// faces and vertices about node nd ranked anticlockwise from face e (degrees,
// wrapped to (-360, 1e-8]), and the control-volume area summed over the
// ranked vertices, from the node's absolute angles (StepNodeAngles): the same
// subtraction, wrap and scaling as angle_about, so the same ranking bits
struct Ranking {
    geo::Ranked fr[6], vr[6];
    double area_cv;
};

ODIS_HD inline void rank_angles(const MeshView& m, int nd, double te, geo::Ranked* fr, geo::Ranked* vr)
{
    const int k = m.nfriends(nd);
    for (int j = 0; j < k; j++) {
        double a = geo::angle_between(te, m.th_f[nd * 6 + j]) * 180. / geo::kGeoPi;
        if (a > 0.0 + 1e-8) a -= 360.0;
        fr[j] = {m.faces[nd * 6 + j], j, a};
        double b = geo::angle_between(te, m.th_v[nd * 6 + j]) * 180. / geo::kGeoPi;
        if (b > 0.0 + 1e-8) b -= 360.0;
        vr[j] = {m.vertexes[nd * 6 + j], j, b};
    }
    geo::sort_desc(fr, k);
    geo::sort_desc(vr, k);
}

ODIS_HD inline void rank_about(const MeshView& m, int nd, int e, Ranking& o)
{
    const int k = m.nfriends(nd);
    int je = -1;
    for (int j = 0; j < k; j++)
        if (m.faces[nd * 6 + j] == e) je = j;
    if (je < 0) m.fail();
    const double te = je < 0 ? 0.0 : m.th_f[nd * 6 + je];
    rank_angles(m, nd, te, o.fr, o.vr);
    double area_cv = 0.0;
    for (int j = 0; j < k; j++) area_cv += m.kcv[nd * 6 + o.vr[j].slot];
    o.area_cv = area_cv;
}

// node nd: absolute angles of its faces' intercepts and vertices, and the kite
// areas (src/mesh.cpp:680-907: the control volume's triangles of consecutive
// vertices, the two triangles of each vertex with its neighbouring faces'
// intercepts).  A vertex lies between the faces ranked just before and after
// it, whatever face the ranking starts from, so these areas serve every
// ranking about the node; each face's ranking sums them in its own order.
struct StepNodeAngles {
    MeshView m;
    ODIS_HD void operator()(int nd) const
    {
        const int k = m.nfriends(nd);
        const geo::LL c = m.node(nd);
        for (int j = 0; j < k; j++) {
            m.th_f[nd * 6 + j] = geo::angle_in_plane(m.ipos(m.faces[nd * 6 + j]), c);
            m.th_v[nd * 6 + j] = geo::angle_in_plane(m.vpos(m.vertexes[nd * 6 + j]), c);
        }
        geo::Ranked fr[6], vr[6];
        rank_angles(m, nd, m.th_f[nd * 6], fr, vr);
        for (int j = 0; j < k; j++) {
            const geo::LL v = m.vpos(vr[j].id);
            const int q = nd * 6 + vr[j].slot;
            m.kcv[q] = geo::sph_tri_area(c, v, m.vpos(vr[(j + 1) % k].id), m.r);
            m.ka1[q] = geo::sph_tri_area(c, v, m.ipos(fr[j].id), m.r);
            m.ka2[q] = geo::sph_tri_area(c, v, m.ipos(fr[(j + 1) % k].id), m.r);
        }
    }
};

// TRiSK weights of face e (src/mesh.cpp:680-907): w = (sum_{j'<j} R_j' - 1/2) n_{e',node} t_{e,node}
struct StepTrisk {
    MeshView m;
    ODIS_HD void operator()(int e) const
    {
        int slot = 0;
        for (int side = 0; side < 2; side++) {
            const int nd = m.face_nodes[e * 2 + side];
            const int k = m.nfriends(nd);
            Ranking rk;
            rank_about(m, nd, e, rk);
            double R[6];
            for (int j = 0; j < k; j++) {
                const int q = nd * 6 + rk.vr[j].slot;
                R[j] = (m.ka1[q] + m.ka2[q]) / rk.area_cv;
            }
            const int tev = (m.face_nodes[e * 2] == nd) ? 1 : -1;
            for (int j = 0; j < k; j++) {
                if (rk.fr[j].id == e) continue;
                if (slot >= 10) { m.fail(); break; }
                double w = 0.0;
                for (int q = 0; q < j; q++) w += R[q];
                w -= 0.5;
                for (int q = 0; q < k; q++)
                    if (rk.fr[j].id == m.faces[nd * 6 + q]) w *= m.node_face_dir[nd * 6 + q];
                w *= tev;
                m.interp_friends[e * 10 + slot] = rk.fr[j].id;
                m.interp_w[e * 10 + slot] = w;
                slot++;
            }
        }
        for (int s = slot; s < 10; s++) {
            m.interp_friends[e * 10 + s] = 0;
            m.interp_w[e * 10 + s] = 0.0;
        }
        m.interp_n[e] = slot;
    }
};

// kite fractions of the vertices about node nd, ranked about the node's
// highest-numbered face: the reference assigns vertex_R once per face about
// the node and that face writes last (src/mesh.cpp:826-866)
struct StepVertexR {
    MeshView m;
    ODIS_HD void operator()(int nd) const
    {
        const int k = m.nfriends(nd);
        int e = -1;
        for (int j = 0; j < k; j++) e = m.faces[nd * 6 + j] > e ? m.faces[nd * 6 + j] : e;
        Ranking rk;
        rank_about(m, nd, e, rk);
        for (int j = 0; j < k; j++) {
            const int vid = rk.vr[j].id;
            const int q = nd * 6 + rk.vr[j].slot;
            const double a1 = m.ka1[q], a2 = m.ka2[q];
            int slot = -1;
            for (int q = 0; q < 3; q++)
                if (m.vert_nodes[vid * 3 + q] == nd) { slot = q; break; }
            if (slot < 0) { m.fail(); continue; }
            m.vert_R[vid * 3 + slot] = (a1 + a2) / rk.area_cv;
        }
    }
};

// the three faces about vertex v in ascending order (the faces between its node
// pairs), their circulation signs, and the area of its node triangle
// (src/mesh.cpp:911-1029, 1117-1148)
struct StepVertexFaces {
    MeshView m;
    ODIS_HD int face_between(int a, int b) const
    {
        const int k = m.nfriends(a);
        for (int q = 0; q < k; q++)
            if (m.friends[a * 6 + q] == b) return m.faces[a * 6 + q];
        return -1;
    }
    ODIS_HD void operator()(int v) const
    {
        const int* vn = m.vert_nodes + v * 3;
        int fc[3];
        for (int j = 0; j < 3; j++) {
            fc[j] = face_between(vn[j], vn[(j + 1) % 3]);
            if (fc[j] < 0 || (m.face_verts[fc[j] * 2] != v && m.face_verts[fc[j] * 2 + 1] != v)) { m.fail(); return; }
        }
        for (int a = 1; a < 3; a++)
            for (int b = a; b > 0 && fc[b - 1] > fc[b]; b--) { const int t = fc[b]; fc[b] = fc[b - 1]; fc[b - 1] = t; }
        const geo::LL vp = m.vpos(v);
        for (int j = 0; j < 3; j++) {
            const int e = fc[j];
            m.vert_faces[v * 3 + j] = e;
            double mm, xv, yv;
            geo::stereo(geo::LL{m.face_centre[e * 2], m.face_centre[e * 2 + 1]}, vp, m.r, mm, xv, yv);
            const double cross = xv * m.face_normal[e * 2 + 1] - yv * m.face_normal[e * 2];
            m.vert_face_dir[v * 3 + j] = cross > 0 ? 1 : -1;
        }
        double area = 0.0;
        for (int j = 0; j < 3; j++) area += fabs(geo::sph_tri_area(vp, m.node(vn[j]), m.node(vn[(j + 1) % 3]), m.r));
        m.vert_area[v] = area;
    }
};

}  // namespace odis

#include "odis_internal.h"

#include <vector>

namespace odis {

// The build as a sequence of per-element steps over an executor (odis_exec.cuh).
// Inputs are range-checked on the host before any step runs, so every index a
// step forms from them is inside its array.
template <class X>
int build_mesh_steps(X& x, int N, const double* node_sph, const int* friends, const double* cent_sph,
                     double radius, Mesh& m)
{
    if (N < 12 || !node_sph || !friends || !cent_sph || !(radius > 0.0)) return ODIS_ERR_ARG;
    for (int i = 0; i < N; i++) {
        for (int j = 0; j < 5; j++) {
            const int f = friends[i * 6 + j];
            if (f < 0 || f >= N || f == i) return ODIS_ERR_MESH;
        }
        const int f5 = friends[i * 6 + 5];
        if (f5 < -1 || f5 >= N || f5 == i) return ODIS_ERR_MESH;
    }
    m.N = N;
    m.r = radius;
    m.node_sph.assign(node_sph, node_sph + (size_t)N * 2);
    m.friends.assign(friends, friends + (size_t)N * 6);
    m.cent_sph.assign(cent_sph, cent_sph + (size_t)N * 12);

    MeshView v;
    v.N = N;
    v.r = radius;
    v.node_sph = x.in(m.node_sph.data(), m.node_sph.size());
    v.friends = x.in(m.friends.data(), m.friends.size());
    v.cent_sph = x.in(m.cent_sph.data(), m.cent_sph.size());
    auto vbase = x.template tmp<int>(N + 1, 0), fbase = x.template tmp<int>(N + 1, 0);
    auto err = x.template tmp<int>(1, 0);
    v.vbase = vbase.ptr;
    v.fbase = fbase.ptr;
    v.err = err.ptr;
    v.cv_area = x.out(m.cv_area, N, 0.0);
    v.vertexes = x.out(m.vertexes, (size_t)N * 6, -1);
    v.faces = x.out(m.faces, (size_t)N * 6, -1);
    v.node_face_dir = x.out(m.node_face_dir, (size_t)N * 6, 0);
    x.run(N, StepCounts{v});

    // exclusive scans of the per-node counts
    std::vector<int> vb(N + 1), fb(N + 1);
    x.to_host(vb.data(), vbase.ptr, N + 1);
    x.to_host(fb.data(), fbase.ptr, N + 1);
    long long sv = 0, sf = 0;
    for (int i = 0; i < N; i++) {
        const int cv = vb[i], cf = fb[i];
        vb[i] = (int)sv;
        fb[i] = (int)sf;
        sv += cv;
        sf += cf;
    }
    vb[N] = (int)sv;
    fb[N] = (int)sf;
    const int E = 3 * N - 6;
    if (x.status()) return x.status();
    if (sf != E || sv != 2 * N - 4) return ODIS_ERR_MESH;
    x.to_dev(vbase.ptr, vb.data(), N + 1);
    x.to_dev(fbase.ptr, fb.data(), N + 1);
    const int V = (int)sv;
    m.E = v.E = E;
    m.V = v.V = V;

    v.vert_sph = x.out(m.vert_sph, (size_t)V * 2, 0.0);
    v.vert_nodes = x.out(m.vert_nodes, (size_t)V * 3, -1);
    v.face_nodes = x.out(m.face_nodes, (size_t)E * 2, -1);
    auto fslot = x.template tmp<int>(E, -1);
    v.face_slot = fslot.ptr;
    x.run(N, StepSlots{v});
    if (x.failed(err.ptr)) return x.status() ? x.status() : ODIS_ERR_MESH;

    v.face_len = x.out(m.face_len, E, 0.0);
    v.face_dist = x.out(m.face_dist, E, 0.0);
    v.face_area = x.out(m.face_area, E, 0.0);
    v.face_centre = x.out(m.face_centre, (size_t)E * 2, 0.0);
    v.face_m = x.out(m.face_m, (size_t)E * 2, 0.0);
    v.face_normal = x.out(m.face_normal, (size_t)E * 2, 0.0);
    v.face_int = x.out(m.face_int, (size_t)E * 2, 0.0);
    v.face_nxyz = x.out(m.face_nxyz, (size_t)E * 3, 0.0);
    v.face_verts = x.out(m.face_verts, (size_t)E * 2, -1);
    x.run(E, StepFaceGeometry{v});
    if (x.failed(err.ptr)) return x.status() ? x.status() : ODIS_ERR_MESH;

    auto th_f = x.template tmp<double>((size_t)N * 6, 0.0), th_v = x.template tmp<double>((size_t)N * 6, 0.0);
    auto kcv = x.template tmp<double>((size_t)N * 6, 0.0), ka1 = x.template tmp<double>((size_t)N * 6, 0.0);
    auto ka2 = x.template tmp<double>((size_t)N * 6, 0.0);
    v.th_f = th_f.ptr;
    v.th_v = th_v.ptr;
    v.kcv = kcv.ptr;
    v.ka1 = ka1.ptr;
    v.ka2 = ka2.ptr;
    x.run(N, StepNodeAngles{v});
    v.interp_friends = x.out(m.interp_friends, (size_t)E * 10, 0);
    v.interp_w = x.out(m.interp_w, (size_t)E * 10, 0.0);
    v.interp_n = x.out(m.interp_n, E, 0);
    v.vert_R = x.out(m.vert_R, (size_t)V * 3, 0.0);
    v.vert_faces = x.out(m.vert_faces, (size_t)V * 3, -1);
    v.vert_face_dir = x.out(m.vert_face_dir, (size_t)V * 3, 0);
    v.vert_area = x.out(m.vert_area, V, 0.0);
    x.run(E, StepTrisk{v});
    x.run(N, StepVertexR{v});
    x.run(V, StepVertexFaces{v});
    if (x.failed(err.ptr)) return x.status() ? x.status() : ODIS_ERR_MESH;
    return x.finish();
}

}  // namespace odis
