// Icosahedral-geodesic grid generation as independent per-element steps, run
// by the host generator (odis_grid.cpp, OpenMP loops) and the device generator
// (odis_mesh_dev.cu, one kernel per step).
//
// The grid: a regular icosahedron (poles at +-90 deg) whose 20 faces are
// bisected `level` times, every new point the re-normalised sum of its edge's
// end points; nodes numbered by first appearance in the depth-first walk of
// the triangle hierarchy; friends clockwise seen from outside; the vertex of
// node i between friends j and j+1 the circumcentre of their triangle;
// coordinates in degrees rounded through the grid file's text form.  (The
// format is the one src/mesh.cpp:4016-4089 reads; the reference ships such
// files but not their generator.)
//
// Closed forms that make the steps independent:
//   * face F's points are the lattice (x, y, z), x + y + z = S = 2^level, in
//     weights of its corners A, B, C.  A point first appears at the level where
//     its coordinates are all multiples of s = 2^(level - L) and not all of 2s;
//     then exactly two are odd multiples of s, say i and j, and the point is the
//     midpoint of p + s (e_i - e_j) and p - s (e_i - e_j) of the level before.
//     Positions are built level by level; a point on a shared base edge gets the
//     same bits from both faces (the sum of two vectors is symmetric);
//   * every point has a key: a base vertex, a base edge and a position along
//     it, or a face interior point;
//   * leaf t of the walk (face t / 4^level, quadrant digits of t % 4^level) has
//     corners computed from its digits; the node number of a key is the rank of
//     its first appearance 3 t + q in the walk (an atomic minimum per key, a
//     count per leaf and a scan).
#pragma once

#include "odis_exec.cuh"
#include "odis_internal.h"
#include "odis_text_round.cuh"

#include <cmath>

namespace odis {

struct GV3 { double x, y, z; };

ODIS_HD inline GV3 gv_add(GV3 a, GV3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
ODIS_HD inline GV3 gv_sub(GV3 a, GV3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
ODIS_HD inline double gv_dot(GV3 a, GV3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
ODIS_HD inline GV3 gv_cross(GV3 a, GV3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
ODIS_HD inline GV3 gv_unit(GV3 a) { const double n = sqrt(gv_dot(a, a)); return {a.x / n, a.y / n, a.z / n}; }

constexpr double kGridPi = 3.14159265358979323846;

struct GenView {
    int level = 0, S = 1;             // S = 2^level
    long long T = 0;                  // leaves, 20 * 4^level
    int N = 0;                        // nodes, 10 S^2 + 2
    int P = 0;                        // lattice points per face, (S + 1)(S + 2) / 2
    int corner[20][3];                // base vertices of each face, in walk order
    int eid[12][12];                  // base edge index of a vertex pair
    GV3* fpos = nullptr;              // [20][P] positions of every face's lattice points
    int* first = nullptr;             // [N] first appearance 3 t + q of each key
    int* leafbase = nullptr;          // [T + 1] new keys in earlier leaves (after the scan)
    int* keyid = nullptr;             // [N] node number of each key
    GV3* pos = nullptr;               // [N] node positions
    int* tri = nullptr;               // [T][3] node numbers of each leaf's corners
    GV3* cc = nullptr;                // [T] circumcentre of each leaf
    int* inc_n = nullptr;             // [N] incident leaves
    int* inc = nullptr;               // [N][6]
    double* node_deg = nullptr;       // [N][2]
    int* friends = nullptr;           // [N][6]
    double* cent_deg = nullptr;       // [N][6][2]
    int* err = nullptr;

    ODIS_HD int pidx(int x, int y) const { return y * (S + 1) - y * (y - 1) / 2 + x; }
    // key of lattice point (x, y, S - x - y) of face F
    ODIS_HD int key(int F, int x, int y) const
    {
        const int z = S - x - y;
        const int a = corner[F][0], b = corner[F][1], c = corner[F][2];
        if (x == S) return a;
        if (y == S) return b;
        if (z == S) return c;
        int u = -1, w = -1, wu = 0, ww = 0;                  // edge end points and their weights
        if (z == 0) { u = a; w = b; wu = x; ww = y; }
        else if (y == 0) { u = a; w = c; wu = x; ww = z; }
        else if (x == 0) { u = b; w = c; wu = y; ww = z; }
        if (u >= 0) {
            const int lo = u < w ? u : w, hi = u < w ? w : u;
            const int along = u < w ? ww : wu;               // weight on the higher-numbered end
            return 12 + eid[lo][hi] * (S - 1) + along - 1;
        }
        const int off = (y - 1) * (S - 1) - (y - 1) * y / 2;
        return 12 + 30 * (S - 1) + F * ((S - 1) * (S - 2) / 2) + off + x - 1;
    }
    // lattice corners (x, y) of leaf t, and its face
    ODIS_HD int leaf(long long t, int cx[3], int cy[3]) const
    {
        const int F = (int)(t >> (2 * level));
        const long long l = t & ((1LL << (2 * level)) - 1);
        int ax = S, ay = 0, bx = 0, by = S, qx = 0, qy = 0;  // corners a, b, c
        for (int d = level - 1; d >= 0; d--) {
            const int dig = (int)((l >> (2 * d)) & 3);
            const int abx = (ax + bx) / 2, aby = (ay + by) / 2;
            const int bcx = (bx + qx) / 2, bcy = (by + qy) / 2;
            const int cax = (qx + ax) / 2, cay = (qy + ay) / 2;
            if (dig == 0) { bx = abx; by = aby; qx = cax; qy = cay; }
            else if (dig == 1) { ax = abx; ay = aby; bx = bcx; by = bcy; qx = cax; qy = cay; }
            else if (dig == 2) { ax = abx; ay = aby; qx = bcx; qy = bcy; }
            else { ax = cax; ay = cay; bx = bcx; by = bcy; }
        }
        cx[0] = ax; cy[0] = ay; cx[1] = bx; cy[1] = by; cx[2] = qx; cy[2] = qy;
        return F;
    }
};

// points that first appear at level L (L >= 1), over the level-L lattice of every face
struct GenLevel {
    GenView g;
    int L;
    ODIS_HD void operator()(long long idx) const
    {
        const int SL = 1 << L, s = g.S >> L;
        const long long per = (long long)(SL + 1) * (SL + 1);
        const int F = (int)(idx / per);
        const int r = (int)(idx % per);
        const int xl = r % (SL + 1), yl = r / (SL + 1);
        if (xl + yl > SL) return;
        const int zl = SL - xl - yl;
        const int ox = xl & 1, oy = yl & 1, oz = zl & 1;
        if (!ox && !oy && !oz) return;                       // a point of the level before
        const int x = xl * s, y = yl * s;
        // parents: move by s along the two odd coordinates, in opposite senses
        int x1 = x, y1 = y, x2 = x, y2 = y;
        if (ox && oy) { x1 += s; y1 -= s; x2 -= s; y2 += s; }
        else if (ox) { x1 += s; x2 -= s; }                   // x and z odd: z absorbs the change
        else { y1 += s; y2 -= s; }                           // y and z odd
        const GV3* f = g.fpos + (size_t)F * g.P;
        g.fpos[(size_t)F * g.P + g.pidx(x, y)] = gv_unit(gv_add(f[g.pidx(x1, y1)], f[g.pidx(x2, y2)]));
    }
};

// first appearance of every key in the walk
struct GenFirst {
    GenView g;
    ODIS_HD void operator()(long long t) const
    {
        int cx[3], cy[3];
        const int F = g.leaf(t, cx, cy);
        for (int q = 0; q < 3; q++) exec_atomic_min(&g.first[g.key(F, cx[q], cy[q])], (int)(3 * t + q));
    }
};

// keys that appear first in leaf t
struct GenCount {
    GenView g;
    ODIS_HD void operator()(long long t) const
    {
        int cx[3], cy[3];
        const int F = g.leaf(t, cx, cy);
        int n = 0;
        for (int q = 0; q < 3; q++) n += g.first[g.key(F, cx[q], cy[q])] == (int)(3 * t + q);
        g.leafbase[t] = n;
    }
};

// node numbers and positions of the keys that appear first in leaf t
struct GenNumber {
    GenView g;
    ODIS_HD void operator()(long long t) const
    {
        int cx[3], cy[3];
        const int F = g.leaf(t, cx, cy);
        int id = g.leafbase[t];
        for (int q = 0; q < 3; q++) {
            const int k = g.key(F, cx[q], cy[q]);
            if (g.first[k] != (int)(3 * t + q)) continue;
            if (id >= g.N) { exec_flag(g.err); return; }
            g.keyid[k] = id;
            g.pos[id] = g.fpos[(size_t)F * g.P + g.pidx(cx[q], cy[q])];
            id++;
        }
    }
};

// corners of leaf t as node numbers, its circumcentre (outward), its incidence
struct GenLeaf {
    GenView g;
    ODIS_HD void operator()(long long t) const
    {
        int cx[3], cy[3];
        const int F = g.leaf(t, cx, cy);
        GV3 p[3];
        for (int q = 0; q < 3; q++) {
            const int id = g.keyid[g.key(F, cx[q], cy[q])];
            if (id < 0 || id >= g.N) { exec_flag(g.err); return; }
            g.tri[3 * t + q] = id;
            p[q] = g.fpos[(size_t)F * g.P + g.pidx(cx[q], cy[q])];
            const int slot = exec_atomic_add(&g.inc_n[id], 1);
            if (slot < 6) g.inc[id * 6 + slot] = (int)t;
            else exec_flag(g.err);
        }
        GV3 n = gv_unit(gv_cross(gv_sub(p[1], p[0]), gv_sub(p[2], p[0])));
        if (gv_dot(n, gv_add(gv_add(p[0], p[1]), p[2])) < 0) n = {-n.x, -n.y, -n.z};
        g.cc[t] = n;
    }
};

ODIS_HD inline void grid_latlon(GV3 p, double& lat, double& lon)
{
    lat = atan2(p.z, sqrt(p.x * p.x + p.y * p.y)) * 180.0 / kGridPi;
    lon = atan2(p.y, p.x) * 180.0 / kGridPi;
    if (lon < 0.0) lon += 360.0;
    if (lon >= 360.0) lon -= 360.0;
}

// node i: its coordinates, friends ordered clockwise (descending angle in the
// local east/north frame) and the circumcentres between consecutive friends
struct GenNode {
    GenView g;
    ODIS_HD void operator()(long long ii) const
    {
        const int i = (int)ii;
        const GV3 p = g.pos[i];
        double lat, lon;
        grid_latlon(p, lat, lon);
        g.node_deg[i * 2] = text_round16(lat);
        g.node_deg[i * 2 + 1] = text_round16(lon);
        const int ni = g.inc_n[i];
        if (ni != 5 && ni != 6) { exec_flag(g.err); return; }
        int inc[6];
        for (int q = 0; q < ni; q++) inc[q] = g.inc[i * 6 + q];
        for (int a = 1; a < ni; a++)                          // ascending leaf order
            for (int b = a; b > 0 && inc[b - 1] > inc[b]; b--) { const int s = inc[b]; inc[b] = inc[b - 1]; inc[b - 1] = s; }
        int nb[12];
        int k = 0;
        for (int q = 0; q < ni; q++)
            for (int c = 0; c < 3; c++) {
                const int v = g.tri[3 * (long long)inc[q] + c];
                bool seen = v == i;
                for (int r = 0; r < k && !seen; r++) seen = nb[r] == v;
                if (!seen && k < 12) nb[k++] = v;
            }
        if (k != ni) { exec_flag(g.err); return; }
        const double lr = atan2(p.y, p.x);
        const GV3 east = {-sin(lr), cos(lr), 0.0};
        const GV3 north = gv_cross(p, east);
        // a neighbour due west sits on atan2's branch cut, where a rounding-level north
        // component (its sign differs between math libraries) decides between +pi and
        // -pi: it is put at +pi, first
        double ang[6];
        for (int j = 0; j < k; j++) {
            const GV3 d = gv_sub(g.pos[nb[j]], p);
            const double dn = gv_dot(d, north), de = gv_dot(d, east);
            ang[j] = (de < 0.0 && fabs(dn) <= 1e-12 * fabs(de)) ? kGridPi : atan2(dn, de);
        }
        for (int a = 1; a < k; a++)                           // descending angle, stable
            for (int b = a; b > 0 && ang[b - 1] < ang[b]; b--) {
                const double t = ang[b]; ang[b] = ang[b - 1]; ang[b - 1] = t;
                const int s = nb[b]; nb[b] = nb[b - 1]; nb[b - 1] = s;
            }
        for (int j = 0; j < k; j++) g.friends[i * 6 + j] = nb[j];
        for (int j = 0; j < k; j++) {
            const int fa = nb[j], fb = nb[(j + 1) % k];
            int found = -1;
            for (int q = 0; q < ni && found < 0; q++) {
                const int* tv = g.tri + 3 * (long long)inc[q];
                const bool ha = tv[0] == fa || tv[1] == fa || tv[2] == fa;
                const bool hb = tv[0] == fb || tv[1] == fb || tv[2] == fb;
                if (ha && hb) found = inc[q];
            }
            if (found < 0) { exec_flag(g.err); return; }
            double clat, clon;
            grid_latlon(g.cc[found], clat, clon);
            g.cent_deg[(i * 6 + j) * 2] = text_round16(clat);
            g.cent_deg[(i * 6 + j) * 2 + 1] = text_round16(clon);
        }
    }
};

// base positions set on the host (the generators agree on them bit for bit)
struct GenBase {
    GenView g;
    GV3 base[12];
    ODIS_HD void operator()(long long idx) const
    {
        const int F = (int)(idx / 3), q = (int)(idx % 3);
        const int x = q == 0 ? g.S : 0, y = q == 1 ? g.S : 0;
        g.fpos[(size_t)F * g.P + g.pidx(x, y)] = base[g.corner[F][q]];
    }
};

template <class X>
int generate_grid_steps(X& x, int level, GridArrays& out)
{
    if (level < 0 || level > 10) return ODIS_ERR_ARG;
    GenView g;
    g.level = level;
    g.S = 1 << level;
    g.T = 20LL << (2 * level);
    g.N = 10 * g.S * g.S + 2;
    g.P = (g.S + 1) * (g.S + 2) / 2;
    GenBase gb;
    {
        const double lat0 = std::atan(0.5);
        gb.base[0] = {0.0, 0.0, 1.0};
        for (int k = 0; k < 5; k++) {
            const double lon = 2.0 * kGridPi * k / 5.0;
            gb.base[1 + k] = {std::cos(lat0) * std::cos(lon), std::cos(lat0) * std::sin(lon), std::sin(lat0)};
        }
        for (int k = 0; k < 5; k++) {
            const double lon = 2.0 * kGridPi * k / 5.0 + kGridPi / 5.0;
            gb.base[6 + k] = {std::cos(lat0) * std::cos(lon), std::cos(lat0) * std::sin(lon), -std::sin(lat0)};
        }
        gb.base[11] = {0.0, 0.0, -1.0};
        // the 20 faces walked around the body, neighbouring faces adjacent
        for (int k = 0; k < 5; k++) {
            const int u0 = 1 + k, u1 = 1 + (k + 1) % 5, l0 = 6 + k, l1 = 6 + (k + 1) % 5;
            const int f[4][3] = {{0, u0, u1}, {u0, l0, u1}, {u1, l0, l1}, {11, l1, l0}};
            for (int q = 0; q < 4; q++)
                for (int c = 0; c < 3; c++) g.corner[4 * k + q][c] = f[q][c];
        }
        for (int a = 0; a < 12; a++)
            for (int b = 0; b < 12; b++) g.eid[a][b] = -1;
        int ne = 0;
        for (int F = 0; F < 20; F++)
            for (int c = 0; c < 3; c++) {
                const int u = g.corner[F][c], w = g.corner[F][(c + 1) % 3];
                const int lo = u < w ? u : w, hi = u < w ? w : u;
                if (g.eid[lo][hi] < 0) g.eid[lo][hi] = ne++;
            }
        if (ne != 30) return ODIS_ERR_MESH;
    }
    const int N = g.N;
    auto fpos = x.template tmp<GV3>((size_t)20 * g.P, GV3{0.0, 0.0, 0.0});
    auto first = x.template tmp<int>(N, 0x7fffffff);
    auto leafbase = x.template tmp<int>(g.T + 1, 0);
    auto keyid = x.template tmp<int>(N, -1);
    auto pos = x.template tmp<GV3>(N, GV3{0.0, 0.0, 0.0});
    auto tri = x.template tmp<int>(3 * g.T, -1);
    auto cc = x.template tmp<GV3>(g.T, GV3{0.0, 0.0, 0.0});
    auto inc_n = x.template tmp<int>(N, 0);
    auto inc = x.template tmp<int>((size_t)N * 6, -1);
    auto err = x.template tmp<int>(1, 0);
    g.fpos = fpos.ptr;
    g.first = first.ptr;
    g.leafbase = leafbase.ptr;
    g.keyid = keyid.ptr;
    g.pos = pos.ptr;
    g.tri = tri.ptr;
    g.cc = cc.ptr;
    g.inc_n = inc_n.ptr;
    g.inc = inc.ptr;
    g.err = err.ptr;
    out.N = N;
    g.node_deg = x.out(out.node_deg, (size_t)N * 2, 0.0);
    g.friends = x.out(out.friends, (size_t)N * 6, -1);
    g.cent_deg = x.out(out.cent_deg, (size_t)N * 12, -1.0);
    if (x.status()) return x.status();

    gb.g = g;
    x.run(60, gb);
    for (int L = 1; L <= level; L++) {
        const long long SL = 1LL << L;
        x.run(20 * (SL + 1) * (SL + 1), GenLevel{g, L});
    }
    x.run(g.T, GenFirst{g});
    x.run(g.T, GenCount{g});
    if (x.scan(g.leafbase, g.T + 1) != N) return x.status() ? x.status() : ODIS_ERR_MESH;
    x.run(g.T, GenNumber{g});
    x.run(g.T, GenLeaf{g});
    if (x.failed(g.err)) return x.status() ? x.status() : ODIS_ERR_MESH;
    x.run(N, GenNode{g});
    if (x.failed(g.err)) return x.status() ? x.status() : ODIS_ERR_MESH;
    return x.finish();
}

}  // namespace odis
