// Icosahedral-geodesic grid generator and reader/writer for the GeodesicODIS
// grid-file format.
//
// File format (one header line, then one line per node), as read by
// ReadMeshFile in src/mesh.cpp:4016-4089 of the reference:
//   ID  LAT  LON  {f0, f1, f2, f3, f4, f5}, {(lat0, lon0), ..., (lat5, lon5)}
// angles in degrees; pentagons have f5 = -1 and centroid 5 = (-1, -1).
// Centroid j of node i is the vertex shared by node i, friend j and friend
// j+1 (src/mesh.cpp:546-561 builds the edge to friend j from centroids j-1
// and j); friends are listed clockwise as seen from outside the sphere, so
// that the map normal of that edge points from node i to friend j
// (include/mathRoutines.h:214-248).  Vertices are spherical circumcentres of
// the Delaunay triangles, which is what the shipped grid files hold.
//
// Generation: regular icosahedron (poles at +-90 deg), recursive 4-way
// bisection with re-normalisation.  Level n has 10*4^n+2 nodes.  Nodes are
// numbered in order of first appearance in a depth-first walk of the
// triangle hierarchy, so cells that are close on the sphere are close in
// memory (which keeps the 10-edge TRiSK gathers inside L2 sectors).
#include "odis_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

namespace odis {

namespace {

struct V3 { double x, y, z; };

inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline V3 unit(V3 a) { double n = std::sqrt(dot(a, a)); return {a.x / n, a.y / n, a.z / n}; }

struct Builder {
    std::vector<V3> pos;
    std::unordered_map<uint64_t, int> mid;
    std::vector<int> leaf;                 // leaf triangles, 3 ints each

    int midpoint(int a, int b) {
        uint64_t key = a < b ? ((uint64_t)a << 32) | (uint32_t)b : ((uint64_t)b << 32) | (uint32_t)a;
        auto it = mid.find(key);
        if (it != mid.end()) return it->second;
        int id = (int)pos.size();
        pos.push_back(unit(add(pos[a], pos[b])));   // p+q == q+p bitwise, so both parents agree
        mid.emplace(key, id);
        return id;
    }
    void split(int a, int b, int c, int depth) {
        if (depth == 0) { leaf.push_back(a); leaf.push_back(b); leaf.push_back(c); return; }
        int ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
        split(a, ab, ca, depth - 1);
        split(ab, bc, ca, depth - 1);
        split(ab, b, bc, depth - 1);
        split(ca, bc, c, depth - 1);
    }
};

void fmt_deg(double v, char* buf) { std::snprintf(buf, 64, "%.16f", v); }

// Round a value through the grid file's text form, so an in-memory grid is
// bit-identical to the same grid written out and read back.
double text_round(double v) { char b[64]; fmt_deg(v, b); return std::strtod(b, nullptr); }

}  // namespace

int generate_grid(int level, GridArrays& g)
{
    if (level < 0 || level > 10) return ODIS_ERR_ARG;
    Builder B;
    const double pi = 3.14159265358979323846;
    const double lat0 = std::atan(0.5);
    B.pos.push_back({0.0, 0.0, 1.0});
    for (int k = 0; k < 5; k++) {
        double lon = 2.0 * pi * k / 5.0;
        B.pos.push_back({std::cos(lat0) * std::cos(lon), std::cos(lat0) * std::sin(lon), std::sin(lat0)});
    }
    for (int k = 0; k < 5; k++) {
        double lon = 2.0 * pi * k / 5.0 + pi / 5.0;
        B.pos.push_back({std::cos(lat0) * std::cos(lon), std::cos(lat0) * std::sin(lon), -std::sin(lat0)});
    }
    B.pos.push_back({0.0, 0.0, -1.0});
    // 20 base faces, walked around the body so neighbouring faces are adjacent
    for (int k = 0; k < 5; k++) {
        int u0 = 1 + k, u1 = 1 + (k + 1) % 5, l0 = 6 + k, l1 = 6 + (k + 1) % 5;
        B.split(0, u0, u1, level);
        B.split(u0, l0, u1, level);
        B.split(u1, l0, l1, level);
        B.split(11, l1, l0, level);
    }
    const int Nraw = (int)B.pos.size();
    const int N = 10 * (1 << (2 * level)) + 2;
    if (Nraw != N) return ODIS_ERR_MESH;
    const int T = (int)B.leaf.size() / 3;

    // renumber by first appearance in the leaf walk
    std::vector<int> perm(Nraw, -1);
    int next = 0;
    for (int t = 0; t < 3 * T; t++) {
        int v = B.leaf[t];
        if (perm[v] < 0) perm[v] = next++;
    }
    std::vector<V3> P(N);
    for (int v = 0; v < Nraw; v++) P[perm[v]] = B.pos[v];
    std::vector<int> tri(3 * T);
    for (int t = 0; t < 3 * T; t++) tri[t] = perm[B.leaf[t]];

    // circumcentre of every leaf triangle, computed once so that the three
    // nodes sharing it see identical values
    std::vector<V3> cc(T);
    for (int t = 0; t < T; t++) {
        V3 a = P[tri[3 * t]], b = P[tri[3 * t + 1]], c = P[tri[3 * t + 2]];
        V3 n = unit(cross(sub(b, a), sub(c, a)));
        if (dot(n, add(add(a, b), c)) < 0) n = {-n.x, -n.y, -n.z};
        cc[t] = n;
    }
    // node -> incident triangles
    std::vector<int> deg(N, 0);
    for (int t = 0; t < 3 * T; t++) deg[tri[t]]++;
    std::vector<int> start(N + 1, 0);
    for (int i = 0; i < N; i++) start[i + 1] = start[i] + deg[i];
    std::vector<int> inc(start[N]), fill(N, 0);
    for (int t = 0; t < T; t++)
        for (int q = 0; q < 3; q++) { int v = tri[3 * t + q]; inc[start[v] + fill[v]++] = t; }

    g.N = N;
    g.node_deg.assign((size_t)N * 2, 0.0);
    g.friends.assign((size_t)N * 6, -1);
    g.cent_deg.assign((size_t)N * 12, -1.0);
    auto latlon = [&](V3 p, double& lat, double& lon) {
        lat = std::atan2(p.z, std::sqrt(p.x * p.x + p.y * p.y)) * 180.0 / pi;
        lon = std::atan2(p.y, p.x) * 180.0 / pi;
        if (lon < 0.0) lon += 360.0;
        if (lon >= 360.0) lon -= 360.0;
    };
    for (int i = 0; i < N; i++) {
        V3 p = P[i];
        double lat, lon;
        latlon(p, lat, lon);
        g.node_deg[i * 2] = text_round(lat);
        g.node_deg[i * 2 + 1] = text_round(lon);
        // neighbours: the other two corners of each incident triangle
        std::vector<int> nb;
        for (int k = start[i]; k < start[i + 1]; k++) {
            int t = inc[k];
            for (int q = 0; q < 3; q++) {
                int v = tri[3 * t + q];
                if (v != i && std::find(nb.begin(), nb.end(), v) == nb.end()) nb.push_back(v);
            }
        }
        int k = (int)nb.size();
        if (k != 5 && k != 6) return ODIS_ERR_MESH;
        // local east/north frame; clockwise seen from outside = descending angle
        double lr = std::atan2(p.y, p.x);
        V3 east = {-std::sin(lr), std::cos(lr), 0.0};
        V3 north = cross(p, east);
        std::vector<std::pair<double, int>> ang(k);
        for (int j = 0; j < k; j++) {
            V3 d = sub(P[nb[j]], p);
            ang[j] = {std::atan2(dot(d, north), dot(d, east)), nb[j]};
        }
        std::sort(ang.begin(), ang.end(), [](const std::pair<double, int>& a, const std::pair<double, int>& b) {
            return a.first > b.first;
        });
        for (int j = 0; j < k; j++) g.friends[i * 6 + j] = ang[j].second;
        for (int j = 0; j < k; j++) {
            int fa = ang[j].second, fb = ang[(j + 1) % k].second;
            int found = -1;
            for (int q = start[i]; q < start[i + 1]; q++) {
                int t = inc[q];
                int* tv = &tri[3 * t];
                bool ha = tv[0] == fa || tv[1] == fa || tv[2] == fa;
                bool hb = tv[0] == fb || tv[1] == fb || tv[2] == fb;
                if (ha && hb) { found = t; break; }
            }
            if (found < 0) return ODIS_ERR_MESH;
            double clat, clon;
            latlon(cc[found], clat, clon);
            g.cent_deg[(i * 6 + j) * 2] = text_round(clat);
            g.cent_deg[(i * 6 + j) * 2 + 1] = text_round(clon);
        }
    }
    return ODIS_OK;
}

int write_grid(const GridArrays& g, const char* path)
{
    FILE* fp = std::fopen(path, "w");
    if (!fp) return ODIS_ERR_IO;
    std::fprintf(fp, "ID    NODE LAT     NODE LON     FRIENDS LIST                           CENTROID COORD LIST \n");
    char a[64], b[64];
    for (int i = 0; i < g.N; i++) {
        fmt_deg(g.node_deg[i * 2], a);
        fmt_deg(g.node_deg[i * 2 + 1], b);
        std::fprintf(fp, "%-5d %s %s {", i, a, b);
        for (int j = 0; j < 6; j++) std::fprintf(fp, "%5d%s", g.friends[i * 6 + j], j < 5 ? ", " : "}, {");
        for (int j = 0; j < 6; j++) {
            fmt_deg(g.cent_deg[(i * 6 + j) * 2], a);
            fmt_deg(g.cent_deg[(i * 6 + j) * 2 + 1], b);
            std::fprintf(fp, "(%s, %s)%s", a, b, j < 5 ? ", " : "} \n");
        }
    }
    return std::fclose(fp) == 0 ? ODIS_OK : ODIS_ERR_IO;
}

// Same column parsing as ReadMeshFile (src/mesh.cpp:4016-4089).
int read_grid(const char* path, GridArrays& g)
{
    FILE* fp = std::fopen(path, "r");
    if (!fp) return ODIS_ERR_IO;
    std::vector<char> buf(1 << 16);
    if (!std::fgets(buf.data(), (int)buf.size(), fp)) { std::fclose(fp); return ODIS_ERR_IO; }
    g.N = 0;
    g.node_deg.clear(); g.friends.clear(); g.cent_deg.clear();
    int status = ODIS_OK;
    while (std::fgets(buf.data(), (int)buf.size(), fp)) {
        char* p = buf.data();
        while (*p == ' ' || *p == '\t') p++;
        if (*p == '\n' || *p == '\r' || *p == 0) continue;
        char* q;
        long id = std::strtol(p, &q, 10);
        if (q == p || id < 0 || id > 100000000) { status = ODIS_ERR_IO; break; }
        p = q;
        double lat = std::strtod(p, &p), lon = std::strtod(p, &p);
        if ((int)id >= g.N) {
            g.N = (int)id + 1;
            g.node_deg.resize((size_t)g.N * 2, 0.0);
            g.friends.resize((size_t)g.N * 6, -2);
            g.cent_deg.resize((size_t)g.N * 12, 0.0);
        }
        g.node_deg[id * 2] = lat; g.node_deg[id * 2 + 1] = lon;
        p = std::strchr(p, '{');
        if (!p) { status = ODIS_ERR_IO; break; }
        p++;
        for (int k = 0; k < 6; k++) {
            g.friends[id * 6 + k] = (int)std::strtol(p, &p, 10);
            while (*p == ',' || *p == ' ' || *p == '}') p++;
        }
        for (int k = 0; k < 6; k++) {
            p = std::strchr(p, '(');
            if (!p) { status = ODIS_ERR_IO; break; }
            p++;
            double a = std::strtod(p, &p);
            while (*p == ',' || *p == ' ') p++;
            double b = std::strtod(p, &p);
            g.cent_deg[(id * 6 + k) * 2] = a; g.cent_deg[(id * 6 + k) * 2 + 1] = b;
        }
        if (status != ODIS_OK) break;
    }
    std::fclose(fp);
    if (status != ODIS_OK) return status;
    if (g.N < 12) return ODIS_ERR_IO;
    for (int i = 0; i < g.N * 6; i++)
        if (g.friends[i] < -1 || g.friends[i] >= g.N) return ODIS_ERR_MESH;
    return ODIS_OK;
}

}  // namespace odis
