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
// Generation: odis_grid_gen.cuh (steps shared with the device generator),
// here as OpenMP loops.  Nodes are numbered in order of first appearance in a
// depth-first walk of the triangle hierarchy, so cells that are close on the
// sphere are close in memory (which keeps the 10-edge TRiSK gathers inside L2
// sectors).
#include "odis_internal.h"
#include "odis_grid_gen.cuh"

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

void fmt_deg(double v, char* buf) { std::snprintf(buf, 64, "%.16f", v); }

}  // namespace

int generate_grid(int level, GridArrays& g)
{
    HostExec x;
    return generate_grid_steps(x, level, g);
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
