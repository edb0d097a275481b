// Internal declarations shared by the host (C++) and device (CUDA) parts of
// libodis_gpu.so.  Nothing here crosses the C ABI.
#pragma once

#include "../../include/odis_gpu.h"

#include <cstdint>
#include <vector>

namespace odis {

// Grid in the reference's file layout, angles in degrees.
struct GridArrays {
    int N = 0;
    std::vector<double> node_deg;   // [N][2]
    std::vector<int> friends;       // [N][6]
    std::vector<double> cent_deg;   // [N][6][2]
};

int generate_grid(int level, GridArrays& g);
int write_grid(const GridArrays& g, const char* path);
int read_grid(const char* path, GridArrays& g);

// Host-side geometry and operator data, numbered exactly as the reference
// numbers cells (file order) and faces (AssignFaces loop order).
struct Mesh {
    int N = 0, E = 0, V = 0;
    double r = 0.0;
    std::vector<double> node_sph;      // [N][2] rad
    std::vector<int> friends;          // [N][6]
    std::vector<double> cent_sph;      // [N][6][2] rad
    std::vector<double> cv_area;       // [N]
    std::vector<int> vertexes;         // [N][6]
    std::vector<double> vert_sph;      // [V][2]
    std::vector<int> faces;            // [N][6]
    std::vector<int> node_face_dir;    // [N][6]
    std::vector<int> face_nodes;       // [E][2]
    std::vector<double> face_len, face_dist, face_area;  // [E]
    std::vector<double> face_centre;   // [E][2]
    std::vector<double> face_m;        // [E][2]
    std::vector<double> face_normal;   // [E][2]
    std::vector<double> face_int;      // [E][2]
    std::vector<double> face_nxyz;     // [E][3] unit normal of the great circle through the face's vertices
    std::vector<int> interp_friends;   // [E][10]
    std::vector<double> interp_w;      // [E][10]
    std::vector<int> interp_n;         // [E]
    // vertex geometry of the nonlinear terms (src/mesh.cpp:436-506, 826-866, 911-1029, 1117-1148)
    std::vector<int> vert_nodes;       // [V][3] the creating node and its two friends
    std::vector<int> face_verts;       // [E][2] the face's two vertices (centroids j-1, j of its first node)
    std::vector<double> vert_R;        // [V][3] kite fraction of the vertex in the control volume of vert_nodes
    std::vector<int> vert_faces;       // [V][3] ascending face ids
    std::vector<int> vert_face_dir;    // [V][3] +1 / -1: circulation sign of the face normal about the vertex
    std::vector<double> vert_area;     // [V] spherical area of the triangle of the vertex's nodes
    int nfriends(int i) const { return friends[i * 6 + 5] < 0 ? 5 : 6; }
};

int build_mesh(int N, const double* node_sph, const int* friends, const double* cent_sph,
               double radius, Mesh& m);
// The same grid and mesh computed by kernels on the current device
// (odis_mesh_dev.cu): integers identical to the host's, geometry to the last
// bit of CUDA's transcendental functions.
int generate_grid_device(int level, GridArrays& g);
int build_mesh_device(int N, const double* node_sph, const int* friends, const double* cent_sph,
                      double radius, Mesh& m);

// Forcing as a single-frequency pair: U_i(t) = cos(M) Ua_i + sin(M) Ub_i with
// M = angvel * t, for the ECC / OBLIQ / OBLIQ_WEST / FULL potentials; zero for
// the other valid types (unforced, or evaluated at the nodes every step).
int forcing_basis(const Mesh& m, const odis_params& p, std::vector<double>& Ua, std::vector<double>& Ub);

// RBF reconstruction of Cartesian velocity at the nodes from the face-normal
// velocities: rbf[(i * 3 + c) * 6 + j] multiplies v at faces(i, j).
void build_rbf(const Mesh& m, std::vector<double>& rbf);

// operatorDirectionalSecondDeriv (src/mesh.cpp:2364-2716) as rows of 7 (node,
// coefficient) pairs, ascending node order, padded with zero coefficients:
// row 2e is the inner node's second derivative normal to face e, 2e+1 the
// outer node's.  eps is the Gaussian RBF shape parameter ("rbf epsilon").
int build_lsq_rows(const Mesh& m, double eps, std::vector<int>& col, std::vector<double>& val);
constexpr double kRbfEps = 0.25;     // the reference's default "rbf epsilon" (src/globals.cpp:570)

// sqrt(largest eigenvalue of -g h D G), power iteration
double gravity_wave_omega(const Mesh& m, double g, double h, int iters);

// Parse input.in (src/globals.cpp:325-477 semantics).
int parse_input(const char* path, odis_input& out);

}  // namespace odis

struct odis_mesh {
    odis::Mesh m;
};
