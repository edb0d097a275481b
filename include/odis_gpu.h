/*
 * odis_gpu.h -- C ABI of libodis_gpu.so, the GB300 (sm_103a) implementation of
 * the GeodesicODIS linear Laplace Tidal Equation timestep.
 *
 * Plain pointers and sizes only.  Every call returns an odis_status; nothing
 * throws across the boundary.  One context per host thread; each context owns
 * one CUDA stream (or uses the one given by odis_set_stream).
 *
 * Reference interfaces replaced (hamishHay/GeodesicODIS v1.11):
 *   odis_update_momentum   <- updateMomentum      include/updateMomentum.h:8,   src/updateMomentum.cpp:16-46
 *   odis_update_eta        <- updateEta           include/updateEta.h:8,        src/updateEta.cpp:7-44
 *   odis_forcing           <- forcing             include/tidalPotentials.h:16, src/tidalPotentials.cpp:29-334
 *   odis_ab3               <- integrateAB3scalar  include/temporalOperators.h:14, src/temporalOperators.cpp:17-68
 *   odis_interpolate_velocity <- interpolateVelocity include/interpolation.h:12, src/interpolation.cpp:26-62
 *   odis_interpolate_cartesian <- interpolateVelocityCartRBF include/interpolation.h:16, src/interpolation.cpp:64-174
 *   odis_update_energy     <- updateEnergy        include/energy.h:10,          src/energy.cpp:13-61
 *   odis_momentum_advection <- calculateMomentumAdvection src/momAdvection.cpp:11-267 (updateMomentum's
 *                             advection branch, src/updateMomentum.cpp:35-39)
 *   odis_lsq_flux          <- interpolateLSQFlux  src/interpolation.cpp:311-356 (updateEta's advection
 *                             branch, src/updateEta.cpp:22-32)
 *   odis_run_steps         <- the body of ab3Explicit's time loop, src/timeIntegrator.cpp:205-313
 *   odis_get_state / odis_set_state <- writeInitialConditions / loadInitialConditions,
 *                                      src/initialConditions.cpp:19,209
 *   odis_analytical_state  <- analyticalInitialConditions + analyticalLTE (OBLIQ_WEST),
 *                             src/initialConditions.cpp:150-211, src/analyticalLTE.cpp:22-181
 *   odis_mesh_*            <- Mesh::Mesh + ReadMeshFile + AssignFaces + Calc*OperatorCoeffs,
 *                             src/mesh.cpp:32-197, :508-1154, :2808-3288, :4016-4089
 *   odis_params_from_input <- Globals::Globals + ReadGlobals + CalcMaxTimeStep,
 *                             src/globals.cpp:35-323,325-477; src/mesh.cpp:1566-1621
 *   odis_h5_*              <- the HDF5 calls of OutFiles::CreateHDF5Framework, DumpGridData
 *                             and DumpData (H5Fcreate, H5Dcreate, H5Dwrite of one row),
 *                             include/outFiles.h:9, src/outFiles.cpp:138-823
 */
#ifndef ODIS_GPU_H
#define ODIS_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int odis_status;
#define ODIS_OK 0
#define ODIS_ERR_ARG 1          /* bad argument or unsupported option */
#define ODIS_ERR_CUDA 2         /* a CUDA runtime call failed */
#define ODIS_ERR_OOB 3          /* index outside the mesh seen by a kernel */
#define ODIS_ERR_NONFINITE 4    /* NaN/Inf appeared in the state */
#define ODIS_ERR_TIMEOUT 5      /* a bounded device wait ran out */
#define ODIS_ERR_IO 6           /* file could not be read/written/parsed */
#define ODIS_ERR_MESH 7         /* inconsistent grid */
#define ODIS_ERR_NOMEM 8        /* allocation failed */

/* forcing types: the values of the reference's enum Potential
 * (include/globals.h:60-76), so that globals->tide_type passes through
 * unchanged.  forcing() (src/tidalPotentials.cpp:29-334) has cases for ECC,
 * OBLIQ, OBLIQ_WEST, FULL, FULL2, PLANET and GENERAL; the other types leave
 * the potential array untouched (a run with one of them is unforced). */
#define ODIS_POT_OBLIQ 0
#define ODIS_POT_OBLIQ_WEST 1
#define ODIS_POT_OBLIQ_EAST 2
#define ODIS_POT_ECC_RAD 3
#define ODIS_POT_ECC_LIB 4
#define ODIS_POT_ECC 5
#define ODIS_POT_ECC_WEST 6
#define ODIS_POT_ECC_EAST 7
#define ODIS_POT_FULL 8
#define ODIS_POT_FULL2 9
#define ODIS_POT_TOTAL 10
#define ODIS_POT_ECC_W3 11
#define ODIS_POT_OBLIQ_W3 12
#define ODIS_POT_PLANET 13
#define ODIS_POT_PLANET_OBL 14
#define ODIS_POT_GENERAL 15
#define ODIS_POT_NONE 16

/* arithmetic of the state and stencils */
#define ODIS_FP64 0             /* everything in FP64 (the reference's method) */
#define ODIS_FP32 1             /* FP32 state and stencils; time accumulation at FP64 accuracy (double-float
                                   residual per unknown), power reductions FP64 across warps */
#define ODIS_DF64 2             /* the FP64 method in double-float (2 x FP32, 48-bit significand) on the
                                   FP32 pipes; meets the FP64 parity bar (1e-10 against the FP64 oracle) */

/* friction type (input.in "friction type"): the dissipation per face is
 * alpha 1000 h |u|^2 (LINEAR) or alpha / h |u|^3 (QUADRATIC) */
#define ODIS_FRIC_LINEAR 0
#define ODIS_FRIC_QUADRATIC 1

/* where the pointers passed to per-operator calls live */
#define ODIS_MEM_HOST 0
#define ODIS_MEM_DEVICE 1

typedef struct odis_mesh odis_mesh;
typedef struct odis_ctx odis_ctx;

/* Physical and numerical parameters, in the units of input.in after the
 * reference's own post-processing (obliquity in radians, angvel after the
 * period has been rounded, dt after snapping).  odis_params_from_input fills
 * one from an input.in file. */
typedef struct odis_params {
    double radius;          /* m */
    double g;               /* m s^-2 */
    double angvel;          /* rad s^-1 */
    double h;               /* ocean thickness, m */
    double alpha;           /* linear drag, s^-1 */
    double ecc;             /* eccentricity */
    double obliq;           /* obliquity, rad */
    double love_reduct;     /* 1 + k2 - h2 */
    double dt;              /* s */
    int potential;          /* ODIS_POT_* */
    int init_load;          /* 1: AB3 from the first step (initial conditions LOAD) */
    int precision;          /* ODIS_FP64 or ODIS_FP32 */
    int sh_lmax;            /* 0: no self-gravity/loading; else maximum degree (<= 64) */
    const double* sh_factors; /* [sh_lmax+1] per-degree factors (0 and 1 unused); may be NULL if sh_lmax == 0 */
    int advection;          /* 1: the nonlinear equations ("advection true"): momentum advection
                               (src/momAdvection.cpp) and the LSQ thickness flux in the continuity
                               equation (src/updateEta.cpp:22-32); ODIS_FP64 or ODIS_DF64, no self-gravity */
    int friction;           /* ODIS_FRIC_LINEAR (0) or ODIS_FRIC_QUADRATIC (1): which dissipation
                               updateEnergy reports (src/energy.cpp:30-53); the momentum equation
                               keeps the linear drag -alpha v in both, as in the reference */
    double semimajor_axis;  /* m, input.in "semimajor axis" (src/globals.cpp:82): the orbit radius a2
                               of the PLANET forcing (src/tidalPotentials.cpp:176-225) */
    int fourier_freq;       /* input.in "fourier freq" (src/globals.cpp:130): the harmonic q_max of
                               the GENERAL forcing (src/tidalPotentials.cpp:227-281) */
} odis_params;

/* Parsed input.in (src/globals.cpp:58-203 keys).  Strings are fixed-size. */
typedef struct odis_input {
    odis_params params;
    double period;           /* s, after rounding */
    double end_time;         /* orbits */
    int steps_per_orbit;     /* totalIter after CalcMaxTimeStep */
    int grid_level;          /* "geodesic grid level" as written in the file */
    int output_time;         /* dumps per orbit */
    int sh_degree;           /* "sh degree" */
    int advection;           /* 1 if advection true (also set in params.advection) */
    int fric_linear;         /* 1 LINEAR, 0 QUADRATIC */
    int surface_free;        /* 1 FREE */
    int init_kind;           /* 0 NONE, 1 LOAD, 2 ANALYTICAL */
    int out_flags;           /* bit0 velocity, 1 cartesian, 2 displacement, 3 dissipation,
                                4 dissipation avg, 5 kinetic avg, 6 dummy1 */
    char potential_name[32];
    char friction_name[32];
    char surface_name[32];
    char solver_name[32];
    char init_name[32];
} odis_input;

/* ---- output file (DATA/data.h5) ---------------------------------------- */
/* An HDF5 file of float32 datasets in the root group, with the structure the
 * HDF5 library gives H5Fcreate/H5Dcreate under default property lists
 * (superblock 0, symbol-table root group, contiguous storage), written without
 * the library.  Dataset k has rank ranks[k] (1 or 2) and extents dims[2k],
 * dims[2k+1] (the second unused for rank 1); names are unique, non-empty and
 * at most 2 x 4 x 2 x 16 = 256 of them.  Storage is allocated and zero-filled at
 * creation (unwritten rows read as the fill value 0).  Host-only: no GPU needed. */
typedef struct odis_h5 odis_h5;
odis_status odis_h5_create(const char* path, int n, const char* const* names, const int* ranks,
                           const long long* dims, odis_h5** out);
/* rows [row0, row0 + nrows) of dataset k; a row is dims[2k+1] values (rank 2)
 * or one value (rank 1).  ODIS_ERR_ARG past the extent. */
odis_status odis_h5_write_rows(odis_h5* h, int k, long long row0, long long nrows, const float* data);
odis_status odis_h5_close(odis_h5* h);

/* ---- grid -------------------------------------------------------------- */
/* Icosahedral grid at level n (10*4^n+2 cells), written in the reference's
 * grid-file format. */
odis_status odis_grid_generate_file(int level, const char* path);

/* ---- mesh (host side geometry, operators and device-ready layout) ------ */
odis_status odis_mesh_from_file(const char* path, double radius, odis_mesh** out);
odis_status odis_mesh_generate(int level, double radius, odis_mesh** out);
/* node_sph [N][2] and cent_sph [N][6][2] in radians, friends [N][6] (-1 in slot 5 for pentagons) */
odis_status odis_mesh_from_arrays(int n_nodes, const double* node_sph, const int* friends,
                                  const double* cent_sph, double radius, odis_mesh** out);
odis_status odis_mesh_sizes(const odis_mesh* m, int* n_cells, int* n_edges, int* n_vertices);
/* Geometry the operators are built from (for checks): which = 0 face_len,
 * 1 face_node_dist, 2 face_area, 3 control-volume area [N], 4 face-centre lat,
 * 5 face-centre lon, 6 map factor at node 0, 7 map factor at node 1,
 * 8/9 face normal (x, y), 10/11 intercept (lat, lon), 12/13 node lat/lon [N]. */
odis_status odis_mesh_field(const odis_mesh* m, int which, double* out);
/* face_nodes [E][2], faces [N][6], node_face_dir [N][6], interp_friends [E][10],
 * interp_w [E][10], interp_n [E]; any may be NULL */
odis_status odis_mesh_topology(const odis_mesh* m, int* face_nodes, int* faces, int* node_face_dir,
                               int* interp_friends, double* interp_w, int* interp_n);
/* Vertex geometry of the nonlinear terms (src/mesh.cpp:436-506, 826-866,
 * 911-1029, 1117-1148), per vertex [V]: which = 0 area of the triangle of its
 * three nodes, 1..3 kite fraction R(v, j) of the vertex in the control volume
 * of its node j, 4 sin(latitude). */
odis_status odis_mesh_vertex_field(const odis_mesh* m, int which, double* out);
/* vert_nodes [V][3], vert_faces [V][3] (ascending), vert_face_dir [V][3],
 * face_verts [E][2] (the two vertices bounding each face); any may be NULL */
odis_status odis_mesh_vertex_topology(const odis_mesh* m, int* vert_nodes, int* vert_faces, int* vert_face_dir,
                                      int* face_verts);
void odis_mesh_destroy(odis_mesh* m);

/* ---- grid generation and mesh build on the GPU ------------------------- */
/* The same steps as odis_grid_generate_file / odis_mesh_from_arrays
 * (ReadMeshFile + AssignFaces + the geometry and TRiSK weights of
 * src/mesh.cpp:436-1154), one kernel per step over nodes, faces, vertices and
 * lattice points of the current device; the result is an ordinary odis_mesh
 * (host arrays).  Numbering, friends, stencils and every other integer array
 * are identical to the host build's; the geometry agrees with it to the last
 * bit of the device's transcendental functions (odis_mesh_compare reports by
 * how much).  Temporary device memory only, freed before return; level 8 needs
 * about 0.5 GB. */
odis_status odis_mesh_generate_device(int level, double radius, odis_mesh** out);
odis_status odis_mesh_from_file_device(const char* path, double radius, odis_mesh** out);
odis_status odis_mesh_from_arrays_device(int n_nodes, const double* node_sph, const int* friends,
                                         const double* cent_sph, double radius, odis_mesh** out);
/* The level-n icosahedral grid as arrays (what odis_grid_generate_file
 * writes): node_deg [N][2], friends [N][6] and cent_deg [N][6][2] in degrees,
 * N = 10*4^n+2, generated on the host (on_device = 0) or the current device. */
odis_status odis_grid_generate_arrays(int level, int on_device, double* node_deg, int* friends, double* cent_deg);
/* out[i] = the double that strtod returns for printf("%.16f", in[i]): the
 * coordinates' round trip through the reference's grid-file text
 * (src/mesh.cpp:4016-4089), which the grid generators apply to every node and
 * circumcentre coordinate they store, computed in exact integer arithmetic
 * (host; in and out may be the same array). */
odis_status odis_text_round16(const double* in, double* out, long long n);
/* Compare two meshes array by array: *int_mismatches counts differing entries
 * of the integer arrays (sizes included), *max_rel is the largest
 * max|a - b| / max|b| over the floating-point arrays (longitudes modulo 2 pi). */
odis_status odis_mesh_compare(const odis_mesh* a, const odis_mesh* b, double* max_rel, long long* int_mismatches);
/* Largest gravity-wave frequency (rad/s) of the discrete operator: sqrt of the
 * largest eigenvalue of -g h D G, by `iters` power iterations (host).  The
 * reference's time loop (AB3 momentum with the old eta, then AB3 continuity
 * with the new velocity, src/timeIntegrator.cpp:213-253) is stable only for
 * omega_max * dt <= 6/11; the reference itself never checks this
 * (src/mesh.cpp:1566-1621 only snaps dt). */
odis_status odis_mesh_gravity_wave_omega(const odis_mesh* m, double g, double h, int iters, double* omega_max);
/* Self-attraction/loading factor gamma_l (l = 0..lmax) of the FREE_LOADING
 * surface (src/boundaryConditions.cpp:29-76, elastic body of rigidity 40 GPa).
 * odis_params.sh_factors[l] = gamma_l reproduces the reference's loading term;
 * a per-degree scaling f_l multiplies it (sh_factors[l] = f_l * gamma_l). */
odis_status odis_loading_factors(double g, double radius, int lmax, double* out);
/* Smallest multiple of 100 steps per orbit with omega_max * dt <= margin * 6/11. */
odis_status odis_stable_steps_per_orbit(double period, double omega_max, double margin, int* steps);

/* ---- parameters -------------------------------------------------------- */
/* Period rounding (src/globals.cpp:209-214) and dt snapping (src/mesh.cpp:1566-1621). */
odis_status odis_derive_time(double angvel_in, double dt_target, double* angvel, double* period,
                             double* dt, int* steps_per_orbit);
odis_status odis_params_from_input(const char* input_in_path, odis_input* out);

/* ---- context ----------------------------------------------------------- */
odis_status odis_create(const odis_params* p, const odis_mesh* m, odis_ctx** out);
void odis_destroy(odis_ctx* c);
/* Use the caller's stream (a cudaStream_t) instead of the context's own. */
odis_status odis_set_stream(odis_ctx* c, void* cuda_stream);
odis_status odis_synchronize(odis_ctx* c);
/* Last status recorded by a kernel's own checks (OOB / NONFINITE / TIMEOUT), 0 if none; clears it. */
odis_status odis_device_status(odis_ctx* c);

/* ---- per-operator calls (mirror the reference's free functions) -------- */
/* dvdt[E] = -g*G*eta + C*v */
odis_status odis_update_momentum(odis_ctx* c, double* dvdt, const double* v, const double* eta, int mem);
/* detadt[N] = h*D*v */
odis_status odis_update_eta(odis_ctx* c, double* detadt, const double* v, int mem);
/* forcing(globals, grid, U, type, t, ecc, obl): U[N] = tidal potential of type
 * `type` (ODIS_POT_*, the reference's Potential values) at time t (s) with
 * eccentricity ecc and obliquity obl (rad).  Types without a case in the
 * reference's switch, and NONE, leave U untouched (ODIS_OK).  GENERAL uses the
 * 4pi-normalised Pbar_20 and Pbar_22 at the nodes; the reference's v1.11 never
 * fills those arrays (CalcLegendreFuncs is commented out), so there its GENERAL
 * potential is zero.  ODIS_ERR_ARG for a type outside 0..16. */
odis_status odis_forcing(odis_ctx* c, double* U, int type, double t, double ecc, double obl, int mem);
/* integrateAB3scalar on s[num] with history hist[num][3] at iteration iter */
odis_status odis_ab3(odis_ctx* c, double* s, double* hist, int iter, int num, int mem);
/* uv[E][2] = (east, north) velocity at faces from normal velocity v[E] */
odis_status odis_interpolate_velocity(odis_ctx* c, double* uv, const double* v, int mem);
/* interpolateVelocityCartRBF (src/interpolation.cpp:64-174; operatorRBFinterp,
 * src/mesh.cpp:355-430 and :2263-2362): Cartesian velocity uxyz [N][3] at the
 * nodes from the face-normal velocities v [E], by the reference's Gaussian
 * radial-basis reconstruction over each node's faces (the "x/y/z velocity"
 * output fields). */
odis_status odis_interpolate_cartesian(odis_ctx* c, double* uxyz, const double* v, int mem);
/* calculateMomentumAdvection (include/momAdvection.h, src/momAdvection.cpp:11-267):
 * dvdt[E] += potential-vorticity flux - G KE for the face velocities v[E] and
 * the column thickness h_total[N] (h + eta).  The PV is (curl v + f) / h at the
 * vertices, with h from the nodes by area x kite-fraction weights (Ringler et
 * al. 2010 eq. 25); the flux is the TRiSK sum with the mean PV (eq. 49); KE is
 * half the squared RBF Cartesian velocity at the nodes.  ekin[N] (nullable)
 * receives KE.  `mesh` is the one the context was created from; the first
 * call builds the vertex operators from it. */
odis_status odis_momentum_advection(odis_ctx* c, const odis_mesh* mesh, double* dvdt, const double* v,
                                    const double* h_total, double* ekin, int mem);
/* interpolateLSQFlux (include/interpolation.h:18, src/interpolation.cpp:311-356),
 * third order (beta = 1): flux[E] of the node scalar h_total[N] across each
 * face with velocity v[E], from the Gaussian-RBF directional second
 * derivatives at the face's two nodes (operatorDirectionalSecondDeriv,
 * src/mesh.cpp:2364-2716, shape parameter 0.25).  The advective continuity
 * equation takes the divergence of this flux.  `mesh` as for
 * odis_momentum_advection. */
odis_status odis_lsq_flux(odis_ctx* c, const odis_mesh* mesh, double* flux, const double* v, const double* h_total,
                          int mem);
/* e[E] (nullable) per-face dissipation and *avg area-mean (W m^-2) from uv[E][2] */
odis_status odis_update_energy(odis_ctx* c, double* avg, double* e, const double* uv, int mem);

/* ---- the fused time loop ----------------------------------------------- */
/* Advance n steps.  power (nullable, ODIS_MEM_HOST or ODIS_MEM_DEVICE per
 * `mem`) receives the dissipated power (W m^-2) after each step. */
odis_status odis_run_steps(odis_ctx* c, int n, double* power, int mem);
/* State in the reference's layout: v[E], eta[N], dvdt[E][3], detadt[N][3]
 * (history slot 0 = latest tendency).  iter = steps taken. Host pointers. */
odis_status odis_get_state(odis_ctx* c, int* iter, double* v, double* eta, double* dvdt, double* detadt);
odis_status odis_set_state(odis_ctx* c, int iter, const double* v, const double* eta,
                           const double* dvdt, const double* detadt);
/* "initial conditions ANALYTICAL": the closed-form westward obliquity-tide
 * solution at time t in the same layout (v at the face centres along the face
 * normals, eta at the nodes, tendencies at t, t - dt, t - 2 dt), for
 * odis_set_state at iter 0.  p->potential must be ODIS_POT_OBLIQ_WEST (the one
 * case the reference's solution has), else ODIS_ERR_ARG.  Outputs are host
 * arrays, each nullable.  Host-only.  Exact for the undamped equations; with
 * drag it is the reference's truncated form. */
odis_status odis_analytical_state(const odis_params* p, const odis_mesh* mesh, double t, double* v, double* eta,
                                  double* dvdt, double* detadt);

/* ---- allocation-free dissipation --------------------------------------- */
/* Same result as odis_update_energy for LINEAR friction (the only dissipation it
 * computes), for callers that cannot allocate device
 * memory (host callbacks or graph host nodes, fixed-budget real-time loops,
 * plugins handed only device buffers): no context, no cudaMalloc/cudaFree.
 * No counterpart in the reference (its updateEnergy, src/energy.cpp:13-61, is
 * the computation, not this calling convention).  All pointers are device
 * pointers: uv [n_faces][2], area [n_faces], e_out [n_faces] (nullable),
 * avg_out [1]; the area-mean dissipation alpha*1000*h*|uv|^2*area/(4 pi r^2)
 * is written to *avg_out on `stream` (a cudaStream_t, NULL = legacy default).
 * The reduction scratch is a fixed 64 KiB __device__ array held by every GPU
 * that loads the library until exit: n_faces above 2,097,152 returns
 * ODIS_ERR_ARG.  The first call on a device sets up that device's scratch
 * address (make it before any stream capture).  Calls share the scratch, so
 * calls that overlap on the GPU race: serialise them.  The cached per-device
 * address goes stale if the process resets the device (cudaDeviceReset): do
 * not call this entry point after a reset. */
odis_status odis_update_energy_noalloc(const double* uv, const double* area, int n_faces, double alpha, double h,
                                       double radius, double* e_out, double* avg_out, void* stream);

/* ---- execution strategy ------------------------------------------------ */
/* FP64 and DF64 runs without self-gravity execute a whole odis_run_steps call
 * as one persistent cooperative launch (one CTA per SM, coefficients and AB3
 * histories resident in shared memory, neighbour-only step synchronisation
 * with bounded waits) when the mesh partition fits; otherwise, and for the
 * other methods, steps are CUDA-graph-replayed pairs of face and cell kernels.
 * Where both are possible, odis_create times each over 192 steps from the
 * zero state on this device, keeps the faster one and restores the zero
 * state.  enable = 0 forces the graph path, 1 the persistent loop (where
 * possible), -1 returns to the choice made at creation.  *active (nullable)
 * reports whether runs will use the persistent loop. */
odis_status odis_set_persistent(odis_ctx* c, int enable, int* active);

/* ---- failure detection ------------------------------------------------- */
/* No reference counterpart (the reference is one single-threaded process).
 * Every wait of the persistent loop on a neighbour CTA's step flag is bounded:
 * after `polls` polls (0: the default, about a second) the CTA records
 * ODIS_ERR_TIMEOUT, leaves the loop, and odis_run_steps returns
 * ODIS_ERR_TIMEOUT; the state of that run is then undefined, the context stays
 * usable (odis_set_state, then run again).  withhold >= 0 makes that CTA of
 * the persistent launch skip its step-flag publications, so the waits on it
 * run out: the test hook that shows the timeout path ends cleanly.  -1 off. */
odis_status odis_set_wait_limit(odis_ctx* c, unsigned polls, int withhold);

/* ---- measurement ------------------------------------------------------- */
/* The FP64 FMA rate this GPU sustains (TFLOP/s, an FMA = 2 flops), measured
 * by a kernel of independent FMA chains on every SM: the FP64 method's second
 * ceiling beside HBM bandwidth.  Takes some tens of milliseconds; no context
 * needed. */
odis_status odis_measure_fp64_rate(double* tflops);
/* Number of this library's kernels launched so far by the context. */
odis_status odis_launch_count(odis_ctx* c, long long* n);
/* Average device time (ms) per launch of each kernel group, each launched
 * `reps` times back to back in a CUDA graph on the context stream:
 * ms[0] face step kernel, ms[1] cell step kernel, ms[2] self-gravity
 * analysis+solve+synthesis (0 if off).  Leaves the state undefined. */
odis_status odis_profile_kernels(odis_ctx* c, int reps, double* ms);
/* Tiles of the self-gravity transforms (0 without self-gravity): the analysis
 * covers tile_l degrees per block with the cells split in `chunks`, and with
 * pre = 1 reads the trig-weighted values of every order formed once per step
 * (else each tile forms them); the synthesis gives each cell `lanes` threads
 * splitting the orders, or with lanes = 16 (32, 48) one warp per pair of
 * orders (m, l_max - m) for 32 x `cells` cells (1, 2, 3 groups of them) per
 * block; each synthesis thread covers `cells` adjacent cells.  lanes = -W is
 * the dense synthesis usg = Z t with Z = Y F (Y^T Y)^-1 precomputed (K rows of
 * the basis's cells, no K x K product per step): W warps per block split the
 * rows, each lane covers `cells` cells.  odis_create times every combination
 * on this device and keeps the fastest; the dense synthesis, whose matrix
 * competes for L2 with the rest of the step, is kept only if whole steps run
 * faster with it.  The environment variable
 * ODIS_SH_TILES="tile_l,chunks,lanes[,cells[,pre]]" names a combination
 * instead.  Any pointer may be NULL.
 * ODIS_FP32 also has tensor-core transforms (tcgen05, fp16 hi/lo operand pairs,
 * FP32 accumulation), retired from the default path because they are slower.
 * They need the full basis, so they are built only with ODIS_SH_TC=1 (which
 * selects them) or on a mesh without antipodal pairs, where odis_create times
 * them against the CUDA-core transforms and keeps the faster (ODIS_SH_TC=0
 * keeps the CUDA cores).  With the tensor-core transforms tile_l = 0, chunks =
 * analysis chunks and lanes = 128-cell tiles per synthesis pass. */
odis_status odis_sh_tiles(const odis_ctx* c, int* tile_l, int* chunks, int* lanes, int* cells, int* pre);

/* Storage of the self-gravity basis (0s without self-gravity).  On a centrally
 * symmetric mesh (every cell has an antipodal partner; the icosahedral grids
 * do) Y_lm(-x) = (-1)^l Y_lm(x), so the basis is stored for one cell of each
 * pair and both transforms run over half the cells: the analysis sums even
 * degrees against eta_a + eta_b and odd degrees against eta_a - eta_b, the
 * synthesis gives the pair E + O and E - O (E, O: the even- and odd-degree
 * sums).  *half = 1 then, *cells = N/2.  ODIS_SH_HALF=0 in the environment at
 * odis_create keeps the full basis.  *basis_bytes = the Legendre and trig rows
 * one transform reads. */
odis_status odis_sh_layout(const odis_ctx* c, int* half, int* cells, long long* basis_bytes);

/* ---- batched sweep ----------------------------------------------------- */
/* Many configurations of the LTE time loop (src/timeIntegrator.cpp:57-322,
 * linear branch) advanced together by one persistent cooperative kernel.  No
 * reference counterpart: it replaces running the reference binary once per
 * configuration.  State FP32 with double-float (FP64-accurate) AB3
 * accumulation; dissipated power summed in FP64 across tiles.  Members share
 * the `common` parameters (radius, g, angvel, potential, love_reduct,
 * init_load; the rest is ignored) and each has its own mesh (an index into
 * `meshes`, which must outlive odis_batch_create only), thickness, drag,
 * eccentricity, obliquity and steps per orbit. */
typedef struct odis_batch odis_batch;
typedef struct odis_batch_member {
    int mesh;                /* index into the meshes array */
    int steps_per_orbit;     /* even; dt = (2 pi / angvel) / steps_per_orbit */
    double h;                /* ocean thickness, m */
    double alpha;            /* linear drag, s^-1 */
    double ecc;              /* eccentricity */
    double obliq;            /* obliquity, radians */
} odis_batch_member;
odis_status odis_batch_create(const odis_params* common, const odis_mesh* const* meshes, int n_meshes,
                              const odis_batch_member* members, int count, odis_batch** out);
void odis_batch_destroy(odis_batch* b);
/* Advances every member by orbits * steps_per_orbit steps (orbits > 0, steps = 0;
 * fractions allowed where that is a whole even number for every member) or by
 * `steps` steps (orbits = 0, steps > 0 and even).  Host outputs, nullable:
 * orbit_power[member * orbit_stride + o] = mean dissipated power (W/m^2 as
 * updateEnergy, src/energy.cpp:13-61) over orbit o of this run;
 * step_power[member * step_stride + k] = power after step k of this run.
 * chunk = steps per cooperative launch (0: 2048).  Returns ODIS_ERR_NONFINITE
 * if a member's state became non-finite, ODIS_ERR_TIMEOUT if a grid barrier
 * wait ran out. */
odis_status odis_batch_run(odis_batch* b, double orbits, int steps, double* orbit_power, int orbit_stride,
                           double* step_power, int step_stride, int chunk);
/* One member's v[E] and eta[N] (FP64 from the double-float master) and its step count. */
odis_status odis_batch_get_member(odis_batch* b, int member, int* iter, double* v, double* eta);
/* Sets one member's v and eta (nullable: zero), clears its AB3 history and
 * restarts its step count at 0 (forcing phase 0, forward-Euler start): the
 * warm-start entry point. */
odis_status odis_batch_set_member(odis_batch* b, int member, const double* v, const double* eta);
/* Layout and launch facts: member groups, padded member slots, CTAs of the
 * cooperative launch, launches so far, and the face/cell rows each thread
 * handles per tile (1, 2 or 4: timed at creation, or ODIS_BATCH_ROWS). */
odis_status odis_batch_info(const odis_batch* b, int* n_groups, int* padded_members, int* grid, long long* launches,
                            int* rows_per_thread);
/* Bulk state access for the members on mesh `mesh`, in increasing member index
 * (v [m][E], eta [m][N]).  set_mesh_members also clears their AB3 histories
 * and restarts their step counts at 0, as odis_batch_set_member. */
odis_status odis_batch_get_mesh_members(odis_batch* b, int mesh, double* v, double* eta);
odis_status odis_batch_set_mesh_members(odis_batch* b, int mesh, const double* v, const double* eta);
/* Projections of the current state of the members on `mesh` onto row bases:
 * out[member * out_stride + k] = sum_e basis_v[k][e] v_e (k < kv), then
 * sum_i basis_eta[k][i] eta_i (kv <= k < kv + ke); FP32 products and slice
 * sums, FP64 across slices.  Members on other meshes are left untouched. */
odis_status odis_batch_project(odis_batch* b, int mesh, const float* basis_v, int kv, const float* basis_eta, int ke,
                               double* out, int out_stride);

/* Runs so far that executed as one CUDA graph launch (every run captures its
 * chunks' cooperative launches in one graph and replays it; a device that
 * refuses the capture gets plain launches). */
odis_status odis_batch_graph_runs(const odis_batch* b, long long* runs);
/* The batch kernel's grid barriers, as odis_set_wait_limit: each wait gives
 * up after `polls` polls (0: the default, about a second) and odis_batch_run
 * returns ODIS_ERR_TIMEOUT; withhold >= 0 makes that CTA never arrive. */
odis_status odis_batch_set_wait_limit(odis_batch* b, unsigned polls, int withhold);

/* ---- warm-start surrogate network -------------------------------------- */
/* No reference counterpart.  MLP n_in -> width (GELU) x depth -> n_mix * n_out,
 * output y = sum_k mix[k] * R_k (n_mix = 0: y = R).  FP32 master weights,
 * BF16 operands with FP32 accumulation in every GEMM (tensor cores), FP32
 * bias/GELU/loss/Adam.  Loss = sum_i w_i ||y_i - t_i||^2 / n (w nullable: 1).
 * Host arrays, row-major: x [n][n_in], mix [n][n_mix], t/y [n][n_out], w [n].
 * Parameters flat: for each layer W [out][in] then b [out]. */
typedef struct odis_mlp odis_mlp;
odis_status odis_mlp_create(int n_in, int width, int depth, int n_out, int n_mix, unsigned long long seed,
                            odis_mlp** out);
void odis_mlp_destroy(odis_mlp* m);
odis_status odis_mlp_num_params(const odis_mlp* m, long long* n);
odis_status odis_mlp_get_params(odis_mlp* m, float* out);
/* also resets the Adam state */
odis_status odis_mlp_set_params(odis_mlp* m, const float* in);
odis_status odis_mlp_predict(odis_mlp* m, const float* x, const float* mix, int n, float* y);
/* one forward + backward pass over n rows: loss and the gradient (flat, FP32) */
odis_status odis_mlp_gradient(odis_mlp* m, const float* x, const float* mix, const float* t, const float* w, int n,
                              double* loss, float* grad);
/* Adam (0.9, 0.999, 1e-8), shuffled minibatches (whole batches only), cosine
 * learning-rate decay from lr; loss_per_epoch (nullable) = mean minibatch loss. */
odis_status odis_mlp_train(odis_mlp* m, const float* x, const float* mix, const float* t, const float* w, int n,
                           int epochs, int batch, float lr, unsigned long long seed, double* loss_per_epoch);

#ifdef __cplusplus
}
#endif
#endif /* ODIS_GPU_H */
