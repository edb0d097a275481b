/*
 * odis_oracle.c -- FP64 CPU oracle for the GeodesicODIS linear Laplace Tidal
 * Equation (LTE) timestep on the icosahedral-geodesic finite-volume mesh.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: it is linked by the
 * test-suite, by __graft_entry__.smoke() and by bench.py's cpu_baseline /
 * reference arm, never by the product library (libodis_gpu.so).
 *
 * It restates, formula by formula and in the reference's own evaluation
 * order, the live path of GeodesicODIS v1.11 (hamishHay/GeodesicODIS):
 *
 *   mesh reading ............ src/mesh.cpp:4016-4089 (ReadMeshFile)
 *   map coordinates ......... src/mesh.cpp:1384-1486 (CalcMappingCoords)
 *   CV area (map coords) .... src/mesh.cpp:1828-1866 (CalcControlVolumeArea)
 *   vertices ................ src/mesh.cpp:436-506   (CalcControlVolumeVertexR)
 *   faces + TRiSK weights ... src/mesh.cpp:508-1154  (AssignFaces)
 *   trig tables ............. src/mesh.cpp:2122-2152 (CalcTrigFunctions)
 *   dt snapping ............. src/mesh.cpp:1566-1621 (CalcMaxTimeStep)
 *   period rounding ......... src/globals.cpp:209-214
 *   gradient operator ....... src/mesh.cpp:3005-3120 (CalcGradOperatorCoeffs)
 *   divergence operator ..... src/mesh.cpp:3177-3288 (CalcDivOperatorCoeffs)
 *   Coriolis operator ....... src/mesh.cpp:2808-2901 (CalcCoriolisOperatorCoeffs)
 *   linear drag ............. src/mesh.cpp:2903-3003 (CalcLinearDragOperatorCoeffs)
 *   geometry helpers ........ include/mathRoutines.h:29-439
 *   forcing ................. src/tidalPotentials.cpp:29-334 (every live case)
 *   updateMomentum .......... src/updateMomentum.cpp:16-46 (linear branch :42)
 *   updateEta ............... src/updateEta.cpp:7-44 (linear branch :39)
 *   integrateAB3scalar ...... src/temporalOperators.cpp:17-68
 *   interpolateVelocity ..... src/interpolation.cpp:26-62
 *   updateEnergy ............ src/energy.cpp:13-61 (LINEAR and QUADRATIC branches)
 *   time loop ............... src/timeIntegrator.cpp:205-272 (ab3Explicit)
 *
 * Sparse operators are held as CSR with each row sorted by ascending column,
 * which is the layout Eigen's setFromTriplets()/makeCompressed() produces for
 * the reference's row-major SpMat; SpMV sums each row left to right from 0,
 * as Eigen's row-major sparse*dense kernel does.
 *
 * Self-gravity / loading (spherical harmonics) follows the commented-out
 * pressureGradientSH (src/spatialOperators.cpp:387-462) and
 * CalcLegendreFuncs (src/mesh.cpp:2154-2258): 4pi-normalised associated
 * Legendre functions with the Condon-Shortley phase (SHTOOLS PlmBar,
 * csphase=-1, as called at src/legendre.f95:20) and an ordinary least-squares
 * analysis (SHTOOLS SHExpandLSQ, src/extractSHCoeffGG.f95:17).  SHTOOLS is not
 * vendored by the reference and that code is dead in v1.11, so this part is
 * "parity unpinned" by the reference; it is pinned by exact analysis/
 * synthesis round trips in the tests.
 *
 * Built with -ffp-contract=off so that results do not depend on whether the
 * host compiler fuses multiply-adds (x86_64 and aarch64 give the same bits).
 * OpenMP parallelises only loops without cross-iteration reductions (rows of
 * an SpMV, cells, SH coefficients), so the results are bit-identical for any
 * thread count; OMP_NUM_THREADS=1 is the reference's own single-threaded build.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.1415926535897932384626433832795028841971693993751058
#define ORC_RADCONV (ORC_PI / 180.0)

void orc_plmbar(int L, double z, double *P);

/* forcing types: the values of the reference's enum Potential
 * (include/globals.h:60-76), which ab3Explicit passes to forcing() as
 * globals->tide_type.  Types without a case in forcing()'s switch
 * (OBLIQ_EAST, ECC_RAD, ECC_LIB, ECC_WEST, ECC_EAST, TOTAL, ECC_W3, OBLIQ_W3,
 * PLANET_OBL) leave the potential array as it was, like NONE. */
enum { ORC_OBLIQ = 0, ORC_OBLIQ_WEST = 1, ORC_OBLIQ_EAST = 2, ORC_ECC_RAD = 3, ORC_ECC_LIB = 4,
       ORC_ECC = 5, ORC_ECC_WEST = 6, ORC_ECC_EAST = 7, ORC_FULL = 8, ORC_FULL2 = 9, ORC_TOTAL = 10,
       ORC_ECC_W3 = 11, ORC_OBLIQ_W3 = 12, ORC_PLANET = 13, ORC_PLANET_OBL = 14, ORC_GENERAL = 15,
       ORC_NONE = 16 };

/* ------------------------------------------------------------------------ */
/* mathRoutines.h restatements (include/mathRoutines.h:29-439)               */
/* ------------------------------------------------------------------------ */
static void map_factor(double *m, double lat1, double lat2, double lon1, double lon2)
{   /* mapFactorAtPoint, include/mathRoutines.h:29-33 */
    *m = 2.0 / (1.0 + sin(lat1) * sin(lat2) + cos(lat1) * cos(lat2) * cos(lon2 - lon1));
}

static void map_at_point(double *m, double *x, double *y, double lat1, double lat2,
                         double lon1, double lon2, double r)
{   /* mapAtPoint, include/mathRoutines.h:61-68 */
    map_factor(m, lat1, lat2, lon1, lon2);
    *x = *m * r * (cos(lat2) * sin(lon2 - lon1));
    *y = *m * r * (sin(lat2) * cos(lat1) - cos(lat2) * sin(lat1) * cos(lon2 - lon1));
}

static double dist_sph(double lat1, double lat2, double lon1, double lon2, double r)
{   /* distanceBetweenSph, include/mathRoutines.h:134-138 */
    return r * acos(sin(lat1) * sin(lat2) + cos(lat1) * cos(lat2) * cos(lon2 - lon1));
}

static void sph2cart(double *x, double *y, double *z, double r, double colat, double lon)
{   /* include/mathRoutines.h:19-25 */
    *x = r * sin(colat) * cos(lon);
    *y = r * sin(colat) * sin(lon);
    *z = r * cos(colat);
}

static double dist_sph2(const double s1[2], const double s2[2])
{   /* distanceBetweenSph2, include/mathRoutines.h:143-163 */
    double a[3], b[3];
    sph2cart(&a[0], &a[1], &a[2], 1.0, ORC_PI * 0.5 - s1[0], s1[1]);
    sph2cart(&b[0], &b[1], &b[2], 1.0, ORC_PI * 0.5 - s2[0], s2[1]);
    double c = pow(a[1] * b[2] - a[2] * b[1], 2.0);
    c += pow(-(a[0] * b[2] - a[2] * b[0]), 2.0);
    c += pow(a[0] * b[1] - a[1] * b[0], 2.0);
    c = sqrt(c);
    double d = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
    return atan2(c, d);
}

static void midpoint_sph(const double s1[2], const double s2[2], double sc[2])
{   /* midpointBetweenSph, include/mathRoutines.h:172-192 */
    double p1[3], p2[3], pc[3];
    p1[0] = cos(s1[0]) * cos(s1[1]); p1[1] = cos(s1[0]) * sin(s1[1]); p1[2] = sin(s1[0]);
    p2[0] = cos(s2[0]) * cos(s2[1]); p2[1] = cos(s2[0]) * sin(s2[1]); p2[2] = sin(s2[0]);
    for (int k = 0; k < 3; k++) pc[k] = 0.5 * (p1[k] + p2[k]);
    sc[0] = atan2(pc[2], sqrt(pow(pc[0], 2.0) + pow(pc[1], 2.0)));
    sc[1] = atan2(pc[1], pc[0]);
}

static void normal_map(double n[2], const double s1[2], const double s2[2])
{   /* normalVectorBetweenMap, include/mathRoutines.h:214-248 */
    double mid[2], c1[2], c2[2], m;
    midpoint_sph(s1, s2, mid);
    double latc = mid[0], lonc = mid[1];
    double lat1 = s1[0], lon1 = s1[1];
    map_factor(&m, latc, lat1, lonc, lon1);
    c1[0] = m * 1.0 * (cos(lat1) * sin(lon1 - lonc));
    c1[1] = m * 1.0 * (sin(lat1) * cos(latc) - cos(lat1) * sin(latc) * cos(lon1 - lonc));
    lat1 = s2[0]; lon1 = s2[1];
    map_factor(&m, latc, lat1, lonc, lon1);
    c2[0] = m * 1.0 * (cos(lat1) * sin(lon1 - lonc));
    c2[1] = m * 1.0 * (sin(lat1) * cos(latc) - cos(lat1) * sin(latc) * cos(lon1 - lonc));
    double xx = c2[0] - c1[0], yy = c2[1] - c1[1];
    double mag = sqrt(xx * xx + yy * yy);
    xx /= mag; yy /= mag;
    n[0] = -yy;
    n[1] = xx;
}

static void intersect_sph(const double s1[2], const double s2[2], const double s3[2],
                          const double s4[2], double si[2])
{   /* intersectPointSph, include/mathRoutines.h:320-383 */
    double c1[3], c2[3], c3[3], c4[3], n1[3], n2[3], mp[3];
    c1[0] = cos(s1[0]) * cos(s1[1]); c2[0] = cos(s2[0]) * cos(s2[1]);
    c3[0] = cos(s3[0]) * cos(s3[1]); c4[0] = cos(s4[0]) * cos(s4[1]);
    c1[1] = cos(s1[0]) * sin(s1[1]); c2[1] = cos(s2[0]) * sin(s2[1]);
    c3[1] = cos(s3[0]) * sin(s3[1]); c4[1] = cos(s4[0]) * sin(s4[1]);
    c1[2] = sin(s1[0]); c2[2] = sin(s2[0]); c3[2] = sin(s3[0]); c4[2] = sin(s4[0]);
    n1[0] = c1[1] * c2[2] - c1[2] * c2[1];
    n1[1] = -(c1[0] * c2[2] - c1[2] * c2[0]);
    n1[2] = c1[0] * c2[1] - c1[1] * c2[0];
    n2[0] = c3[1] * c4[2] - c3[2] * c4[1];
    n2[1] = -(c3[0] * c4[2] - c3[2] * c4[0]);
    n2[2] = c3[0] * c4[1] - c3[1] * c4[0];
    double m1 = sqrt(n1[0] * n1[0] + n1[1] * n1[1] + n1[2] * n1[2]);
    double m2 = sqrt(n2[0] * n2[0] + n2[1] * n2[1] + n2[2] * n2[2]);
    for (int k = 0; k < 3; k++) { n1[k] /= m1; n2[k] /= m2; }
    mp[0] = n1[1] * n2[2] - n2[1] * n1[2];
    mp[1] = n2[0] * n1[2] - n1[0] * n2[2];
    mp[2] = n1[0] * n2[1] - n2[0] * n1[1];
    m1 = sqrt(mp[0] * mp[0] + mp[1] * mp[1] + mp[2] * mp[2]);
    for (int k = 0; k < 3; k++) mp[k] /= m1;
    si[0] = asin(mp[2] / 1.0);
    si[1] = atan2(mp[1], mp[0]);
    if (si[1] < 0.0) si[1] += 2 * ORC_PI;
}

static double angle_map(const double s1[2], const double s2[2], const double sc[2])
{   /* angleBetweenMap, include/mathRoutines.h:385-410 (final form: ang1-ang2) */
    double m, x1, y1, x2, y2;
    map_at_point(&m, &x1, &y1, sc[0], s1[0], sc[1], s1[1], 1.0);
    map_at_point(&m, &x2, &y2, sc[0], s2[0], sc[1], s2[1], 1.0);
    double a1 = atan2(y1 - 0.0, x1 - 0.0);
    double a2 = atan2(y2 - 0.0, x2 - 0.0);
    double a = a1 - a2;
    if (a > ORC_PI) a -= 2 * ORC_PI;
    else if (a < -ORC_PI) a += 2 * ORC_PI;
    return a;
}

static double tri_area_map(double xc, double yc, double x1, double x2, double y1, double y2)
{   /* triangularArea, include/mathRoutines.h:415-420 */
    return 0.5 * fabs(xc * (y1 - y2) + x1 * (y2 - yc) + x2 * (yc - y1));
}

static double tri_area_sph(double lat1, double lat2, double lat3,
                           double lon1, double lon2, double lon3, double r)
{   /* triangularAreaSph, include/mathRoutines.h:422-439 */
    double c = fabs(acos(sin(lat1) * sin(lat2) + cos(lat1) * cos(lat2) * cos(fabs(lon2 - lon1))));
    double a = fabs(acos(sin(lat2) * sin(lat3) + cos(lat2) * cos(lat3) * cos(fabs(lon3 - lon2))));
    double b = fabs(acos(sin(lat3) * sin(lat1) + cos(lat3) * cos(lat1) * cos(fabs(lon1 - lon3))));
    double A = fabs(acos((cos(a) - cos(b) * cos(c)) / (sin(b) * sin(c))));
    double B = fabs(acos((cos(b) - cos(a) * cos(c)) / (sin(a) * sin(c))));
    double C = fabs(acos((cos(c) - cos(b) * cos(a)) / (sin(b) * sin(a))));
    return pow(r, 2.0) * fabs((A + B + C) - ORC_PI);
}

/* ------------------------------------------------------------------------ */
/* CSR                                                                       */
/* ------------------------------------------------------------------------ */
typedef struct { int rows, cols, nnz; int *rowptr; int *col; double *val; } orc_csr;

static void csr_free(orc_csr *m) { free(m->rowptr); free(m->col); free(m->val); memset(m, 0, sizeof(*m)); }

/* Sort each row's (col,val) pairs by ascending column and merge duplicates:
 * the compressed layout of Eigen::SparseMatrix<double,RowMajor>::setFromTriplets. */
static void csr_finalise_rows(orc_csr *m)
{
    int out = 0;
    int *newptr = (int *)malloc(sizeof(int) * (m->rows + 1));
    for (int i = 0; i < m->rows; i++) {
        int b = m->rowptr[i], e = m->rowptr[i + 1];
        for (int p = b + 1; p < e; p++) {          /* insertion sort, rows are short */
            int c = m->col[p]; double v = m->val[p]; int q = p - 1;
            while (q >= b && m->col[q] > c) { m->col[q + 1] = m->col[q]; m->val[q + 1] = m->val[q]; q--; }
            m->col[q + 1] = c; m->val[q + 1] = v;
        }
        newptr[i] = out;
        for (int p = b; p < e; p++) {
            if (out > newptr[i] && m->col[out - 1] == m->col[p]) m->val[out - 1] += m->val[p];
            else { m->col[out] = m->col[p]; m->val[out] = m->val[p]; out++; }
        }
    }
    newptr[m->rows] = out;
    free(m->rowptr); m->rowptr = newptr; m->nnz = out;
}

/* y = alpha * (A x), row sums left to right from zero (Eigen row-major SpMV) */
static void csr_spmv(const orc_csr *A, const double *x, double alpha, double *y)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < A->rows; i++) {
        double t = 0.0;
        for (int p = A->rowptr[i]; p < A->rowptr[i + 1]; p++) t += A->val[p] * x[A->col[p]];
        y[i] = 0.0 + alpha * t;
    }
}

/* ------------------------------------------------------------------------ */
/* mesh                                                                      */
/* ------------------------------------------------------------------------ */
typedef struct {
    int N, E, V;
    double r;
    double *node_sph;     /* [N][2] lat, lon (rad) */
    int *friends;         /* [N][6], -1 in slot 5 for pentagons */
    double *cent_sph;     /* [N][6][2] */
    double *cent_map;     /* [N][6][2] map coords about the node */
    double *cv_area;      /* [N]  control_volume_surf_area_map */
    int *vertexes;        /* [N][6] */
    double *vert_sph;     /* [V][2] */
    int *vert_nodes;      /* [V][3] */
    int *faces;           /* [N][6] */
    int *node_face_dir;   /* [N][6] */
    int *face_nodes;      /* [E][2] */
    double *face_len, *face_dist, *face_area;   /* [E] */
    double *face_centre;  /* [E][2] */
    double *face_m;       /* [E][2] */
    double *face_normal;  /* [E][2] */
    double *face_int;     /* [E][2] */
    double *face_nxyz;    /* [E][3] Cartesian face normal */
    int *interp_friends;  /* [E][10] */
    double *interp_w;     /* [E][10] */
    int *interp_n;        /* [E] number of valid entries (10, 9 or 8) */
    double *trig;         /* [N][10]: cosLat sinLat cosLon sinLon cos2Lat sin2Lat cos2Lon sin2Lon cosSqLat sinSqLat */
    double *pbar2;        /* [N][2]: 4pi-normalised Pbar_20, Pbar_22 (GENERAL forcing) */
    int *face_verts;      /* [E][2] face_vertexes */
    double *vert_R;       /* [V][3] kite fraction of vertex v in the control volume of vert_nodes(v, j) */
    int *vert_faces;      /* [V][3] */
    int *vert_face_dir;   /* [V][3] */
    double *vert_area;    /* [V] */
    orc_csr Curl;         /* V x E, operatorCurl */
    orc_csr D2;           /* 2E x N, operatorDirectionalSecondDeriv (built on first use) */
    orc_csr G, D, C0;     /* gradient (E x N), divergence (N x E), Coriolis without Omega factor is not kept: C0 = Coriolis with Omega=1 */
} orc_mesh;

static int nfriends(const orc_mesh *M, int i) { return M->friends[i * 6 + 5] < 0 ? 5 : 6; }

void orc_mesh_free(orc_mesh *M)
{
    if (!M) return;
    free(M->node_sph); free(M->friends); free(M->cent_sph); free(M->cent_map); free(M->cv_area);
    free(M->vertexes); free(M->vert_sph); free(M->vert_nodes); free(M->faces); free(M->node_face_dir);
    free(M->face_nodes); free(M->face_len); free(M->face_dist); free(M->face_area); free(M->face_centre);
    free(M->face_m); free(M->face_normal); free(M->face_int); free(M->face_nxyz); free(M->interp_friends); free(M->interp_w);
    free(M->interp_n); free(M->trig); free(M->pbar2);
    free(M->face_verts); free(M->vert_R); free(M->vert_faces); free(M->vert_face_dir); free(M->vert_area);
    csr_free(&M->G); csr_free(&M->D); csr_free(&M->C0); csr_free(&M->Curl); csr_free(&M->D2);
    free(M);
}

/* CalcControlVolumeVertexR, src/mesh.cpp:436-506 */
static int build_vertices(orc_mesh *M)
{
    int N = M->N;
    M->vertexes = (int *)malloc(sizeof(int) * N * 6);
    int Vmax = 2 * N;                    /* (6(N-12)+60)/3 = 2N-4 */
    M->vert_sph = (double *)calloc((size_t)Vmax * 2, sizeof(double));
    M->vert_nodes = (int *)calloc((size_t)Vmax * 3, sizeof(int));
    for (int i = 0; i < N * 6; i++) M->vertexes[i] = -1;
    int vc = 0;
    for (int i = 0; i < N; i++) {
        int fn = nfriends(M, i);
        for (int j = 0; j < fn; j++) {
            if (M->vertexes[i * 6 + j] >= 0) continue;
            if (vc >= Vmax) return -1;
            M->vertexes[i * 6 + j] = vc;
            double vlat = M->cent_sph[(i * 6 + j) * 2], vlon = M->cent_sph[(i * 6 + j) * 2 + 1];
            M->vert_sph[vc * 2] = vlat; M->vert_sph[vc * 2 + 1] = vlon;
            int f1 = M->friends[i * 6 + (j % fn)];
            int f2 = M->friends[i * 6 + ((j + 1) % fn)];
            M->vert_nodes[vc * 3] = i; M->vert_nodes[vc * 3 + 1] = f1; M->vert_nodes[vc * 3 + 2] = f2;
            int ff[2] = {f1, f2};
            for (int q = 0; q < 2; q++) {
                int f = ff[q], nf = nfriends(M, f);
                for (int k = 0; k < nf; k++) {
                    double a = M->cent_sph[(f * 6 + k) * 2], b = M->cent_sph[(f * 6 + k) * 2 + 1];
                    if (a < vlat + 1e-9 && a > vlat - 1e-9 && b < vlon + 1e-9 && b > vlon - 1e-9)
                        M->vertexes[f * 6 + k] = vc;
                }
            }
            vc++;
        }
    }
    M->V = vc;
    return 0;
}

typedef struct { int id; double angle; } orc_ang;
static int cmp_desc(const void *a, const void *b)
{
    double x = ((const orc_ang *)a)->angle, y = ((const orc_ang *)b)->angle;
    return (x > y) ? -1 : (x < y) ? 1 : 0;
}

/* AssignFaces, src/mesh.cpp:508-1154 (face ids, geometry, TRiSK weights) */
static int assign_faces(orc_mesh *M)
{
    int N = M->N, E = 3 * N - 6;
    double r = M->r;
    M->E = E;
    M->faces = (int *)malloc(sizeof(int) * N * 6);
    M->node_face_dir = (int *)calloc((size_t)N * 6, sizeof(int));
    M->face_nodes = (int *)calloc((size_t)E * 2, sizeof(int));
    M->face_len = (double *)calloc(E, sizeof(double));
    M->face_dist = (double *)calloc(E, sizeof(double));
    M->face_area = (double *)calloc(E, sizeof(double));
    M->face_centre = (double *)calloc((size_t)E * 2, sizeof(double));
    M->face_m = (double *)calloc((size_t)E * 2, sizeof(double));
    M->face_normal = (double *)calloc((size_t)E * 2, sizeof(double));
    M->face_nxyz = (double *)calloc((size_t)E * 3, sizeof(double));
    M->face_int = (double *)calloc((size_t)E * 2, sizeof(double));
    M->interp_friends = (int *)calloc((size_t)E * 10, sizeof(int));
    M->interp_w = (double *)calloc((size_t)E * 10, sizeof(double));
    M->interp_n = (int *)calloc(E, sizeof(int));
    M->face_verts = (int *)calloc((size_t)E * 2, sizeof(int));
    M->vert_R = (double *)calloc((size_t)M->V * 3, sizeof(double));
    for (int i = 0; i < N * 6; i++) M->faces[i] = -1;

    int fc = 0;
    for (int i = 0; i < N; i++) {
        int fn = nfriends(M, i);
        for (int j = 0; j < fn; j++) {
            if (M->faces[i * 6 + j] >= 0) continue;
            if (fc >= E) return -1;
            M->faces[i * 6 + j] = fc;
            M->face_nodes[fc * 2] = i;
            M->node_face_dir[i * 6 + j] = 1;
            int f = M->friends[i * 6 + j];
            double s1[2], s2[2], sc[2], s3[2], s4[2];
            for (int k = 0; k < 2; k++) {
                s1[k] = M->cent_sph[(i * 6 + (j + fn - 1) % fn) * 2 + k];
                s2[k] = M->cent_sph[(i * 6 + j % fn) * 2 + k];
            }
            M->face_len[fc] = fabs(dist_sph(s1[0], s2[0], s1[1], s2[1], r));     /* :551-561 */
            midpoint_sph(s1, s2, sc);                                              /* :564-570 */
            if (sc[1] < 0.0) sc[1] += 2 * ORC_PI;
            M->face_centre[fc * 2] = sc[0]; M->face_centre[fc * 2 + 1] = sc[1];
            double m, x, y;
            map_at_point(&m, &x, &y, sc[0], M->node_sph[i * 2], sc[1], M->node_sph[i * 2 + 1], r);
            M->face_m[fc * 2] = m;                                                 /* :600-613 */
            map_at_point(&m, &x, &y, sc[0], M->node_sph[f * 2], sc[1], M->node_sph[f * 2 + 1], r);
            M->face_m[fc * 2 + 1] = m;
            double n1[2] = {M->node_sph[i * 2], M->node_sph[i * 2 + 1]};
            double n2[2] = {M->node_sph[f * 2], M->node_sph[f * 2 + 1]};
            M->face_dist[fc] = dist_sph2(n1, n2) * r;                              /* :617-624 */
            double nv[2];
            normal_map(nv, s1, s2);                                                /* :632-637 */
            M->face_normal[fc * 2] = nv[0]; M->face_normal[fc * 2 + 1] = nv[1];
            {   /* normalVectorBetweenXYZ, include/mathRoutines.h:246-267; src/mesh.cpp:640-644 */
                double a[3], b[3];
                sph2cart(&a[0], &a[1], &a[2], 1.0, ORC_PI * 0.5 - s1[0], s1[1]);
                sph2cart(&b[0], &b[1], &b[2], 1.0, ORC_PI * 0.5 - s2[0], s2[1]);
                double nx = a[1] * b[2] - a[2] * b[1], ny = -(a[0] * b[2] - a[2] * b[0]), nz = a[0] * b[1] - a[1] * b[0];
                double mag = sqrt(nx * nx + ny * ny + nz * nz);
                M->face_nxyz[fc * 3] = nx / mag; M->face_nxyz[fc * 3 + 1] = ny / mag; M->face_nxyz[fc * 3 + 2] = nz / mag;
            }
            for (int k = 0; k < 2; k++) { s3[k] = M->node_sph[i * 2 + k]; s4[k] = M->node_sph[f * 2 + k]; }
            intersect_sph(s1, s2, s3, s4, sc);                                     /* :660-670 */
            M->face_int[fc * 2] = sc[0]; M->face_int[fc * 2 + 1] = sc[1];
            int fn2 = nfriends(M, f), found = 0;
            for (int j2 = 0; j2 < fn2; j2++) {
                if (M->friends[f * 6 + j2] == i) {
                    M->faces[f * 6 + j2] = fc;
                    M->face_nodes[fc * 2 + 1] = f;
                    M->node_face_dir[f * 6 + j2] = -1;
                    found = 1;
                }
            }
            if (!found) return -2;        /* inconsistent friend lists */
            fc++;
        }
    }
    if (fc != E) return -3;

    /* TRiSK weights, src/mesh.cpp:680-907 */
    orc_ang fl[6], vl[6];
    double R[6];
    for (int i = 0; i < E; i++) {
        int jadd = 0;
        for (int k = 0; k < 2; k++) {
            int nd = M->face_nodes[i * 2 + k];
            int fn = nfriends(M, nd);
            const double *sn = &M->node_sph[nd * 2];
            for (int j = 0; j < fn; j++) {
                int id = M->faces[nd * 6 + j];
                fl[j].id = id;
                double a = angle_map(&M->face_int[i * 2], &M->face_int[id * 2], sn) * 180. / ORC_PI;
                if (a > 0.0 + 1e-8) a -= 360.0;
                fl[j].angle = a;
            }
            for (int j = 0; j < fn; j++) {
                int vid = M->vertexes[nd * 6 + j];
                vl[j].id = vid;
                double a = angle_map(&M->face_int[i * 2], &M->vert_sph[vid * 2], sn) * 180. / ORC_PI;
                if (a > 0.0 + 1e-8) a -= 360.0;
                vl[j].angle = a;
            }
            qsort(fl, fn, sizeof(orc_ang), cmp_desc);
            qsort(vl, fn, sizeof(orc_ang), cmp_desc);
            double area_cv = 0.0;
            for (int j = 0; j < fn; j++) {
                const double *v1 = &M->vert_sph[vl[j].id * 2];
                const double *v2 = &M->vert_sph[vl[(j + 1) % fn].id * 2];
                area_cv += tri_area_sph(sn[0], v1[0], v2[0], sn[1], v1[1], v2[1], r);
            }
            for (int j = 0; j < fn; j++) {
                const double *v1 = &M->vert_sph[vl[j].id * 2];
                const double *p1 = &M->face_int[fl[j].id * 2];
                const double *p2 = &M->face_int[fl[(j + 1) % fn].id * 2];
                double a1 = tri_area_sph(sn[0], v1[0], p1[0], sn[1], v1[1], p1[1], r);
                double a2 = tri_area_sph(sn[0], v1[0], p2[0], sn[1], v1[1], p2[1], r);
                R[j] = (a1 + a2) / area_cv;
                /* face_vertexes of the face ranked 1, src/mesh.cpp:826-829 (the last face to rank it wins) */
                if (j == 1) { M->face_verts[fl[1].id * 2] = vl[1].id; M->face_verts[fl[1].id * 2 + 1] = vl[0].id; }
                /* vertex_R(v, slot of this node), src/mesh.cpp:857-866 */
                for (int c = 0; c < 3; c++)
                    if (M->vert_nodes[vl[j].id * 3 + c] == nd) { M->vert_R[vl[j].id * 3 + c] = R[j]; break; }
            }
            for (int j = 0; j < fn; j++) {
                if (fl[j].id == i) continue;
                if (jadd >= 10) return -4;
                M->interp_friends[i * 10 + jadd] = fl[j].id;
                double w = 0.0;
                for (int j2 = 0; j2 < j; j2++) w += R[j2];
                w -= 0.5;
                for (int j2 = 0; j2 < fn; j2++)
                    if (fl[j].id == M->faces[nd * 6 + j2]) w *= M->node_face_dir[nd * 6 + j2];
                int tev = (M->face_nodes[i * 2] == nd) ? 1 : -1;
                w *= tev;
                M->interp_w[i * 10 + jadd] = w;
                jadd++;
            }
        }
        M->interp_n[i] = jadd;
        M->face_area[i] = M->face_dist[i] * M->face_len[i];                        /* :1093 */
    }
    return 0;
}

/* vertex_faces, vertex_face_dir and vertex areas (src/mesh.cpp:911-1029,
 * 1117-1148); operatorCurl (src/mesh.cpp:3122-3175) */
static int build_vertex_geometry(orc_mesh *M)
{
    int V = M->V, E = M->E;
    double r = M->r;
    M->vert_faces = (int *)malloc(sizeof(int) * V * 3);
    M->vert_face_dir = (int *)calloc((size_t)V * 3, sizeof(int));
    M->vert_area = (double *)calloc(V, sizeof(double));
    for (int i = 0; i < V * 3; i++) M->vert_faces[i] = -1;
    for (int i = 0; i < E; i++) {
        for (int s = 0; s < 2; s++) {
            int v = M->face_verts[i * 2 + s];
            for (int j = 0; j < 3; j++) {
                if (M->vert_faces[v * 3 + j] >= 0) continue;
                M->vert_faces[v * 3 + j] = i;
                double m, xv, yv;
                map_at_point(&m, &xv, &yv, M->face_centre[i * 2], M->vert_sph[v * 2], M->face_centre[i * 2 + 1],
                             M->vert_sph[v * 2 + 1], r);
                double cross = xv * M->face_normal[i * 2 + 1] - yv * M->face_normal[i * 2];
                M->vert_face_dir[v * 3 + j] = cross > 0 ? 1 : -1;
                break;
            }
        }
    }
    for (int i = 0; i < V; i++) {
        double area = 0.0;
        const double *sv = &M->vert_sph[i * 2];
        for (int j = 0; j < 3; j++) {
            const double *s1 = &M->node_sph[M->vert_nodes[i * 3 + j] * 2];
            const double *s2 = &M->node_sph[M->vert_nodes[i * 3 + (j + 1) % 3] * 2];
            area += fabs(tri_area_sph(sv[0], s1[0], s2[0], sv[1], s1[1], s2[1], r));
        }
        M->vert_area[i] = area;
    }
    orc_csr *C = &M->Curl;
    C->rows = V; C->cols = E;
    C->rowptr = (int *)malloc(sizeof(int) * (V + 1));
    C->col = (int *)malloc(sizeof(int) * 3 * V);
    C->val = (double *)malloc(sizeof(double) * 3 * V);
    for (int i = 0; i < V; i++) {
        C->rowptr[i] = 3 * i;
        for (int j = 0; j < 3; j++) {
            int f = M->vert_faces[i * 3 + j];
            if (f < 0) return -5;
            C->col[3 * i + j] = f;
            C->val[3 * i + j] = M->face_dist[f] * M->vert_face_dir[i * 3 + j] / M->vert_area[i];
        }
    }
    C->rowptr[V] = 3 * V;
    csr_finalise_rows(C);
    return 0;
}

static void build_operators(orc_mesh *M)
{
    int N = M->N, E = M->E;
    /* gradient, src/mesh.cpp:3005-3120 */
    orc_csr *G = &M->G;
    G->rows = E; G->cols = N;
    G->rowptr = (int *)malloc(sizeof(int) * (E + 1));
    G->col = (int *)malloc(sizeof(int) * 2 * E);
    G->val = (double *)malloc(sizeof(double) * 2 * E);
    for (int i = 0; i < E; i++) {
        double d = M->face_dist[i];
        G->rowptr[i] = 2 * i;
        G->col[2 * i] = M->face_nodes[i * 2];     G->val[2 * i] = (-M->face_m[i * 2]) / d;
        G->col[2 * i + 1] = M->face_nodes[i * 2 + 1]; G->val[2 * i + 1] = (M->face_m[i * 2 + 1]) / d;
    }
    G->rowptr[E] = 2 * E;
    csr_finalise_rows(G);
    /* divergence, src/mesh.cpp:3177-3288 */
    orc_csr *D = &M->D;
    D->rows = N; D->cols = E;
    D->rowptr = (int *)malloc(sizeof(int) * (N + 1));
    D->col = (int *)malloc(sizeof(int) * 6 * N);
    D->val = (double *)malloc(sizeof(double) * 6 * N);
    int c = 0;
    for (int i = 0; i < N; i++) {
        D->rowptr[i] = c;
        int fn = nfriends(M, i);
        for (int j = 0; j < fn; j++) {
            int fid = M->faces[i * 6 + j];
            int dir = M->node_face_dir[i * 6 + j];
            D->col[c] = fid;
            D->val[c] = -dir * M->face_len[fid] / M->cv_area[i];
            c++;
        }
    }
    D->rowptr[N] = c;
    csr_finalise_rows(D);
}

/* Coriolis operator for a given rotation rate, src/mesh.cpp:2808-2901 */
static void build_coriolis(const orc_mesh *M, double omega, orc_csr *C)
{
    int E = M->E;
    C->rows = E; C->cols = E;
    C->rowptr = (int *)malloc(sizeof(int) * (E + 1));
    C->col = (int *)malloc(sizeof(int) * 10 * E);
    C->val = (double *)malloc(sizeof(double) * 10 * E);
    int c = 0;
    for (int i = 0; i < E; i++) {
        C->rowptr[i] = c;
        int fn = 10;
        if (M->friends[M->face_nodes[i * 2] * 6 + 5] < 0) fn--;
        if (M->friends[M->face_nodes[i * 2 + 1] * 6 + 5] < 0) fn--;
        for (int j = 0; j < fn; j++) {
            int fid = M->interp_friends[i * 10 + j];
            C->col[c] = fid;
            C->val[c] = -2.0 * omega * sin(M->face_centre[i * 2]) * M->interp_w[i * 10 + j] *
                        M->face_len[fid] / M->face_dist[i];
            c++;
        }
    }
    C->rowptr[E] = c;
    csr_finalise_rows(C);
}

/* Build a mesh from node positions, friend lists and centroid lists in the
 * reference grid-file layout (angles in radians). */
orc_mesh *orc_mesh_from_arrays(int N, const double *node_sph, const int *friends,
                               const double *cent_sph, double radius, int *status)
{
    orc_mesh *M = (orc_mesh *)calloc(1, sizeof(orc_mesh));
    M->N = N; M->r = radius;
    M->node_sph = (double *)malloc(sizeof(double) * N * 2);
    M->friends = (int *)malloc(sizeof(int) * N * 6);
    M->cent_sph = (double *)malloc(sizeof(double) * N * 12);
    memcpy(M->node_sph, node_sph, sizeof(double) * N * 2);
    memcpy(M->friends, friends, sizeof(int) * N * 6);
    memcpy(M->cent_sph, cent_sph, sizeof(double) * N * 12);
    double r = radius;
    /* CalcMappingCoords (centroid part), src/mesh.cpp:1453-1482 */
    M->cent_map = (double *)calloc((size_t)N * 12, sizeof(double));
    M->cv_area = (double *)calloc(N, sizeof(double));
    M->trig = (double *)calloc((size_t)N * 10, sizeof(double));
    M->pbar2 = (double *)calloc((size_t)N * 2, sizeof(double));
    for (int i = 0; i < N; i++) {
        double lat1 = M->node_sph[i * 2], lon1 = M->node_sph[i * 2 + 1];
        for (int j = 0; j < 6; j++) {
            double *xy = &M->cent_map[(i * 6 + j) * 2];
            if (M->friends[i * 6 + j] == -1) { xy[0] = -1.0; xy[1] = -1.0; continue; }
            double m;
            map_at_point(&m, &xy[0], &xy[1], lat1, M->cent_sph[(i * 6 + j) * 2], lon1,
                         M->cent_sph[(i * 6 + j) * 2 + 1], r);
        }
        /* node-centred map coords of the node itself: mapAtPoint(lat1,lat1,lon1,lon1) */
        double m0, xc, yc;
        map_at_point(&m0, &xc, &yc, lat1, lat1, lon1, lon1, r);
        /* CalcControlVolumeArea, src/mesh.cpp:1828-1866 */
        int fn = nfriends(M, i);
        double area = 0.0;
        for (int j = 0; j < fn; j++) {
            const double *p1 = &M->cent_map[(i * 6 + j) * 2];
            const double *p2 = &M->cent_map[(i * 6 + (j + 1) % fn) * 2];
            area += tri_area_map(xc, yc, p1[0], p2[0], p1[1], p2[1]);
        }
        M->cv_area[i] = area;
        /* CalcTrigFunctions, src/mesh.cpp:2122-2152 */
        double *t = &M->trig[i * 10];
        t[0] = cos(lat1); t[1] = sin(lat1); t[2] = cos(lon1); t[3] = sin(lon1);
        t[4] = cos(2.0 * lat1); t[5] = sin(2.0 * lat1); t[6] = cos(2.0 * lon1); t[7] = sin(2.0 * lon1);
        t[8] = pow(cos(lat1), 2.0); t[9] = pow(sin(lat1), 2.0);
        {   /* Pbar_20, Pbar_22 at the node (src/mesh.cpp:2193-2194, dead in v1.11) */
            double P[6];
            orc_plmbar(2, cos(ORC_PI * 0.5 - lat1), P);
            M->pbar2[i * 2] = P[3];
            M->pbar2[i * 2 + 1] = P[5];
        }
    }
    int st = build_vertices(M);
    if (st == 0) st = assign_faces(M);
    if (st == 0) st = build_vertex_geometry(M);
    if (st != 0) { if (status) *status = st; orc_mesh_free(M); return NULL; }
    build_operators(M);
    build_coriolis(M, 1.0, &M->C0);
    if (status) *status = 0;
    return M;
}

/* ReadMeshFile, src/mesh.cpp:4016-4089: same columns, degrees * (pi/180) */
orc_mesh *orc_mesh_load(const char *path, double radius, int *status)
{
    FILE *fp = fopen(path, "r");
    if (!fp) { if (status) *status = -10; return NULL; }
    int cap = 1024, N = 0;
    double *ns = (double *)malloc(sizeof(double) * cap * 2);
    int *fr = (int *)malloc(sizeof(int) * cap * 6);
    double *cs = (double *)malloc(sizeof(double) * cap * 12);
    char *line = NULL; size_t ln = 0;
    if (getline(&line, &ln, fp) < 0) { fclose(fp); if (status) *status = -11; return NULL; }
    while (getline(&line, &ln, fp) > 0) {
        char *p = line;
        while (*p == ' ' || *p == '\t') p++;
        if (*p == '\n' || *p == 0) continue;
        int id = (int)strtol(p, &p, 10);
        double lat = strtod(p, &p), lon = strtod(p, &p);
        if (id < 0) { N = -1; break; }
        while (id >= cap) {
            cap *= 2;
            ns = (double *)realloc(ns, sizeof(double) * cap * 2);
            fr = (int *)realloc(fr, sizeof(int) * cap * 6);
            cs = (double *)realloc(cs, sizeof(double) * cap * 12);
        }
        if (id + 1 > N) N = id + 1;
        ns[id * 2] = lat * ORC_RADCONV; ns[id * 2 + 1] = lon * ORC_RADCONV;
        p = strchr(p, '{'); if (!p) { N = -1; break; } p++;
        for (int k = 0; k < 6; k++) { fr[id * 6 + k] = (int)strtol(p, &p, 10); while (*p == ',' || *p == ' ' || *p == '}') p++; }
        for (int k = 0; k < 6; k++) {
            p = strchr(p, '('); if (!p) { N = -1; break; } p++;
            double a = strtod(p, &p); while (*p == ',' || *p == ' ') p++;
            double b = strtod(p, &p);
            cs[(id * 6 + k) * 2] = a * ORC_RADCONV; cs[(id * 6 + k) * 2 + 1] = b * ORC_RADCONV;
        }
        if (N < 0) break;
    }
    free(line); fclose(fp);
    if (N <= 0) { free(ns); free(fr); free(cs); if (status) *status = -12; return NULL; }
    orc_mesh *M = orc_mesh_from_arrays(N, ns, fr, cs, radius, status);
    free(ns); free(fr); free(cs);
    return M;
}

/* ------------------------------------------------------------------------ */
/* accessors for the tests                                                   */
/* ------------------------------------------------------------------------ */
void orc_mesh_sizes(const orc_mesh *M, int *N, int *E, int *V) { *N = M->N; *E = M->E; *V = M->V; }

/* which: 0 face_len, 1 face_dist, 2 face_area, 3 cv_area(N), 4 face_centre lat,
 *        5 face_centre lon, 6 face_m0, 7 face_m1, 8 normal x, 9 normal y,
 *        10 intercept lat, 11 intercept lon */
int orc_mesh_get_field(const orc_mesh *M, int which, double *out)
{
    int E = M->E;
    switch (which) {
    case 0: memcpy(out, M->face_len, sizeof(double) * E); return E;
    case 1: memcpy(out, M->face_dist, sizeof(double) * E); return E;
    case 2: memcpy(out, M->face_area, sizeof(double) * E); return E;
    case 3: memcpy(out, M->cv_area, sizeof(double) * M->N); return M->N;
    case 12: case 13:
        for (int i = 0; i < M->N; i++) out[i] = M->node_sph[i * 2 + (which - 12)];
        return M->N;
    default: break;
    }
    const double *src = NULL; int off = 0;
    switch (which) {
    case 4: src = M->face_centre; off = 0; break;
    case 5: src = M->face_centre; off = 1; break;
    case 6: src = M->face_m; off = 0; break;
    case 7: src = M->face_m; off = 1; break;
    case 8: src = M->face_normal; off = 0; break;
    case 9: src = M->face_normal; off = 1; break;
    case 10: src = M->face_int; off = 0; break;
    case 11: src = M->face_int; off = 1; break;
    default: return -1;
    }
    for (int i = 0; i < E; i++) out[i] = src[i * 2 + off];
    return E;
}

void orc_mesh_get_topology(const orc_mesh *M, int *face_nodes, int *faces, int *node_face_dir,
                           int *interp_friends, double *interp_w, int *interp_n)
{
    if (face_nodes) memcpy(face_nodes, M->face_nodes, sizeof(int) * M->E * 2);
    if (faces) memcpy(faces, M->faces, sizeof(int) * M->N * 6);
    if (node_face_dir) memcpy(node_face_dir, M->node_face_dir, sizeof(int) * M->N * 6);
    if (interp_friends) memcpy(interp_friends, M->interp_friends, sizeof(int) * M->E * 10);
    if (interp_w) memcpy(interp_w, M->interp_w, sizeof(double) * M->E * 10);
    if (interp_n) memcpy(interp_n, M->interp_n, sizeof(int) * M->E);
}

/* op: 0 gradient (E x N), 1 divergence (N x E), 2 Coriolis with Omega=1 (E x E).
 * Returns nnz; with NULL arrays only nnz is returned. */
int orc_mesh_get_csr(const orc_mesh *M, int op, int *rowptr, int *col, double *val)
{
    const orc_csr *A = op == 0 ? &M->G : op == 1 ? &M->D : &M->C0;
    if (rowptr) memcpy(rowptr, A->rowptr, sizeof(int) * (A->rows + 1));
    if (col) memcpy(col, A->col, sizeof(int) * A->nnz);
    if (val) memcpy(val, A->val, sizeof(double) * A->nnz);
    return A->nnz;
}

/* ------------------------------------------------------------------------ */
/* parameters                                                                */
/* ------------------------------------------------------------------------ */
/* Globals constructor, src/globals.cpp:209-214 (period rounded to an even
 * number of seconds) and CalcMaxTimeStep, src/mesh.cpp:1566-1621. */
void orc_derive_time(double angvel_in, double dt_target, double *angvel, double *period,
                     double *dt, int *steps_per_orbit)
{
    double P = 2. * ORC_PI / angvel_in;
    int it = (int)round(P / 2) * 2;
    *period = (double)it;
    *angvel = 2 * ORC_PI / (double)it;
    double d = *period;
    int n = 100;
    while (d > dt_target) { d = *period / n; n += 100; }
    n -= 100;
    *dt = d;
    *steps_per_orbit = n;
}

typedef struct {
    double radius, g, angvel, h, alpha, ecc, obliq, love_reduct, dt;
    int potential;        /* ORC_* (the reference's Potential values) */
    int init_load;
    int advection;        /* 1: the nonlinear branch (momentum advection, LSQ thickness flux) */
    int friction;         /* 0 LINEAR, 1 QUADRATIC (src/globals.cpp:232-234) */
    double semimajor_axis;   /* "semimajor axis" (src/globals.cpp:82), m: PLANET's a2 */
    int fourier_freq;        /* "fourier freq" (src/globals.cpp:130): GENERAL's q_max */
} orc_params;

/* ------------------------------------------------------------------------ */
/* per-operator restatements                                                 */
/* ------------------------------------------------------------------------ */
typedef struct {
    orc_mesh *M;
    orc_params p;
    orc_csr C;            /* Coriolis operator at the run's rotation rate */
    /* optional self-gravity / loading */
    int sh_lmax;          /* 0: off */
    double *sh_R;         /* [K][K] Cholesky factor (lower) of the Gram matrix Y^T Y, K=(L+1)^2 */
    double *sh_Y;         /* [K][N] basis rows Y_k(node) */
    double *sh_f;         /* [L+1] per-degree factor */
} orc_solver;

orc_solver *orc_solver_create(orc_mesh *M, const orc_params *p)
{
    orc_solver *S = (orc_solver *)calloc(1, sizeof(orc_solver));
    S->M = M; S->p = *p;
    build_coriolis(M, p->angvel, &S->C);
    return S;
}

void orc_solver_free(orc_solver *S)
{
    if (!S) return;
    csr_free(&S->C);
    free(S->sh_R); free(S->sh_Y); free(S->sh_f);
    free(S);
}

/* updateMomentum, linear branch: dvdt = -g*G*eta + C*v (src/updateMomentum.cpp:42) */
void orc_update_momentum(const orc_solver *S, double *dvdt, const double *v, const double *eta)
{
    const orc_mesh *M = S->M;
    int E = M->E;
    double *tmp = (double *)malloc(sizeof(double) * E);
    csr_spmv(&M->G, eta, -S->p.g * (1 - 0.5 * 0.0), dvdt);
    csr_spmv(&S->C, v, 1.0, tmp);
    for (int i = 0; i < E; i++) dvdt[i] = dvdt[i] + tmp[i];
    free(tmp);
}

/* updateEta, linear branch: detadt = h*D*v (src/updateEta.cpp:39) */
void orc_update_eta(const orc_solver *S, double *detadt, const double *v)
{
    csr_spmv(&S->M->D, v, S->p.h, detadt);
}

/* forcing, src/tidalPotentials.cpp:29-334: the potential of type `type` at time
 * t with the caller's eccentricity and obliquity, as forcing(consts, grid,
 * potential, type, time, ecc, obl).  Types without a case leave U untouched.
 * GENERAL reads Pbar_20 and Pbar_22 at the nodes (src/tidalPotentials.cpp:238-
 * 239); v1.11 never fills those arrays (their filler, CalcLegendreFuncs, is
 * commented out at src/mesh.cpp:2154-2258, so they stay zero and the live
 * reference's GENERAL potential is zero).  Here they hold the 4pi-normalised
 * P20 and P22 that the dead code would assign (src/mesh.cpp:2193-2194). */
void orc_forcing(const orc_solver *S, double *U, int type, double t, double ecc, double obl)
{
    const orc_mesh *M = S->M;
    double radius = S->p.radius, omega = S->p.angvel;
    double lr = S->p.love_reduct;
    if (type != ORC_ECC && type != ORC_OBLIQ && type != ORC_OBLIQ_WEST && type != ORC_FULL2 &&
        type != ORC_FULL && type != ORC_PLANET && type != ORC_GENERAL)
        return;                                                   /* no case, or NONE */
    double cosM = cos(omega * t), sinM = sin(omega * t);
    double cos2M = cos(2 * omega * t);
    double cos3M = cos(3 * omega * t), cos4M = cos(4 * omega * t);
    /* PLANET (:176-225): Io-like perturber m2 at a1, this body at a2 = semimajor axis */
    double pl_factor = 0.0, pl_p = 0.0, pl_cosphi = 0.0, pl_sinphi = 0.0;
    if (type == ORC_PLANET) {
        double m2 = 8.931938e+22, a1 = 421800000.0, a2 = S->p.semimajor_axis;
        double n2 = omega, n1 = n2 * 2.0, nij = n1 - n2;
        double cosnt = cos(nij * t), sinnt = sin(nij * t);
        pl_p = pow(a1, 2.0) + pow(a2, 2.0) - 2. * a1 * a2 * cosnt;
        pl_cosphi = (a1 - a2 * cosnt);
        pl_sinphi = a2 * sinnt;
        pl_factor = 0.5 * 6.67408e-11 * m2 * pow(radius / pl_p, 2.0) / sqrt(pl_p);
    }
    /* GENERAL (:227-281) */
    double ge_cos = 0.0, ge_sin = 0.0;
    const double a20 = -9.991062592506567e-05 * 2.0, a22 = 0.0012049514054640862 * 2.0,
                 b22 = -0.0012017622891820471 * 2.0;
    if (type == ORC_GENERAL) {
        double n2 = omega, n1 = n2 * 2.0, nij = n1 - n2;
        ge_cos = cos((double)S->p.fourier_freq * nij * t);
        ge_sin = sin((double)S->p.fourier_freq * nij * t);
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < M->N; i++) {
        const double *tr = &M->trig[i * 10];
        double cosLat = tr[0], sinLat = tr[1], cosLon = tr[2], sinLon = tr[3];
        double cos2Lat = tr[4], sin2Lat = tr[5], cos2Lon = tr[6], sin2Lon = tr[7];
        double cosSqLat = tr[8], sinSqLat = tr[9];
        double factor, factor2;
        switch (type) {
        case ORC_ECC:                                                 /* :82-101 */
            factor = 0.75 * lr * pow(omega, 2.0) * pow(radius, 2.0) * ecc;
            U[i] = factor * ((1. - 3. * sinSqLat) * cosM + cosSqLat * (3. * cosM * cos2Lon + 4. * sinM * sin2Lon));
            break;
        case ORC_OBLIQ:                                               /* :104-116 */
            factor = -3. / 2. * lr * pow(omega, 2.0) * pow(radius, 2.0) * obl;
            U[i] = factor * cosM * sin2Lat * cosLon;
            break;
        case ORC_OBLIQ_WEST:                                          /* :118-131 */
            factor = 0.5 * lr * pow(omega, 2.0) * pow(radius, 2.0) * obl;
            U[i] = 3 * factor * sinLat * cosLat * (cosLon * cosM - sinLon * sinM);
            break;
        case ORC_FULL:                                                /* :158-174 */
            factor = 0.75 * lr * pow(omega, 2.0) * pow(radius, 2.0) * ecc;
            factor2 = -3. / 2. * lr * pow(omega, 2.0) * pow(radius, 2.0) * obl;
            U[i] = factor * ((1 - 3 * sinSqLat) * cosM + cosSqLat * (3 * cosM * cos2Lon + 4 * sinM * sin2Lon))
                   + factor2 * cosM * sin2Lat * cosLon;
            break;
        case ORC_FULL2: {                                             /* :133-156 */
            factor = 1 / 32. * lr * pow(omega, 2.0) * pow(radius, 2.0);
            double T1, T2, T3;
            T1 = 3. * ecc * (4. - 7. * obl * obl) * cosM + 6 * (obl * obl + ecc * ecc * (3 - 7 * obl * obl)) * cos2M;
            T1 += 3 * ecc * obl * obl * (7 * cos3M + 17 * ecc * cos4M);
            T1 *= -(1 - 3 * cos2Lat);
            T2 = (4 + 15 * ecc * ecc + 20 * ecc * cosM + 43 * ecc * ecc * cos2M) * cosLon;
            T2 += 2 * ecc * (4 + 25 * ecc * cosM) * sinM * sinLon;
            T2 *= 24 * obl * cosLat * sinLat * sinM;
            T3 = obl * obl * (2 + 3 * ecc * ecc + 6 * ecc * cosM + 9 * ecc * ecc * cos2M) * (cosM * cosLon + sinM * sinLon);
            T3 += -(obl * obl - 2) * ((6 * ecc * cosM + 17 * ecc * ecc * cos2M) * cos2Lon + 2 * ecc * (4 + 17 * ecc * cosM) * sinM * sin2Lon);
            T3 *= 6 * cosSqLat;
            U[i] = factor * (T1 + T2 + T3);
            break; }
        case ORC_PLANET: {                                            /* :176-225 */
            double cosgam = cosLat * (cosLon * pl_cosphi + sinLon * pl_sinphi);
            U[i] = pl_factor * (3. * pow(cosgam, 2.0) - pl_p);
            break; }
        case ORC_GENERAL: {                                           /* :227-281 */
            double U20 = 0.0, U22a = 0.0, U22b = 0.0;
            U20 += (a20 * ge_cos);
            U22a += (a22 * ge_cos);
            U22b += (b22 * ge_sin);
            U20 = (U20) * M->pbar2[i * 2];
            U22a = (U22a) * M->pbar2[i * 2 + 1] * cos2Lon;
            U22b = (U22b) * M->pbar2[i * 2 + 1] * sin2Lon;
            U[i] = (U20 + U22a + U22b);
            break; }
        }
    }
}

/* integrateAB3scalar, src/temporalOperators.cpp:17-68; hist is [num][3] */
void orc_ab3(double dt, double *s, double *hist, int iter, int num, int init_load)
{
    double a = 23. / 12., b = -16. / 12., c = 5. / 12.;
    if (iter > 1 || init_load) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < num; ++i) {
            s[i] += (a * hist[i * 3] + b * hist[i * 3 + 1] + c * hist[i * 3 + 2]) * dt;
            hist[i * 3 + 2] = hist[i * 3 + 1];
            hist[i * 3 + 1] = hist[i * 3];
        }
    } else if (iter == 0) {
        for (int i = 0; i < num; i++) { s[i] += hist[i * 3] * dt; hist[i * 3 + 2] = hist[i * 3]; }
    } else if (iter == 1) {
        for (int i = 0; i < num; i++) { s[i] += hist[i * 3] * dt; hist[i * 3 + 1] = hist[i * 3]; }
    }
}

/* interpolateVelocity, src/interpolation.cpp:26-62; uv is [E][2] */
void orc_interpolate_velocity(const orc_mesh *M, double *uv, const double *vn)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < M->E; ++i) {
        double vt = 0.0;
        int fn = 10;
        if (M->friends[M->face_nodes[i * 2] * 6 + 5] < 0) fn--;
        if (M->friends[M->face_nodes[i * 2 + 1] * 6 + 5] < 0) fn--;
        for (int j = 0; j < fn; j++) {
            int f = M->interp_friends[i * 10 + j];
            vt += vn[f] * M->interp_w[i * 10 + j] * M->face_len[f];
        }
        vt /= M->face_dist[i];
        double nx = M->face_normal[i * 2], ny = M->face_normal[i * 2 + 1];
        double ty = -nx, tx = ny;
        uv[i * 2] = nx * vn[i] + tx * vt;
        uv[i * 2 + 1] = ny * vn[i] + ty * vt;
    }
}

/* interpolateVelocityCartRBF, src/interpolation.cpp:64-174, with the operator
 * of src/mesh.cpp:355-430 and :2263-2362: per node i with faces j,
 * A[j1][j2] = phi(arc(f_j1, f_j2)) n_j1 . n_j2, w[j] = phi(arc(i, f_j)),
 * phi(d) = exp(-d^2) (1 below 1e-8, include/mathRoutines.h:431-439),
 * u_c(i) = sum_j1 w[j1] n_j1,c (A^-1 v_faces)[j1].  The k x k systems are solved
 * by Gaussian elimination with partial pivoting. */
static double orc_rbf(double d) { return d < 1e-8 ? 1.0 : exp(-pow(d, 2.0)); }

void orc_interpolate_cartesian(const orc_mesh *M, double *uxyz, const double *vn)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < M->N; i++) {
        int k = nfriends(M, i);
        double a[6][7], x[6];
        double sn[2] = {M->node_sph[i * 2], M->node_sph[i * 2 + 1]};
        double w[6];
        for (int j1 = 0; j1 < k; j1++) {
            int f1 = M->faces[i * 6 + j1];
            double s1[2] = {M->face_centre[f1 * 2], M->face_centre[f1 * 2 + 1]};
            for (int j2 = 0; j2 < k; j2++) {
                int f2 = M->faces[i * 6 + j2];
                double s2[2] = {M->face_centre[f2 * 2], M->face_centre[f2 * 2 + 1]};
                double dot = M->face_nxyz[f1 * 3] * M->face_nxyz[f2 * 3] + M->face_nxyz[f1 * 3 + 1] * M->face_nxyz[f2 * 3 + 1] +
                             M->face_nxyz[f1 * 3 + 2] * M->face_nxyz[f2 * 3 + 2];
                a[j1][j2] = orc_rbf(dist_sph2(s1, s2)) * dot;
            }
            a[j1][k] = vn[f1];
            w[j1] = orc_rbf(dist_sph2(sn, s1));
        }
        /* solve A x = v_faces */
        for (int c = 0; c < k; c++) {
            int piv = c;
            for (int r = c + 1; r < k; r++) if (fabs(a[r][c]) > fabs(a[piv][c])) piv = r;
            if (piv != c) for (int q = 0; q <= k; q++) { double t = a[c][q]; a[c][q] = a[piv][q]; a[piv][q] = t; }
            for (int r = c + 1; r < k; r++) {
                double f = a[r][c] / a[c][c];
                for (int q = c; q <= k; q++) a[r][q] -= f * a[c][q];
            }
        }
        for (int r = k - 1; r >= 0; r--) {
            double t = a[r][k];
            for (int q = r + 1; q < k; q++) t -= a[r][q] * x[q];
            x[r] = t / a[r][r];
        }
        for (int c = 0; c < 3; c++) {
            double u = 0.0;
            for (int j = 0; j < k; j++) u += w[j] * M->face_nxyz[M->faces[i * 6 + j] * 3 + c] * x[j];
            uxyz[i * 3 + c] = u;
        }
    }
}

/* calculateMomentumAdvection, src/momAdvection.cpp:11-267: dvdt += PV flux - G KE.
 * PV at vertices from the curl and the thickness interpolated with the kite
 * fractions (Ringler et al. 2010 eq. 25), averaged to faces, TRiSK flux of the
 * thickness flux h_e v_e with the mean PV (eq. 49); the kinetic energy from
 * the RBF Cartesian velocity at the nodes.  ekin [N] receives the kinetic energy. */
void orc_momentum_advection(const orc_mesh *M, double omega, double *dvdt, const double *vel, const double *h_total,
                            double *ekin)
{
    int V = M->V, E = M->E, N = M->N;
    double *qv = (double *)malloc(sizeof(double) * V);
    double *qe = (double *)malloc(sizeof(double) * E);
    double *he = (double *)malloc(sizeof(double) * E);
    double *uxyz = (double *)malloc(sizeof(double) * N * 3);
    double *gk = (double *)malloc(sizeof(double) * E);
    csr_spmv(&M->Curl, vel, 1.0, qv);                                         /* step 1 */
    for (int i = 0; i < V; i++) {                                              /* steps 2-3 */
        double f = -2 * omega * sin(M->vert_sph[i * 2]);
        double thickness = 0.0;
        for (int j = 0; j < 3; j++) {
            int n = M->vert_nodes[i * 3 + j];
            thickness += h_total[n] * M->cv_area[n] * M->vert_R[i * 3 + j];
        }
        thickness *= 1.0 / M->vert_area[i];
        qv[i] = (qv[i] + f) / thickness;
    }
    for (int i = 0; i < E; i++) {                                              /* steps 4-5 */
        qe[i] = 0.5 * (qv[M->face_verts[i * 2]] + qv[M->face_verts[i * 2 + 1]]);
        he[i] = 0.5 * (h_total[M->face_nodes[i * 2]] + h_total[M->face_nodes[i * 2 + 1]]);
    }
    for (int i = 0; i < E; i++) {                                              /* step 6 */
        double F = 0.0, dr = 1.0 / M->face_dist[i];
        for (int j = 0; j < M->interp_n[i]; j++) {
            int f = M->interp_friends[i * 10 + j];
            double coeff = M->interp_w[i * 10 + j] * M->face_len[f] * dr;
            F += coeff * (he[f] * vel[f]) * (qe[i] + qe[f]) * 0.5;
        }
        dvdt[i] -= -F;
    }
    orc_interpolate_cartesian(M, uxyz, vel);                                   /* step 7 */
    for (int i = 0; i < N; i++)
        ekin[i] = 0.5 * (uxyz[i * 3] * uxyz[i * 3] + uxyz[i * 3 + 1] * uxyz[i * 3 + 1] + uxyz[i * 3 + 2] * uxyz[i * 3 + 2]);
    csr_spmv(&M->G, ekin, 1.0, gk);                                            /* step 8 */
    for (int i = 0; i < E; i++) dvdt[i] += -gk[i];
    free(qv); free(qe); free(he); free(uxyz); free(gk);
}

/* RBF(dist, eps), include/mathRoutines.h:432-439 */
static double rbf_gauss(double dist, double eps)
{
    double phi = exp(-pow(eps * dist, 2.0));
    if (dist < 1e-8) phi = 1;
    return phi;
}

/* In-place inverse of the n x n row-major matrix a (n <= 7) by Gauss-Jordan
 * elimination with partial pivoting; 0 on success. */
static int gj_inverse(int n, double *a)
{
    double b[7 * 7];
    for (int i = 0; i < n * n; i++) b[i] = 0.0;
    for (int i = 0; i < n; i++) b[i * n + i] = 1.0;
    for (int c = 0; c < n; c++) {
        int piv = c;
        for (int r = c + 1; r < n; r++) if (fabs(a[r * n + c]) > fabs(a[piv * n + c])) piv = r;
        if (a[piv * n + c] == 0.0) return -1;
        if (piv != c)
            for (int q = 0; q < n; q++) {
                double t = a[c * n + q]; a[c * n + q] = a[piv * n + q]; a[piv * n + q] = t;
                t = b[c * n + q]; b[c * n + q] = b[piv * n + q]; b[piv * n + q] = t;
            }
        double d = a[c * n + c];
        for (int q = 0; q < n; q++) { a[c * n + q] /= d; b[c * n + q] /= d; }
        for (int r = 0; r < n; r++) {
            if (r == c) continue;
            double f = a[r * n + c];
            if (f == 0.0) continue;
            for (int q = 0; q < n; q++) { a[r * n + q] -= f * a[c * n + q]; b[r * n + q] -= f * b[c * n + q]; }
        }
    }
    for (int i = 0; i < n * n; i++) a[i] = b[i];
    return 0;
}

/* operatorDirectionalSecondDeriv = N R operatorSecondDeriv (src/mesh.cpp:2364-2716):
 * per node, the second derivatives (xx, xy, yy) of the Gaussian-RBF interpolant
 * over the node and its friends in node-centred map coordinates
 * (CalcControlVolumeInterpMatrix, :199-360, inverted as in :2413-2440), rotated
 * into each face's frame (face_node_vel_trans, :1222-1383) and projected on the
 * face normal.  Rows 2e (inner node) and 2e+1 (outer node). */
static int build_lsq(orc_mesh *M, double eps)
{
    int N = M->N, E = M->E;
    double r = M->r, r_recip = 1.0 / M->r;
    double *S = (double *)calloc((size_t)N * 3 * 7, sizeof(double));       /* [N][3][7] */
    for (int i = 0; i < N; i++) {
        int k = nfriends(M, i), K = k + 1;
        double lat1 = M->node_sph[i * 2], lon1 = M->node_sph[i * 2 + 1];
        double px[7], py[7];
        for (int j = 0; j < K; j++) {                /* node_pos_map(i, j), CalcMappingCoords :1384-1450 */
            double m, x, y;
            int f = j == 0 ? i : M->friends[i * 6 + j - 1];
            map_at_point(&m, &x, &y, lat1, M->node_sph[f * 2], lon1, M->node_sph[f * 2 + 1], r);
            px[j] = x; py[j] = y;
        }
        double A[7 * 7], nnr[7];
        A[0] = 1.0;
        for (int j1 = 0; j1 < k; j1++) {
            double x1 = px[j1 + 1] / r, y1 = py[j1 + 1] / r;
            double arc = sqrt(x1 * x1 + y1 * y1);
            A[0 * K + j1 + 1] = rbf_gauss(arc, eps);
        }
        for (int j1 = 0; j1 < k; j1++) {
            double x1 = px[j1 + 1] / r, y1 = py[j1 + 1] / r;
            double arc = sqrt(x1 * x1 + y1 * y1);
            A[(j1 + 1) * K + 0] = rbf_gauss(arc, eps);
            nnr[j1 + 1] = rbf_gauss(arc, eps);
            for (int j2 = 0; j2 < k; j2++) {
                double x2 = px[j2 + 1] / r, y2 = py[j2 + 1] / r;
                arc = sqrt((x1 - x2) * (x1 - x2) + (y1 - y2) * (y1 - y2));
                A[(j1 + 1) * K + j2 + 1] = rbf_gauss(arc, eps);
            }
        }
        if (gj_inverse(K, A) != 0) { free(S); return -6; }
        /* rbfDeriv2 rows (:2472-2548), scaled by r_recip^2 */
        double D[3][7];
        for (int c = 0; c < 3; c++) for (int j = 0; j < K; j++) D[c][j] = 0.0;
        D[0][0] = -2.0 * eps * eps;
        D[2][0] = -2.0 * eps * eps;
        for (int j = 0; j < k; j++) {
            double x1 = px[j + 1] * r_recip, y1 = py[j + 1] * r_recip;
            double arc = sqrt(x1 * x1 + y1 * y1);
            double xx = x1 * x1, yy = y1 * y1, xy = x1 * y1;
            double arc2 = 1.0 / (arc * arc), arc3 = 1.0 / (arc * arc * arc);
            double rbf = nnr[j + 1];
            double d2phidr2 = 2 * eps * eps * rbf * (2 * arc * arc * eps * eps - 1);
            double dphidr = -2 * arc * eps * eps * rbf;
            D[0][j + 1] = (yy * arc3 * dphidr + xx * arc2 * d2phidr2);
            D[1][j + 1] = (-xy * arc3 * dphidr + xy * arc2 * d2phidr2);
            D[2][j + 1] = (xx * arc3 * dphidr + yy * arc2 * d2phidr2);
        }
        double sc = r_recip * r_recip;
        for (int c = 0; c < 3; c++)
            for (int j = 0; j < K; j++) {
                double t = 0.0;
                for (int q = (c == 1 ? 1 : 0); q < K; q++) t += (sc * D[c][q]) * A[q * K + j];
                S[((size_t)i * 3 + c) * 7 + j] = t;
            }
    }
    orc_csr *C = &M->D2;
    C->rows = 2 * E; C->cols = N;
    C->rowptr = (int *)malloc(sizeof(int) * (2 * E + 1));
    C->col = (int *)malloc(sizeof(int) * 14 * E);
    C->val = (double *)malloc(sizeof(double) * 14 * E);
    int nz = 0;
    for (int e = 0; e < E; e++)
        for (int side = 0; side < 2; side++) {
            int n = M->face_nodes[e * 2 + side];
            int k = nfriends(M, n), K = k + 1;
            double ca, sa;                            /* velTransform, include/mathRoutines.h:79-87 */
            {
                double lat1 = M->face_int[e * 2], lon1 = M->face_int[e * 2 + 1];
                double lat2 = M->node_sph[n * 2], lon2 = M->node_sph[n * 2 + 1];
                ca = cos(lat1) * cos(lat2);
                ca += (1.0 + sin(lat1) * sin(lat2)) * cos(lon2 - lon1);
                ca /= (1.0 + sin(lat1) * sin(lat2) + cos(lat1) * cos(lat2) * cos(lon2 - lon1));
                sa = -(sin(lat1) + sin(lat2)) * sin(lon2 - lon1);
                sa /= (1.0 + sin(lat1) * sin(lat2) + cos(lat1) * cos(lat2) * cos(lon2 - lon1));
            }
            double R[3][3] = {{ca * ca, -2 * ca * sa, sa * sa},
                              {ca * sa, ca * ca - sa * sa, -sa * ca},
                              {sa * sa, 2 * ca * sa, ca * ca}};
            double nx = M->face_normal[e * 2], ny = M->face_normal[e * 2 + 1];
            double Nv[3] = {nx * nx, 2 * nx * ny, ny * ny};
            double NR[3];
            for (int c = 0; c < 3; c++) {
                double t = 0.0;
                for (int q = 0; q < 3; q++) t += Nv[q] * R[q][c];
                NR[c] = t;
            }
            C->rowptr[2 * e + side] = nz;
            for (int j = 0; j < K; j++) {
                double t = 0.0;
                for (int c = 0; c < 3; c++) t += NR[c] * S[((size_t)n * 3 + c) * 7 + j];
                C->col[nz] = j == 0 ? n : M->friends[n * 6 + j - 1];
                C->val[nz] = t;
                nz++;
            }
        }
    C->rowptr[2 * E] = nz;
    csr_finalise_rows(C);
    free(S);
    return 0;
}

/* interpolateLSQFlux, src/interpolation.cpp:311-356 (beta = 1, third order):
 * flux_e = v (h_in + h_out) / 2 - dx^2/12 (d2_out + d2_in) v + dx^2/12 |v| (d2_out - d2_in) */
int orc_lsq_flux(orc_mesh *M, double eps, double *flux, const double *vel, const double *h)
{
    if (!M->D2.rowptr) { int st = build_lsq(M, eps); if (st) return st; }
    int E = M->E;
    double *d2 = (double *)malloc(sizeof(double) * 2 * E);
    csr_spmv(&M->D2, h, 1.0, d2);
    double fact = 1. / 12.0, beta = 1.0;
    for (int i = 0; i < E; i++) {
        double dx = M->face_dist[i];
        double dx2 = dx * dx * fact;
        double v = vel[i];
        int in = M->face_nodes[i * 2], out = M->face_nodes[i * 2 + 1];
        double d2o = d2[2 * i + 1], d2i = d2[2 * i];
        flux[i] = v * 0.5 * (h[in] + h[out]) - dx2 * (d2o + d2i) * v + dx2 * beta * fabs(v) * (d2o - d2i);
    }
    free(d2);
    return 0;
}

/* vertex fields for checks: which = 0 area, 1..3 kite fractions R(v, j), 4 sin(lat) */
int orc_mesh_vertex_field(const orc_mesh *M, int which, double *out)
{
    for (int i = 0; i < M->V; i++) {
        if (which == 0) out[i] = M->vert_area[i];
        else if (which >= 1 && which <= 3) out[i] = M->vert_R[i * 3 + which - 1];
        else if (which == 4) out[i] = sin(M->vert_sph[i * 2]);
        else return -1;
    }
    return M->V;
}

/* vertex topology: nodes [V][3], faces [V][3], face directions [V][3], face vertices [E][2] */
void orc_mesh_vertex_topology(const orc_mesh *M, int *vert_nodes, int *vert_faces, int *vert_face_dir, int *face_verts)
{
    memcpy(vert_nodes, M->vert_nodes, sizeof(int) * M->V * 3);
    memcpy(vert_faces, M->vert_faces, sizeof(int) * M->V * 3);
    memcpy(vert_face_dir, M->vert_face_dir, sizeof(int) * M->V * 3);
    memcpy(face_verts, M->face_verts, sizeof(int) * M->E * 2);
}

/* updateEnergy, src/energy.cpp:13-61: LINEAR (:30-43) alpha 1000 h |u|^2,
 * QUADRATIC (:45-53) alpha / h |u| |u|^2; area-weighted sum over 4 pi r^2 */
double orc_update_energy_fric(const orc_mesh *M, double alpha, double h, int friction, double *e, const double *uv)
{
    double avg = 0.0;
    for (int i = 0; i < M->E; i++) {
        double q = uv[i * 2] * uv[i * 2] + uv[i * 2 + 1] * uv[i * 2 + 1];
        double ei = friction ? alpha / h * sqrt(q) * q : alpha * 1000.0 * h * q;
        if (e) e[i] = ei;
        avg += ei * M->face_area[i];
    }
    avg /= (4 * ORC_PI * pow(M->r, 2.0));
    return avg;
}

/* updateEnergy, LINEAR branch */
double orc_update_energy(const orc_mesh *M, double alpha, double h, double *e, const double *uv)
{
    return orc_update_energy_fric(M, alpha, h, 0, e, uv);
}

/* ------------------------------------------------------------------------ */
/* spherical harmonics (self-gravity / loading)                              */
/* ------------------------------------------------------------------------ */
/* 4pi-normalised associated Legendre functions with the Condon-Shortley phase,
 * P[l(l+1)/2+m] for z = cos(colatitude); standard three-term recurrences
 * (Holmes & Featherstone 2002, unscaled form). */
void orc_plmbar(int L, double z, double *P)
{
    double s = sqrt(fmax(0.0, 1.0 - z * z));
    /* sectoral terms */
    P[0] = 1.0;
    double pmm = 1.0;
    for (int m = 1; m <= L; m++) {
        double f = (m == 1) ? sqrt(3.0) : sqrt((2.0 * m + 1.0) / (2.0 * m));
        pmm = -f * s * pmm;                /* Condon-Shortley phase */
        P[m * (m + 1) / 2 + m] = pmm;
    }
    for (int m = 0; m <= L; m++) {
        if (m + 1 <= L) {
            double a = sqrt(2.0 * m + 3.0);
            P[(m + 1) * (m + 2) / 2 + m] = a * z * P[m * (m + 1) / 2 + m];
        }
        for (int l = m + 2; l <= L; l++) {
            double a = sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)m * m));
            double b = sqrt(((2.0 * l + 1.0) * ((l - 1.0) * (l - 1.0) - (double)m * m)) /
                            ((2.0 * l - 3.0) * ((double)l * l - (double)m * m)));
            P[l * (l + 1) / 2 + m] = a * z * P[(l - 1) * l / 2 + m] - b * P[(l - 2) * (l - 1) / 2 + m];
        }
    }
}

/* column index of the real harmonic (l, m, cos|sin) in a K=(L+1)^2 basis:
 * k = l*l + 2m - (m>0) for cos, l*l + 2m for sin (m>0) */
static int sh_col(int l, int m, int is_sin) { return l * l + (m == 0 ? 0 : 2 * m - 1 + is_sin); }

static int cholesky_factor(double *A, int n)
{   /* A (n x n, SPD) overwritten by its lower Cholesky factor R, A = R R^T */
    for (int j = 0; j < n; j++) {
        double d = A[(size_t)j * n + j];
        for (int k = 0; k < j; k++) d -= A[(size_t)j * n + k] * A[(size_t)j * n + k];
        if (d <= 0.0) return -1;
        d = sqrt(d);
        A[(size_t)j * n + j] = d;
#pragma omp parallel for schedule(static)
        for (int i = j + 1; i < n; i++) {
            double s = A[(size_t)i * n + j];
            for (int k = 0; k < j; k++) s -= A[(size_t)i * n + k] * A[(size_t)j * n + k];
            A[(size_t)i * n + j] = s / d;
        }
    }
    return 0;
}

static void cholesky_solve(const double *R, int n, double *x)
{   /* x <- (R R^T)^-1 x: forward then backward substitution */
    for (int i = 0; i < n; i++) {
        double s = x[i];
        for (int k = 0; k < i; k++) s -= R[(size_t)i * n + k] * x[k];
        x[i] = s / R[(size_t)i * n + i];
    }
    for (int i = n - 1; i >= 0; i--) {
        double s = x[i];
        for (int k = i + 1; k < n; k++) s -= R[(size_t)k * n + i] * x[k];
        x[i] = s / R[(size_t)i * n + i];
    }
}

/* Real SH basis rows at the nodes, Y[k][i] = Pbar_lm(sin lat_i) * (cos m lon_i | sin m lon_i),
 * the columns of sh_matrix in src/mesh.cpp:2219-2252 (with l = 0, 1 kept). */
void orc_sh_basis(const orc_mesh *M, int L, double *Y)
{
    int N = M->N;
#pragma omp parallel
    {
        double *P = (double *)malloc(sizeof(double) * (L + 1) * (L + 2) / 2);
#pragma omp for schedule(static)
        for (int i = 0; i < N; i++) {
            double lat = M->node_sph[i * 2], lon = M->node_sph[i * 2 + 1];
            orc_plmbar(L, cos(ORC_PI * 0.5 - lat), P);
            for (int l = 0; l <= L; l++)
                for (int m = 0; m <= l; m++) {
                    double p = P[l * (l + 1) / 2 + m];
                    Y[(size_t)sh_col(l, m, 0) * N + i] = p * cos((double)m * lon);
                    if (m > 0) Y[(size_t)sh_col(l, m, 1) * N + i] = p * sin((double)m * lon);
                }
        }
        free(P);
    }
}

/* Enable self-gravity/loading: U_eff = U + g * sum_{l=2..L} f_l * sum_m c_lm Y_lm,
 * with c = (Y^T Y)^-1 Y^T eta (ordinary least squares over the nodes, as
 * SHExpandLSQ).  factors has L+1 entries (entries 0 and 1 unused). */
int orc_solver_set_loading(orc_solver *S, int L, const double *factors)
{
    const orc_mesh *M = S->M;
    int N = M->N, K = (L + 1) * (L + 1);
    free(S->sh_R); free(S->sh_Y); free(S->sh_f);
    S->sh_R = S->sh_Y = S->sh_f = NULL;
    S->sh_lmax = 0;
    if (L <= 0) return 0;
    if (N < K) return -1;
    double *Y = (double *)malloc(sizeof(double) * (size_t)N * K);
    if (!Y) return -3;
    orc_sh_basis(M, L, Y);
    /* Gram matrix of the basis rows: each entry a dot product over the nodes in
     * four interleaved partial sums (the setup's own order; setup only) */
    double *A = (double *)calloc((size_t)K * K, sizeof(double));
#pragma omp parallel for schedule(dynamic)
    for (int a = 0; a < K; a++)
        for (int b = 0; b <= a; b++) {
            const double *ya = &Y[(size_t)a * N], *yb = &Y[(size_t)b * N];
            double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
            int i = 0;
            for (; i + 3 < N; i += 4) {
                s0 += ya[i] * yb[i]; s1 += ya[i + 1] * yb[i + 1];
                s2 += ya[i + 2] * yb[i + 2]; s3 += ya[i + 3] * yb[i + 3];
            }
            for (; i < N; i++) s0 += ya[i] * yb[i];
            A[(size_t)a * K + b] = (s0 + s1) + (s2 + s3);
        }
    for (int a = 0; a < K; a++) for (int b = a + 1; b < K; b++) A[(size_t)a * K + b] = A[(size_t)b * K + a];
    if (cholesky_factor(A, K) != 0) { free(A); free(Y); return -2; }
    S->sh_R = A; S->sh_Y = Y;
    S->sh_f = (double *)malloc(sizeof(double) * (L + 1));
    memcpy(S->sh_f, factors, sizeof(double) * (L + 1));
    S->sh_lmax = L;
    return 0;
}

/* coefficients c[K] of eta (LSQ): t = Y^T eta, then c = (Y^T Y)^-1 t */
void orc_sh_analysis(const orc_solver *S, const double *eta, double *c)
{
    int N = S->M->N, K = (S->sh_lmax + 1) * (S->sh_lmax + 1);
#pragma omp parallel for schedule(static)
    for (int a = 0; a < K; a++) {
        double s = 0.0;
        const double *y = &S->sh_Y[(size_t)a * N];
        for (int i = 0; i < N; i++) s += y[i] * eta[i];
        c[a] = s;
    }
    cholesky_solve(S->sh_R, K, c);
}

/* U[i] += g * sum_{l>=2} f_l c_lm Y_lm(i), each node's sum in ascending harmonic order */
void orc_sh_add_loading(const orc_solver *S, const double *eta, double *U)
{
    int L = S->sh_lmax, N = S->M->N, K = (L + 1) * (L + 1);
    double *c = (double *)malloc(sizeof(double) * K);
    orc_sh_analysis(S, eta, c);
    for (int l = 0; l <= L; l++)
        for (int k = l * l; k < (l + 1) * (l + 1); k++) c[k] = (l >= 2) ? c[k] * S->sh_f[l] : 0.0;
    const int B = 256;
#pragma omp parallel for schedule(static)
    for (int i0 = 0; i0 < N; i0 += B) {
        double s[256];
        int n = N - i0 < B ? N - i0 : B;
        for (int q = 0; q < n; q++) s[q] = 0.0;
        for (int k = 4; k < K; k++) {
            const double *y = &S->sh_Y[(size_t)k * N + i0];
            double ck = c[k];
            for (int q = 0; q < n; q++) s[q] += y[q] * ck;
        }
        for (int q = 0; q < n; q++) U[i0 + q] += S->p.g * s[q];
    }
    free(c);
}

/* ------------------------------------------------------------------------ */
/* the time loop (ab3Explicit, src/timeIntegrator.cpp:205-272)               */
/* ------------------------------------------------------------------------ */
typedef struct {
    orc_solver *S;
    int iter;
    double time;
    double *v, *eta, *dvdt, *detadt;   /* v[E], eta[N], dvdt[E][3], detadt[N][3] */
    double *U, *drag, *dv0, *dp0, *uv, *ediss, *tmp;
    double *h_total, *ekin, *flux;      /* advection: column thickness h + eta [N], KE [N], thickness flux [E] */
    double power;                       /* last dissipated power, W/m^2 */
} orc_sim;

orc_sim *orc_sim_create(orc_solver *S)
{
    orc_sim *X = (orc_sim *)calloc(1, sizeof(orc_sim));
    int N = S->M->N, E = S->M->E;
    X->S = S;
    X->v = (double *)calloc(E, sizeof(double));
    X->eta = (double *)calloc(N, sizeof(double));
    X->dvdt = (double *)calloc((size_t)E * 3, sizeof(double));
    X->detadt = (double *)calloc((size_t)N * 3, sizeof(double));
    X->U = (double *)calloc(N, sizeof(double));
    X->drag = (double *)calloc(E, sizeof(double));
    X->dv0 = (double *)calloc(E, sizeof(double));
    X->dp0 = (double *)calloc(N, sizeof(double));
    X->uv = (double *)calloc((size_t)E * 2, sizeof(double));
    X->ediss = (double *)calloc(E, sizeof(double));
    X->tmp = (double *)calloc(E, sizeof(double));
    X->h_total = (double *)calloc(N, sizeof(double));
    X->ekin = (double *)calloc(N, sizeof(double));
    X->flux = (double *)calloc(E, sizeof(double));
    for (int i = 0; i < N; i++) X->h_total[i] = S->p.h + X->eta[i];      /* :203 */
    return X;
}

void orc_sim_free(orc_sim *X)
{
    if (!X) return;
    free(X->v); free(X->eta); free(X->dvdt); free(X->detadt); free(X->U); free(X->drag);
    free(X->dv0); free(X->dp0); free(X->uv); free(X->ediss); free(X->tmp);
    free(X->h_total); free(X->ekin); free(X->flux);
    free(X);
}

void orc_sim_set_state(orc_sim *X, int iter, const double *v, const double *eta,
                       const double *dvdt, const double *detadt)
{
    int N = X->S->M->N, E = X->S->M->E;
    X->iter = iter;
    X->time = X->S->p.dt * iter;
    if (v) memcpy(X->v, v, sizeof(double) * E);
    if (eta) memcpy(X->eta, eta, sizeof(double) * N);
    if (dvdt) memcpy(X->dvdt, dvdt, sizeof(double) * E * 3);
    if (detadt) memcpy(X->detadt, detadt, sizeof(double) * N * 3);
    for (int i = 0; i < N; i++) X->h_total[i] = X->S->p.h + X->eta[i];   /* src/timeIntegrator.cpp:203 */
}

void orc_sim_get_state(const orc_sim *X, int *iter, double *v, double *eta, double *dvdt, double *detadt)
{
    int N = X->S->M->N, E = X->S->M->E;
    if (iter) *iter = X->iter;
    if (v) memcpy(v, X->v, sizeof(double) * E);
    if (eta) memcpy(eta, X->eta, sizeof(double) * N);
    if (dvdt) memcpy(dvdt, X->dvdt, sizeof(double) * E * 3);
    if (detadt) memcpy(detadt, X->detadt, sizeof(double) * N * 3);
}

/* One pass of the time-loop body; returns the dissipated power (W/m^2). */
double orc_sim_step(orc_sim *X)
{
    orc_solver *S = X->S;
    const orc_mesh *M = S->M;
    int N = M->N, E = M->E;
    double dt = S->p.dt;
    if (S->p.advection) {                /* updateMomentum's advection branch, src/updateMomentum.cpp:35-39 */
        csr_spmv(&M->G, X->eta, -S->p.g * (1 - 0.5 * 0.0), X->dv0);
        orc_momentum_advection(M, S->p.angvel, X->dv0, X->v, X->h_total, X->ekin);
    } else {
        orc_update_momentum(S, X->dv0, X->v, X->eta);                  /* :213 */
    }
    for (int i = 0; i < E; ++i) X->dvdt[i * 3] = X->dv0[i];              /* :215 */
    orc_forcing(S, X->U, S->p.potential, X->time + dt, S->p.ecc, S->p.obliq);   /* :218 */
    if (S->sh_lmax > 0) orc_sh_add_loading(S, X->eta, X->U);
    /* drag_term = Ldrag*v + G*U (:219); Ldrag is the diagonal -alpha */
    csr_spmv(&M->G, X->U, 1.0, X->tmp);
    for (int i = 0; i < E; i++) X->drag[i] = (0.0 + 1.0 * ((-S->p.alpha) * X->v[i])) + X->tmp[i];
    orc_ab3(dt, X->v, X->dvdt, X->iter, E, S->p.init_load);              /* :239 */
    for (int i = 0; i < E; i++) X->v[i] += dt * X->drag[i];              /* :242 */
    if (S->p.advection) {                /* updateEta's advection branch, src/updateEta.cpp:22-32 */
        int st = orc_lsq_flux((orc_mesh *)M, 0.25, X->flux, X->v, X->h_total);
        if (st) return NAN;
        csr_spmv(&M->D, X->flux, 1.0, X->dp0);
    } else {
        orc_update_eta(S, X->dp0, X->v);                                 /* :249 */
    }
    for (int i = 0; i < N; ++i) X->detadt[i * 3] = X->dp0[i];
    orc_ab3(dt, X->eta, X->detadt, X->iter, N, S->p.init_load);          /* :253 */
    orc_interpolate_velocity(M, X->uv, X->v);                            /* :261 */
    X->power = orc_update_energy_fric(M, S->p.alpha, S->p.h, S->p.friction, X->ediss, X->uv);
    if (S->p.advection)                  /* column thickness for the next step, :266-269 */
        for (int i = 0; i < N; i++) X->h_total[i] = S->p.h + X->eta[i];
    X->iter++;
    X->time = dt * X->iter;
    return X->power;
}

int orc_sim_run(orc_sim *X, int nsteps, double *power)
{
    for (int s = 0; s < nsteps; s++) {
        double p = orc_sim_step(X);
        if (power) power[s] = p;
    }
    return X->iter;
}

double orc_sim_power(const orc_sim *X) { return X->power; }
void orc_sim_energy_field(const orc_sim *X, double *e) { memcpy(e, X->ediss, sizeof(double) * X->S->M->E); }

/* ------------------------------------------------------------------------ */
/* Icosahedral grid in the reference's grid-file format (test infrastructure: */
/* the CPU baseline's own copy of the benchmark grids)                        */
/* ------------------------------------------------------------------------ */
/* The grid is defined by: a regular icosahedron with vertices at the poles
 * and at latitude +-atan(1/2) (longitudes 72 k and 72 k + 36 degrees), each
 * triangle split into four through its edge midpoints, level times, every
 * new vertex the normalised sum of its edge's end points.  Its Voronoi cells
 * are what the reference reads (src/mesh.cpp:4016-4089): per node its
 * friends in clockwise order as seen from outside the sphere, and per friend
 * j the spherical circumcentre of the triangle (node, friend j, friend j+1).
 * The node numbering here is the order of creation (12 icosahedron vertices,
 * then each level's midpoints); any numbering describes the same mesh. */
typedef struct { double x, y, z; } orc_v3;

static orc_v3 v3_unit(orc_v3 a)
{
    double n = sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    orc_v3 r = {a.x / n, a.y / n, a.z / n};
    return r;
}

typedef struct { long long *key; int *val; size_t cap; } orc_edge_map;

static int edge_midpoint(orc_edge_map *h, orc_v3 *pos, int *npos, int a, int b)
{
    long long lo = a < b ? a : b, hi = a < b ? b : a;
    long long key = (lo << 32) | hi;
    size_t slot = (size_t)((unsigned long long)key * 0x9E3779B97F4A7C15ull >> 17) & (h->cap - 1);
    while (h->key[slot] != -1) {
        if (h->key[slot] == key) return h->val[slot];
        slot = (slot + 1) & (h->cap - 1);
    }
    orc_v3 s = {pos[a].x + pos[b].x, pos[a].y + pos[b].y, pos[a].z + pos[b].z};
    int id = (*npos)++;
    pos[id] = v3_unit(s);
    h->key[slot] = key;
    h->val[slot] = id;
    return id;
}

static void deg_latlon(orc_v3 p, double *lat, double *lon)
{
    *lat = atan2(p.z, sqrt(p.x * p.x + p.y * p.y)) * 180.0 / ORC_PI;
    *lon = atan2(p.y, p.x) * 180.0 / ORC_PI;
    if (*lon < 0.0) *lon += 360.0;
    if (*lon >= 360.0) *lon -= 360.0;
}

typedef struct { double ang; int node; } orc_nbr_ang;

static int ang_desc(const void *a, const void *b)
{
    double x = ((const orc_nbr_ang *)a)->ang, y = ((const orc_nbr_ang *)b)->ang;
    return x < y ? 1 : (x > y ? -1 : 0);
}

int orc_generate_grid_file(int level, const char *path)
{
    if (level < 0 || level > 10) return -1;
    long long N = 10ll * (1ll << (2 * level)) + 2, T = 20ll * (1ll << (2 * level));
    orc_v3 *pos = (orc_v3 *)malloc(sizeof(orc_v3) * N);
    int *tri = (int *)malloc(sizeof(int) * 3 * T), *tri2 = (int *)malloc(sizeof(int) * 3 * T);
    orc_edge_map h;
    h.cap = 1;
    while (h.cap < (size_t)(4 * N)) h.cap <<= 1;
    h.key = (long long *)malloc(sizeof(long long) * h.cap);
    h.val = (int *)malloc(sizeof(int) * h.cap);
    if (!pos || !tri || !tri2 || !h.key || !h.val) { free(pos); free(tri); free(tri2); free(h.key); free(h.val); return -2; }
    memset(h.key, 0xff, sizeof(long long) * h.cap);
    const double pi = 3.14159265358979323846, lat0 = atan(0.5);
    int npos = 0;
    pos[npos++] = (orc_v3){0.0, 0.0, 1.0};
    for (int k = 0; k < 5; k++) {
        double lon = 2.0 * pi * k / 5.0;
        pos[npos++] = (orc_v3){cos(lat0) * cos(lon), cos(lat0) * sin(lon), sin(lat0)};
    }
    for (int k = 0; k < 5; k++) {
        double lon = 2.0 * pi * k / 5.0 + pi / 5.0;
        pos[npos++] = (orc_v3){cos(lat0) * cos(lon), cos(lat0) * sin(lon), -sin(lat0)};
    }
    pos[npos++] = (orc_v3){0.0, 0.0, -1.0};
    long long nt = 0;
    for (int k = 0; k < 5; k++) {
        int u0 = 1 + k, u1 = 1 + (k + 1) % 5, l0 = 6 + k, l1 = 6 + (k + 1) % 5;
        int base[4][3] = {{0, u0, u1}, {u0, l0, u1}, {u1, l0, l1}, {11, l1, l0}};
        for (int q = 0; q < 4; q++, nt++)
            for (int c = 0; c < 3; c++) tri[3 * nt + c] = base[q][c];
    }
    for (int lv = 0; lv < level; lv++) {           /* one level of 4-way splits */
        long long nn = 0;
        for (long long t = 0; t < nt; t++) {
            int a = tri[3 * t], b = tri[3 * t + 1], c = tri[3 * t + 2];
            int ab = edge_midpoint(&h, pos, &npos, a, b);
            int bc = edge_midpoint(&h, pos, &npos, b, c);
            int ca = edge_midpoint(&h, pos, &npos, c, a);
            int kids[4][3] = {{a, ab, ca}, {ab, bc, ca}, {ab, b, bc}, {ca, bc, c}};
            for (int q = 0; q < 4; q++, nn++)
                for (int e = 0; e < 3; e++) tri2[3 * nn + e] = kids[q][e];
        }
        int *sw = tri; tri = tri2; tri2 = sw;
        nt = nn;
    }
    free(h.key); free(h.val); free(tri2);
    int st = 0;
    if (npos != N || nt != T) st = -3;
    /* node -> incident triangles */
    int *start = (int *)calloc((size_t)N + 1, sizeof(int)), *inc = (int *)malloc(sizeof(int) * 3 * T);
    int *fill = (int *)calloc((size_t)N, sizeof(int));
    orc_v3 *cc = (orc_v3 *)malloc(sizeof(orc_v3) * T);
    if (!start || !inc || !fill || !cc) st = -2;
    FILE *fp = st == 0 ? fopen(path, "w") : NULL;
    if (st == 0 && !fp) st = -4;
    if (st == 0) {
        for (long long t = 0; t < 3 * T; t++) start[tri[t] + 1]++;
        for (long long i = 0; i < N; i++) start[i + 1] += start[i];
        for (long long t = 0; t < T; t++)
            for (int q = 0; q < 3; q++) { int v = tri[3 * t + q]; inc[start[v] + fill[v]++] = (int)t; }
        /* circumcentre direction of each triangle: (b - a) x (c - a), outward */
        for (long long t = 0; t < T; t++) {
            orc_v3 a = pos[tri[3 * t]], b = pos[tri[3 * t + 1]], c = pos[tri[3 * t + 2]];
            orc_v3 u = {b.x - a.x, b.y - a.y, b.z - a.z}, w = {c.x - a.x, c.y - a.y, c.z - a.z};
            orc_v3 n = {u.y * w.z - u.z * w.y, u.z * w.x - u.x * w.z, u.x * w.y - u.y * w.x};
            if (n.x * (a.x + b.x + c.x) + n.y * (a.y + b.y + c.y) + n.z * (a.z + b.z + c.z) < 0) {
                n.x = -n.x; n.y = -n.y; n.z = -n.z;
            }
            cc[t] = v3_unit(n);
        }
        fprintf(fp, "ID    NODE LAT     NODE LON     FRIENDS LIST                           CENTROID COORD LIST \n");
        for (long long i = 0; i < N && st == 0; i++) {
            orc_v3 p = pos[i];
            int nb[6], k = 0;
            for (int q = start[i]; q < start[i + 1]; q++) {
                const int *tv = &tri[3 * (size_t)inc[q]];
                for (int c = 0; c < 3; c++) {
                    int v = tv[c], seen = (v == (int)i);
                    for (int j = 0; j < k && !seen; j++) seen = nb[j] == v;
                    if (!seen) { if (k == 6) { st = -5; break; } nb[k++] = v; }
                }
            }
            if (st != 0 || (k != 5 && k != 6)) { st = -5; break; }
            /* clockwise seen from outside: descending angle in the local east/north plane; a
             * neighbour due west (on atan2's branch cut, where a rounding-level north component
             * decides between +pi and -pi) is put at +pi, first */
            double lr = atan2(p.y, p.x);
            orc_v3 east = {-sin(lr), cos(lr), 0.0};
            orc_v3 north = {p.y * east.z - p.z * east.y, p.z * east.x - p.x * east.z, p.x * east.y - p.y * east.x};
            orc_nbr_ang ang[6];
            for (int j = 0; j < k; j++) {
                orc_v3 d = {pos[nb[j]].x - p.x, pos[nb[j]].y - p.y, pos[nb[j]].z - p.z};
                double dn = d.x * north.x + d.y * north.y + d.z * north.z, de = d.x * east.x + d.y * east.y + d.z * east.z;
                ang[j].ang = (de < 0.0 && fabs(dn) <= 1e-12 * fabs(de)) ? 3.14159265358979323846 : atan2(dn, de);
                ang[j].node = nb[j];
            }
            qsort(ang, k, sizeof(orc_nbr_ang), ang_desc);
            double lat, lon;
            deg_latlon(p, &lat, &lon);
            fprintf(fp, "%-5lld %.16f %.16f {", i, lat, lon);
            for (int j = 0; j < 6; j++) fprintf(fp, "%5d%s", j < k ? ang[j].node : -1, j < 5 ? ", " : "}, {");
            for (int j = 0; j < 6; j++) {
                double clat = -1.0, clon = -1.0;
                if (j < k) {
                    int fa = ang[j].node, fb = ang[(j + 1) % k].node, found = -1;
                    for (int q = start[i]; q < start[i + 1] && found < 0; q++) {
                        const int *tv = &tri[3 * (size_t)inc[q]];
                        int ha = tv[0] == fa || tv[1] == fa || tv[2] == fa;
                        int hb = tv[0] == fb || tv[1] == fb || tv[2] == fb;
                        if (ha && hb) found = inc[q];
                    }
                    if (found < 0) { st = -6; break; }
                    deg_latlon(cc[found], &clat, &clon);
                }
                fprintf(fp, "(%.16f, %.16f)%s", clat, clon, j < 5 ? ", " : "} \n");
            }
        }
        if (fclose(fp) != 0 && st == 0) st = -4;
    }
    free(pos); free(tri); free(start); free(inc); free(fill); free(cc);
    return st;
}

/* FREE_LOADING degree factors, src/boundaryConditions.cpp:29-76: loading Love
 * numbers of a uniform elastic body (rigidity 40 GPa, bulk density
 * 1609.22 kg/m^3, ocean 1000 kg/m^3), gamma_l = (1 + k_l - h_l) 3 rho_o /
 * ((2l+1) rho_b), for l = 0..lmax in the reference's loop order and form. */
void orc_loading_factors(double g, double r, int lmax, double *out)
{
    double ocean_den = 1000.0, bulk_den = 1609.22, rig = 40e9;
    for (int l = 0; l < lmax + 1; l++) {
        double eff_rig = (double)(2 * l * l + 4 * l + 3);
        eff_rig /= (double)l;
        eff_rig *= rig / (bulk_den * g * r);
        double k_l = -(1.0 / (1.0 + eff_rig));
        double h_l = -(1.0 / (1.0 + eff_rig)) * (2.0 * (double)l + 1.0) / 3.0;
        out[l] = (1.0 + k_l - h_l);
        out[l] *= 3. * ocean_den / ((2. * (double)l + 1.0) * bulk_den);
    }
}
