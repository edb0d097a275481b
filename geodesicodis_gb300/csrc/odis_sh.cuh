// Self-gravity / ocean-loading potential through spherical harmonics.
//
// The reference's form (commented-out pressureGradientSH,
// src/spatialOperators.cpp:387-462, with the basis of CalcLegendreFuncs,
// src/mesh.cpp:2154-2258): eta is expanded to degree L in 4pi-normalised real
// harmonics with the Condon-Shortley phase (SHTOOLS PlmBar csphase=-1,
// src/legendre.f95:20) by least squares over the cells (SHExpandLSQ,
// src/extractSHCoeffGG.f95:17), each degree l >= 2 is scaled by a factor f_l
// and the field is synthesised back and added to the tidal potential times g.
//
// Per step:  t = Y^T eta  (K sums over the cells),  c = F (Y^T Y)^-1 t  (K x K),
//            usg = Y c    (N dot products of length K);
// the face kernel then adds G (g usg) to the forcing gradient.
#pragma once

#include <cuda_runtime.h>

#include "odis_internal.h"

namespace odis {

// column of harmonic (l, m, cos|sin) in t and c: l^2 for m=0, l^2 + 2m-1 (cos), l^2 + 2m (sin)
__host__ __device__ inline int sh_col(int l, int m, int is_sin) { return l * l + (m == 0 ? 0 : 2 * m - 1 + is_sin); }
// stored Legendre row of (l, m): rows ordered by order m, then degree l
__host__ __device__ inline int p_row(int L, int l, int m) { return m * (L + 1) - m * (m - 1) / 2 + (l - m); }

struct ShLoading;

// status: the context's device status word (bounded waits record ODIS_ERR_TIMEOUT there)
int sh_create(ShLoading** out, const Mesh& m, int lmax, const double* factors, int precision, int Np, int* status);
void sh_destroy(ShLoading* s);
// usg buffer ([Np], FP64 or FP32 according to the precision)
const double* sh_usg64(ShLoading* s);
const float* sh_usg32(ShLoading* s);
const float2* sh_usgdf(ShLoading* s);
// enqueue analysis + synthesis of the current eta (double* or float*)
void sh_enqueue(ShLoading* s, const void* eta, cudaStream_t stream);
// kernels launched by one sh_enqueue
int sh_kernels_per_step(const ShLoading* s);
// tile shapes chosen by the setup-time autotuner; tl = 0 for the tensor-core
// transforms (nchunk = analysis chunks, lanes = cell tiles per synthesis pass)
// (cells = synthesis cells per thread, pre = 1 for the analysis from trig-weighted values)
void sh_tuning(const ShLoading* s, int* tl, int* nchunk, int* lanes, int* cells, int* pre);
// Dense synthesis (usg = Z t, Z = Y F G^-1) offered by the setup timing for a
// whole-step comparison: sh_try_dense switches between it and the factored
// synthesis; sh_set_dense makes the choice final (off frees Z).
bool sh_dense_candidate(const ShLoading* s);
void sh_try_dense(ShLoading* s, bool on);
void sh_set_dense(ShLoading* s, bool on);
// the stored basis: half = 1 for the antipodal half basis, the cells it covers,
// and its bytes (Legendre rows + trig rows in the method's type)
void sh_layout(const ShLoading* s, int* half, int* cells, long long* basis_bytes);
// host helpers for checks: real SH basis at the nodes, [N][K]
void sh_basis_host(const Mesh& m, int lmax, std::vector<double>& Y);

}  // namespace odis
