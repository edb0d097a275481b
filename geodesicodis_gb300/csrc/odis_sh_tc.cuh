// Tensor-core (tcgen05) form of the self-gravity transforms for the FP32-state
// method.  Internal to the library; odis_sh.cu chooses between this path and the
// CUDA-core transforms by timing both at setup.
#pragma once

#include <cuda_runtime.h>

namespace odis {

struct ShTc;

// Build the operand tiles from the FP32 Legendre rows P[MP][Np] (device, rows
// ordered by order m then degree l) and keep the trig rows trig[2(L+1)][Np].
// pmax = max |P| (host, FP64).  Returns ODIS_ERR_ARG when the degree does not
// fit the kernels' tile limits (the caller then keeps the CUDA-core path).
int shtc_create(ShTc** out, const float* P, const float* trig, double pmax, int L, int N, int Np, int* status);
void shtc_destroy(ShTc* s);
// partial sums part[k][chunk] of t = Y^T eta (the fold sums over the chunks)
void shtc_analysis(ShTc* s, const float* eta, cudaStream_t st);
const float* shtc_partials(const ShTc* s);
int shtc_chunks(const ShTc* s);
// scaled fp16 pairs of the coefficients c[K] as the synthesis operand
void shtc_pack(ShTc* s, const float* coef, cudaStream_t st);
// usg = Y c
void shtc_synth(ShTc* s, float* usg, cudaStream_t st);
// cell tiles per synthesis pass (1 or 2; setup-time choice)
int shtc_tiles_per_pass(const ShTc* s);
bool shtc_tiles_per_pass_ok(const ShTc* s, int tp);
void shtc_set_tiles_per_pass(ShTc* s, int tp);
int shtc_kernels_per_step();

}  // namespace odis
