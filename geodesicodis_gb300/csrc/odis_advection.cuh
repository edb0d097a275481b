// Nonlinear momentum advection on the device (see odis_advection.cu).
#pragma once

#include <cuda_runtime.h>

#include "odis_internal.h"

namespace odis {

struct AdvDev;

int adv_create(AdvDev** out, const Mesh& m, double angvel, int Ep, int Np);
void adv_destroy(AdvDev* a);
// dvdt[E] += PV flux - G KE for velocity v[E] and column thickness h_total[N];
// ekin[N] receives the kinetic energy (device; adv_ekin_scratch gives a buffer).
// rbf / cell_face: the context's Cartesian reconstruction blocks and cell-face table.
void adv_momentum(AdvDev* a, const double* rbf, const int* cell_face, double* dvdt, const double* v,
                  const double* h_total, double* ekin, cudaStream_t s);
double* adv_ekin_scratch(AdvDev* a);
// state of an advective run, reference layout: v[E], eta[N], dvdt history [E][3],
// detadt history [N][3], column thickness h + eta [N], forcing [N], uv [E][2]
struct AdvState {
    double *v, *eta, *hv, *hp, *ht, *U, *uv;
};
// Ua/Ub: the forcing basis at the nodes, U(t) = cos(Omega t) Ua + sin(Omega t) Ub
int adv_state_alloc(AdvDev* a, double h0, const std::vector<double>& Ua, const std::vector<double>& Ub, double angvel);
AdvState adv_state(AdvDev* a);
// one step of the advective loop up to the continuity update (forcing phase
// from the device step counter, AB3 mode from iter); the caller then computes the
// power from v and calls adv_thickness, which advances the counter
void adv_step(AdvDev* a, const double* rbf, const int* cell_face, double g, double alpha, double h0, double dt,
              int iter, int init_load, cudaStream_t s);
void adv_thickness(AdvDev* a, double h0, cudaStream_t s, bool advance = true);
void adv_set_step(AdvDev* a, long long step, cudaStream_t s);
int adv_kernels_per_step();
// captured graph of adv_graph_steps() steps (owned by AdvDev) and its power buffer
int adv_graph_steps();
double* adv_graph_power(AdvDev* a);
cudaGraphExec_t* adv_graph(AdvDev* a);
// flux[E]: the reference's interpolateLSQFlux of the column thickness h_total[N] with velocities v[E]
void adv_lsq_flux(AdvDev* a, double* flux, const double* v, const double* h_total, cudaStream_t s);
int adv_kernels_per_call();

}  // namespace odis
