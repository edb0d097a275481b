// Nonlinear momentum advection on the device (see odis_advection.cu).
#pragma once

#include <cuda_runtime.h>

#include "odis_internal.h"

namespace odis {

struct AdvDev;

// df64_run: the context will run the loop in double-float (keeps the host copies of
// the tables until adv_state_alloc converts them)
int adv_create(AdvDev** out, const Mesh& m, double angvel, int Ep, int Np, bool df64_run = false);
void adv_destroy(AdvDev* a);
// dvdt[E] += PV flux - G KE for velocity v[E] and column thickness h_total[N];
// ekin[N] receives the kinetic energy (device; adv_ekin_scratch gives a buffer).
// rbf / cell_face / nbr / tw: the context's Cartesian reconstruction blocks, cell-face
// table and TRiSK table ([10][Ep] neighbours and weights w_ee' l_e' / d_e, FP64).
void adv_momentum(AdvDev* a, const double* rbf, const int* cell_face, const int* nbr, const double* tw, double* dvdt,
                  const double* v, const double* h_total, double* ekin, cudaStream_t s);
double* adv_ekin_scratch(AdvDev* a);
// Run state in the method's number type (ODIS_FP64: double; ODIS_DF64: double-float
// pairs), allocated once: v, eta, the AB3 histories, h + eta, the forcing at the
// nodes.  Ua/Ub: the forcing basis at the nodes, U(t) = cos(Omega t) Ua + sin(Omega t) Ub.
int adv_state_alloc(AdvDev* a, int precision, double h0, const std::vector<double>& Ua, const std::vector<double>& Ub);
// reference layout on the host: v[E], eta[N], dvdt history [E][3], detadt history [N][3] (each nullable)
int adv_get_state(AdvDev* a, double* v, double* eta, double* dvdt, double* detadt);
int adv_set_state(AdvDev* a, const double* v, const double* eta, const double* dvdt, const double* detadt);
// what one advective step needs from the context; the typed tables are in the
// run's number type (double, or df64 for an ODIS_DF64 run)
struct AdvStepArgs {
    const void* rbf;          // [3][6][Np] Cartesian reconstruction blocks
    const int* cell_face;     // [6][Np] cell-face table
    const int* nbr;           // [10][Ep] TRiSK neighbour faces
    const void* w;            // [10][Ep] TRiSK weights (tangential velocity)
    const void* nrm;          // [2][Ep] face normals
    const void* area;         // [Ep] face areas
    double g, alpha, h0, dt;
    double divisor;           // 4 pi r^2
    int init_load;
    int quad;                 // QUADRATIC friction: dissipation alpha / h |u|^3
};
// one whole step of the advective loop (7 kernels): momentum with advection, the
// continuity update, the power of the updated velocity into *power (device), and
// h + eta, step counter and forcing phase for the next step.  AB3 mode from iter.
void adv_step(AdvDev* a, const AdvStepArgs& x, int iter, double* power, cudaStream_t s);
// h + eta from the current eta (after a state is loaded)
void adv_thickness(AdvDev* a, double h0, cudaStream_t s);
// step counter and the forcing phase of that step
void adv_set_step(AdvDev* a, long long step, double dt, cudaStream_t s);
int adv_kernels_per_step();
// captured graph of adv_graph_steps() steps (owned by AdvDev) and its power buffer
int adv_graph_steps();
double* adv_graph_power(AdvDev* a);
cudaGraphExec_t* adv_graph(AdvDev* a);
// flux[E]: the reference's interpolateLSQFlux of the column thickness h_total[N] with velocities v[E]
void adv_lsq_flux(AdvDev* a, double* flux, const double* v, const double* h_total, cudaStream_t s);
int adv_kernels_per_call();

}  // namespace odis
