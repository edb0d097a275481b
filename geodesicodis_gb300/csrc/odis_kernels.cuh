// Launchers of the LTE kernels (odis_kernels.cu), called by the C ABI.
#pragma once

#include "../../include/odis_gpu.h"
#include "odis_device.cuh"
#include "odis_forcing.cuh"

namespace odis {

constexpr int kStepThreads = 256;

template <class T, bool kMaster>
void launch_edge(const FaceCoef<T>& fc, const State<T>& st, const StepConst& sc, int offset, cudaStream_t s);
template <class T, bool kMaster>
void launch_cell(const CellCoef<T>& cc, const State<T>& st, const StepConst& sc, int offset, cudaStream_t s);
template <class T, bool kMaster>
void launch_step(const FaceCoef<T>& fc, const CellCoef<T>& cc, const State<T>& st, const StepConst& sc,
                 int offset, cudaStream_t s);
template <class T>
void launch_power_tail(const FaceCoef<T>& fc, const State<T>& st, const StepConst& sc, int n, cudaStream_t s);
// power[k] = sum of row k+1 of a run's partial table [n+1][nb] (no-op without power)
void launch_power_fold(const double* part, int nb, int n, double* power, cudaStream_t s);
// uxyz[i][c] = sum_j rbf[(c*6+j)*Np + i] * v[edge[j*Np + i]]
void launch_rbf(const double* rbf, const int* edge, int N, int Np, const double* v, double* uxyz, cudaStream_t s);
// CTAs of the face step kernel: one face per thread, or a face pair per thread (FP32 variant)
int face_blocks(const StepConst& sc, bool pairs);
void launch_bump(long long* iter, int n, cudaStream_t s);
// forcing-phase table of a run: out[2k], out[2k+1] = cos, sin of Omega*(dt*(first+k) + dt)
void launch_phase(void* out, int precision, long long first, int n, double dt, double angvel, cudaStream_t s);

// ODIS_DF64 method (odis_kernels_df.cu)
void launch_edge_df(const FaceCoef<float2>& fc, const State<float2>& st, const StepConst& sc, int offset, cudaStream_t s);
void launch_cell_df(const CellCoef<float2>& cc, const State<float2>& st, const StepConst& sc, int offset, cudaStream_t s);
void launch_power_tail_df(const FaceCoef<float2>& fc, const State<float2>& st, const StepConst& sc, int n, cudaStream_t s);

void launch_momentum(const FaceCoef<double>& fc, int E, int Ep, double* dvdt, const double* v, const double* eta,
                     cudaStream_t s);
void launch_divergence(const CellCoef<double>& cc, int N, int Np, double* q, const double* v, cudaStream_t s);
void launch_ab3_ref(double* x, double* h, int iter, int num, double dt, int init_load, cudaStream_t s);
void launch_interp(const FaceCoef<double>& fc, const double* nrm, int E, int Ep, double* uv, const double* v,
                   cudaStream_t s);
int energy_blocks(int E);
// Dissipation coefficient of updateEnergy (src/energy.cpp:30-53): e_e = coef |u|^2
// for LINEAR friction (coef = alpha 1000 h) and coef |u|^3 for QUADRATIC
// (coef = alpha / h).
inline double energy_coef(const odis_params& p)
{
    return p.friction == ODIS_FRIC_QUADRATIC ? p.alpha / p.h : p.alpha * 1000.0 * p.h;
}

void launch_energy(const double* area, int E, double coef, int quad, double divisor, const double* uv, double* e_out,
                   double* partial, double* out, cudaStream_t s);

}  // namespace odis
