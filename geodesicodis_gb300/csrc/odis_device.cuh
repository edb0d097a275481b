// Device-side data layout of the LTE step (shared by the kernels and the C ABI).
//
// All per-face and per-cell arrays are structure-of-arrays with the slot index
// outermost ([k][Ep] / [k][Np]), so that consecutive threads (consecutive
// faces or cells) read consecutive words: every coefficient load of a warp is
// one fully used 128-byte line (FP32) or two (FP64).  Ep and Np are padded
// to a multiple of 128.  Missing stencil entries (faces next to one of the
// twelve pentagons have 9 or 8 TRiSK neighbours, pentagons have 5 faces)
// carry weight 0 and point at the face/cell itself, so kernels need no
// branches and never read out of range.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace odis {

constexpr int kTrisk = 10;    // TRiSK stencil width
constexpr int kCellFaces = 6;

template <class T>
struct FaceCoef {
    const int* nbr;      // [10][Ep] TRiSK neighbour faces
    const T* w;          // [10][Ep] w_ee' * l_e' / d_e
    const int* n0;       // [Ep] first node (face_nodes(e,0))
    const int* n1;       // [Ep] second node
    const T* gg0;        // [Ep] -g * (-m_e0 / d_e)
    const T* gg1;        // [Ep] -g * ( m_e1 / d_e)
    const T* cor;        // [Ep] -2 Omega sin(lat of face centre)
    const T* fP;         // [Ep] (G Ua)_e : forcing gradient, cos(M) part
    const T* fQ;         // [Ep] (G Ub)_e : forcing gradient, sin(M) part
    const T* diss;       // [Ep] alpha * 1000 * h * A_e / (4 pi r^2)
};

template <class T>
struct CellCoef {
    const int* edge;     // [6][Np] faces of the cell
    const T* hw;         // [6][Np] h * (-dir * l_e / A_i)
};

// Step constants (identical for every step of a run).
struct StepConst {
    int E, N, Ep, Np;
    double dt, alpha, angvel;
    double ab3a, ab3b, ab3c;  // 23/12, -16/12, 5/12
    int init_load;            // 1: AB3 from the first step
    int use_sg;               // 1: add the self-gravity / loading potential
    int quad;                 // 1: QUADRATIC friction (dissipation diss_e |u|^3 instead of diss_e |u|^2)
    // the same constants as double-float (hi, lo) pairs for the ODIS_DF64 method
    float2 df_dt, df_malpha, df_a, df_b, df_c;
    // and rounded to FP32 for the FP32-state variant (no per-thread conversions)
    float f_dt, f_malpha, f_a, f_b, f_c;
};

// Mutable state of one instance.  The time level of v alternates between
// v[0] and v[1]; the AB3 history alternates between hv[0] and hv[1]:
// step `it` reads v[it&1], writes v[(it+1)&1], reads f(it-1) from
// hv[(it+1)&1] and f(it-2) from hv[it&1] and then stores f(it) in hv[it&1].
// The FP32-state variant keeps v and eta as double-float pairs: the FP32 value
// the stencils gather (v, eta) plus its rounding residual (vlo, etalo), which
// only the owning thread reads and writes.  The AB3 increment, formed in FP32
// from FP32 stencils, is accumulated into the pair with an error-free FP32
// two-sum, i.e. at FP64 accuracy without FP64 instructions (GB300's FP64 and
// FP64-conversion rates are a small fraction of its FP32 rate).
template <class T>
struct State {
    T* v[2];
    float* vlo;          // FP32 variant: rounding residual of v (nullptr otherwise)
    T* hv[2];
    T* eta;
    float* etalo;        // FP32 variant: rounding residual of eta
    T* he[2];
    const T* usg;        // [N] self-gravity potential / g (nullable)
    const long long* iter;   // device step counter (base of the current chunk)
    const long long* run_first;  // first step index of the current run
    const T* phase;      // [2n] cos, sin of the forcing phase Omega*t^{n+1} for each step of the current run
    double* partial;     // [steps of the run chunk + 1][edge blocks] per-block dissipation partial sums
    double* power;       // [n] output power series of the current run chunk (nullable; written by the fold only)
    int* status;         // device status word
};

}  // namespace odis
