// Batched sweep: many ocean configurations, of uneven mesh level, advanced by
// one persistent cooperative kernel.
//
// Each member is one run of the time loop of src/timeIntegrator.cpp:205-272
// (linear branch, same operators as the single-instance kernels) with its own
// thickness h, drag alpha, eccentricity, obliquity and steps per orbit.  The
// state is FP32 (the stencils gather FP32 values) and the AB3 accumulation is
// kept at FP64 accuracy as a double-float master (hi, lo) pair: hi is the FP32
// value the stencils read, lo the rounding residual that only the owning thread
// reads and writes.  The dissipated power is summed in FP32 per thread and per
// quad within a CTA's share of a group (non-negative terms) and in FP64 beyond.
//
// Layout.  Members are grouped by mesh; inside a group they are sorted by
// steps per orbit (descending) and padded to a multiple of four.  Every state
// array is instance-minor, [row][member]: one face or cell row holds the
// group's members contiguously, so a thread handles one face (or cell) for a
// quad of four members with float4 loads, the mesh coefficients are read once
// per quad (one broadcast load per warp row) instead of once per member, and
// the neighbour gathers of a warp read whole rows.
//
// Schedule.  One launch runs a chunk of steps j of the current run.  Per step:
// face phase (tiles of every group, grid-stride over CTAs), grid barrier, cell
// phase plus the fold of the per-CTA power partials of the face phase, grid
// barrier.  Members stop updating once they have made their own number of
// steps; the sort makes whole quads retire together except at group borders.
// Every barrier wait is bounded: on timeout the CTA records ODIS_ERR_TIMEOUT
// and returns, so the launch always ends.
#include "../../include/odis_gpu.h"
#include "odis_internal.h"
#include "odis_forcing.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <numeric>
#include <vector>

namespace odis {
namespace {

constexpr int kBatchThreads = 256;
constexpr int kRowChoices[3] = {1, 2, 4};  // face / cell rows per thread per tile: a template choice, timed at creation
constexpr int kMaxQuads = kBatchThreads; // members per group <= 4 * 256
constexpr int kMaxGroups = 32;
constexpr unsigned kBarrierSpins = 1u << 22;
constexpr double kPiB = 3.1415926535897932384626433832795028841971693993751058;

struct GroupDev {
    int E, N, Bq, ny;                  // rows, quads of members, tile height (rows per thread pass)
    int ftile0, ftiles, ctile0, ctiles;
    int moff;                          // first padded member slot of the group
    const int* nbr;                    // [10][E]
    const float* w;                    // [10][E]  w_ee' l_e' / d_e
    const int* n0;
    const int* n1;
    const float* gg0;                  // -g (-m_e0 / d_e)
    const float* gg1;                  // -g ( m_e1 / d_e)
    const float* cor;                  // -2 Omega sin(lat_e)
    const float* pe;                   // G of the unit-eccentricity forcing, cos part
    const float* qe;                   //                                     sin part
    const float* po;                   // G of the unit-obliquity forcing, cos part
    const float* qo;                   //                                  sin part
    const float* dbase;                // 1000 A_e / (4 pi r^2)
    const int* edge;                   // [6][N] faces of the cell
    const float* dv;                   // [6][N] -dir l_e / A_i (missing faces weight 0)
    float* vhi[2];                     // [E][4 Bq]
    float* vlo;
    float* hv[2];
    float* ehi;                        // [N][4 Bq]
    float* elo;
    float* he[2];
};

struct MemberDev {                     // structure of arrays over padded member slots
    const float* dt;
    const float* malpha;               // -alpha
    const float* h;
    const float* ecc;
    const float* obl;
    const float* dah;                  // alpha * h
    const int* n;                      // steps per orbit
    const int* S;                      // steps of the current run
    const int* base;                   // step index at the start of the current run
    const int* user;                   // caller's member index (-1: padding)
};

struct BatchArgs {
    const GroupDev* groups;
    int ngroups, ftiles, ctiles, P;    // P: padded member slots
    MemberDev mem;
    double* part;                      // [2][gridDim][P]
    double* step_power;                // [user][step_stride] (nullable)
    int step_stride;
    double* orbit_power;               // [user][orbit_stride] (nullable)
    int orbit_stride;
    unsigned* bar_count;
    unsigned* bar_gen;
    int* status;
    int init_load;
    float ab3a, ab3b, ab3c;
    unsigned spin_limit;               // polls of one barrier wait before it gives up
    int withhold;                      // >= 0: this CTA never arrives at a barrier (failure-detection test hook)
};

__device__ __forceinline__ float4 f4(float s) { return make_float4(s, s, s, s); }
__device__ __forceinline__ float4 fma4(float a, float4 b, float4 c)
{
    return make_float4(fmaf(a, b.x, c.x), fmaf(a, b.y, c.y), fmaf(a, b.z, c.z), fmaf(a, b.w, c.w));
}
__device__ __forceinline__ float4 fma4v(float4 a, float4 b, float4 c)
{
    return make_float4(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y), fmaf(a.z, b.z, c.z), fmaf(a.w, b.w, c.w));
}
__device__ __forceinline__ float4 mul4(float a, float4 b) { return make_float4(a * b.x, a * b.y, a * b.z, a * b.w); }
__device__ __forceinline__ float4 mul4v(float4 a, float4 b) { return make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
__device__ __forceinline__ float4 add4v(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ float4 sel4(int4 m, float4 a, float4 b)
{
    return make_float4(m.x ? a.x : b.x, m.y ? a.y : b.y, m.z ? a.z : b.z, m.w ? a.w : b.w);
}

// (hi, lo) += x in double-float arithmetic (Knuth two-sum, then renormalise).
__device__ __forceinline__ void df_acc(float& hi, float& lo, float x)
{
    const float s = __fadd_rn(hi, x);
    const float bb = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
    const float t = __fadd_rn(lo, err);
    const float h2 = __fadd_rn(s, t);
    lo = __fsub_rn(t, __fsub_rn(h2, s));
    hi = h2;
}
__device__ __forceinline__ void df_acc4(float4& hi, float4& lo, float4 x)
{
    df_acc(hi.x, lo.x, x.x);
    df_acc(hi.y, lo.y, x.y);
    df_acc(hi.z, lo.z, x.z);
    df_acc(hi.w, lo.w, x.w);
}

// store only the components selected by m (all four: one vector store)
__device__ __forceinline__ void st4m(float4* p, float4 v, int4 m)
{
    if (m.x && m.y && m.z && m.w) { *p = v; return; }
    float* q = reinterpret_cast<float*>(p);
    if (m.x) q[0] = v.x;
    if (m.y) q[1] = v.y;
    if (m.z) q[2] = v.z;
    if (m.w) q[3] = v.w;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned* p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid-wide barrier of a cooperative launch with a bounded wait; returns false
// (in every thread of the CTA) if this CTA gave up waiting.
__device__ bool grid_barrier(const BatchArgs& a, int* s_ok)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned gen = ld_acquire(a.bar_gen);
        __threadfence();
        const unsigned arrived = (int)blockIdx.x == a.withhold ? 0u : atomicAdd(a.bar_count, 1u);
        if ((int)blockIdx.x != a.withhold && arrived == gridDim.x - 1) {
            atomicExch(a.bar_count, 0u);
            __threadfence();
            st_release(a.bar_gen, gen + 1);
        } else {
            unsigned spins = 0;
            while (ld_acquire(a.bar_gen) == gen) {
                if (++spins > a.spin_limit) { ok = 0; atomicOr(a.status, 1 << ODIS_ERR_TIMEOUT); break; }
                __nanosleep(32);
            }
        }
        __threadfence();
        *s_ok = ok;
    }
    __syncthreads();
    return *s_ok != 0;
}

struct QuadInfo {
    float4 dt, malpha, ce, co, se, so;   // forcing weights: cos/sin of the phase times eccentricity/obliquity
    float4 w;                            // face phase: alpha * h (dissipation); cell phase: h
    unsigned mask;                       // bits 0-3 member advances, 4-7 its power is recorded, 8-11 forward-Euler step
};

__device__ __forceinline__ int4 bits4(unsigned m, int shift)
{
    return make_int4((m >> shift) & 1u, (m >> (shift + 1)) & 1u, (m >> (shift + 2)) & 1u, (m >> (shift + 3)) & 1u);
}

__device__ __forceinline__ QuadInfo quad_info(const BatchArgs& a, int slot, int j, const float* s_cos,
                                              const float* s_sin, bool face)
{
    QuadInfo q;
    const MemberDev& m = a.mem;
    const int4 S = __ldg(reinterpret_cast<const int4*>(m.S + slot));
    const int4 b = __ldg(reinterpret_cast<const int4*>(m.base + slot));
    const int Sv[4] = {S.x, S.y, S.z, S.w}, bv[4] = {b.x, b.y, b.z, b.w};
    unsigned mask = 0;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        mask |= (unsigned)(j < Sv[c]) << c;
        mask |= (unsigned)(j >= 1 && j <= Sv[c]) << (4 + c);
        mask |= (unsigned)!(a.init_load || bv[c] + j > 1) << (8 + c);
    }
    q.mask = mask;
    q.dt = __ldg(reinterpret_cast<const float4*>(m.dt + slot));
    if (face) {
        q.malpha = __ldg(reinterpret_cast<const float4*>(m.malpha + slot));
        const float4 ecc = __ldg(reinterpret_cast<const float4*>(m.ecc + slot));
        const float4 obl = __ldg(reinterpret_cast<const float4*>(m.obl + slot));
        const float4 cm = *reinterpret_cast<const float4*>(s_cos + slot);
        const float4 sm = *reinterpret_cast<const float4*>(s_sin + slot);
        q.ce = mul4v(cm, ecc);
        q.co = mul4v(cm, obl);
        q.se = mul4v(sm, ecc);
        q.so = mul4v(sm, obl);
        q.w = __ldg(reinterpret_cast<const float4*>(m.dah + slot));
    } else {
        q.w = __ldg(reinterpret_cast<const float4*>(m.h + slot));
    }
    return q;
}

// Face phase of step j for one tile; returns the tile's power partial of this
// thread's quad (components outside pow_on are zero).  State arrays are read
// with plain (L1-cacheable) loads: the grid barrier before each phase is an
// acquire at GPU scope, so no line cached before it is used after it.
template <int R>
__device__ __forceinline__ float4 face_tile(const BatchArgs& a, const GroupDev& G, const QuadInfo& q, int x, int y,
                                            int ny, int e0, int j, bool& bad)
{
    const int Bq = G.Bq, E = G.E, p = j & 1;
    const float4* __restrict__ vcur = reinterpret_cast<const float4*>(p ? G.vhi[1] : G.vhi[0]);
    float4* __restrict__ vnext = reinterpret_cast<float4*>(p ? G.vhi[0] : G.vhi[1]);
    float4* __restrict__ vlo = reinterpret_cast<float4*>(G.vlo);
    float4* __restrict__ hcur = reinterpret_cast<float4*>(p ? G.hv[1] : G.hv[0]);            // f(j-2) in, f(j) out
    const float4* __restrict__ hprev = reinterpret_cast<const float4*>(p ? G.hv[0] : G.hv[1]); // f(j-1)
    const float4* __restrict__ eta = reinterpret_cast<const float4*>(G.ehi);
    const int* __restrict__ nbr = G.nbr;
    const float* __restrict__ w = G.w;
    float4 pw = f4(0.f);
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int e = e0 + y + ny * r;
        if (e < E) {
            float4 ts = f4(0.f);
#pragma unroll
            for (int k = 0; k < 10; k++) ts = fma4(__ldg(&w[k * E + e]), vcur[(size_t)__ldg(&nbr[k * E + e]) * Bq + x], ts);
            const size_t o = (size_t)e * Bq + x;
            const float4 ve = vcur[o];
            if (q.mask & 0xF0u) {
                const float4 ke = fma4v(ve, ve, mul4v(ts, ts));
                const float4 d = mul4(__ldg(&G.dbase[e]), mul4v(q.w, ke));
                pw = add4v(pw, sel4(bits4(q.mask, 4), d, f4(0.f)));
            }
            if (q.mask & 0xFu) {
                const int4 upd = bits4(q.mask, 0);
                const int i0 = __ldg(&G.n0[e]), i1 = __ldg(&G.n1[e]);
                const float g0 = __ldg(&G.gg0[e]), g1 = __ldg(&G.gg1[e]);
                const float4 f0 = fma4(__ldg(&G.cor[e]), ts, fma4(g0, eta[(size_t)i0 * Bq + x], mul4(g1, eta[(size_t)i1 * Bq + x])));
                const float4 gu = fma4v(q.ce, f4(__ldg(&G.pe[e])), fma4v(q.co, f4(__ldg(&G.po[e])),
                                        fma4v(q.se, f4(__ldg(&G.qe[e])), mul4v(q.so, f4(__ldg(&G.qo[e]))))));
                const float4 drag = fma4v(q.malpha, ve, gu);
                const float4 f1 = hprev[o], f2 = hcur[o];
                const float4 ab = fma4(a.ab3c, f2, fma4(a.ab3b, f1, mul4(a.ab3a, f0)));
                const float4 inc = sel4(bits4(q.mask, 8), f0, ab);
                st4m(&hcur[o], f0, upd);
                float4 hi = ve, lo = vlo[o];
                df_acc4(hi, lo, mul4v(q.dt, add4v(inc, drag)));
                st4m(&vnext[o], hi, upd);
                st4m(&vlo[o], lo, upd);
                bad |= (upd.x && !isfinite(hi.x)) || (upd.y && !isfinite(hi.y)) || (upd.z && !isfinite(hi.z)) ||
                       (upd.w && !isfinite(hi.w));
            }
        }
    }
    return pw;
}

template <int R>
__device__ __forceinline__ void cell_tile(const GroupDev& G, const QuadInfo& q, const BatchArgs& a, int x, int y,
                                          int ny, int c0, int j)
{
    const int Bq = G.Bq, N = G.N, p = j & 1;
    const float4* __restrict__ vn = reinterpret_cast<const float4*>(p ? G.vhi[0] : G.vhi[1]);
    float4* __restrict__ hcur = reinterpret_cast<float4*>(p ? G.he[1] : G.he[0]);
    const float4* __restrict__ hprev = reinterpret_cast<const float4*>(p ? G.he[0] : G.he[1]);
    float4* __restrict__ ehi = reinterpret_cast<float4*>(G.ehi);
    float4* __restrict__ elo = reinterpret_cast<float4*>(G.elo);
    const int* __restrict__ edge = G.edge;
    const float* __restrict__ dv = G.dv;
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int i = c0 + y + ny * r;
        if (i < N) {
            float4 qd = f4(0.f);
#pragma unroll
            for (int k = 0; k < 6; k++) qd = fma4(__ldg(&dv[k * N + i]), vn[(size_t)__ldg(&edge[k * N + i]) * Bq + x], qd);
            qd = mul4v(q.w, qd);
            const size_t o = (size_t)i * Bq + x;
            const float4 f1 = hprev[o], f2 = hcur[o];
            const float4 ab = fma4(a.ab3c, f2, fma4(a.ab3b, f1, mul4(a.ab3a, qd)));
            const int4 upd = bits4(q.mask, 0);
            const float4 inc = sel4(bits4(q.mask, 8), qd, ab);
            st4m(&hcur[o], qd, upd);
            float4 hi = ehi[o], lo = elo[o];
            df_acc4(hi, lo, mul4v(q.dt, inc));
            st4m(&ehi[o], hi, upd);
            st4m(&elo[o], lo, upd);
        }
    }
}

// Adds the per-thread FP32 power sums of group g's quads (threads x = tid % qa,
// y = tid / qa < ny) to the CTA's FP64 accumulators.  Called by every thread.
__device__ __forceinline__ void fold_group_power(const BatchArgs& a, int g, int qa, int ny, float4 pw, float4* s_pw,
                                                 double* s_acc)
{
    const int tid = threadIdx.x;
    s_pw[tid] = tid < qa * ny ? pw : f4(0.f);
    __syncthreads();
    if (tid < qa) {
        float4 sm = f4(0.f);
        for (int yy = 0; yy < ny; yy++) sm = add4v(sm, s_pw[yy * qa + tid]);
        double* acc = s_acc + a.groups[g].moff + 4 * tid;
        acc[0] += (double)sm.x;
        acc[1] += (double)sm.y;
        acc[2] += (double)sm.z;
        acc[3] += (double)sm.w;
    }
    __syncthreads();
}

// Active quads of group g at step j: members are sorted by run length
// (descending), so the quads whose first member still updates or records power
// (S >= max(j, 1)) are a prefix; binary search over the quads' first slots.
__device__ __forceinline__ int active_quads(const BatchArgs& a, const GroupDev& G, int j)
{
    const int need = j > 1 ? j : 1;
    int lo = 0, hi = G.Bq;                       // first quad with S < need
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&a.mem.S[G.moff + 4 * mid]) >= need) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

template <int R>
__global__ void __launch_bounds__(kBatchThreads) k_batch(BatchArgs a, int j0, int j1)
{
    extern __shared__ double s_dyn[];
    double* s_acc = s_dyn;                                   // [P] power of this CTA's tiles, per member slot
    float* s_cos = reinterpret_cast<float*>(s_dyn + a.P);    // [P] forcing phase of this step, per member slot
    float* s_sin = s_cos + a.P;
    __shared__ float4 s_pw[kBatchThreads];
    __shared__ double s_red[kBatchThreads / 32];
    __shared__ int s_qa[kMaxGroups], s_ny[kMaxGroups], s_ft0[kMaxGroups + 1], s_ct0[kMaxGroups + 1];
    __shared__ int s_ok, s_bad;
    const int tid = threadIdx.x;
    const int ng = a.ngroups;
    // a previous chunk of this run gave up on a barrier: the run is over
    if (*(volatile const int*)a.status & (1 << ODIS_ERR_TIMEOUT)) return;
    if (tid == 0) s_bad = 0;
    for (int j = j0; j < j1; j++) {
        // ---- per-step tables: forcing phase of every member, active quads and tiles of every group ----
        for (int k = tid; k < a.P; k += blockDim.x) {
            s_acc[k] = 0.0;
            // Omega t^{k+1} = 2 pi ((k+1) mod n) / n with dt = P / n
            const int n = max(__ldg(&a.mem.n[k]), 1);
            const int r = (int)(((long long)__ldg(&a.mem.base[k]) + j + 1) % n);
            sincospif(2.0f * (float)r / (float)n, &s_sin[k], &s_cos[k]);
        }
        if (tid < ng) {
            const GroupDev& G = a.groups[tid];
            const int qa = active_quads(a, G, j);
            const int ny = qa ? kBatchThreads / qa : 1;
            const int rows = ny * R;
            s_qa[tid] = qa;
            s_ny[tid] = ny;
            s_ft0[tid + 1] = qa ? (G.E + rows - 1) / rows : 0;
            s_ct0[tid + 1] = qa ? (G.N + rows - 1) / rows : 0;
        }
        __syncthreads();
        if (tid == 0) {
            s_ft0[0] = 0;
            s_ct0[0] = 0;
            for (int g = 0; g < ng; g++) {
                s_ft0[g + 1] += s_ft0[g];
                s_ct0[g + 1] += s_ct0[g];
            }
        }
        __syncthreads();
        // ---- face phase ----
        // Power: each thread sums its quad's faces over all of this CTA's tiles of a group in FP32
        // (non-negative terms); the block folds the threads of a quad once per group, into FP64.
        bool bad = false;
        float4 pw = f4(0.f);
        int cur = -1;
        for (int t = blockIdx.x; t < s_ft0[ng]; t += gridDim.x) {
            int g = 0;
            while (g + 1 < ng && t >= s_ft0[g + 1]) g++;
            if (g != cur) {                                          // uniform over the CTA
                if (cur >= 0) fold_group_power(a, cur, s_qa[cur], s_ny[cur], pw, s_pw, s_acc);
                cur = g;
                pw = f4(0.f);
            }
            const GroupDev& G = a.groups[g];
            const int qa = s_qa[g], ny = s_ny[g];
            const int x = tid % qa, y = tid / qa;
            if (y < ny) {
                const QuadInfo q = quad_info(a, G.moff + 4 * x, j, s_cos, s_sin, true);
                if (q.mask & 0xFFu)
                    pw = add4v(pw, face_tile<R>(a, G, q, x, y, ny, (t - s_ft0[g]) * ny * R, j, bad));
            }
        }
        if (cur >= 0) fold_group_power(a, cur, s_qa[cur], s_ny[cur], pw, s_pw, s_acc);
        if (bad) s_bad = 1;
        double* part = a.part + (size_t)(j & 1) * gridDim.x * a.P + (size_t)blockIdx.x * a.P;
        for (int k = tid; k < a.P; k += blockDim.x) __stcg(&part[k], s_acc[k]);
        if (!grid_barrier(a, &s_ok)) return;
        // ---- fold of the power partials of step j, then the cell phase ----
        const double* pj = a.part + (size_t)(j & 1) * gridDim.x * a.P;
        for (int b = blockIdx.x; b < a.P; b += gridDim.x) {
            const int u = __ldg(&a.mem.user[b]);
            const int S = __ldg(&a.mem.S[b]);
            if (u < 0 || j < 1 || j > S) continue;               // uniform over the CTA
            double sm = 0.0;
            for (int k = tid; k < (int)gridDim.x; k += blockDim.x) sm += __ldcg(&pj[(size_t)k * a.P + b]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) sm += __shfl_down_sync(0xffffffffu, sm, o);
            if ((tid & 31) == 0) s_red[tid >> 5] = sm;
            __syncthreads();
            if (tid == 0) {
                double t = 0.0;
                for (int w = 0; w < kBatchThreads / 32; w++) t += s_red[w];
                if (a.step_power) a.step_power[(size_t)u * a.step_stride + (j - 1)] = t;
                if (a.orbit_power) {
                    const int n = __ldg(&a.mem.n[b]);
                    a.orbit_power[(size_t)u * a.orbit_stride + (j - 1) / n] += t / n;
                }
            }
            __syncthreads();
        }
        for (int t = blockIdx.x; t < s_ct0[ng]; t += gridDim.x) {
            int g = 0;
            while (g + 1 < ng && t >= s_ct0[g + 1]) g++;
            const GroupDev& G = a.groups[g];
            const int qa = s_qa[g], ny = s_ny[g];
            const int x = tid % qa, y = tid / qa;
            if (y < ny) {
                const QuadInfo q = quad_info(a, G.moff + 4 * x, j, s_cos, s_sin, false);
                if (q.mask & 0xFu) cell_tile<R>(G, q, a, x, y, ny, (t - s_ct0[g]) * ny * R, j);
            }
        }
        if (j + 1 < j1 && !grid_barrier(a, &s_ok)) return;
        __syncthreads();                                     // per-step tables are rewritten next step
    }
    __syncthreads();
    if (tid == 0 && s_bad) atomicOr(a.status, 1 << ODIS_ERR_NONFINITE);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct Arena {
    std::vector<void*> ptrs;
    template <class T>
    T* alloc(size_t n) {
        void* p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T) + 16) != cudaSuccess) return nullptr;
        cudaMemset(p, 0, std::max<size_t>(n, 1) * sizeof(T) + 16);
        ptrs.push_back(p);
        return (T*)p;
    }
    template <class T>
    T* upload(const std::vector<T>& h) {
        T* d = alloc<T>(h.size());
        if (d && !h.empty()) cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
        return d;
    }
    ~Arena() { for (void* p : ptrs) cudaFree(p); }
};

}  // namespace
}  // namespace odis

using namespace odis;

struct odis_batch {
    odis_params p{};
    int count = 0, P = 0;
    double period = 0.0;
    std::vector<GroupDev> groups;
    std::vector<int> slot_of;            // user member -> padded slot
    std::vector<int> group_of;           // user member -> group
    std::vector<odis_batch_member> members;
    std::vector<int> base;               // per slot
    std::vector<int> n;                  // per slot
    Arena mem;
    GroupDev* d_groups = nullptr;
    MemberDev md{};
    int* d_S = nullptr;
    int* d_base = nullptr;
    double* d_part = nullptr;
    unsigned* d_bar = nullptr;           // [0] count, [1] generation
    bool use_graph = true;               // runs replay their chunk launches from one CUDA graph
    long long graph_runs = 0;            // runs executed as one graph launch
    unsigned spin_limit = 0;             // odis_batch_set_wait_limit: polls of a barrier wait (0: kBarrierSpins)
    int withhold = -1;                   // odis_batch_set_wait_limit: CTA that never arrives (-1: none)
    int* d_status = nullptr;
    int grid = 0;                        // CTAs of the chosen variant
    int variant = 2;                     // index into kRowChoices
    int grid_v[3] = {0, 0, 0};           // co-resident CTAs of each variant (0: cannot launch)
    int ftiles = 0, ctiles = 0;
    cudaStream_t stream = nullptr;
    long long launches = 0;
    ~odis_batch() {
        if (stream) cudaStreamDestroy(stream);
    }
};

#define ODIS_BCK(call)                                 \
    do {                                               \
        cudaError_t _e = (call);                       \
        if (_e != cudaSuccess) return ODIS_ERR_CUDA;   \
    } while (0)

static const void* batch_kernel(int v)
{
    return v == 0 ? (const void*)k_batch<1> : v == 1 ? (const void*)k_batch<2> : (const void*)k_batch<4>;
}

static void (*batch_kernel_fn(int v))(BatchArgs, int, int)
{
    return v == 0 ? k_batch<1> : v == 1 ? k_batch<2> : k_batch<4>;
}

static int zero_state(odis_batch* b)
{
    for (GroupDev& G : b->groups) {
        const size_t ev = (size_t)G.E * 4 * G.Bq, cv = (size_t)G.N * 4 * G.Bq;
        for (int k = 0; k < 2; k++) {
            ODIS_BCK(cudaMemset(G.vhi[k], 0, sizeof(float) * ev));
            ODIS_BCK(cudaMemset(G.hv[k], 0, sizeof(float) * ev));
            ODIS_BCK(cudaMemset(G.he[k], 0, sizeof(float) * cv));
        }
        ODIS_BCK(cudaMemset(G.vlo, 0, sizeof(float) * ev));
        ODIS_BCK(cudaMemset(G.ehi, 0, sizeof(float) * cv));
        ODIS_BCK(cudaMemset(G.elo, 0, sizeof(float) * cv));
    }
    std::fill(b->base.begin(), b->base.end(), 0);
    return ODIS_OK;
}

// Rows per thread per tile: ODIS_BATCH_ROWS=1|2|4 fixes it; otherwise each
// variant runs 24 steps from rest (after a 4-step warm-up) and the fastest is
// kept.  The members are then put back at rest, step 0.
static int choose_rows(odis_batch* b)
{
    const char* e = std::getenv("ODIS_BATCH_ROWS");
    int forced = -1;
    if (e) for (int v = 0; v < 3; v++) if (std::atoi(e) == kRowChoices[v]) forced = v;
    double best = 1e300;
    int pick = -1;
    for (int v = 0; v < 3; v++) {
        if (!b->grid_v[v] || (forced >= 0 && v != forced)) continue;
        b->variant = v;
        b->grid = b->grid_v[v];
        if (forced >= 0) { pick = v; break; }
        int st = odis_batch_run(b, 0.0, 4, nullptr, 0, nullptr, 0, 0);
        const auto t0 = std::chrono::steady_clock::now();
        if (st == ODIS_OK || st == ODIS_ERR_NONFINITE) st = odis_batch_run(b, 0.0, 24, nullptr, 0, nullptr, 0, 0);
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (st != ODIS_OK && st != ODIS_ERR_NONFINITE) return st;
        if (ms < best) { best = ms; pick = v; }
    }
    if (pick < 0) return ODIS_ERR_CUDA;
    b->variant = pick;
    b->grid = b->grid_v[pick];
    b->launches = 0;
    return zero_state(b);
}

static int build_group(odis_batch* b, const Mesh& m, GroupDev& G)
{
    const int E = m.E, N = m.N;
    std::vector<int> nbr((size_t)10 * E), n0(E), n1(E), edge((size_t)6 * N);
    std::vector<float> w((size_t)10 * E, 0.f), gg0(E), gg1(E), cor(E), pe(E), qe(E), po(E), qo(E), dbase(E);
    std::vector<float> dv((size_t)6 * N, 0.f);
    odis_params pe_p = b->p, po_p = b->p;
    pe_p.ecc = 1.0;
    pe_p.obliq = 0.0;
    po_p.ecc = 0.0;
    po_p.obliq = 1.0;
    std::vector<double> Uae, Ube, Uao, Ubo;
    int st = forcing_basis(m, pe_p, Uae, Ube);
    if (st != ODIS_OK) return st;
    st = forcing_basis(m, po_p, Uao, Ubo);
    if (st != ODIS_OK) return st;
    const double four_pi_r2 = 4 * kPiB * m.r * m.r;
    for (int e = 0; e < E; e++) {
        for (int k = 0; k < 10; k++) {
            const bool ok = k < m.interp_n[e];
            const int f = ok ? m.interp_friends[(size_t)e * 10 + k] : e;
            nbr[(size_t)k * E + e] = f;
            w[(size_t)k * E + e] = ok ? (float)(m.interp_w[(size_t)e * 10 + k] * m.face_len[f] / m.face_dist[e]) : 0.f;
        }
        const int a0 = m.face_nodes[(size_t)e * 2], a1 = m.face_nodes[(size_t)e * 2 + 1];
        n0[e] = a0;
        n1[e] = a1;
        const double d = m.face_dist[e];
        const double g0 = (-m.face_m[(size_t)e * 2]) / d, g1 = (m.face_m[(size_t)e * 2 + 1]) / d;
        gg0[e] = (float)(-b->p.g * g0);
        gg1[e] = (float)(-b->p.g * g1);
        cor[e] = (float)(-2.0 * b->p.angvel * std::sin(m.face_centre[(size_t)e * 2]));
        pe[e] = (float)(g0 * Uae[a0] + g1 * Uae[a1]);
        qe[e] = (float)(g0 * Ube[a0] + g1 * Ube[a1]);
        po[e] = (float)(g0 * Uao[a0] + g1 * Uao[a1]);
        qo[e] = (float)(g0 * Ubo[a0] + g1 * Ubo[a1]);
        dbase[e] = (float)(1000.0 * m.face_area[e] / four_pi_r2);
    }
    for (int i = 0; i < N; i++) {
        const int k5 = m.nfriends(i);
        for (int k = 0; k < 6; k++) {
            const bool ok = k < k5;
            const int f = ok ? m.faces[(size_t)i * 6 + k] : m.faces[(size_t)i * 6];
            edge[(size_t)k * N + i] = f;
            if (ok) dv[(size_t)k * N + i] = (float)(-m.node_face_dir[(size_t)i * 6 + k] * m.face_len[f] / m.cv_area[i]);
        }
    }
    for (int x : nbr) if (x < 0 || x >= E) return ODIS_ERR_MESH;
    for (int x : n0) if (x < 0 || x >= N) return ODIS_ERR_MESH;
    for (int x : n1) if (x < 0 || x >= N) return ODIS_ERR_MESH;
    for (int x : edge) if (x < 0 || x >= E) return ODIS_ERR_MESH;
    Arena& A = b->mem;
    G.E = E;
    G.N = N;
    G.nbr = A.upload(nbr);
    G.w = A.upload(w);
    G.n0 = A.upload(n0);
    G.n1 = A.upload(n1);
    G.gg0 = A.upload(gg0);
    G.gg1 = A.upload(gg1);
    G.cor = A.upload(cor);
    G.pe = A.upload(pe);
    G.qe = A.upload(qe);
    G.po = A.upload(po);
    G.qo = A.upload(qo);
    G.dbase = A.upload(dbase);
    G.edge = A.upload(edge);
    G.dv = A.upload(dv);
    const size_t ev = (size_t)E * 4 * G.Bq, cv = (size_t)N * 4 * G.Bq;
    for (int k = 0; k < 2; k++) {
        G.vhi[k] = A.alloc<float>(ev);
        G.hv[k] = A.alloc<float>(ev);
        G.he[k] = A.alloc<float>(cv);
    }
    G.vlo = A.alloc<float>(ev);
    G.ehi = A.alloc<float>(cv);
    G.elo = A.alloc<float>(cv);
    if (!G.nbr || !G.w || !G.n0 || !G.n1 || !G.gg0 || !G.gg1 || !G.cor || !G.pe || !G.qe || !G.po || !G.qo ||
        !G.dbase || !G.edge || !G.dv || !G.vhi[0] || !G.vhi[1] || !G.hv[0] || !G.hv[1] || !G.he[0] || !G.he[1] ||
        !G.vlo || !G.ehi || !G.elo)
        return ODIS_ERR_NOMEM;
    return ODIS_OK;
}

extern "C" odis_status odis_batch_create(const odis_params* common, const odis_mesh* const* meshes, int n_meshes,
                                         const odis_batch_member* members, int count, odis_batch** out)
{
    if (!common || !meshes || n_meshes <= 0 || !members || count <= 0 || !out) return ODIS_ERR_ARG;
    *out = nullptr;
    if (!(common->g > 0.0) || !(common->radius > 0.0) || !(common->angvel > 0.0)) return ODIS_ERR_ARG;
    // a member's forcing is ecc x (the unit-eccentricity potential) + obliq x (the unit-obliquity one):
    // the single-frequency potentials (and the unforced types), not FULL2 / PLANET / GENERAL
    if (!pot_valid(common->potential) || pot_nodal(common->potential)) return ODIS_ERR_ARG;
    // the batch reports LINEAR dissipation (alpha 1000 h |u|^2) only
    if (common->friction != ODIS_FRIC_LINEAR) return ODIS_ERR_ARG;
    for (int k = 0; k < n_meshes; k++) if (!meshes[k]) return ODIS_ERR_ARG;
    for (int i = 0; i < count; i++) {
        const odis_batch_member& mb = members[i];
        if (mb.mesh < 0 || mb.mesh >= n_meshes || mb.steps_per_orbit <= 0 || (mb.steps_per_orbit & 1)) return ODIS_ERR_ARG;
        if (!(mb.h > 0.0) || mb.alpha < 0.0) return ODIS_ERR_ARG;
    }
    std::unique_ptr<odis_batch> b(new (std::nothrow) odis_batch);
    if (!b) return ODIS_ERR_NOMEM;
    b->p = *common;
    b->count = count;
    b->period = 2.0 * kPiB / common->angvel;
    b->members.assign(members, members + count);
    // groups: one per mesh (split above 4 * kMaxQuads members), members sorted by steps per orbit, descending
    std::vector<std::vector<int>> by_mesh(n_meshes);
    for (int i = 0; i < count; i++) by_mesh[members[i].mesh].push_back(i);
    std::vector<std::vector<int>> glist;
    std::vector<int> gmesh;
    for (int k = 0; k < n_meshes; k++) {
        std::vector<int>& v = by_mesh[k];
        if (v.empty()) continue;
        std::stable_sort(v.begin(), v.end(), [&](int x, int y) { return members[x].steps_per_orbit > members[y].steps_per_orbit; });
        for (size_t s = 0; s < v.size(); s += 4 * kMaxQuads) {
            glist.emplace_back(v.begin() + s, v.begin() + std::min(v.size(), s + 4 * (size_t)kMaxQuads));
            gmesh.push_back(k);
        }
    }
    const int ng = (int)glist.size();
    if (ng > kMaxGroups || count > 8192) return ODIS_ERR_ARG;
    b->groups.resize(ng);
    b->slot_of.assign(count, -1);
    b->group_of.assign(count, -1);
    int P = 0, ft = 0, ct = 0;
    for (int g = 0; g < ng; g++) {
        GroupDev& G = b->groups[g];
        std::memset(&G, 0, sizeof(G));
        const Mesh& m = meshes[gmesh[g]]->m;
        G.Bq = (int)(glist[g].size() + 3) / 4;
        G.ny = kBatchThreads / G.Bq;
        G.moff = P;
        for (size_t s = 0; s < glist[g].size(); s++) {
            b->slot_of[glist[g][s]] = P + (int)s;
            b->group_of[glist[g][s]] = g;
        }
        P += 4 * G.Bq;
        const int st = build_group(b.get(), m, G);
        if (st != ODIS_OK) return st;
        const int rows = G.ny * 4;
        G.ftile0 = ft;
        G.ftiles = (G.E + rows - 1) / rows;
        ft += G.ftiles;
        G.ctile0 = ct;
        G.ctiles = (G.N + rows - 1) / rows;
        ct += G.ctiles;
    }
    b->P = P;
    b->ftiles = ft;
    b->ctiles = ct;
    std::vector<float> dt(P, 0.f), ma(P, 0.f), h(P, 0.f), ecc(P, 0.f), obl(P, 0.f), dah(P, 0.f);
    std::vector<int> user(P, -1);
    b->n.assign(P, 2);
    b->base.assign(P, 0);
    for (int i = 0; i < count; i++) {
        const int s = b->slot_of[i];
        const odis_batch_member& mb = members[i];
        dt[s] = (float)(b->period / mb.steps_per_orbit);
        ma[s] = (float)(-mb.alpha);
        h[s] = (float)mb.h;
        ecc[s] = (float)mb.ecc;
        obl[s] = (float)mb.obliq;
        dah[s] = (float)(mb.alpha * mb.h);
        b->n[s] = mb.steps_per_orbit;
        user[s] = i;
    }
    Arena& A = b->mem;
    b->md.dt = A.upload(dt);
    b->md.malpha = A.upload(ma);
    b->md.h = A.upload(h);
    b->md.ecc = A.upload(ecc);
    b->md.obl = A.upload(obl);
    b->md.dah = A.upload(dah);
    b->md.n = A.upload(b->n);
    b->md.user = A.upload(user);
    b->d_S = A.alloc<int>(P);
    b->d_base = A.alloc<int>(P);
    b->md.S = b->d_S;
    b->md.base = b->d_base;
    b->d_groups = A.upload(b->groups);
    b->d_bar = A.alloc<unsigned>(2);
    b->d_status = A.alloc<int>(1);
    if (!b->md.dt || !b->md.malpha || !b->md.h || !b->md.ecc || !b->md.obl || !b->md.dah || !b->md.n || !b->md.user ||
        !b->d_S || !b->d_base || !b->d_groups || !b->d_bar || !b->d_status)
        return ODIS_ERR_NOMEM;
    // one CTA per SM slot the kernel can keep resident: a cooperative launch needs them all co-resident
    int dev = 0, sms = 0, per_sm = 0, coop = 0;
    ODIS_BCK(cudaGetDevice(&dev));
    ODIS_BCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    ODIS_BCK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) return ODIS_ERR_CUDA;
    const size_t smem = (sizeof(double) + 2 * sizeof(float)) * (size_t)P;
    int gmax = 0;
    for (int v = 0; v < 3; v++) {
        const void* f = batch_kernel(v);
        if (smem > 48 * 1024) ODIS_BCK(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        ODIS_BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, kBatchThreads, smem));
        b->grid_v[v] = per_sm >= 1 ? sms * std::min(per_sm, 4) : 0;
        gmax = std::max(gmax, b->grid_v[v]);
    }
    if (gmax < 1) return ODIS_ERR_CUDA;
    b->d_part = A.alloc<double>((size_t)2 * gmax * P);
    if (!b->d_part) return ODIS_ERR_NOMEM;
    ODIS_BCK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    ODIS_BCK(cudaDeviceSynchronize());
    const int st = choose_rows(b.get());
    if (st != ODIS_OK) return st;
    *out = b.release();
    return ODIS_OK;
}

extern "C" void odis_batch_destroy(odis_batch* b)
{
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    delete b;
}

extern "C" odis_status odis_batch_info(const odis_batch* b, int* n_groups, int* padded_members, int* grid,
                                       long long* launches, int* rows_per_thread)
{
    if (!b) return ODIS_ERR_ARG;
    if (rows_per_thread) *rows_per_thread = kRowChoices[b->variant];
    if (n_groups) *n_groups = (int)b->groups.size();
    if (padded_members) *padded_members = b->P;
    if (grid) *grid = b->grid;
    if (launches) *launches = b->launches;
    return ODIS_OK;
}

extern "C" odis_status odis_batch_run(odis_batch* b, double orbits, int steps, double* orbit_power, int orbit_stride,
                                      double* step_power, int step_stride, int chunk)
{
    if (!b || !(orbits >= 0.0) || steps < 0 || (orbits > 0.0) == (steps > 0) || (steps & 1)) return ODIS_ERR_ARG;
    std::vector<int> S(b->P, 0);
    int smax = 0, omax = 0;
    for (int i = 0; i < b->count; i++) {
        const int s = b->slot_of[i];
        const double x = orbits * b->n[s];
        const long long run = orbits > 0.0 ? std::llround(x) : steps;
        // each member's step count must be a whole, even number (its state then ends in buffer 0)
        if (run > (1LL << 30) || (run & 1)) return ODIS_ERR_ARG;
        if (orbits > 0.0 && std::fabs(x - (double)run) > 1e-6 * std::max(1.0, x)) return ODIS_ERR_ARG;
        S[s] = (int)run;
        smax = std::max(smax, S[s]);
        omax = std::max(omax, (S[s] + b->n[s] - 1) / b->n[s]);
    }
    if (step_power && step_stride < smax) return ODIS_ERR_ARG;
    if (orbit_power && orbit_stride < omax) return ODIS_ERR_ARG;
    if (chunk <= 0) chunk = 2048;
    double* d_sp = nullptr;
    double* d_op = nullptr;
    const size_t sp_n = step_power ? (size_t)b->count * step_stride : 0, op_n = orbit_power ? (size_t)b->count * orbit_stride : 0;
    if (sp_n) ODIS_BCK(cudaMalloc(&d_sp, sp_n * sizeof(double)));
    if (op_n && cudaMalloc(&d_op, op_n * sizeof(double)) != cudaSuccess) { cudaFree(d_sp); return ODIS_ERR_CUDA; }
    auto cleanup = [&]() { if (d_sp) cudaFree(d_sp); if (d_op) cudaFree(d_op); };
    cudaStream_t s = b->stream;
    int st = ODIS_OK;
    bool nonfinite = false;
    do {
        if (sp_n && cudaMemsetAsync(d_sp, 0, sp_n * sizeof(double), s) != cudaSuccess) { st = ODIS_ERR_CUDA; break; }
        if (op_n && cudaMemsetAsync(d_op, 0, op_n * sizeof(double), s) != cudaSuccess) { st = ODIS_ERR_CUDA; break; }
        if (cudaMemcpyAsync(b->d_S, S.data(), sizeof(int) * b->P, cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(b->d_base, b->base.data(), sizeof(int) * b->P, cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemsetAsync(b->d_status, 0, sizeof(int), s) != cudaSuccess ||
            cudaMemsetAsync(b->d_bar, 0, 2 * sizeof(unsigned), s) != cudaSuccess) { st = ODIS_ERR_CUDA; break; }
        BatchArgs a{};
        a.groups = b->d_groups;
        a.ngroups = (int)b->groups.size();
        a.ftiles = b->ftiles;
        a.ctiles = b->ctiles;
        a.P = b->P;
        a.mem = b->md;
        a.part = b->d_part;
        a.step_power = d_sp;
        a.step_stride = step_stride;
        a.orbit_power = d_op;
        a.orbit_stride = orbit_stride;
        a.bar_count = b->d_bar;
        a.bar_gen = b->d_bar + 1;
        a.status = b->d_status;
        a.init_load = b->p.init_load ? 1 : 0;
        a.ab3a = (float)(23. / 12.);
        a.ab3b = (float)(-16. / 12.);
        a.ab3c = (float)(5. / 12.);
        a.spin_limit = b->spin_limit ? b->spin_limit : kBarrierSpins;
        a.withhold = b->withhold;
        const size_t smem = (sizeof(double) + 2 * sizeof(float)) * (size_t)b->P;
        // steps j = 0 .. smax (the last one only records the power of the final state), in
        // cooperative launches of `chunk` steps.  The whole run is one CUDA graph: the chunks'
        // launches are captured in stream order and replayed by one cudaGraphLaunch; a chunk
        // that starts after a barrier wait ran out returns at once (the kernel reads the status
        // word on entry), and a member that went non-finite is reported while the others run on.
        void (*kern)(BatchArgs, int, int) = batch_kernel_fn(b->variant);
        auto launch_chunk = [&](int j0, int j1) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(b->grid);
            cfg.blockDim = dim3(kBatchThreads);
            cfg.dynamicSmemBytes = smem;
            cfg.stream = s;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeCooperative;
            attr[0].val.cooperative = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            return cudaLaunchKernelEx(&cfg, kern, a, j0, j1);
        };
        int nchunks = 0;
        for (int j0 = 0; j0 <= smax; j0 += chunk) nchunks++;
        bool graphed = false;
        if (b->use_graph) {
            cudaGraph_t gr = nullptr;
            cudaGraphExec_t ge = nullptr;
            bool ok = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
            if (ok) {
                for (int j0 = 0; j0 <= smax; j0 += chunk) ok = launch_chunk(j0, std::min(smax + 1, j0 + chunk)) == cudaSuccess && ok;
                ok = cudaStreamEndCapture(s, &gr) == cudaSuccess && ok;
            }
            ok = ok && cudaGraphInstantiate(&ge, gr, 0) == cudaSuccess;
            ok = ok && cudaGraphLaunch(ge, s) == cudaSuccess;
            if (ge) cudaGraphExecDestroy(ge);       // freed once the launch completes
            if (gr) cudaGraphDestroy(gr);
            if (ok) { graphed = true; b->graph_runs++; }
            else { (void)cudaGetLastError(); b->use_graph = false; }   // plain launches from now on
        }
        if (!graphed)
            for (int j0 = 0; j0 <= smax; j0 += chunk)
                if (launch_chunk(j0, std::min(smax + 1, j0 + chunk)) != cudaSuccess) { st = ODIS_ERR_CUDA; break; }
        if (st != ODIS_OK) break;
        b->launches += nchunks;
        int h = 0;
        if (cudaMemcpyAsync(&h, b->d_status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) { st = ODIS_ERR_CUDA; break; }
        if (h & (1 << ODIS_ERR_TIMEOUT)) st = ODIS_ERR_TIMEOUT;
        else if (h & (1 << ODIS_ERR_NONFINITE)) nonfinite = true;
        if (st != ODIS_OK) break;
        if (step_power && cudaMemcpyAsync(step_power, d_sp, sp_n * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess) { st = ODIS_ERR_CUDA; break; }
        if (orbit_power && cudaMemcpyAsync(orbit_power, d_op, op_n * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess) { st = ODIS_ERR_CUDA; break; }
        if (cudaStreamSynchronize(s) != cudaSuccess) { st = ODIS_ERR_CUDA; break; }
        for (int p = 0; p < b->P; p++) b->base[p] += S[p];
    } while (0);
    cleanup();
    return st == ODIS_OK && nonfinite ? ODIS_ERR_NONFINITE : st;
}

// Member state in the reference's layout: v[E], eta[N] (FP64 from the (hi, lo) pairs).
extern "C" odis_status odis_batch_get_member(odis_batch* b, int member, int* iter, double* v, double* eta)
{
    if (!b || member < 0 || member >= b->count) return ODIS_ERR_ARG;
    const int s = b->slot_of[member];
    const GroupDev& G = b->groups[b->group_of[member]];
    const int col = s - G.moff, pitch = 4 * G.Bq;
    ODIS_BCK(cudaStreamSynchronize(b->stream));
    if (iter) *iter = b->base[s];
    auto col_get = [&](const float* hi, const float* lo, int rows, double* out) -> int {
        std::vector<float> a(rows), c(rows);
        ODIS_BCK(cudaMemcpy2D(a.data(), sizeof(float), hi + col, sizeof(float) * pitch, sizeof(float), rows, cudaMemcpyDeviceToHost));
        ODIS_BCK(cudaMemcpy2D(c.data(), sizeof(float), lo + col, sizeof(float) * pitch, sizeof(float), rows, cudaMemcpyDeviceToHost));
        for (int r = 0; r < rows; r++) out[r] = (double)a[r] + (double)c[r];
        return ODIS_OK;
    };
    int st = ODIS_OK;
    // runs are an even number of steps, so the current velocity is always in buffer 0
    if (v) st = col_get(G.vhi[0], G.vlo, G.E, v);
    if (st == ODIS_OK && eta) st = col_get(G.ehi, G.elo, G.N, eta);
    return st;
}

// Sets one member's v and eta (nullable: zero), clears its AB3 history and
// restarts its step count at 0 (forcing phase t = 0, forward-Euler start).
extern "C" odis_status odis_batch_set_member(odis_batch* b, int member, const double* v, const double* eta)
{
    if (!b || member < 0 || member >= b->count) return ODIS_ERR_ARG;
    const int s = b->slot_of[member];
    const GroupDev& G = b->groups[b->group_of[member]];
    const int col = s - G.moff, pitch = 4 * G.Bq;
    ODIS_BCK(cudaStreamSynchronize(b->stream));
    auto col_set = [&](float* hi, float* lo, int rows, const double* in) -> int {
        std::vector<float> a(rows, 0.f), c(rows, 0.f);
        for (int r = 0; in && r < rows; r++) {
            a[r] = (float)in[r];
            c[r] = (float)(in[r] - (double)a[r]);
        }
        ODIS_BCK(cudaMemcpy2D(hi + col, sizeof(float) * pitch, a.data(), sizeof(float), sizeof(float), rows, cudaMemcpyHostToDevice));
        if (lo) ODIS_BCK(cudaMemcpy2D(lo + col, sizeof(float) * pitch, c.data(), sizeof(float), sizeof(float), rows, cudaMemcpyHostToDevice));
        return ODIS_OK;
    };
    int st = col_set(G.vhi[0], G.vlo, G.E, v);
    if (st == ODIS_OK) st = col_set(G.vhi[1], nullptr, G.E, nullptr);
    if (st == ODIS_OK) st = col_set(G.ehi, G.elo, G.N, eta);
    for (int k = 0; k < 2 && st == ODIS_OK; k++) {
        st = col_set(G.hv[k], nullptr, G.E, nullptr);
        if (st == ODIS_OK) st = col_set(G.he[k], nullptr, G.N, nullptr);
    }
    if (st == ODIS_OK) b->base[s] = 0;
    return st;
}

// ---------------------------------------------------------------------------
// bulk state access and projections (one mesh's members at a time)
// ---------------------------------------------------------------------------
namespace odis {
namespace {

constexpr int kProjK = 8;        // basis rows per thread
constexpr int kProjQ = 32;       // member quads per block (threadIdx.x)
constexpr int kProjS = 8;        // row slices per block (threadIdx.y)

// out[k][4 q + c] = sum_r basis[k][r] * state[r][4 q + c] for one group: each
// thread sums kProjK basis rows for one quad over a slice of the rows (FP32),
// the slices are added in FP64.
__global__ void __launch_bounds__(kProjQ * kProjS) k_project(const float* __restrict__ basis, int K, int rows,
                                                            const float4* __restrict__ state, int Bq,
                                                            double* __restrict__ out)
{
    __shared__ float4 s_acc[kProjS][kProjK][kProjQ];
    const int x = threadIdx.x, y = threadIdx.y;
    const int q = blockIdx.x * kProjQ + x, k0 = blockIdx.y * kProjK;
    float4 acc[kProjK];
#pragma unroll
    for (int kk = 0; kk < kProjK; kk++) acc[kk] = f4(0.f);
    if (q < Bq) {
        for (int r = y; r < rows; r += kProjS) {
            const float4 v = state[(size_t)r * Bq + q];
#pragma unroll
            for (int kk = 0; kk < kProjK; kk++) {
                const float bk = k0 + kk < K ? __ldg(&basis[(size_t)(k0 + kk) * rows + r]) : 0.f;
                acc[kk] = fma4(bk, v, acc[kk]);
            }
        }
    }
#pragma unroll
    for (int kk = 0; kk < kProjK; kk++) s_acc[y][kk][x] = acc[kk];
    __syncthreads();
    if (y == 0 && q < Bq) {
        for (int kk = 0; kk < kProjK && k0 + kk < K; kk++) {
            double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
            for (int yy = 0; yy < kProjS; yy++) {
                const float4 a = s_acc[yy][kk][x];
                s0 += a.x; s1 += a.y; s2 += a.z; s3 += a.w;
            }
            double* o = out + (size_t)(k0 + kk) * 4 * Bq + 4 * q;
            o[0] = s0; o[1] = s1; o[2] = s2; o[3] = s3;
        }
    }
}

}  // namespace
}  // namespace odis

static std::vector<int> mesh_members(const odis_batch* b, int mesh)
{
    std::vector<int> out;
    for (int i = 0; i < b->count; i++)
        if (b->members[i].mesh == mesh) out.push_back(i);
    return out;
}

extern "C" odis_status odis_batch_project(odis_batch* b, int mesh, const float* basis_v, int kv, const float* basis_eta,
                                          int ke, double* out, int out_stride)
{
    if (!b || !out || kv < 0 || ke < 0 || (kv && !basis_v) || (ke && !basis_eta) || out_stride < kv + ke) return ODIS_ERR_ARG;
    const std::vector<int> mem = mesh_members(b, mesh);
    if (mem.empty()) return ODIS_ERR_ARG;
    const GroupDev& G0 = b->groups[b->group_of[mem[0]]];
    const int E = G0.E, N = G0.N;
    ODIS_BCK(cudaStreamSynchronize(b->stream));
    float* d_basis = nullptr;
    double* d_out = nullptr;
    const int K = std::max(kv, ke);
    int maxBq = 0;
    for (size_t g = 0; g < b->groups.size(); g++) maxBq = std::max(maxBq, b->groups[g].Bq);
    const size_t bn = std::max((size_t)kv * E, (size_t)ke * N);
    if (cudaMalloc(&d_basis, sizeof(float) * std::max<size_t>(bn, 1)) != cudaSuccess) return ODIS_ERR_NOMEM;
    if (cudaMalloc(&d_out, sizeof(double) * (size_t)std::max(K, 1) * 4 * maxBq) != cudaSuccess) { cudaFree(d_basis); return ODIS_ERR_NOMEM; }
    int st = ODIS_OK;
    std::vector<double> h;
    for (int which = 0; which < 2 && st == ODIS_OK; which++) {
        const int k = which == 0 ? kv : ke;
        if (!k) continue;
        const int rows = which == 0 ? E : N;
        if (cudaMemcpy(d_basis, which == 0 ? basis_v : basis_eta, sizeof(float) * (size_t)k * rows, cudaMemcpyHostToDevice) != cudaSuccess) { st = ODIS_ERR_CUDA; break; }
        for (size_t g = 0; g < b->groups.size() && st == ODIS_OK; g++) {
            const GroupDev& G = b->groups[g];
            bool mine = false;
            for (int i : mem) mine |= b->group_of[i] == (int)g;
            if (!mine) continue;
            const float4* state = reinterpret_cast<const float4*>(which == 0 ? G.vhi[0] : G.ehi);
            dim3 grid((G.Bq + kProjQ - 1) / kProjQ, (k + kProjK - 1) / kProjK), block(kProjQ, kProjS);
            k_project<<<grid, block, 0, b->stream>>>(d_basis, k, rows, state, G.Bq, d_out);
            h.assign((size_t)k * 4 * G.Bq, 0.0);
            if (cudaMemcpyAsync(h.data(), d_out, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, b->stream) != cudaSuccess ||
                cudaStreamSynchronize(b->stream) != cudaSuccess) { st = ODIS_ERR_CUDA; break; }
            b->launches++;
            for (int i : mem) {
                if (b->group_of[i] != (int)g) continue;
                const int col = b->slot_of[i] - G.moff;
                for (int kk = 0; kk < k; kk++) out[(size_t)i * out_stride + (which == 0 ? 0 : kv) + kk] = h[(size_t)kk * 4 * G.Bq + col];
            }
        }
    }
    cudaFree(d_basis);
    cudaFree(d_out);
    return st;
}

// Members on `mesh`, in increasing member index: v [m][E], eta [m][N].
extern "C" odis_status odis_batch_get_mesh_members(odis_batch* b, int mesh, double* v, double* eta)
{
    if (!b) return ODIS_ERR_ARG;
    const std::vector<int> mem = mesh_members(b, mesh);
    if (mem.empty()) return ODIS_ERR_ARG;
    ODIS_BCK(cudaStreamSynchronize(b->stream));
    std::vector<float> hi, lo;
    for (int which = 0; which < 2; which++) {
        double* out = which == 0 ? v : eta;
        if (!out) continue;
        for (size_t g = 0; g < b->groups.size(); g++) {
            const GroupDev& G = b->groups[g];
            std::vector<int> here;
            for (size_t k = 0; k < mem.size(); k++) if (b->group_of[mem[k]] == (int)g) here.push_back((int)k);
            if (here.empty()) continue;
            const int rows = which == 0 ? G.E : G.N, pitch = 4 * G.Bq;
            hi.resize((size_t)rows * pitch);
            lo.resize((size_t)rows * pitch);
            ODIS_BCK(cudaMemcpy(hi.data(), which == 0 ? G.vhi[0] : G.ehi, sizeof(float) * hi.size(), cudaMemcpyDeviceToHost));
            ODIS_BCK(cudaMemcpy(lo.data(), which == 0 ? G.vlo : G.elo, sizeof(float) * lo.size(), cudaMemcpyDeviceToHost));
            for (int k : here) {
                const int col = b->slot_of[mem[k]] - G.moff;
                double* o = out + (size_t)k * rows;
                for (int r = 0; r < rows; r++) o[r] = (double)hi[(size_t)r * pitch + col] + (double)lo[(size_t)r * pitch + col];
            }
        }
    }
    return ODIS_OK;
}

// Sets every member on `mesh` (increasing member index; v [m][E], eta [m][N],
// nullable: zero), clears their AB3 histories and restarts their step counts
// at 0 (forcing phase 0, forward-Euler start): the bulk warm-start entry point.
extern "C" odis_status odis_batch_set_mesh_members(odis_batch* b, int mesh, const double* v, const double* eta)
{
    if (!b) return ODIS_ERR_ARG;
    const std::vector<int> mem = mesh_members(b, mesh);
    if (mem.empty()) return ODIS_ERR_ARG;
    ODIS_BCK(cudaStreamSynchronize(b->stream));
    std::vector<float> hi, lo;
    for (size_t g = 0; g < b->groups.size(); g++) {
        GroupDev& G = b->groups[g];
        std::vector<int> here;
        for (size_t k = 0; k < mem.size(); k++) if (b->group_of[mem[k]] == (int)g) here.push_back((int)k);
        if (here.empty()) continue;
        const int pitch = 4 * G.Bq;
        for (int which = 0; which < 2; which++) {
            const double* in = which == 0 ? v : eta;
            const int rows = which == 0 ? G.E : G.N;
            float* dhi = which == 0 ? G.vhi[0] : G.ehi;
            float* dlo = which == 0 ? G.vlo : G.elo;
            hi.resize((size_t)rows * pitch);
            lo.resize((size_t)rows * pitch);
            // keep the columns of members on other meshes (none share a group) and of padding
            ODIS_BCK(cudaMemcpy(hi.data(), dhi, sizeof(float) * hi.size(), cudaMemcpyDeviceToHost));
            ODIS_BCK(cudaMemcpy(lo.data(), dlo, sizeof(float) * lo.size(), cudaMemcpyDeviceToHost));
            for (int k : here) {
                const int col = b->slot_of[mem[k]] - G.moff;
                for (int r = 0; r < rows; r++) {
                    const double x = in ? in[(size_t)k * rows + r] : 0.0;
                    const float xh = (float)x;
                    hi[(size_t)r * pitch + col] = xh;
                    lo[(size_t)r * pitch + col] = (float)(x - (double)xh);
                }
            }
            ODIS_BCK(cudaMemcpy(dhi, hi.data(), sizeof(float) * hi.size(), cudaMemcpyHostToDevice));
            ODIS_BCK(cudaMemcpy(dlo, lo.data(), sizeof(float) * lo.size(), cudaMemcpyHostToDevice));
        }
        const size_t ev = (size_t)G.E * pitch, cv = (size_t)G.N * pitch;
        ODIS_BCK(cudaMemset(G.vhi[1], 0, sizeof(float) * ev));
        for (int k = 0; k < 2; k++) {
            ODIS_BCK(cudaMemset(G.hv[k], 0, sizeof(float) * ev));
            ODIS_BCK(cudaMemset(G.he[k], 0, sizeof(float) * cv));
        }
        for (int k : here) b->base[b->slot_of[mem[k]]] = 0;
    }
    return ODIS_OK;
}

extern "C" odis_status odis_batch_graph_runs(const odis_batch* b, long long* runs)
{
    if (!b || !runs) return ODIS_ERR_ARG;
    *runs = b->graph_runs;
    return ODIS_OK;
}

extern "C" odis_status odis_batch_set_wait_limit(odis_batch* b, unsigned polls, int withhold)
{
    if (!b || withhold < -1) return ODIS_ERR_ARG;
    b->spin_limit = polls;
    b->withhold = withhold;
    return ODIS_OK;
}
