// Self-gravity transforms of the FP32-state method on the 5th-generation tensor
// cores (tcgen05: operands in shared memory, accumulators in tensor memory).
//
// The transforms of odis_sh.cu, with P[r][i] the Legendre row r = row(l, m) at
// cell i and (cos|sin)(m lon_i) the trig rows, are written as two GEMMs:
//   analysis   C[r][j] = sum_i P[r][i] B[i][j],    B[i][2m + s] = eta_i (cos|sin)(m lon_i)
//              t(l, m, s) = C[row(l, m)][2m + s]
//   synthesis  D[i][j] = sum_r P[r][i] Cf[r][j],   Cf[row(l, m)][2m + s] = c(l, m, s)
//              usg_i   = sum_j (cos|sin)(m_j lon_i) D[i][j]
// Every Legendre row meets every trig column, of which it needs two: the tensor
// pipe does (L+1) times the useful multiply-adds, and in exchange a transform is
// a stream of the Legendre rows through shared memory.  The analysis limits the
// waste: each 128-row tile of P meets only the columns of the orders it holds.
//
// Precision.  Each operand is a power-of-two-scaled FP32 value x split into two
// fp16 numbers, hi = fp16(x) and lo = fp16(x - hi) (22 significant bits), and
// each K step accumulates hi*hi + hi*lo + lo*hi in FP32 in tensor memory.  The
// scales: 2^sA for the Legendre rows (fixed at setup from max |P|), 2^sB per
// chunk of cells for the analysis (from the chunk's max |eta|), 2^s per trig
// column for the coefficients; each keeps the scaled values below 2^14.  The
// analysis partials of a chunk are unscaled and folded in FP64 by k_sh_fold.
//
// Data movement.  The Legendre rows are stored twice, once per GEMM, as fp16
// pairs already in the K-major "core matrix" order of the MMA operands (8 rows
// x 16 bytes per 128-byte core matrix, no swizzle), so one bulk copy
// (cp.async.bulk, completion on an mbarrier) moves one pipeline stage; the
// analysis stage also carries the stage's trig tile and eta, from which the
// workers build the B operand in shared memory.  Four stages; warp roles: one
// lane copies, one lane issues MMAs (tcgen05.commit arrives on a per-stage
// mbarrier when they have read the stage), four warps build operands and read
// the accumulators, which alternate between two tensor-memory buffers.  Every
// wait is bounded (about a second of SM clocks); on expiry the kernel stops,
// records ODIS_ERR_TIMEOUT in the context status word, waits (bounded) for its
// copies and MMAs in flight and releases its tensor memory.
#include "odis_sh_tc.cuh"
#include "odis_sh.cuh"

#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <memory>
#include <vector>

namespace odis {

namespace {

constexpr int kS = 6;              // most pipeline stages (the count in use fits shared memory)
constexpr int kMaxTiles = 8;       // 128-row tiles of P in the analysis
constexpr int kMaxCols = 256;
constexpr long long kWaitCycles = 2000000000ll;

// ---- PTX wrappers --------------------------------------------------------

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// wait for the completion of the phase with the given parity; false after ~1 s
__device__ __noinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    const long long t0 = clock64();
    while (!mbar_try(bar, parity))
        if (clock64() - t0 > kWaitCycles) return false;
    return true;
}

// global -> shared bulk copy (TMA engine), completion counted on bar in bytes
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// whole warp: allocate ncols tensor-memory columns, address written to shared memory
__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// shared-memory matrix descriptor: K-major, no swizzle; lbo = byte distance of
// adjacent core matrices along K, sbo = along M/N
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
    d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
    d |= (uint64_t)1 << 46;                      // descriptor version of tcgen05
    return d;                                    // base offset 0, no swizzle
}

// instruction descriptor, kind::f16: fp16 A and B, both K-major, FP32 accumulator
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N)
{
    return (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread
__device__ __forceinline__ void mma_f16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

// arrive on bar once every MMA issued so far by this thread has completed
__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 16 consecutive FP32 columns of this thread's tensor-memory lane (whole warp)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int q = 0; q < 16; q++) v[q] = __uint_as_float(r[q]);
}

// ---- scaling and splitting -----------------------------------------------

// exponent e with mx * 2^e < 2^14 (0 for zero, NaN or Inf), clamped to +-60
__device__ __forceinline__ int scale_exp(float mx)
{
    if (!(mx > 0.f)) return 0;
    const int E = (__float_as_int(mx) >> 23) & 0xff;
    if (E == 0xff) return 0;
    const int e = E == 0 ? -126 : E - 126;
    return max(-60, min(60, 14 - e));
}

__device__ __forceinline__ float exp2i(int e) { return __int_as_float((127 + e) << 23); }   // e in [-126, 127]

__device__ __forceinline__ void split_f16(float x, __half& hi, __half& lo)
{
    hi = __float2half_rn(x);
    lo = __float2half_rn(x - __half2float(hi));
}

// offset (in halves) of element (row, k) in a K-major block with kb = K/8 core matrices per row group
__host__ __device__ __forceinline__ int cm_off(int row, int k, int kb)
{
    return ((row >> 3) * kb + (k >> 3)) * 64 + (row & 7) * 8 + (k & 7);
}

struct Ctl {
    unsigned long long full[kS];    // stage copied (producer -> all)
    unsigned long long done[kS];    // MMAs of the stage completed (tcgen05.commit)
    unsigned long long bready[kS];  // B operand of the stage built (workers -> MMA)
    unsigned long long accf[2];     // accumulator buffer complete (tcgen05.commit -> workers)
    unsigned long long acce[2];     // accumulator buffer read out (workers -> MMA)
    unsigned long long tfull[2];    // synthesis: trig tile of a pass copied
    unsigned long long tempty[2];   // synthesis: trig tile read by the workers
    uint32_t tslot;
    int abort;
    float red[4];
    float fcol[kMaxCols];
};

// named barrier 1 over the 4 worker warps; returns the OR of p over them
__device__ __forceinline__ bool workers_or(bool p)
{
    uint32_t r;
    asm volatile("{\n\t.reg .pred a, b;\n\tsetp.ne.u32 a, %1, 0;\n\tbar.red.or.pred b, 1, 128, a;\n\tselp.u32 %0, 1, 0, b;\n\t}"
                 : "=r"(r)
                 : "r"((uint32_t)p)
                 : "memory");
    return r != 0;
}

__device__ __forceinline__ void workers_sync() { asm volatile("bar.sync 1, 128;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(bar) : "memory");
}

__device__ float workers_max(float v, float* red, int w)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) red[w] = v;
    workers_sync();
    v = fmaxf(fmaxf(red[0], red[1]), fmaxf(red[2], red[3]));
    workers_sync();
    return v;
}

// Warp roles (192 threads): warp 0 lane 0 copies stages (bulk copies), warp 1
// lane 0 issues the MMAs and owns the tensor-memory allocation, warps 2-5 (128
// threads, one per tensor-memory lane) build operands and read accumulators.
constexpr int kRoleThreads = 192;

__device__ __forceinline__ void set_abort(Ctl* ctl, int* status)
{
    if (atomicExch(&ctl->abort, 1) == 0) atomicOr(status, 1 << ODIS_ERR_TIMEOUT);
}
__device__ __forceinline__ bool aborted(const Ctl* ctl) { return *(volatile const int*)&ctl->abort != 0; }

// ---- analysis ----------------------------------------------------------------

struct TcAnaArgs {
    const __half* A;        // [nstage][2][MR][KA] core-matrix order
    const float* T;         // [nstage][ncol][KA] trig tiles
    const float* eta;       // [Np]
    const int* rowlm;       // [MPAD] (l << 8) | m, -1 on padding rows
    float* part;            // [K][nchunk]
    int* status;
    int N, L, MR, MPAD, KA, NB, nstage, spc, nchunk, ntile, sA, cols, tmem_cols;
    int nst;                // pipeline stages (<= kS)
    unsigned stage_bytes;
    int c0[kMaxTiles], nn[kMaxTiles], toff[kMaxTiles];
};

// One CTA per SM over chunks of spc stages of KA cells.  Stage smem: A hi, A lo
// (MPAD rows, rows >= MR zero), trig tile, eta, B hi, B lo.  The accumulators of
// a chunk (all row tiles) alternate between two tensor-memory buffers.
__global__ void __launch_bounds__(kRoleThreads, 1) k_shtc_analysis(const TcAnaArgs a)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    Ctl* ctl = reinterpret_cast<Ctl*>(sm + a.nst * a.stage_bytes);
    const int ncol = 2 * (a.L + 1);
    const uint32_t aslice = (uint32_t)a.MPAD * a.KA * 2, acopy = (uint32_t)a.MR * a.KA * 2;
    const uint32_t tbytes = (uint32_t)ncol * a.KA * 4, ebytes = (uint32_t)a.KA * 4;
    const uint32_t toffs = 2 * aslice, eoffs = toffs + ((tbytes + 127) & ~127u), boffs = eoffs + 128;
    const uint32_t bslice = (uint32_t)a.NB * a.KA * 2;
    const uint32_t sbase = smem_u32(sm);
    if (tid == 0) {
        for (int b = 0; b < a.nst; b++) {
            mbar_init(smem_u32(&ctl->full[b]), 1);
            mbar_init(smem_u32(&ctl->done[b]), 1);
            mbar_init(smem_u32(&ctl->bready[b]), 128);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(smem_u32(&ctl->accf[b]), 1);
            mbar_init(smem_u32(&ctl->acce[b]), 128);
        }
        ctl->abort = 0;
        fence_barrier_init();
    }
    const uint32_t padb = aslice - acopy;    // rows MR..MPAD of every A slice: zero, never copied
    if (padb > 0)
        for (uint32_t o = tid * 16; o < a.nst * 2 * padb; o += kRoleThreads * 16) {
            const uint32_t buf = o / padb, r = o % padb;
            *reinterpret_cast<uint4*>(sm + (buf >> 1) * a.stage_bytes + (buf & 1) * aslice + acopy + r) =
                make_uint4(0u, 0u, 0u, 0u);
        }
    fence_async_smem();
    if (warp == 1) tmem_alloc(smem_u32(&ctl->tslot), (uint32_t)a.tmem_cols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = ctl->tslot;

    const int G = gridDim.x;
    const int nmine = (a.nchunk - (int)blockIdx.x + G - 1) / G;
    int ns = 0;
    if (nmine > 0) {
        const int lastc = (int)blockIdx.x + (nmine - 1) * G;
        ns = (nmine - 1) * a.spc + min(a.spc, a.nstage - lastc * a.spc);
    }
    const int kb = a.KA >> 3;
    const uint32_t sbo = (uint32_t)kb * 128;

    if (warp == 0) {                                   // ---- producer
        if (lane == 0) {
            int issued = 0;
            for (int g = 0; g < ns && !aborted(ctl); g++) {
                const int b = g % a.nst;
                if (g >= a.nst && !mbar_wait(smem_u32(&ctl->done[b]), ((g - a.nst) / a.nst) & 1)) { set_abort(ctl, a.status); break; }
                const int s = ((int)blockIdx.x + (g / a.spc) * G) * a.spc + g % a.spc;
                const uint32_t dst = sbase + b * a.stage_bytes, bar = smem_u32(&ctl->full[b]);
                const __half* src = a.A + (size_t)s * 2 * a.MR * a.KA;
                mbar_expect_tx(bar, 2 * acopy + tbytes + ebytes);
                bulk_g2s(dst, src, acopy, bar);
                bulk_g2s(dst + aslice, src + (size_t)a.MR * a.KA, acopy, bar);
                bulk_g2s(dst + toffs, a.T + (size_t)s * ncol * a.KA, tbytes, bar);
                bulk_g2s(dst + eoffs, a.eta + (size_t)s * a.KA, ebytes, bar);
                issued = g + 1;
            }
            if (aborted(ctl))      // let the copies in flight land before the CTA ends
                for (int g = max(0, issued - a.nst); g < issued; g++) mbar_wait(smem_u32(&ctl->full[g % a.nst]), (g / a.nst) & 1);
        }
        __syncwarp();
    } else if (warp == 1) {                            // ---- MMA issuer
        if (lane == 0) {
            int mmas = 0;
            for (int g = 0; g < ns && !aborted(ctl); g++) {
                const int b = g % a.nst, k = g % a.spc, r = g / a.spc, ab = r & 1;
                const int chunk = (int)blockIdx.x + r * G;
                const int klast = min(a.spc, a.nstage - chunk * a.spc) - 1;
                if (k == 0 && r >= 2 && !mbar_wait(smem_u32(&ctl->acce[ab]), ((r - 2) >> 1) & 1)) { set_abort(ctl, a.status); break; }
                if (!mbar_wait(smem_u32(&ctl->full[b]), (g / a.nst) & 1) ||
                    !mbar_wait(smem_u32(&ctl->bready[b]), (g / a.nst) & 1)) { set_abort(ctl, a.status); break; }
                tc_fence_after();
                const uint32_t abase = sbase + b * a.stage_bytes, bbase = abase + boffs;
                for (int j = 0; j < a.KA / 16; j++)
                    for (int t = 0; t < a.ntile; t++) {
                        const uint32_t idesc = idesc_f16(128, a.nn[t]);
                        const uint32_t d = tmem + (uint32_t)(ab * a.cols + a.toff[t]);
                        const uint32_t ao = abase + (uint32_t)t * 16 * sbo + j * 256;
                        const uint32_t bo = bbase + (uint32_t)(a.c0[t] >> 3) * sbo + j * 256;
                        mma_f16(d, sdesc(ao, 128, sbo), sdesc(bo, 128, sbo), idesc, (k == 0 && j == 0) ? 0u : 1u);
                        mma_f16(d, sdesc(ao, 128, sbo), sdesc(bo + bslice, 128, sbo), idesc, 1u);
                        mma_f16(d, sdesc(ao + aslice, 128, sbo), sdesc(bo, 128, sbo), idesc, 1u);
                    }
                mma_commit(smem_u32(&ctl->done[b]));
                if (k == klast) mma_commit(smem_u32(&ctl->accf[ab]));
                mmas = g + 1;
            }
            if (aborted(ctl) && mmas > 0) mbar_wait(smem_u32(&ctl->done[(mmas - 1) % a.nst]), ((mmas - 1) / a.nst) & 1);
        }
        __syncwarp();
    } else {                                           // ---- workers
        const int w = warp & 3;                        // tensor-memory subpartition of this warp
        const int q = w * 32 + lane;                   // its lane = row of each accumulator tile
        const int wt = tid - 64;                       // 0..127
        float scale_b = 1.f;
        int sB = 0;
        for (int g = 0; g < ns; g++) {
            const int b = g % a.nst, k = g % a.spc, r = g / a.spc, ab = r & 1;
            const int chunk = (int)blockIdx.x + r * G;
            const int klast = min(a.spc, a.nstage - chunk * a.spc) - 1;
            if (k == 0) {                              // the chunk's scale of the B operand
                const int i0 = chunk * a.spc * a.KA, i1 = min(a.N, i0 + (klast + 1) * a.KA);
                float mx = 0.f;
                for (int i = i0 + wt; i < i1; i += 128) mx = fmaxf(mx, fabsf(a.eta[i]));
                mx = workers_max(mx, ctl->red, w);
                sB = scale_exp(mx);
                scale_b = exp2i(sB);
            }
            const bool ok = mbar_wait(smem_u32(&ctl->full[b]), (g / a.nst) & 1);
            if (workers_or(!ok || aborted(ctl))) { if (!ok) set_abort(ctl, a.status); break; }
            {   // B[c][k] = eta_k trig[c][k] 2^sB as fp16 pairs, 8 cells (one core-matrix row) per task
                const unsigned char* st = sm + b * a.stage_bytes;
                const float* T = reinterpret_cast<const float*>(st + toffs);
                const float* E = reinterpret_cast<const float*>(st + eoffs);
                unsigned char* bb = sm + b * a.stage_bytes + boffs;
                const int s = chunk * a.spc + k;
                const int ntask = a.NB * kb;
                for (int e = wt; e < ntask; e += 128) {
                    const int c = e / kb, kg = e - c * kb;
                    uint32_t hi[4], lo[4];
#pragma unroll
                    for (int u = 0; u < 8; u += 2) {
                        float x0 = 0.f, x1 = 0.f;
                        const int kk = kg * 8 + u, i = s * a.KA + kk;
                        if (c < ncol) {
                            if (i < a.N) x0 = E[kk] * T[c * a.KA + kk] * scale_b;
                            if (i + 1 < a.N) x1 = E[kk + 1] * T[c * a.KA + kk + 1] * scale_b;
                        }
                        __half h0, l0, h1, l1;
                        split_f16(x0, h0, l0);
                        split_f16(x1, h1, l1);
                        hi[u >> 1] = (uint32_t)__half_as_ushort(h0) | ((uint32_t)__half_as_ushort(h1) << 16);
                        lo[u >> 1] = (uint32_t)__half_as_ushort(l0) | ((uint32_t)__half_as_ushort(l1) << 16);
                    }
                    const int off = cm_off(c, kg * 8, kb) * 2;          // bytes
                    *reinterpret_cast<uint4*>(bb + off) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
                    *reinterpret_cast<uint4*>(bb + bslice + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
                }
                fence_async_smem();
                mbar_arrive(smem_u32(&ctl->bready[b]));
            }
            if (k == klast) {                          // read out the chunk's accumulators
                const bool ok2 = mbar_wait(smem_u32(&ctl->accf[ab]), (r >> 1) & 1);
                if (workers_or(!ok2 || aborted(ctl))) { if (!ok2) set_abort(ctl, a.status); break; }
                tc_fence_after();
                const float inv = exp2i(-(a.sA + sB));
                const uint32_t lanes = tmem + ((uint32_t)(w * 32) << 16) + (uint32_t)(ab * a.cols);
                for (int t = 0; t < a.ntile; t++) {
                    const int lm = a.rowlm[t * 128 + q];
                    const int l = lm >> 8, m = lm & 255;
                    const int cc = 2 * m - a.c0[t];
                    float vc = 0.f, vs = 0.f;
                    for (int j0 = 0; j0 < a.nn[t]; j0 += 16) {
                        float v[16];
                        tmem_ld16(lanes + (uint32_t)(a.toff[t] + j0), v);
#pragma unroll
                        for (int u = 0; u < 16; u++) {
                            if (j0 + u == cc) vc = v[u];
                            if (j0 + u == cc + 1) vs = v[u];
                        }
                    }
                    if (lm >= 0) {
                        a.part[(size_t)sh_col(l, m, 0) * a.nchunk + chunk] = vc * inv;
                        if (m > 0) a.part[(size_t)sh_col(l, m, 1) * a.nchunk + chunk] = vs * inv;
                    }
                }
                tc_fence_before();
                mbar_arrive(smem_u32(&ctl->acce[ab]));
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1) tmem_dealloc(tmem, (uint32_t)a.tmem_cols);
}

// ---- synthesis ------------------------------------------------------------

struct TcSynArgs {
    const __half* A;        // [NKC][NU][2][128 x 32] core-matrix order
    const __half* B;        // [NKC][2][NS x 32]
    const float* fcol;      // [NS] 2^-(sA + s_col)
    const float* T;         // [NU][2(L+1)][128] trig tiles
    float* usg;
    int* status;
    int N, L, NS, NKC, NU, npass, tmem_cols;
    int nst;                // pipeline stages (<= kS)
    unsigned stage_bytes;
};

// One CTA per SM over passes of TP x 128 cells; the K chunks of 32 Legendre
// rows stream through the stages, the accumulators of a pass alternate between
// two tensor-memory buffers, and the workers (one cell per lane) combine the
// columns of one buffer with the pass's trig tile (copied into one of two
// shared-memory buffers) while the MMAs fill the other.
template <int TP>
__global__ void __launch_bounds__(kRoleThreads, 1) k_shtc_synth(const TcSynArgs a)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    Ctl* ctl = reinterpret_cast<Ctl*>(sm + a.nst * a.stage_bytes);
    const int ncol = 2 * (a.L + 1);
    const uint32_t abytes = TP * 16384u, bbytes = (uint32_t)a.NS * 128u, tbytes = (uint32_t)TP * ncol * 512u;
    const uint32_t sbase = smem_u32(sm);
    const uint32_t tsm = a.nst * a.stage_bytes + ((sizeof(Ctl) + 127) & ~(size_t)127);   // trig buffers
    if (tid == 0) {
        for (int b = 0; b < a.nst; b++) {
            mbar_init(smem_u32(&ctl->full[b]), 1);
            mbar_init(smem_u32(&ctl->done[b]), 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(smem_u32(&ctl->accf[b]), 1);
            mbar_init(smem_u32(&ctl->acce[b]), 128);
            mbar_init(smem_u32(&ctl->tfull[b]), 1);
            mbar_init(smem_u32(&ctl->tempty[b]), 128);
        }
        ctl->abort = 0;
        fence_barrier_init();
    }
    for (int c = tid; c < a.NS; c += kRoleThreads) ctl->fcol[c] = a.fcol[c];
    if (warp == 1) tmem_alloc(smem_u32(&ctl->tslot), (uint32_t)a.tmem_cols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = ctl->tslot;

    const int G = gridDim.x;
    const int nmine = max(0, (a.npass - (int)blockIdx.x + G - 1) / G);
    const int ns = nmine * a.NKC;
    const int span = TP * a.NS;                        // columns of one accumulator buffer

    if (warp == 0) {                                   // ---- producer
        if (lane == 0) {
            int issued = 0, tissued = 0;
            for (int g = 0; g < ns && !aborted(ctl); g++) {
                const int b = g % a.nst, kc = g % a.NKC, r = g / a.NKC, p = (int)blockIdx.x + r * G;
                if (kc == 0) {       // the pass's trig tile, into the buffer freed by pass r - 2
                    const int tb = r & 1;
                    if (r >= 2 && !mbar_wait(smem_u32(&ctl->tempty[tb]), ((r - 2) >> 1) & 1)) { set_abort(ctl, a.status); break; }
                    const uint32_t bar = smem_u32(&ctl->tfull[tb]);
                    mbar_expect_tx(bar, tbytes);
                    bulk_g2s(sbase + tsm + tb * tbytes, a.T + (size_t)p * TP * ncol * 128, tbytes, bar);
                    tissued = r + 1;
                }
                if (g >= a.nst && !mbar_wait(smem_u32(&ctl->done[b]), ((g - a.nst) / a.nst) & 1)) { set_abort(ctl, a.status); break; }
                const uint32_t dst = sbase + b * a.stage_bytes, bar = smem_u32(&ctl->full[b]);
                mbar_expect_tx(bar, abytes + bbytes);
                bulk_g2s(dst, a.A + ((size_t)kc * a.NU + (size_t)p * TP) * 8192, abytes, bar);
                bulk_g2s(dst + abytes, a.B + (size_t)kc * a.NS * 64, bbytes, bar);
                issued = g + 1;
            }
            if (aborted(ctl)) {
                for (int g = max(0, issued - a.nst); g < issued; g++) mbar_wait(smem_u32(&ctl->full[g % a.nst]), (g / a.nst) & 1);
                for (int r = max(0, tissued - 2); r < tissued; r++) mbar_wait(smem_u32(&ctl->tfull[r & 1]), (r >> 1) & 1);
            }
        }
        __syncwarp();
    } else if (warp == 1) {                            // ---- MMA issuer
        if (lane == 0) {
            int mmas = 0;
            const uint32_t idesc = idesc_f16(128, a.NS);
            for (int g = 0; g < ns && !aborted(ctl); g++) {
                const int b = g % a.nst, kc = g % a.NKC, r = g / a.NKC, ab = r & 1;
                if (kc == 0 && r >= 2 && !mbar_wait(smem_u32(&ctl->acce[ab]), ((r - 2) >> 1) & 1)) { set_abort(ctl, a.status); break; }
                if (!mbar_wait(smem_u32(&ctl->full[b]), (g / a.nst) & 1)) { set_abort(ctl, a.status); break; }
                tc_fence_after();
                const uint32_t abase = sbase + b * a.stage_bytes, bbase = abase + abytes;
#pragma unroll
                for (int j = 0; j < 2; j++)
#pragma unroll
                    for (int t = 0; t < TP; t++) {
                        const uint32_t d = tmem + (uint32_t)(ab * span + t * a.NS);
                        const uint32_t ah = abase + t * 16384u + j * 256u, al = ah + 8192u;
                        const uint32_t bh = bbase + j * 256u, bl = bh + (uint32_t)a.NS * 64u;
                        mma_f16(d, sdesc(ah, 128, 512), sdesc(bh, 128, 512), idesc, (kc == 0 && j == 0) ? 0u : 1u);
                        mma_f16(d, sdesc(ah, 128, 512), sdesc(bl, 128, 512), idesc, 1u);
                        mma_f16(d, sdesc(al, 128, 512), sdesc(bh, 128, 512), idesc, 1u);
                    }
                mma_commit(smem_u32(&ctl->done[b]));
                if (kc == a.NKC - 1) mma_commit(smem_u32(&ctl->accf[ab]));
                mmas = g + 1;
            }
            if (aborted(ctl) && mmas > 0) mbar_wait(smem_u32(&ctl->done[(mmas - 1) % a.nst]), ((mmas - 1) / a.nst) & 1);
        }
        __syncwarp();
    } else {                                           // ---- workers: epilogue
        const int w = warp & 3, q = w * 32 + lane;
        for (int r = 0; r < nmine; r++) {
            const int ab = r & 1, p = (int)blockIdx.x + r * G;
            const bool ok = mbar_wait(smem_u32(&ctl->accf[ab]), (r >> 1) & 1) &&
                            mbar_wait(smem_u32(&ctl->tfull[ab]), (r >> 1) & 1);
            if (workers_or(!ok || aborted(ctl))) { if (!ok) set_abort(ctl, a.status); break; }
            tc_fence_after();
            const uint32_t lanes = tmem + ((uint32_t)(w * 32) << 16) + (uint32_t)(ab * span);
            const float* T = reinterpret_cast<const float*>(sm + tsm + ab * tbytes);
#pragma unroll
            for (int t = 0; t < TP; t++) {
                const int i = (p * TP + t) * 128 + q;
                const float* Tt = T + (size_t)t * ncol * 128 + q;
                float u = 0.f;
                for (int j0 = 0; j0 < a.NS; j0 += 16) {
                    float v[16];
                    tmem_ld16(lanes + (uint32_t)(t * a.NS + j0), v);
#pragma unroll
                    for (int c = 0; c < 16; c++)
                        if (j0 + c < ncol) u = fmaf(Tt[(j0 + c) * 128] * ctl->fcol[j0 + c], v[c], u);
                }
                if (i < a.N) a.usg[i] = u;
            }
            tc_fence_before();
            mbar_arrive(smem_u32(&ctl->tempty[ab]));
            mbar_arrive(smem_u32(&ctl->acce[ab]));
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1) tmem_dealloc(tmem, (uint32_t)a.tmem_cols);
}

// ---- per-step coefficient operand and setup-time tiling --------------------

// coefficients c[K] -> per-column scaled fp16 pairs at their (row, column) of
// the K-major synthesis operand; the other entries stay zero from setup
__global__ void __launch_bounds__(1024) k_shtc_pack(const float* __restrict__ coef, int L, int K, int NS, int sA,
                                                    __half* __restrict__ B, float* __restrict__ fcol)
{
    __shared__ float colscale[kMaxCols];
    const int ncol = 2 * (L + 1), lane = threadIdx.x & 31;
    for (int c = threadIdx.x >> 5; c < NS; c += blockDim.x >> 5) {     // one warp per trig column
        float mx = 0.f;
        const int m = c >> 1, sn = c & 1;
        if (c < ncol && !(m == 0 && sn))
            for (int l = m + lane; l <= L; l += 32) mx = fmaxf(mx, fabsf(coef[sh_col(l, m, sn)]));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0) {
            const int e = scale_exp(mx);
            colscale[c] = exp2i(e);
            fcol[c] = exp2i(-(sA + e));
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        int l = (int)sqrtf((float)k);
        while (l * l > k) l--;
        while ((l + 1) * (l + 1) <= k) l++;
        const int rem = k - l * l;
        const int m = (rem + 1) >> 1, sn = rem == 0 ? 0 : ((rem + 1) & 1);
        const int r = p_row(L, l, m), c = 2 * m + sn;
        __half h, lo;
        split_f16(coef[k] * colscale[c], h, lo);
        const size_t off = (size_t)(r >> 5) * NS * 64 + cm_off(c, r & 31, 4);
        B[off] = h;
        B[off + (size_t)NS * 32] = lo;
    }
}

// analysis operand: stage g holds cells g*KA .. g*KA+KA-1, rows 0..MR-1
__global__ void k_shtc_tile_analysis(const float* __restrict__ P, int MP, int MR, int N, int Np, int KA, int nstage,
                                     float scale, __half* __restrict__ out)
{
    const size_t total = (size_t)nstage * MR * KA;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total; q += (size_t)gridDim.x * blockDim.x) {
        const int g = (int)(q / ((size_t)MR * KA));
        const int rem = (int)(q % ((size_t)MR * KA));
        const int r = rem / KA, k = rem % KA;
        const int i = g * KA + k;
        const float x = (r < MP && i < N) ? P[(size_t)r * Np + i] * scale : 0.f;
        __half h, l;
        split_f16(x, h, l);
        const size_t base = (size_t)g * 2 * MR * KA + cm_off(r, k, KA >> 3);
        out[base] = h;
        out[base + (size_t)MR * KA] = l;
    }
}

// synthesis operand: tile u holds cells u*128 .. u*128+127, chunk kc the rows kc*32 .. kc*32+31
__global__ void k_shtc_tile_synth(const float* __restrict__ P, int MP, int N, int Np, int NKC, int NU, float scale,
                                  __half* __restrict__ out)
{
    const size_t total = (size_t)NKC * NU * 4096;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total; q += (size_t)gridDim.x * blockDim.x) {
        const int kc = (int)(q / ((size_t)NU * 4096));
        const int rem = (int)(q % ((size_t)NU * 4096));
        const int u = rem / 4096, w = rem % 4096;
        const int k = w / 128, c = w % 128;      // consecutive threads read consecutive cells
        const int i = u * 128 + c, r = kc * 32 + k;
        const float x = (r < MP && i < N) ? P[(size_t)r * Np + i] * scale : 0.f;
        __half h, l;
        split_f16(x, h, l);
        const size_t base = ((size_t)kc * NU + u) * 8192 + cm_off(c, k, 4);
        out[base] = h;
        out[base + 4096] = l;
    }
}

// analysis trig tiles: stage g holds trig[c][g*KA + k] as [c][k]
__global__ void k_shtc_tile_trig(const float* __restrict__ trig, int ncol, int N, int Np, int KA, int nstage,
                                 float* __restrict__ out)
{
    const size_t total = (size_t)nstage * ncol * KA;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total; q += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(q % KA), c = (int)((q / KA) % ncol), g = (int)(q / ((size_t)KA * ncol));
        const int i = g * KA + k;
        out[q] = i < N ? trig[(size_t)c * Np + i] : 0.f;
    }
}

// synthesis trig tiles: tile u holds trig[c][u*128 + k] as [c][k]
__global__ void k_shtc_tile_trig_synth(const float* __restrict__ trig, int ncol, int N, int Np, int NU,
                                       float* __restrict__ out)
{
    const size_t total = (size_t)NU * ncol * 128;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total; q += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(q % 128), c = (int)((q / 128) % ncol), u = (int)(q / ((size_t)128 * ncol));
        const int i = u * 128 + k;
        out[q] = i < N ? trig[(size_t)c * Np + i] : 0.f;
    }
}

int pow2_cols(int n)
{
    int c = 32;
    while (c < n) c <<= 1;
    return c;
}

}  // namespace

struct ShTc {
    int L = 0, K = 0, MP = 0, MR = 0, N = 0, Np = 0, nsm = 0, sA = 0, tp = 2;
    int* status = nullptr;
    const float* trig = nullptr;
    // analysis
    __half* Aan = nullptr;
    float* Tan = nullptr;
    int* rowlm = nullptr;
    float* part = nullptr;
    int KA = 32, MPAD = 0, NB = 0, nstage = 0, spc = 0, nchunk = 0, ntile = 0, cols = 0, tmem_a = 0, grid_a = 0;
    int c0[kMaxTiles] = {}, nn[kMaxTiles] = {}, toff[kMaxTiles] = {};
    unsigned stage_a = 0;
    int nst_a = 0;
    size_t smem_a = 0;
    // synthesis
    __half* Asy = nullptr;
    __half* Bsy = nullptr;
    float* fcol = nullptr;
    float* Tsy = nullptr;
    int NS = 0, NKC = 0, NU = 0;
    bool tp_ok[3] = {false, false, false};
    unsigned stage_s[3] = {0, 0, 0};
    int nst_s[3] = {0, 0, 0};
    size_t smem_s[3] = {0, 0, 0};
    int tmem_s[3] = {0, 0, 0};
};

void shtc_destroy(ShTc* s)
{
    if (!s) return;
    cudaFree(s->Aan); cudaFree(s->Tan); cudaFree(s->rowlm); cudaFree(s->part);
    cudaFree(s->Asy); cudaFree(s->Bsy); cudaFree(s->fcol); cudaFree(s->Tsy);
    delete s;
}

int shtc_create(ShTc** out, const float* P, const float* trig, double pmax, int L, int N, int Np, int* status)
{
    *out = nullptr;
    int dev = 0, nsm = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return ODIS_ERR_CUDA;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    std::unique_ptr<ShTc, void (*)(ShTc*)> s(new ShTc, shtc_destroy);
    s->L = L; s->K = (L + 1) * (L + 1); s->MP = (L + 1) * (L + 2) / 2; s->MR = (s->MP + 7) / 8 * 8;
    s->N = N; s->Np = Np; s->nsm = nsm; s->status = status; s->trig = trig;
    int e = 0;
    std::frexp(pmax, &e);                       // pmax < 2^e
    s->sA = pmax > 0.0 ? 14 - e : 0;
    const int ncol = 2 * (L + 1);
    const size_t ctl = sizeof(Ctl);

    // analysis tiles: rows are ordered by order m, so each 128-row tile meets a window of columns
    s->ntile = (s->MP + 127) / 128;
    s->MPAD = s->ntile * 128;
    if (s->ntile > kMaxTiles) return ODIS_ERR_ARG;
    std::vector<int> lm(s->MPAD, -1);
    for (int m = 0; m <= L; m++)
        for (int l = m; l <= L; l++) lm[p_row(L, l, m)] = (l << 8) | m;
    int nb = ncol;
    for (int t = 0; t < s->ntile; t++) {
        const int r0 = t * 128, r1 = std::min(s->MP, r0 + 128) - 1;
        const int mlo = lm[r0] & 255, mhi = lm[r1] & 255;
        s->c0[t] = (2 * mlo) & ~7;
        s->nn[t] = (2 * mhi + 2 - s->c0[t] + 15) / 16 * 16;
        s->toff[t] = s->cols;
        s->cols += s->nn[t];
        nb = std::max(nb, s->c0[t] + s->nn[t]);
    }
    s->NB = (nb + 15) / 16 * 16;
    if (2 * s->cols > 512 || s->NB > kMaxCols) return ODIS_ERR_ARG;
    s->tmem_a = pow2_cols(2 * s->cols);
    // stage depth: as many stages (<= kS) as shared memory holds, at least 4 at the wider KA
    for (int ka : {32, 16}) {
        const size_t tb = ((size_t)ncol * ka * 4 + 127) / 128 * 128;
        const unsigned st = (unsigned)((2ull * s->MPAD * ka * 2 + tb + 128 + 2ull * s->NB * ka * 2 + 1023) / 1024 * 1024);
        const int fit = (int)std::min<size_t>(kS, ((size_t)optin - ctl) / st);
        if (fit >= 4 || (ka == 16 && fit >= 3)) { s->KA = ka; s->stage_a = st; s->nst_a = fit; break; }
    }
    if (!s->stage_a) return ODIS_ERR_ARG;
    s->smem_a = (size_t)s->nst_a * s->stage_a + ctl;
    s->nstage = (N + s->KA - 1) / s->KA;
    // chunks of at most 1024 cells (FP32 accumulation length) in whole waves of one chunk per SM
    const int waves = (s->nstage + nsm * (1024 / s->KA) - 1) / (nsm * (1024 / s->KA));
    s->spc = std::max(1, (s->nstage + nsm * waves - 1) / (nsm * waves));
    s->nchunk = (s->nstage + s->spc - 1) / s->spc;
    s->grid_a = std::min(s->nchunk, nsm);

    // synthesis: 32-row K chunks, 128-cell tiles (an even count, for 2 tiles per pass)
    s->NS = (ncol + 15) / 16 * 16;
    s->NKC = (s->MP + 31) / 32;
    s->NU = (N + 255) / 256 * 2;
    if (s->NS > kMaxCols) return ODIS_ERR_ARG;
    for (int tp = 1; tp <= 2; tp++) {
        s->stage_s[tp] = (unsigned)((tp * 16384ull + (size_t)s->NS * 128 + 1023) / 1024 * 1024);
        const size_t fixed = (ctl + 127) / 128 * 128 + 2ull * tp * ncol * 512;
        s->nst_s[tp] = fixed < (size_t)optin ? (int)std::min<size_t>(kS, ((size_t)optin - fixed) / s->stage_s[tp]) : 0;
        s->smem_s[tp] = (size_t)s->nst_s[tp] * s->stage_s[tp] + fixed;
        s->tmem_s[tp] = pow2_cols(2 * tp * s->NS);
        s->tp_ok[tp] = s->nst_s[tp] >= 3 && 2 * tp * s->NS <= 512;
    }
    if (!s->tp_ok[1]) return ODIS_ERR_ARG;
    if (!s->tp_ok[2]) s->tp = 1;

    const size_t na = (size_t)s->nstage * 2 * s->MR * s->KA, nt = (size_t)s->nstage * ncol * s->KA;
    const size_t nsy = (size_t)s->NKC * s->NU * 8192, nbs = (size_t)s->NKC * s->NS * 64, nts = (size_t)s->NU * ncol * 128;
    if (cudaMalloc(&s->Aan, na * sizeof(__half)) != cudaSuccess || cudaMalloc(&s->Tan, nt * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&s->Asy, nsy * sizeof(__half)) != cudaSuccess || cudaMalloc(&s->Bsy, nbs * sizeof(__half)) != cudaSuccess ||
        cudaMalloc(&s->fcol, kMaxCols * sizeof(float)) != cudaSuccess || cudaMalloc(&s->Tsy, nts * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&s->rowlm, sizeof(int) * s->MPAD) != cudaSuccess ||
        cudaMalloc(&s->part, sizeof(float) * (size_t)s->K * s->nchunk) != cudaSuccess)
        return ODIS_ERR_NOMEM;
    cudaMemcpy(s->rowlm, lm.data(), sizeof(int) * s->MPAD, cudaMemcpyHostToDevice);
    cudaMemset(s->Bsy, 0, nbs * sizeof(__half));
    cudaMemset(s->fcol, 0, kMaxCols * sizeof(float));
    cudaMemset(s->part, 0, sizeof(float) * (size_t)s->K * s->nchunk);
    const float scale = std::ldexp(1.0f, s->sA);
    k_shtc_tile_analysis<<<4 * nsm, 256>>>(P, s->MP, s->MR, N, Np, s->KA, s->nstage, scale, s->Aan);
    k_shtc_tile_trig<<<4 * nsm, 256>>>(trig, ncol, N, Np, s->KA, s->nstage, s->Tan);
    k_shtc_tile_synth<<<4 * nsm, 256>>>(P, s->MP, N, Np, s->NKC, s->NU, scale, s->Asy);
    k_shtc_tile_trig_synth<<<4 * nsm, 256>>>(trig, ncol, N, Np, s->NU, s->Tsy);
    if (cudaFuncSetAttribute(k_shtc_analysis, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->smem_a) != cudaSuccess ||
        cudaFuncSetAttribute(k_shtc_synth<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->smem_s[1]) != cudaSuccess ||
        (s->tp_ok[2] && cudaFuncSetAttribute(k_shtc_synth<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)s->smem_s[2]) != cudaSuccess))
        return ODIS_ERR_CUDA;
    if (cudaDeviceSynchronize() != cudaSuccess) return ODIS_ERR_CUDA;
    *out = s.release();
    return ODIS_OK;
}

void shtc_analysis(ShTc* s, const float* eta, cudaStream_t st)
{
    TcAnaArgs a;
    a.A = s->Aan; a.T = s->Tan; a.eta = eta; a.rowlm = s->rowlm; a.part = s->part; a.status = s->status;
    a.N = s->N; a.L = s->L; a.MR = s->MR; a.MPAD = s->MPAD; a.KA = s->KA; a.NB = s->NB;
    a.nstage = s->nstage; a.spc = s->spc; a.nchunk = s->nchunk; a.ntile = s->ntile; a.sA = s->sA;
    a.cols = s->cols; a.tmem_cols = s->tmem_a; a.stage_bytes = s->stage_a; a.nst = s->nst_a;
    for (int t = 0; t < kMaxTiles; t++) { a.c0[t] = s->c0[t]; a.nn[t] = s->nn[t]; a.toff[t] = s->toff[t]; }
    k_shtc_analysis<<<s->grid_a, kRoleThreads, s->smem_a, st>>>(a);
}

const float* shtc_partials(const ShTc* s) { return s->part; }
int shtc_chunks(const ShTc* s) { return s->nchunk; }

void shtc_pack(ShTc* s, const float* coef, cudaStream_t st)
{
    k_shtc_pack<<<1, 1024, 0, st>>>(coef, s->L, s->K, s->NS, s->sA, s->Bsy, s->fcol);
}

void shtc_synth(ShTc* s, float* usg, cudaStream_t st)
{
    TcSynArgs a;
    a.A = s->Asy; a.B = s->Bsy; a.fcol = s->fcol; a.T = s->Tsy; a.usg = usg; a.status = s->status;
    a.N = s->N; a.L = s->L; a.NS = s->NS; a.NKC = s->NKC; a.NU = s->NU;
    const int tp = s->tp;
    a.npass = s->NU / tp;
    a.tmem_cols = s->tmem_s[tp];
    a.stage_bytes = s->stage_s[tp];
    a.nst = s->nst_s[tp];
    const int grid = std::min(a.npass, s->nsm);
    if (tp == 1) k_shtc_synth<1><<<grid, kRoleThreads, s->smem_s[1], st>>>(a);
    else k_shtc_synth<2><<<grid, kRoleThreads, s->smem_s[2], st>>>(a);
}

int shtc_tiles_per_pass(const ShTc* s) { return s->tp; }
bool shtc_tiles_per_pass_ok(const ShTc* s, int tp) { return (tp == 1 || tp == 2) && s->tp_ok[tp]; }
void shtc_set_tiles_per_pass(ShTc* s, int tp) { s->tp = (tp == 2 && s->tp_ok[2]) ? 2 : 1; }
int shtc_kernels_per_step() { return 5; }

}  // namespace odis
