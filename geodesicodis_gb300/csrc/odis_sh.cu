// Spherical-harmonic self-gravity / loading kernels (see odis_sh.cuh).
//
// Storage: the real harmonic Y_lm(cos|sin) = Pbar_lm(sin lat) * (cos|sin)(m lon)
// is never stored.  Each cell keeps the (L+1)(L+2)/2 normalised Legendre values
// Pbar_lm in rows ordered by order m (P[row(l,m)][Np]) plus cos(m lon) and
// sin(m lon) rows: 187 rows at L = 16 instead of 289 rows of Y.
//
// Half basis.  On a centrally symmetric mesh every cell a has an antipodal
// partner b (x_b = -x_a: lat -> -lat, lon -> lon + pi), and there
// Pbar_lm(-z) cos|sin(m (lon + pi)) = (-1)^(l+m) (-1)^m Y_lm = (-1)^l Y_lm.
// The rows are then stored for one cell of each pair only (half the bytes:
// 31 MB in FP64/DF64 at level 6), and
//   analysis  t_lm = sum_a Y_lm(a) (eta_a + (-1)^l eta_b)
//   synthesis usg_a = E + O, usg_b = E - O  (E, O: the even- and odd-degree sums at a)
// halve the multiply-adds of both transforms.  Without the symmetry (or with
// ODIS_SH_HALF=0) the full basis is used.
//
// Per step:
//   k_sh_pair:     e = eta_a + eta_b, o = eta_a - eta_b per pair (half basis only)
//   k_sh_analysis: blocks of (order m, up to 8 degrees, chunk of cells);
//                  partial sums of Pbar_lm * (cos|sin)(m lon) * eta (or e / o) per
//                  chunk; the last block of each tile folds its chunk partials
//   k_sh_coef:     c = F (Y^T Y)^-1 t  (least squares as SHExpandLSQ, factors F)
//   k_sh_synth:    usg_i = sum_m cos(m lon) sum_l Pbar_lm c_lm,cos + sin(m lon) sum_l Pbar_lm c_lm,sin
// The Legendre values are computed in FP64 on the host (three-term recurrences
// of the fully normalised functions, Holmes & Featherstone 2002), the Gram
// matrix Y^T Y in FP64 on the device over all cells, its inverse in FP64
// (Cholesky) on the host.  The arithmetic of the per-step transforms follows
// the method: FP64, double-float (DF64) or FP32 (FP32-state variant; block sums
// in FP64).
#include "odis_sh.cuh"
#include "odis_sh_tc.cuh"
#include "odis_df64.cuh"
#include "odis_arith.cuh"
#include "odis_pdl.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <cstdio>
#include <cstdlib>
#include <type_traits>
#include <unordered_map>
#include <vector>

namespace odis {

namespace {

constexpr double kPi = 3.1415926535897932384626433832795028841971693993751058;
constexpr int kShThreads = 256;
constexpr int kSynthThreads = 128;
constexpr int kSynthPairs = 16;    // "lanes" value that selects the warp-per-order-pair synthesis
constexpr int kSynthMaxWarps = 17; // its warps per cell group (l_max 32 has 17 order pairs; more pairs share warps)
constexpr int kSynthMaxThreads = 1024;
constexpr int kMaxChunks = 64;     // largest cell-chunk count the autotuner tries

// fully normalised (4pi) associated Legendre functions with the Condon-Shortley
// phase, P[l(l+1)/2 + m], argument z = cos(colatitude)
void plm_bar(int L, double z, std::vector<double>& P)
{
    P.assign((size_t)(L + 1) * (L + 2) / 2, 0.0);
    const double s = std::sqrt(std::fmax(0.0, 1.0 - z * z));
    P[0] = 1.0;
    double pmm = 1.0;
    for (int m = 1; m <= L; m++) {
        const double f = (m == 1) ? std::sqrt(3.0) : std::sqrt((2.0 * m + 1.0) / (2.0 * m));
        pmm = -f * s * pmm;
        P[(size_t)m * (m + 1) / 2 + m] = pmm;
    }
    for (int m = 0; m <= L; m++) {
        if (m + 1 <= L) P[(size_t)(m + 1) * (m + 2) / 2 + m] = std::sqrt(2.0 * m + 3.0) * z * P[(size_t)m * (m + 1) / 2 + m];
        for (int l = m + 2; l <= L; l++) {
            const double ll = (double)l * l - (double)m * m;
            const double a = std::sqrt((4.0 * l * l - 1.0) / ll);
            const double b = std::sqrt(((2.0 * l + 1.0) * ((l - 1.0) * (l - 1.0) - (double)m * m)) / ((2.0 * l - 3.0) * ll));
            P[(size_t)l * (l + 1) / 2 + m] = a * z * P[(size_t)(l - 1) * l / 2 + m] - b * P[(size_t)(l - 2) * (l - 1) / 2 + m];
        }
    }
}

// arithmetic of each method: Ar<T> (odis_arith.cuh)

// partial[k][chunk] = sum over the chunk's cells of Pbar_lm (cos|sin)(m lon) eta,
// for the degrees l0 .. l0+nl-1 of order m of this block's tile.
// kHalf: the basis is stored for one cell of each antipodal pair (N of them,
// row stride Np), and `eta` holds e = eta_a + eta_b in [0, Np) and
// o = eta_a - eta_b in [Np, 2 Np); since Y_lm(-x) = (-1)^l Y_lm(x), even
// degrees sum Y_lm e and odd degrees Y_lm o over the half set.  The tiles then
// hold one parity each (degrees l0, l0 + 2, ...), so a block reads only e or o.
// kPre: `eta` holds the trig-weighted values of every order, written once per
// step by k_sh_prep (rows 4m..4m+3: cos e, sin e, cos o, sin o with the half
// basis; rows 2m, 2m+1: cos eta, sin eta with the full one), so the loop is
// multiply-adds only; otherwise each tile forms those products itself.
//
// The last of a tile's nchunk blocks to finish (a per-tile arrival counter,
// reset by that block for the next step) folds the tile's coefficients over
// the chunks into t in FP64, in the fixed order of k_sh_fold: the result does
// not depend on which block comes last, and the step needs no fold launch.
template <class T, int kTileL, bool kHalf, bool kPre>
__global__ void __launch_bounds__(kShThreads) k_sh_analysis(const T* __restrict__ P, const T* __restrict__ trig,
                                                            const T* __restrict__ eta, int N, int Np, int L,
                                                            const int* __restrict__ tiles, int nchunk,
                                                            T* __restrict__ part, unsigned* __restrict__ arrivals,
                                                            double* __restrict__ t)
{
    pdl_wait();
    using A = Ar<T>;
    // per-thread sums of the block's tile, [coefficient][thread]: 32 KB for 8 degrees in FP64
    __shared__ T red[2 * kTileL][kShThreads];
    const int m = tiles[3 * blockIdx.x], l0 = tiles[3 * blockIdx.x + 1], nl = tiles[3 * blockIdx.x + 2];
    const int chunk = blockIdx.y;
    // chunk bounds are even, so cell pairs (i, i+1) stay inside one chunk and are 2-aligned
    const int per = ((N + nchunk - 1) / nchunk + 1) & ~1;
    const int i0 = min(N, chunk * per), i1 = min(N, i0 + per);
    T ac[kTileL], as[kTileL], bc[kTileL], bs[kTileL];
#pragma unroll
    for (int j = 0; j < kTileL; j++) { ac[j] = A::zero(); as[j] = A::zero(); bc[j] = A::zero(); bs[j] = A::zero(); }
    const T* cm = trig + (size_t)(2 * m) * Np;
    const T* sm = trig + (size_t)(2 * m + 1) * Np;
    const T* prow = P + (size_t)p_row(L, l0, m) * Np;
    // kHalf: a tile's degrees share one parity (l0, l0 + 2, ...), so it needs only e or only o
    constexpr int kStride = kHalf ? 2 : 1;
    const bool odd = kHalf && (l0 & 1);
    const T* xm = eta + (size_t)(kHalf ? 4 * m + (odd ? 2 : 0) : 2 * m) * Np;   // kPre: cos x, sin x rows
    const T* ev = eta + (odd ? (size_t)Np : 0);                                 // otherwise: e or o
    // two adjacent cells per thread and iteration, each row read with one vector load;
    // two iterations unrolled so their loads are in flight together
    int i = i0 + 2 * threadIdx.x;
#pragma unroll 2
    for (; i + 1 < i1; i += 2 * kShThreads) {
        T ec, es, ec2, es2;
        if constexpr (kPre) {
            A::ld2(xm + i, ec, ec2);
            A::ld2(xm + Np + i, es, es2);
        } else {
            T e, e2, c1, c2, s1, s2;
            A::ld2(ev + i, e, e2);
            A::ld2(cm + i, c1, c2);
            A::ld2(sm + i, s1, s2);
            ec = A::mul(c1, e); es = A::mul(s1, e);
            ec2 = A::mul(c2, e2); es2 = A::mul(s2, e2);
        }
#pragma unroll
        for (int j = 0; j < kTileL; j++) {
            if (j < nl) {
                T p, p2;
                A::ld2(prow + (size_t)(kStride * j) * Np + i, p, p2);
                ac[j] = A::fma_acc(p, ec, ac[j]);
                as[j] = A::fma_acc(p, es, as[j]);
                bc[j] = A::fma_acc(p2, ec2, bc[j]);
                bs[j] = A::fma_acc(p2, es2, bs[j]);
            }
        }
    }
    if (i < i1) {           // the last cell of an odd-length final chunk
        T ec, es;
        if constexpr (kPre) {
            ec = xm[i]; es = xm[Np + i];
        } else {
            const T e = ev[i];
            ec = A::mul(cm[i], e); es = A::mul(sm[i], e);
        }
#pragma unroll
        for (int j = 0; j < kTileL; j++) {
            if (j < nl) {
                const T p = prow[(size_t)(kStride * j) * Np + i];
                ac[j] = A::fma_acc(p, ec, ac[j]);
                as[j] = A::fma_acc(p, es, as[j]);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < kTileL; j++) {
        ac[j] = A::add(A::norm(ac[j]), A::norm(bc[j]));
        as[j] = A::add(A::norm(as[j]), A::norm(bs[j]));
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    // block sum of each of the tile's 2 nl coefficients: every thread parks its sums in shared
    // memory, then one warp per coefficient adds eight values per lane and a shuffle tree --
    // a fixed order, and a third of the additions of a per-warp shuffle tree of every sum
#pragma unroll
    for (int j = 0; j < kTileL; j++) {
        if (j < nl) { red[2 * j][threadIdx.x] = ac[j]; red[2 * j + 1][threadIdx.x] = as[j]; }
    }
    __syncthreads();
    for (int q = wid; q < 2 * nl; q += kShThreads / 32) {
        T x = red[q][lane];
#pragma unroll
        for (int r = 1; r < kShThreads / 32; r++) x = A::add(x, red[q][lane + 32 * r]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x = A::add(x, A::shfl(x, o));
        const int j = q >> 1, is_sin = q & 1;
        if (lane == 0 && (m > 0 || !is_sin)) part[(size_t)sh_col(l0 + kStride * j, m, is_sin) * nchunk + chunk] = x;
    }
    // publish the partials, then count this block in
    __threadfence();
    __syncthreads();
    __shared__ bool s_last;
    if (threadIdx.x == 0) s_last = atomicAdd(&arrivals[blockIdx.x], 1u) == (unsigned)(nchunk - 1);
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    for (int q = wid; q < 2 * nl; q += kShThreads / 32) {       // one warp per coefficient of the tile
        const int j = q >> 1, is_sin = q & 1;
        if (m == 0 && is_sin) continue;
        const int k = sh_col(l0 + kStride * j, m, is_sin);
        double x = 0.0;
        for (int c = lane; c < nchunk; c += 32) x += A::to(A::ldcg(&part[(size_t)k * nchunk + c]));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) t[k] = x;
    }
    if (threadIdx.x == 0) arrivals[blockIdx.x] = 0u;             // ready for the next step
}

// e and o of the antipodal pairs (kHalf transforms): eo[h] = eta[ia[h]] + eta[ib[h]],
// eo[Np + h] = eta[ia[h]] - eta[ib[h]]; zero on the padding h >= N
template <class T>
__global__ void __launch_bounds__(256) k_sh_pair(const T* __restrict__ eta, const int* __restrict__ ia,
                                                 const int* __restrict__ ib, int N, int Np, T* __restrict__ eo)
{
    pdl_wait();
    using A = Ar<T>;
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= Np) return;
    T e = A::zero(), o = A::zero();
    if (h < N) {
        const T a = eta[ia[h]], b = eta[ib[h]];
        e = A::add(a, b);
        o = A::sub(a, b);
    }
    eo[h] = e;
    eo[Np + h] = o;
}

// trig-weighted values of every order for the kPre analysis, one (cell, order)
// per thread (grid.y = order): half basis x[4m..4m+3][h] = (cos e, sin e, cos o,
// sin o)(m lon_h) with e, o = eta_a +- eta_b; full basis x[2m], x[2m+1] =
// (cos, sin)(m lon_i) eta_i; zero on the padding
template <class T, bool kHalf>
__global__ void __launch_bounds__(256) k_sh_prep(const T* __restrict__ eta, const int* __restrict__ ia,
                                                 const int* __restrict__ ib, const T* __restrict__ trig, int N,
                                                 int Np, int L, T* __restrict__ x)
{
    pdl_wait();
    using A = Ar<T>;
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    const int m = blockIdx.y;
    if (h >= Np) return;
    T e = A::zero(), o = A::zero();
    if (h < N) {
        if constexpr (kHalf) {
            const T a = eta[__ldg(&ia[h])], b = eta[__ldg(&ib[h])];
            e = A::add(a, b);
            o = A::sub(a, b);
        } else {
            e = eta[h];
        }
    }
    const T c = trig[(size_t)(2 * m) * Np + h], sn = trig[(size_t)(2 * m + 1) * Np + h];
    if constexpr (kHalf) {
        T* xm = x + (size_t)(4 * m) * Np + h;
        xm[0] = A::mul(c, e);
        xm[(size_t)Np] = A::mul(sn, e);
        xm[2 * (size_t)Np] = A::mul(c, o);
        xm[3 * (size_t)Np] = A::mul(sn, o);
    } else {
        T* xm = x + (size_t)(2 * m) * Np + h;
        xm[0] = A::mul(c, e);
        xm[(size_t)Np] = A::mul(sn, e);
    }
}

// t_k = sum over the chunk partials of coefficient k in FP64, one warp per
// coefficient: lane j adds chunks j, j+32, ... then the lanes meet in a fixed
// shuffle tree (the order does not depend on timing)
template <class T>
__global__ void __launch_bounds__(128) k_sh_fold(const T* __restrict__ part, int K, int nchunk, double* __restrict__ t)
{
    pdl_wait();
    using A = Ar<T>;
    const int k = blockIdx.x * 4 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (k >= K) return;
    double s = 0.0;
    for (int c = lane; c < nchunk; c += 32) s += A::to(part[(size_t)k * nchunk + c]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) t[k] = s;
}

// c = (F G^-1) t in FP64, one warp per coefficient, stored in the method's type
template <class T>
__global__ void __launch_bounds__(32) k_sh_coef(const double* __restrict__ t, int K, const double* __restrict__ FGinv,
                                                T* __restrict__ coef)
{
    pdl_wait();
    const int a = blockIdx.x;
    const double* row = FGinv + (size_t)a * K;
    double s = 0.0;
    for (int b = threadIdx.x; b < K; b += 32) s = fma(row[b], t[b], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) coef[a] = Ar<T>::from(s);
}

// usg_i = sum_{m} [cos(m lon) sum_{l>=max(m,2)} Pbar_lm c_lm,cos + sin(m lon) sum_l Pbar_lm c_lm,sin]
// kSynthLanes consecutive threads share a cell and split the orders m between
// them (m = j, j + kSynthLanes, ...); their sums meet by shuffles in a fixed
// order.  Two independent accumulator pairs keep two loads in flight per lane.
// kHalf: the basis covers one cell h of each antipodal pair (N of them); the
// even- and odd-degree sums E and O are kept apart (consecutive degrees go to
// the two accumulator sets in turn) and the pair's cells receive E + O
// (ia[h]) and E - O (ib[h]), since Y_lm(-x) = (-1)^l Y_lm(x).
template <class T, int kSynthLanes, int kCells, bool kHalf>
__global__ void __launch_bounds__(kSynthThreads) k_sh_synth(const T* __restrict__ P, const T* __restrict__ trig,
                                                            const T* __restrict__ coef, int N, int Np, int L, int K,
                                                            const int* __restrict__ ia, const int* __restrict__ ib,
                                                            T* __restrict__ usg)
{
    pdl_wait();
    using A = Ar<T>;
    extern __shared__ unsigned char c_raw[];
    T* c = reinterpret_cast<T*>(c_raw);
    for (int k = threadIdx.x; k < K; k += kSynthThreads) c[k] = coef[k];
    __syncthreads();
    // each thread sums orders m = j, j + lanes, ... for the cell q (kCells = 1) or the
    // adjacent cells 2q and 2q+1 (kCells = 2)
    const int gt = blockIdx.x * kSynthThreads + threadIdx.x;
    const int q = gt / kSynthLanes, j = gt % kSynthLanes;
    const int i = kCells * q, i2 = kCells == 2 ? min(2 * q + 1, N - 1) : i;
    const bool pair = kCells == 2 && i2 == i + 1;   // i is even, so (i, i+1) is one aligned vector
    T u = A::zero(), u2 = A::zero();     // full basis: the sums; kHalf: the even-degree sums E
    T w = A::zero(), w2 = A::zero();     // kHalf: the odd-degree sums O
    if (i < N) {
        for (int m = j; m <= L; m += kSynthLanes) {
            // set X takes degrees lstart, lstart + 2, ...; set Y lstart + 1, lstart + 3, ...
            T xa0 = A::zero(), xb0 = A::zero(), xa1 = A::zero(), xb1 = A::zero();
            T ya0 = A::zero(), yb0 = A::zero(), ya1 = A::zero(), yb1 = A::zero();
            const int lstart = m < 2 ? 2 : m;
            const T* prow = P + (size_t)p_row(L, lstart, m) * Np;
            // the order's trig values are loaded first and are in flight during the degree loop
            const T* cr = trig + (size_t)(2 * m) * Np;
            const T* sr = trig + (size_t)(2 * m + 1) * Np;
            T c0, c1, s0, s1;
            if (pair) { A::ld2(cr + i, c0, c1); A::ld2(sr + i, s0, s1); }
            else { c0 = cr[i]; c1 = cr[i2]; s0 = sr[i]; s1 = sr[i2]; }
            auto stepx = [&](int l, T p0, T p1, T& a0, T& b0, T& a1, T& b1) {
                const T cc = c[sh_col(l, m, 0)];
                a0 = A::fma_acc(p0, cc, a0);
                if (kCells == 2) a1 = A::fma_acc(p1, cc, a1);
                if (m > 0) {
                    const T cs = c[sh_col(l, m, 1)];
                    b0 = A::fma_acc(p0, cs, b0);
                    if (kCells == 2) b1 = A::fma_acc(p1, cs, b1);
                }
            };
            int l = lstart;
            // four rows' loads issued before their multiply-adds (four L2 requests in flight)
            for (; l + 3 <= L; l += 4) {
                T p0[4], p1[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const T* pr = prow + (size_t)(l + q - lstart) * Np;
                    if (pair) A::ld2(pr + i, p0[q], p1[q]);
                    else { p0[q] = pr[i]; p1[q] = kCells == 2 ? pr[i2] : p0[q]; }
                }
                if constexpr (kHalf) {
                    stepx(l, p0[0], p1[0], xa0, xb0, xa1, xb1);
                    stepx(l + 1, p0[1], p1[1], ya0, yb0, ya1, yb1);
                    stepx(l + 2, p0[2], p1[2], xa0, xb0, xa1, xb1);
                    stepx(l + 3, p0[3], p1[3], ya0, yb0, ya1, yb1);
                } else {
#pragma unroll
                    for (int q = 0; q < 4; q++) stepx(l + q, p0[q], p1[q], xa0, xb0, xa1, xb1);
                }
            }
            for (; l <= L; l++) {
                const T* pr = prow + (size_t)(l - lstart) * Np;
                T p0, p1;
                if (pair) A::ld2(pr + i, p0, p1);
                else { p0 = pr[i]; p1 = kCells == 2 ? pr[i2] : p0; }
                if (kHalf && ((l - lstart) & 1)) stepx(l, p0, p1, ya0, yb0, ya1, yb1);
                else stepx(l, p0, p1, xa0, xb0, xa1, xb1);
            }
            if constexpr (kHalf) {
                const bool xodd = lstart & 1;             // set X holds the degrees of lstart's parity
                const T ea0 = xodd ? ya0 : xa0, eb0 = xodd ? yb0 : xb0, oa0 = xodd ? xa0 : ya0, ob0 = xodd ? xb0 : yb0;
                u = A::fma(c0, A::norm(ea0), A::fma(s0, A::norm(eb0), u));
                w = A::fma(c0, A::norm(oa0), A::fma(s0, A::norm(ob0), w));
                if (kCells == 2) {
                    const T ea1 = xodd ? ya1 : xa1, eb1 = xodd ? yb1 : xb1, oa1 = xodd ? xa1 : ya1, ob1 = xodd ? xb1 : yb1;
                    u2 = A::fma(c1, A::norm(ea1), A::fma(s1, A::norm(eb1), u2));
                    w2 = A::fma(c1, A::norm(oa1), A::fma(s1, A::norm(ob1), w2));
                }
            } else {
                u = A::fma(c0, A::norm(xa0), A::fma(s0, A::norm(xb0), u));
                if (kCells == 2) u2 = A::fma(c1, A::norm(xa1), A::fma(s1, A::norm(xb1), u2));
            }
        }
    }
#pragma unroll
    for (int o = kSynthLanes / 2; o > 0; o >>= 1) {
        u = A::add(u, A::shfl(u, o));
        if (kCells == 2) u2 = A::add(u2, A::shfl(u2, o));
        if (kHalf) {
            w = A::add(w, A::shfl(w, o));
            if (kCells == 2) w2 = A::add(w2, A::shfl(w2, o));
        }
    }
    if (i < N && j == 0) {
        if constexpr (kHalf) {
            usg[ia[i]] = A::add(u, w);
            usg[ib[i]] = A::sub(u, w);
            if (kCells == 2 && 2 * q + 1 < N) {
                usg[ia[2 * q + 1]] = A::add(u2, w2);
                usg[ib[2 * q + 1]] = A::sub(u2, w2);
            }
        } else {
            usg[i] = u;
            if (kCells == 2 && 2 * q + 1 < N) usg[2 * q + 1] = u2;
        }
    }
}

// Synthesis with one warp per pair of orders (m, L - m) (the middle order alone
// for even L): the degree counts of a pair add up to L + 2, so the warps of a
// block are balanced without splitting an order's degree sum.  A block covers
// 32 kCells consecutive basis cells (lanes: cells, kCells adjacent cells per
// lane with one vector load per row); every warp sums its orders for every cell
// of the block, and the warps' sums meet in shared memory in warp order.  With
// (L + 2) / 2 warps per block this keeps several times more warps resident than
// the lane-per-order kernel, whose per-cell thread count the half basis halves.
// kGroups: cell groups of 32 kCells cells per block (warp w: order pair w % nw,
// cell group w / nw), so the coefficients are staged once for kGroups groups.
template <class T, int kCells, bool kHalf, int kGroups>
__global__ void __launch_bounds__(kGroups * kSynthMaxWarps * 32 < kSynthMaxThreads ? kGroups * kSynthMaxWarps * 32
                                                                                    : kSynthMaxThreads) k_sh_synth_m(const T* __restrict__ P, const T* __restrict__ trig,
                                                     const T* __restrict__ coef, int N, int Np, int L, int K,
                                                     const int* __restrict__ ia, const int* __restrict__ ib,
                                                     T* __restrict__ usg)
{
    pdl_wait();
    using A = Ar<T>;
    extern __shared__ unsigned char c_raw[];
    T* c = reinterpret_cast<T*>(c_raw);
    T* red = c + ((K + 1) & ~1);               // [warps][32][4]: u, u2, w, w2 of every lane
    for (int k = threadIdx.x; k < K; k += blockDim.x) c[k] = coef[k];
    __syncthreads();
    const int lane = threadIdx.x & 31, nw = (blockDim.x >> 5) / kGroups;
    const int grp = (threadIdx.x >> 5) / nw, wid = (threadIdx.x >> 5) % nw;
    const int i = ((blockIdx.x * kGroups + grp) * 32 + lane) * kCells;
    const int i2 = kCells == 2 ? min(i + 1, N - 1) : i;
    const bool pair = kCells == 2 && i2 == i + 1;
    T u = A::zero(), u2 = A::zero();     // full basis: the sums; kHalf: the even-degree sums E
    T w = A::zero(), w2 = A::zero();     // kHalf: the odd-degree sums O
    const int npairs = L / 2 + 1;
    if (i < N) {
        for (int pr = wid; pr < npairs; pr += nw)
            for (int side = 0; side < 2; side++) {
                const int m = side == 0 ? pr : L - pr;
                if (side == 1 && m == pr) break;
                T xa0 = A::zero(), xb0 = A::zero(), xa1 = A::zero(), xb1 = A::zero();
                T ya0 = A::zero(), yb0 = A::zero(), ya1 = A::zero(), yb1 = A::zero();
                const int lstart = m < 2 ? 2 : m;
                const T* prow = P + (size_t)p_row(L, lstart, m) * Np;
                const T* cr = trig + (size_t)(2 * m) * Np;
                const T* sr = trig + (size_t)(2 * m + 1) * Np;
                T c0, c1, s0, s1;
                if (pair) { A::ld2(cr + i, c0, c1); A::ld2(sr + i, s0, s1); }
                else { c0 = cr[i]; c1 = cr[i2]; s0 = sr[i]; s1 = sr[i2]; }
                auto stepx = [&](int l, T p0, T p1, T& a0, T& b0, T& a1, T& b1) {
                    const T cc = c[sh_col(l, m, 0)];
                    a0 = A::fma_acc(p0, cc, a0);
                    if (kCells == 2) a1 = A::fma_acc(p1, cc, a1);
                    if (m > 0) {
                        const T cs = c[sh_col(l, m, 1)];
                        b0 = A::fma_acc(p0, cs, b0);
                        if (kCells == 2) b1 = A::fma_acc(p1, cs, b1);
                    }
                };
                int l = lstart;
                for (; l + 3 <= L; l += 4) {            // four rows' loads in flight
                    T p0[4], p1[4];
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        const T* prq = prow + (size_t)(l + q - lstart) * Np;
                        if (pair) A::ld2(prq + i, p0[q], p1[q]);
                        else { p0[q] = prq[i]; p1[q] = kCells == 2 ? prq[i2] : p0[q]; }
                    }
                    if constexpr (kHalf) {
                        stepx(l, p0[0], p1[0], xa0, xb0, xa1, xb1);
                        stepx(l + 1, p0[1], p1[1], ya0, yb0, ya1, yb1);
                        stepx(l + 2, p0[2], p1[2], xa0, xb0, xa1, xb1);
                        stepx(l + 3, p0[3], p1[3], ya0, yb0, ya1, yb1);
                    } else {
#pragma unroll
                        for (int q = 0; q < 4; q++) stepx(l + q, p0[q], p1[q], xa0, xb0, xa1, xb1);
                    }
                }
                for (; l <= L; l++) {
                    const T* prq = prow + (size_t)(l - lstart) * Np;
                    T p0, p1;
                    if (pair) A::ld2(prq + i, p0, p1);
                    else { p0 = prq[i]; p1 = kCells == 2 ? prq[i2] : p0; }
                    if (kHalf && ((l - lstart) & 1)) stepx(l, p0, p1, ya0, yb0, ya1, yb1);
                    else stepx(l, p0, p1, xa0, xb0, xa1, xb1);
                }
                if constexpr (kHalf) {
                    const bool xodd = lstart & 1;
                    const T ea0 = xodd ? ya0 : xa0, eb0 = xodd ? yb0 : xb0, oa0 = xodd ? xa0 : ya0, ob0 = xodd ? xb0 : yb0;
                    u = A::fma(c0, A::norm(ea0), A::fma(s0, A::norm(eb0), u));
                    w = A::fma(c0, A::norm(oa0), A::fma(s0, A::norm(ob0), w));
                    if (kCells == 2) {
                        const T ea1 = xodd ? ya1 : xa1, eb1 = xodd ? yb1 : xb1, oa1 = xodd ? xa1 : ya1, ob1 = xodd ? xb1 : yb1;
                        u2 = A::fma(c1, A::norm(ea1), A::fma(s1, A::norm(eb1), u2));
                        w2 = A::fma(c1, A::norm(oa1), A::fma(s1, A::norm(ob1), w2));
                    }
                } else {
                    u = A::fma(c0, A::norm(xa0), A::fma(s0, A::norm(xb0), u));
                    if (kCells == 2) u2 = A::fma(c1, A::norm(xa1), A::fma(s1, A::norm(xb1), u2));
                }
            }
    }
    T* r = red + (size_t)(threadIdx.x) * 4;
    r[0] = u; r[1] = u2; r[2] = w; r[3] = w2;
    __syncthreads();
    if (wid == 0 && i < N) {
        T su = A::zero(), su2 = A::zero(), sw = A::zero(), sw2 = A::zero();
        for (int v = 0; v < nw; v++) {
            const T* x = red + (size_t)((grp * nw + v) * 32 + lane) * 4;
            su = A::add(su, x[0]); su2 = A::add(su2, x[1]); sw = A::add(sw, x[2]); sw2 = A::add(sw2, x[3]);
        }
        if constexpr (kHalf) {
            usg[ia[i]] = A::add(su, sw);
            usg[ib[i]] = A::sub(su, sw);
            if (kCells == 2 && i + 1 < N) {
                usg[ia[i + 1]] = A::add(su2, sw2);
                usg[ib[i + 1]] = A::sub(su2, sw2);
            }
        } else {
            usg[i] = su;
            if (kCells == 2 && i + 1 < N) usg[i + 1] = su2;
        }
    }
}

// Gram matrix G = Y^T Y in FP64 (setup only): 32x32 output tiles, lower triangle
__global__ void __launch_bounds__(256) k_gram(const double* __restrict__ Y, int K, int N, int Np, double* __restrict__ G)
{
    __shared__ double ya[32][33], yb[32][33];
    const int ta = blockIdx.y, tb = blockIdx.x;
    if (tb > ta) return;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;      // 8 rows of threads
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int i0 = 0; i0 < N; i0 += 32) {
        for (int r = ty; r < 32; r += 8) {
            const int ka = ta * 32 + r, kb = tb * 32 + r, i = i0 + tx;
            ya[r][tx] = (ka < K && i < N) ? Y[(size_t)ka * Np + i] : 0.0;
            yb[r][tx] = (kb < K && i < N) ? Y[(size_t)kb * Np + i] : 0.0;
        }
        __syncthreads();
        for (int q = 0; q < 4; q++) {
            const int r = ty + 8 * q;
#pragma unroll 8
            for (int x = 0; x < 32; x++) acc[q] = fma(ya[r][x], yb[tx][x], acc[q]);
        }
        __syncthreads();
    }
    for (int q = 0; q < 4; q++) {
        const int a = ta * 32 + ty + 8 * q, b = tb * 32 + tx;
        if (a < K && b < K) { G[(size_t)a * K + b] = acc[q]; G[(size_t)b * K + a] = acc[q]; }
    }
}

// (l, m, sin) of coefficient k = sh_col(l, m, sin)
__host__ __device__ inline void sh_lms(int k, int& l, int& m, int& s)
{
    l = 0;
    while ((l + 1) * (l + 1) <= k) l++;
    const int r = k - l * l;
    m = (r + 1) >> 1;
    s = r == 0 ? 0 : ((r + 1) & 1);
}

// Dense synthesis matrix Z[k][h] = sum_j Y_j(h) M[j][k] (setup only, FP64):
// usg = Y c = Y M t = Z t, so the per-step synthesis reads t directly and the
// K x K product disappears from the step.  Y_j(h) = P[row(j)][h] trig[2m+s][h]
// is formed while the tile is staged.  64 x 64 output tiles, 16 j per stage,
// 4 x 4 outputs per thread.  Rows k of Z are written in the method's type.
template <class T>
__global__ void __launch_bounds__(256) k_sh_zmat(const double* __restrict__ P, const double* __restrict__ trig,
                                                 const double* __restrict__ M, int L, int K, int np,
                                                 T* __restrict__ Z)
{
    __shared__ double ys[16][64 + 1], ms[16][64 + 1];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int h0 = blockIdx.x * 64, k0 = blockIdx.y * 64;
    double acc[4][4] = {};
    for (int j0 = 0; j0 < K; j0 += 16) {
        for (int q = threadIdx.x; q < 16 * 64; q += 256) {
            const int jj = q >> 6, c = q & 63, j = j0 + jj;
            double y = 0.0, mv = 0.0;
            if (j < K) {
                int l, m, s;
                sh_lms(j, l, m, s);
                y = P[(size_t)p_row(L, l, m) * np + h0 + c] * trig[(size_t)(2 * m + s) * np + h0 + c];
                if (k0 + c < K) mv = M[(size_t)j * K + k0 + c];
            }
            ys[jj][c] = y;
            ms[jj][c] = mv;
        }
        __syncthreads();
#pragma unroll
        for (int jj = 0; jj < 16; jj++)
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) acc[a][b] = fma(ys[jj][tx + 16 * a], ms[jj][ty + 16 * b], acc[a][b]);
        __syncthreads();
    }
#pragma unroll
    for (int b = 0; b < 4; b++) {
        const int k = k0 + ty + 16 * b;
        if (k >= K) continue;
#pragma unroll
        for (int a = 0; a < 4; a++) Z[(size_t)k * np + h0 + tx + 16 * a] = Ar<T>::from(acc[a][b]);
    }
}

// Dense synthesis usg = Z t: kW warps split the K rows (warp w takes rows w, w + kW,
// ...), each lane owns kC cells (h = base + lane + 32 c, so every row load of a warp
// is one coalesced line), t is staged once per block in the method's type.  Rows are
// taken four at a time, so each lane has 4 kC loads in flight.  kHalf: rows of even
// degree add to E, odd to O (a per-row flag in shared memory), and the pair's cells
// receive E + O and E - O.  The warps' partial sums meet in shared memory in warp
// order (a fixed order).
template <class T, bool kHalf, int kW, int kC>
__global__ void __launch_bounds__(32 * kW) k_sh_synth_z(const T* __restrict__ Z, const double* __restrict__ t, int n,
                                                        int np, int K, const int* __restrict__ ia,
                                                        const int* __restrict__ ib, T* __restrict__ usg)
{
    pdl_wait();
    using A = Ar<T>;
    constexpr int kU = 4;
    extern __shared__ unsigned char z_raw[];
    T* tk = reinterpret_cast<T*>(z_raw);                                     // [K]
    T* se = tk + ((K + 1) & ~1);                                             // [kW][32 kC]
    T* so = se + kW * 32 * kC;
    unsigned char* odd = reinterpret_cast<unsigned char*>(so + kW * 32 * kC); // [K] degree parity of row k
    for (int k = threadIdx.x; k < K; k += 32 * kW) {
        tk[k] = A::from(t[k]);
        int l = 0;
        while ((l + 1) * (l + 1) <= k) l++;
        odd[k] = (unsigned char)(kHalf && (l & 1));
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int base = blockIdx.x * 32 * kC;
    T e[kC], o[kC];
#pragma unroll
    for (int c = 0; c < kC; c++) { e[c] = A::zero(); o[c] = A::zero(); }
    const T* zc = Z + base + lane;
    for (int k0 = w; k0 < K; k0 += kU * kW) {
        T z[kU][kC];
#pragma unroll
        for (int u = 0; u < kU; u++) {
            const int k = k0 + u * kW;
#pragma unroll
            for (int c = 0; c < kC; c++) z[u][c] = k < K ? zc[(size_t)k * np + 32 * c] : A::zero();
        }
#pragma unroll
        for (int u = 0; u < kU; u++) {
            const int k = k0 + u * kW;
            if (k >= K) break;
            const T tv = tk[k];
            if (odd[k]) {
#pragma unroll
                for (int c = 0; c < kC; c++) o[c] = A::fma_acc(z[u][c], tv, o[c]);
            } else {
#pragma unroll
                for (int c = 0; c < kC; c++) e[c] = A::fma_acc(z[u][c], tv, e[c]);
            }
        }
    }
#pragma unroll
    for (int c = 0; c < kC; c++) {
        se[w * 32 * kC + 32 * c + lane] = A::norm(e[c]);
        so[w * 32 * kC + 32 * c + lane] = A::norm(o[c]);
    }
    __syncthreads();
    for (int q = threadIdx.x; q < 32 * kC; q += 32 * kW) {
        T E = se[q], O = so[q];
#pragma unroll
        for (int v = 1; v < kW; v++) { E = A::add(E, se[v * 32 * kC + q]); O = A::add(O, so[v * 32 * kC + q]); }
        const int h = base + q;
        if (h >= n) continue;
        if constexpr (kHalf) {
            usg[__ldg(&ia[h])] = A::add(E, O);
            usg[__ldg(&ib[h])] = A::sub(E, O);
        } else {
            usg[h] = E;
        }
    }
}

}  // namespace

int sh_autotune(ShLoading* s);

struct ShLoading {
    int L = 0, K = 0, MP = 0, N = 0, Np = 0, precision = ODIS_FP64, ntiles = 0;
    int tl = 8, nchunk = 16, lanes = 4;   // tile shapes chosen by the autotuner
    bool pre = false;                     // analysis from trig-weighted values formed once per step
    int cells = 2;                        // synthesis cells per thread
    void* P = nullptr;           // [MP][Np] Legendre rows, method type
    void* trig = nullptr;        // [2(L+1)][Np] cos(m lon), sin(m lon), method type
    int* tiles = nullptr;        // [ntiles][3] (m, l0, nl)
    void* part = nullptr;        // [K][nchunk] chunk partials, method type
    double* FGinv = nullptr;     // [K][K]
    double* t = nullptr;
    void* coef = nullptr;        // [K] coefficients, method type
    void* usg = nullptr;         // [Np] method type
    ShTc* tc = nullptr;          // tensor-core transforms (FP32 method), when they fit
    bool use_tc = false;         // setup-time choice between the tc and CUDA-core transforms
    int* status = nullptr;       // context status word (device)
    // antipodal half basis: P and trig hold the Nh cells ia[h] (one of each pair
    // {ia[h], ib[h]} of antipodal cells), rows of stride Nhp
    bool half = false;
    int Nh = 0, Nhp = 0;
    int* ia = nullptr;           // [Nhp] (padding repeats the last pair)
    int* ib = nullptr;
    void* eo = nullptr;          // [2][Nhp] e = eta_a + eta_b, o = eta_a - eta_b, or the trig-weighted values
                                 // [4(L+1)][Nhp] (half) / [2(L+1)][Np] (full) of the pre analysis; method type
    unsigned* arrivals = nullptr; // [analysis tiles] blocks of a tile that finished this step (reset by the last)
    // dense synthesis usg = Z t (Z = Y F G^-1, [K][bp], method type), chosen by the timing when faster than the
    // K x K product plus the factored synthesis: zw warps per block (0: factored), zc cells per lane
    void* Z = nullptr;
    int zw = 0, zc = 1;
    int zw_cand = 0, zc_cand = 1;   // the fastest dense variant in isolation, offered to the whole-step timing
    bool zforced = false;           // ODIS_SH_TILES named the synthesis
    // cells and row stride of the stored basis
    int bn() const { return half ? Nh : N; }
    int bp() const { return half ? Nhp : Np; }
};

// Antipodal pairing of the mesh's cells: b = a(i) with x_b = -x_i to within
// `tol` (unit vectors), a(a(i)) = i, a(i) != i, for every cell; false if the
// mesh has no such symmetry.  The icosahedral grids are centrally symmetric.
static bool antipodal_pairs(const Mesh& m, double tol, std::vector<int>& partner)
{
    const int N = m.N;
    partner.assign(N, -1);
    std::vector<double> x((size_t)3 * N);
    for (int i = 0; i < N; i++) {
        const double lat = m.node_sph[(size_t)i * 2], lon = m.node_sph[(size_t)i * 2 + 1];
        x[3 * i] = std::cos(lat) * std::cos(lon);
        x[3 * i + 1] = std::cos(lat) * std::sin(lon);
        x[3 * i + 2] = std::sin(lat);
    }
    // cells bucketed on a grid of spacing q; a partner lies in the bucket of -x or a neighbour of it
    const double q = 1e-4;
    auto key = [](long long a, long long b, long long c) {
        return (unsigned long long)((a & 0x1fffff) | ((b & 0x1fffff) << 21) | ((c & 0x1fffff) << 42));
    };
    std::unordered_map<unsigned long long, std::vector<int>> grid;
    grid.reserve((size_t)N * 2);
    for (int i = 0; i < N; i++)
        grid[key(std::llround(x[3 * i] / q), std::llround(x[3 * i + 1] / q), std::llround(x[3 * i + 2] / q))].push_back(i);
    for (int i = 0; i < N; i++) {
        const long long k0 = std::llround(-x[3 * i] / q), k1 = std::llround(-x[3 * i + 1] / q),
                        k2 = std::llround(-x[3 * i + 2] / q);
        double best = tol;
        for (int d0 = -1; d0 <= 1; d0++)
            for (int d1 = -1; d1 <= 1; d1++)
                for (int d2 = -1; d2 <= 1; d2++) {
                    auto it = grid.find(key(k0 + d0, k1 + d1, k2 + d2));
                    if (it == grid.end()) continue;
                    for (int j : it->second) {
                        const double d = std::fabs(x[3 * j] + x[3 * i]) + std::fabs(x[3 * j + 1] + x[3 * i + 1]) +
                                         std::fabs(x[3 * j + 2] + x[3 * i + 2]);
                        if (d <= best) { best = d; partner[i] = j; }
                    }
                }
        if (partner[i] < 0 || partner[i] == i) return false;
    }
    for (int i = 0; i < N; i++)
        if (partner[partner[i]] != i) return false;
    return true;
}

void sh_basis_host(const Mesh& m, int L, std::vector<double>& Y)
{
    const int K = (L + 1) * (L + 1);
    Y.assign((size_t)m.N * K, 0.0);
#pragma omp parallel
    {
        std::vector<double> P;
#pragma omp for schedule(static)
        for (int i = 0; i < m.N; i++) {
            const double lat = m.node_sph[(size_t)i * 2], lon = m.node_sph[(size_t)i * 2 + 1];
            plm_bar(L, std::cos(kPi * 0.5 - lat), P);
            for (int l = 0; l <= L; l++)
                for (int mm = 0; mm <= l; mm++) {
                    const double p = P[(size_t)l * (l + 1) / 2 + mm];
                    Y[(size_t)i * K + sh_col(l, mm, 0)] = p * std::cos((double)mm * lon);
                    if (mm > 0) Y[(size_t)i * K + sh_col(l, mm, 1)] = p * std::sin((double)mm * lon);
                }
        }
    }
}

static int chol_inverse(std::vector<double>& A, int n)
{
    // A = R R^T (lower R), then A^-1 by solving for the identity
    std::vector<double> Lw(A);
    for (int j = 0; j < n; j++) {
        double d = Lw[(size_t)j * n + j];
        for (int k = 0; k < j; k++) d -= Lw[(size_t)j * n + k] * Lw[(size_t)j * n + k];
        if (!(d > 0.0)) return ODIS_ERR_ARG;
        d = std::sqrt(d);
        Lw[(size_t)j * n + j] = d;
#pragma omp parallel for schedule(static)
        for (int i = j + 1; i < n; i++) {
            double s = Lw[(size_t)i * n + j];
            for (int k = 0; k < j; k++) s -= Lw[(size_t)i * n + k] * Lw[(size_t)j * n + k];
            Lw[(size_t)i * n + j] = s / d;
        }
    }
    std::vector<double> inv((size_t)n * n, 0.0);
#pragma omp parallel for schedule(dynamic)
    for (int c = 0; c < n; c++) {
        std::vector<double> x(n, 0.0);
        for (int i = 0; i < n; i++) {
            double s = (i == c) ? 1.0 : 0.0;
            for (int k = 0; k < i; k++) s -= Lw[(size_t)i * n + k] * x[k];
            x[i] = s / Lw[(size_t)i * n + i];
        }
        for (int i = n - 1; i >= 0; i--) {
            double s = x[i];
            for (int k = i + 1; k < n; k++) s -= Lw[(size_t)k * n + i] * x[k];
            x[i] = s / Lw[(size_t)i * n + i];
        }
        for (int i = 0; i < n; i++) inv[(size_t)i * n + c] = x[i];
    }
    A.swap(inv);
    return ODIS_OK;
}

template <class T>
static T host_cvt(double x);
template <> double host_cvt<double>(double x) { return x; }
template <> float host_cvt<float>(double x) { return (float)x; }
template <> df64 host_cvt<df64>(double x) { return df_from_double(x); }

template <class T>
static bool upload_rows(void** d, const std::vector<double>& h)
{
    std::vector<T> v(h.size());
    for (size_t q = 0; q < h.size(); q++) v[q] = host_cvt<T>(h[q]);
    if (cudaMalloc(d, sizeof(T) * v.size()) != cudaSuccess) { *d = nullptr; return false; }
    return cudaMemcpy(*d, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice) == cudaSuccess;
}

static bool forced_tiles(int* f);

int sh_create(ShLoading** out, const Mesh& m, int L, const double* factors, int precision, int Np, int* status)
{
    *out = nullptr;
    const int K = (L + 1) * (L + 1), MP = (L + 1) * (L + 2) / 2;
    if (L < 2 || m.N < K) return ODIS_ERR_ARG;
    const int N = m.N;
    // Legendre rows, trig rows (host, FP64)
    std::vector<double> P((size_t)MP * Np, 0.0), trig((size_t)2 * (L + 1) * Np, 0.0);
#pragma omp parallel
    {
        std::vector<double> pl;
#pragma omp for schedule(static)
        for (int i = 0; i < N; i++) {
            const double lat = m.node_sph[(size_t)i * 2], lon = m.node_sph[(size_t)i * 2 + 1];
            plm_bar(L, std::cos(kPi * 0.5 - lat), pl);
            for (int mm = 0; mm <= L; mm++) {
                for (int l = mm; l <= L; l++) P[(size_t)p_row(L, l, mm) * Np + i] = pl[(size_t)l * (l + 1) / 2 + mm];
                trig[(size_t)(2 * mm) * Np + i] = std::cos((double)mm * lon);
                trig[(size_t)(2 * mm + 1) * Np + i] = std::sin((double)mm * lon);
            }
        }
    }
    // Gram matrix on the device from the full basis Y[K][Np] (FP64, setup only)
    std::vector<double> G((size_t)K * K, 0.0);
    {
        std::vector<double> Yt((size_t)K * Np, 0.0);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < N; i++)
            for (int mm = 0; mm <= L; mm++)
                for (int l = mm; l <= L; l++) {
                    const double p = P[(size_t)p_row(L, l, mm) * Np + i];
                    Yt[(size_t)sh_col(l, mm, 0) * Np + i] = p * trig[(size_t)(2 * mm) * Np + i];
                    if (mm > 0) Yt[(size_t)sh_col(l, mm, 1) * Np + i] = p * trig[(size_t)(2 * mm + 1) * Np + i];
                }
        double *dY = nullptr, *dG = nullptr;
        if (cudaMalloc(&dY, sizeof(double) * Yt.size()) != cudaSuccess) return ODIS_ERR_NOMEM;
        if (cudaMalloc(&dG, sizeof(double) * G.size()) != cudaSuccess) { cudaFree(dY); return ODIS_ERR_NOMEM; }
        cudaMemcpy(dY, Yt.data(), sizeof(double) * Yt.size(), cudaMemcpyHostToDevice);
        const int nt = (K + 31) / 32;
        k_gram<<<dim3(nt, nt), 256>>>(dY, K, N, Np, dG);
        const cudaError_t e = cudaMemcpy(G.data(), dG, sizeof(double) * G.size(), cudaMemcpyDeviceToHost);
        cudaFree(dY);
        cudaFree(dG);
        if (e != cudaSuccess) return ODIS_ERR_CUDA;
    }
    if (chol_inverse(G, K) != ODIS_OK) return ODIS_ERR_ARG;
    for (int l = 0; l <= L; l++)
        for (int a = l * l; a < (l + 1) * (l + 1); a++) {
            const double f = l >= 2 ? factors[l] : 0.0;
            for (int b = 0; b < K; b++) G[(size_t)a * K + b] *= f;
        }
    ShLoading* s = new ShLoading;
    s->L = L; s->K = K; s->MP = MP; s->N = N; s->Np = Np; s->precision = precision; s->status = status;
    bool ok = true;
    // Antipodal half basis (ODIS_SH_HALF=0 keeps the full one; the FP32 method's
    // tensor-core transforms, when forced with ODIS_SH_TC=1, need the full one)
    std::vector<int> partner;
    {
        const char* eh = std::getenv("ODIS_SH_HALF");
        const char* et = std::getenv("ODIS_SH_TC");
        const bool want = !(eh && eh[0] == '0') && !(precision == ODIS_FP32 && et && et[0] == '1');
        s->half = want && (N % 2 == 0) && antipodal_pairs(m, 1e-9, partner);
    }
    if (s->half) {
        s->Nh = N / 2;
        s->Nhp = (s->Nh + 127) / 128 * 128;
        std::vector<int> ha(s->Nhp), hb(s->Nhp);
        int h = 0;
        for (int i = 0; i < N; i++)
            if (i < partner[i]) { ha[h] = i; hb[h] = partner[i]; h++; }
        for (int k = h; k < s->Nhp; k++) { ha[k] = ha[h - 1]; hb[k] = hb[h - 1]; }
        std::vector<double> Ph((size_t)MP * s->Nhp, 0.0), th((size_t)2 * (L + 1) * s->Nhp, 0.0);
        for (int r = 0; r < MP; r++)
            for (int k = 0; k < s->Nh; k++) Ph[(size_t)r * s->Nhp + k] = P[(size_t)r * Np + ha[k]];
        for (int r = 0; r < 2 * (L + 1); r++)
            for (int k = 0; k < s->Nh; k++) th[(size_t)r * s->Nhp + k] = trig[(size_t)r * Np + ha[k]];
        P.swap(Ph);
        trig.swap(th);
        ok = cudaMalloc(&s->ia, sizeof(int) * s->Nhp) == cudaSuccess &&
             cudaMemcpy(s->ia, ha.data(), sizeof(int) * s->Nhp, cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMalloc(&s->ib, sizeof(int) * s->Nhp) == cudaSuccess &&
             cudaMemcpy(s->ib, hb.data(), sizeof(int) * s->Nhp, cudaMemcpyHostToDevice) == cudaSuccess;
    }
    {   // e/o (half basis) or the pre analysis's trig-weighted values: (4 | 2) (L+1) rows of the basis stride
        const size_t eo_bytes = (size_t)(s->half ? 4 : 2) * (L + 1) * (s->half ? s->Nhp : Np) * 8;
        ok = ok && cudaMalloc(&s->eo, eo_bytes) == cudaSuccess && cudaMemset(s->eo, 0, eo_bytes) == cudaSuccess;
    }
    if (precision == ODIS_FP64) ok = ok && upload_rows<double>(&s->P, P) && upload_rows<double>(&s->trig, trig);
    else if (precision == ODIS_DF64) ok = ok && upload_rows<df64>(&s->P, P) && upload_rows<df64>(&s->trig, trig);
    else ok = ok && upload_rows<float>(&s->P, P) && upload_rows<float>(&s->trig, trig);
    const size_t esz = precision == ODIS_FP32 ? sizeof(float) : sizeof(double);
    ok = ok && cudaMalloc(&s->usg, esz * Np) == cudaSuccess && cudaMemset(s->usg, 0, esz * Np) == cudaSuccess;
    ok = ok && cudaMalloc(&s->part, 8 * (size_t)K * kMaxChunks) == cudaSuccess &&
         cudaMemset(s->part, 0, 8 * (size_t)K * kMaxChunks) == cudaSuccess;
    ok = ok && cudaMalloc(&s->FGinv, sizeof(double) * G.size()) == cudaSuccess &&
         cudaMemcpy(s->FGinv, G.data(), sizeof(double) * G.size(), cudaMemcpyHostToDevice) == cudaSuccess;
    ok = ok && cudaMalloc(&s->t, sizeof(double) * K) == cudaSuccess && cudaMalloc(&s->coef, 8 * (size_t)K) == cudaSuccess &&
         cudaMemset(s->t, 0, sizeof(double) * K) == cudaSuccess;
    // arrival counters: one per analysis tile, at most (L+1)^2 tiles (one degree per tile)
    ok = ok && cudaMalloc(&s->arrivals, sizeof(unsigned) * (size_t)K) == cudaSuccess &&
         cudaMemset(s->arrivals, 0, sizeof(unsigned) * (size_t)K) == cudaSuccess;
    if (!ok) { sh_destroy(s); return ODIS_ERR_NOMEM; }
    // dense synthesis matrix, from the FP64 rows and F G^-1.  It pays only while it stays in L2 with the
    // rest of the step (measured: FP32 at level 6, 24 MB; FP64 and DF64 at level 6, 48 MB, and every
    // method at level 8 ran slower with it), so it is built up to 32 MB, or when ODIS_SH_TILES names the
    // dense synthesis or ODIS_SH_DENSE=1 asks for it (ODIS_SH_DENSE=0: never).
    {
        const char* ed = std::getenv("ODIS_SH_DENSE");
        const char* et = std::getenv("ODIS_SH_TILES");
        int f[5] = {0, 0, 0, 2, 0};
        const bool named = et && forced_tiles(f) && f[2] < 0;
        const int np = s->bp();
        const size_t zb = (precision == ODIS_FP32 ? sizeof(float) : sizeof(double)) * (size_t)K * np;
        const bool want = !(ed && ed[0] == '0') && (named || (ed && ed[0] == '1') || zb <= ((size_t)32 << 20));
        if (want) {
            double *dP = nullptr, *dT = nullptr;
            bool zok = cudaMalloc(&dP, sizeof(double) * P.size()) == cudaSuccess &&
                       cudaMalloc(&dT, sizeof(double) * trig.size()) == cudaSuccess &&
                       cudaMalloc(&s->Z, zb) == cudaSuccess &&
                       cudaMemcpy(dP, P.data(), sizeof(double) * P.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
                       cudaMemcpy(dT, trig.data(), sizeof(double) * trig.size(), cudaMemcpyHostToDevice) == cudaSuccess;
            if (zok) {
                const dim3 zg(np / 64, (K + 63) / 64);
                if (precision == ODIS_FP64) k_sh_zmat<double><<<zg, 256>>>(dP, dT, s->FGinv, L, K, np, (double*)s->Z);
                else if (precision == ODIS_DF64) k_sh_zmat<df64><<<zg, 256>>>(dP, dT, s->FGinv, L, K, np, (df64*)s->Z);
                else k_sh_zmat<float><<<zg, 256>>>(dP, dT, s->FGinv, L, K, np, (float*)s->Z);
                zok = cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess;
            }
            cudaFree(dP);
            cudaFree(dT);
            if (!zok) {
                (void)cudaGetLastError();
                cudaFree(s->Z);
                s->Z = nullptr;                          // the factored synthesis still works
            }
        }
    }
    if (precision == ODIS_FP32 && !s->half) {
        double pmax = 0.0;
        for (double x : P) pmax = std::fmax(pmax, std::fabs(x));
        const int tst = shtc_create(&s->tc, (const float*)s->P, (const float*)s->trig, pmax, L, N, Np, status);
        if (tst != ODIS_OK && tst != ODIS_ERR_ARG) { sh_destroy(s); return tst; }
    }
    const int st = sh_autotune(s);
    if (st != ODIS_OK) { sh_destroy(s); return st; }
    *out = s;
    return ODIS_OK;
}

void sh_destroy(ShLoading* s)
{
    if (!s) return;
    cudaFree(s->P); cudaFree(s->trig); cudaFree(s->tiles); cudaFree(s->part); cudaFree(s->FGinv);
    cudaFree(s->t); cudaFree(s->coef); cudaFree(s->usg);
    cudaFree(s->ia); cudaFree(s->ib); cudaFree(s->eo); cudaFree(s->arrivals); cudaFree(s->Z);
    shtc_destroy(s->tc);
    delete s;
}

const double* sh_usg64(ShLoading* s) { return s && s->precision == ODIS_FP64 ? (const double*)s->usg : nullptr; }
const float* sh_usg32(ShLoading* s) { return s && s->precision == ODIS_FP32 ? (const float*)s->usg : nullptr; }
const float2* sh_usgdf(ShLoading* s) { return s && s->precision == ODIS_DF64 ? (const float2*)s->usg : nullptr; }

// analysis tiles (m, l0, nl) with nl <= tl: degrees l0 .. l0 + nl - 1, or with the
// half basis l0, l0 + 2, ..., l0 + 2 (nl - 1) (one parity per tile)
static std::vector<int> make_tiles(int L, int tl, bool half)
{
    std::vector<int> tiles;
    for (int mm = 0; mm <= L; mm++) {
        if (!half) {
            for (int l0 = mm; l0 <= L; l0 += tl) {
                tiles.push_back(mm);
                tiles.push_back(l0);
                tiles.push_back(std::min(tl, L - l0 + 1));
            }
            continue;
        }
        for (int start = mm; start <= std::min(L, mm + 1); start++)
            for (int l0 = start; l0 <= L; l0 += 2 * tl) {
                tiles.push_back(mm);
                tiles.push_back(l0);
                tiles.push_back(std::min(tl, (L - l0) / 2 + 1));
            }
    }
    return tiles;
}

template <class T>
static void launch_analysis(const ShLoading* s, int tl, const int* tiles, int ntiles, int nchunk, bool pre,
                            const void* eta, cudaStream_t st)
{
    const dim3 grid(ntiles, nchunk);
    const T* P = (const T*)s->P;
    const T* trig = (const T*)s->trig;
    T* part = (T*)s->part;
    unsigned* arr = s->arrivals;
    double* tt = s->t;
    const int n = s->bn(), np = s->bp();
    const T* e = (const T*)eta;
    if (pre) {            // trig-weighted values of every order, then multiply-adds only
        T* x = (T*)s->eo;
        const dim3 pg((np + 255) / 256, s->L + 1);
        if (s->half) pdl_launch(k_sh_prep<T, true>, pg, 256, 0, st, e, (const int*)s->ia, (const int*)s->ib, trig, n, np, s->L, x);
        else pdl_launch(k_sh_prep<T, false>, pg, 256, 0, st, e, (const int*)s->ia, (const int*)s->ib, trig, n, np, s->L, x);
        e = x;
    } else if (s->half) {
        T* eo = (T*)s->eo;
        pdl_launch(k_sh_pair<T>, (np + 255) / 256, 256, 0, st, e, (const int*)s->ia, (const int*)s->ib, n, np, eo);
        e = eo;
    }
#define ODIS_ANA(TL, H, PRE) pdl_launch(k_sh_analysis<T, TL, H, PRE>, grid, kShThreads, 0, st, P, trig, e, n, np, s->L, tiles, nchunk, part, arr, tt)
#define ODIS_ANA_TL(H, PRE) do { if (tl == 2) ODIS_ANA(2, H, PRE); else if (tl == 4) ODIS_ANA(4, H, PRE); else ODIS_ANA(8, H, PRE); } while (0)
    if (s->half) { if (pre) ODIS_ANA_TL(true, true); else ODIS_ANA_TL(true, false); }
    else { if (pre) ODIS_ANA_TL(false, true); else ODIS_ANA_TL(false, false); }
#undef ODIS_ANA_TL
#undef ODIS_ANA
}

template <class T>
static void launch_synth(const ShLoading* s, int lanes, int cells, cudaStream_t st)
{
    const int n = s->bn(), np = s->bp();
    const int sb = ((n + cells - 1) / cells * lanes + kSynthThreads - 1) / kSynthThreads;
    const size_t sm = sizeof(T) * s->K;
    const T* P = (const T*)s->P;
    const T* trig = (const T*)s->trig;
    const T* c = (const T*)s->coef;
    const int* ia = s->ia;
    const int* ib = s->ib;
    T* u = (T*)s->usg;
#define ODIS_SYNTH(LN, CL, H) pdl_launch(k_sh_synth<T, LN, CL, H>, sb, kSynthThreads, sm, st, P, trig, c, n, np, s->L, s->K, ia, ib, u)
#define ODIS_SYNTH_LANES(CL, H) \
    do { if (lanes == 1) ODIS_SYNTH(1, CL, H); else if (lanes == 2) ODIS_SYNTH(2, CL, H); \
         else if (lanes == 4) ODIS_SYNTH(4, CL, H); else ODIS_SYNTH(8, CL, H); } while (0)
    if (lanes % kSynthPairs == 0) {      // one warp per pair of orders; lanes / 16 groups of 32 * cells cells
        const int groups = lanes / kSynthPairs;
        const int nw = std::min(s->L / 2 + 1, kSynthMaxWarps);
        const int nb = (n + 32 * cells * groups - 1) / (32 * cells * groups);
        const size_t smp = sizeof(T) * ((size_t)((s->K + 1) & ~1) + (size_t)groups * nw * 32 * 4);
#define ODIS_SYNTH_M(CL, H, G) pdl_launch(k_sh_synth_m<T, CL, H, G>, nb, G * nw * 32, smp, st, P, trig, c, n, np, s->L, s->K, ia, ib, u)
#define ODIS_SYNTH_MG(CL, H) do { if (groups == 1) ODIS_SYNTH_M(CL, H, 1); else if (groups == 2) ODIS_SYNTH_M(CL, H, 2); \
                                 else ODIS_SYNTH_M(CL, H, 3); } while (0)
        if (s->half) { if (cells == 2) ODIS_SYNTH_MG(2, true); else ODIS_SYNTH_MG(1, true); }
        else { if (cells == 2) ODIS_SYNTH_MG(2, false); else ODIS_SYNTH_MG(1, false); }
#undef ODIS_SYNTH_MG
#undef ODIS_SYNTH_M
    } else if (s->half) {
        if (cells == 2) ODIS_SYNTH_LANES(2, true); else ODIS_SYNTH_LANES(1, true);
    } else {
        if (cells == 2) ODIS_SYNTH_LANES(2, false); else ODIS_SYNTH_LANES(1, false);
    }
#undef ODIS_SYNTH_LANES
#undef ODIS_SYNTH
}

// Cell-chunk counts the timing tries for an analysis of nt tiles: the powers of
// two, and the counts whose tiles x chunks CTAs fill one, two or three whole
// waves of this kernel's resident CTAs.  The transforms are bound by arithmetic
// issue, so an SM that runs one CTA more than the others sets the time: 85
// tiles x 8 chunks = 680 CTAs on 608 slots leaves some SMs 5 CTAs' work
// against 4.47 on average, 85 x 7 = 595 fits one wave.
template <class T>
static std::vector<int> analysis_chunks(const ShLoading* s, int tl, bool pre, int nt)
{
    std::vector<int> c = {2, 4, 8, 16, 32, 64};
    int dev = 0, sms = 0, nb = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const bool h = s->half;
#define ODIS_AFN(TL) (pre ? (h ? (const void*)k_sh_analysis<T, TL, true, true> : (const void*)k_sh_analysis<T, TL, false, true>) \
                          : (h ? (const void*)k_sh_analysis<T, TL, true, false> : (const void*)k_sh_analysis<T, TL, false, false>))
    const void* f = tl == 2 ? ODIS_AFN(2) : tl == 4 ? ODIS_AFN(4) : ODIS_AFN(8);
#undef ODIS_AFN
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, f, kShThreads, 0) != cudaSuccess || nb <= 0 || sms <= 0 || nt <= 0) {
        (void)cudaGetLastError();
        return c;
    }
    for (int w = 1; w <= 3; w++) {
        const int ch = w * nb * sms / nt;
        if (ch >= 2 && ch <= kMaxChunks && std::find(c.begin(), c.end(), ch) == c.end()) c.push_back(ch);
    }
    return c;
}

// dense synthesis usg = Z t with zw warps per block and zc cells per lane
template <class T>
static cudaError_t launch_synth_z(const ShLoading* s, int zw, int zc, cudaStream_t st)
{
    const int n = s->bn(), np = s->bp(), K = s->K;
    const int nb = (n + 32 * zc - 1) / (32 * zc);
    const size_t sm = sizeof(T) * ((size_t)((K + 1) & ~1) + 2 * (size_t)zw * 32 * zc) + (size_t)K;
    const T* Z = (const T*)s->Z;
    T* u = (T*)s->usg;
#define ODIS_SZ(H, W, C) return pdl_launch(k_sh_synth_z<T, H, W, C>, nb, 32 * W, sm, st, Z, (const double*)s->t, n, np, K, \
                                           (const int*)s->ia, (const int*)s->ib, u)
#define ODIS_SZ_W(H, C) do { if (zw == 4) ODIS_SZ(H, 4, C); if (zw == 8) ODIS_SZ(H, 8, C); ODIS_SZ(H, 16, C); } while (0)
    if (s->half) { if (zc == 2) ODIS_SZ_W(true, 2); ODIS_SZ_W(true, 1); }
    else { if (zc == 2) ODIS_SZ_W(false, 2); ODIS_SZ_W(false, 1); }
#undef ODIS_SZ_W
#undef ODIS_SZ
}

// Self-tuning of the transform tiles: every candidate is timed on this mesh
// and this device (CUDA events, warm L2, median of three runs of 10 launches)
// and the fastest is kept.  Results do not depend on the choice of the
// synthesis lanes; the analysis's chunking changes only the order of the
// partial sums.
// ODIS_SH_TILES="tile_l,chunks,lanes[,cells[,pre]]" (tile_l in {2,4,8}, chunks in
// 2..64, lanes in {1,2,4,8} threads per cell splitting the orders, or
// 16, 32, 48 for one warp per pair of orders (k_sh_synth_m) and 1, 2, 3 cell
// groups per block, or -4, -8, -16 for the dense synthesis with that many warps
// per block, synthesis cells per thread in
// {1,2}, default 2, pre = 1 for the analysis from trig-weighted values formed
// once per step, default 0) fixes the tiles instead of timing them, e.g. to
// reproduce a run bit for bit or to profile a given variant.  Anything else is
// ignored, and so are synthesis lanes whose blocks would exceed 1024 threads at
// this degree (two or three cell groups of 17 order-pair warps at l_max 32).
static bool forced_tiles(int* f)
{
    const char* e = std::getenv("ODIS_SH_TILES");
    if (!e) return false;
    int a = 0, b = 0, c = 0, d = 2, pre = 0;
    const int n = std::sscanf(e, "%d,%d,%d,%d,%d", &a, &b, &c, &d, &pre);
    if (n < 3 || n > 5 || (pre != 0 && pre != 1)) return false;
    const bool ok = (a == 2 || a == 4 || a == 8) && b >= 2 && b <= kMaxChunks &&
                    (c == 1 || c == 2 || c == 4 || c == 8 || c == kSynthPairs || c == 2 * kSynthPairs ||
                     c == 3 * kSynthPairs || c == -4 || c == -8 || c == -16) && (d == 1 || d == 2);
    if (ok) { f[0] = a; f[1] = b; f[2] = c; f[3] = d; f[4] = pre; }
    return ok;
}

template <class T>
static void enqueue_t(ShLoading* s, const void* eta, cudaStream_t st);

template <class T>
static int autotune_t(ShLoading* s)
{
    void* eta = nullptr;
    if (cudaMalloc(&eta, sizeof(T) * s->Np) != cudaSuccess) return ODIS_ERR_NOMEM;
    cudaMemset(eta, 0, sizeof(T) * s->Np);
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    // a candidate whose launch the driver refuses is never chosen
    auto timeit = [&](auto&& body) {
        float best = 1e30f;
        (void)cudaGetLastError();
        body();
        if (cudaGetLastError() != cudaSuccess) return best;
        for (int r = 0; r < 3; r++) {
            cudaEventRecord(a);
            for (int q = 0; q < 10; q++) body();
            cudaEventRecord(b);
            cudaEventSynchronize(b);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, a, b);
            best = std::min(best, ms);
        }
        return best;
    };
    float best = 1e30f;
    int best_tl = 8, best_ch = 16;
    std::vector<int> best_tiles;
    int forced[5] = {0, 0, 0, 2, 0};
    const bool force = forced_tiles(forced);
    int* dt = nullptr;
    cudaMalloc(&dt, sizeof(int) * 3 * (size_t)(s->L + 1) * (s->L + 1));
    bool best_pre = false;
    for (int tl : {2, 4, 8}) {
        if (force && tl != forced[0]) continue;
        const std::vector<int> tiles = make_tiles(s->L, tl, s->half);
        cudaMemcpy(dt, tiles.data(), sizeof(int) * tiles.size(), cudaMemcpyHostToDevice);
        const int nt = (int)tiles.size() / 3;
        for (bool pre : {false, true})
            for (int ch : force ? std::vector<int>{forced[1]} : analysis_chunks<T>(s, tl, pre, nt)) {
                if (force && (ch != forced[1] || (int)pre != forced[4])) continue;
                const float ms = force ? 0.f : timeit([&] { launch_analysis<T>(s, tl, dt, nt, ch, pre, eta, 0); });
                if (ms < best) { best = ms; best_tl = tl; best_ch = ch; best_tiles = tiles; best_pre = pre; }
            }
    }
    if (best_tiles.empty()) {                          // nothing ran (a refused launch in every candidate)
        best_tl = 8;
        best_ch = 16;
        best_pre = false;
        best_tiles = make_tiles(s->L, best_tl, s->half);
    }
    s->pre = best_pre;
    cudaFree(dt);
    s->tl = best_tl;
    s->nchunk = best_ch;
    s->ntiles = (int)best_tiles.size() / 3;
    int st = ODIS_OK;
    if (cudaMalloc(&s->tiles, sizeof(int) * best_tiles.size()) != cudaSuccess ||
        cudaMemcpy(s->tiles, best_tiles.data(), sizeof(int) * best_tiles.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        st = ODIS_ERR_NOMEM;
    best = 1e30f;
    // order-pair blocks hold groups x (warps per group) x 32 threads, at most 1024
    auto synth_fits = [&](int lanes) {
        return lanes % kSynthPairs != 0 ||
               (lanes / kSynthPairs) * std::min(s->L / 2 + 1, kSynthMaxWarps) * 32 <= kSynthMaxThreads;
    };
    const bool force_dense = force && forced[2] < 0 && s->Z;
    const bool force_synth = force && !force_dense && forced[2] > 0 && synth_fits(forced[2]);
    for (int cells : {2, 1})
        for (int lanes : {1, 2, 4, 8, kSynthPairs, 2 * kSynthPairs, 3 * kSynthPairs}) {
            if (!synth_fits(lanes) || force_dense) continue;
            if (force_synth && (lanes != forced[2] || cells != forced[3])) continue;
            const float ms = force_synth ? 0.f : timeit([&] { launch_synth<T>(s, lanes, cells, 0); });
            if (ms < best) { best = ms; s->lanes = lanes; s->cells = cells; }
        }
    // the dense synthesis against the K x K product plus the chosen factored synthesis, in isolation.
    // Z's bytes compete for L2 with the rest of the step, so a dense variant within 5 % is only a
    // candidate: odis_create times whole steps both ways (sh_dense_candidate / sh_set_dense).
    s->zw = 0;
    s->zw_cand = 0;
    s->zforced = force_synth || force_dense;
    if (s->Z && !force_synth) {
        const float fact = force_dense ? 1e30f : timeit([&] {
            pdl_launch(k_sh_coef<T>, s->K, 32, 0, (cudaStream_t)0, s->t, s->K, s->FGinv, (T*)s->coef);
            launch_synth<T>(s, s->lanes, s->cells, 0);
        });
        float bz = 1e30f;
        for (int zc : {1, 2})
            for (int zw : {4, 8, 16}) {
                if (force_dense && (zw != -forced[2] || zc != forced[3])) continue;
                const float ms = force_dense ? 0.f : timeit([&] { launch_synth_z<T>(s, zw, zc, 0); });
                if (ms < bz) { bz = ms; s->zw_cand = zw; s->zc_cand = zc; }
            }
        if (force_dense) { s->zw = s->zw_cand; s->zc = s->zc_cand; }
        else if (!(bz <= 1.05f * fact)) s->zw_cand = 0;
    }
    if (s->zw == 0 && s->zw_cand == 0 && s->Z) {       // the factored synthesis stays: Z is not kept
        cudaDeviceSynchronize();
        cudaFree(s->Z);
        s->Z = nullptr;
    }
    if constexpr (std::is_same<T, float>::value) {
        // tensor-core transforms against the CUDA-core ones, whole per-step sequence;
        // ODIS_SH_TC=1 or 0 fixes the choice
        if (s->tc && st == ODIS_OK) {
            const char* e = std::getenv("ODIS_SH_TC");
            const int want = (e && e[0] == '1') ? 1 : (e && e[0] == '0') ? 0 : -1;
            s->use_tc = false;
            const float cc = want < 0 ? timeit([&] { enqueue_t<float>(s, eta, 0); }) : 0.f;
            float best_tc = 1e30f;
            int best_tp = 2;
            for (int tp : {1, 2}) {
                if (!shtc_tiles_per_pass_ok(s->tc, tp)) continue;
                shtc_set_tiles_per_pass(s->tc, tp);
                s->use_tc = true;
                const float ms = timeit([&] { enqueue_t<float>(s, eta, 0); });
                if (ms < best_tc) { best_tc = ms; best_tp = tp; }
            }
            shtc_set_tiles_per_pass(s->tc, best_tp);
            s->use_tc = want == 1 || (want < 0 && best_tc < cc);
            int h = 0;
            if (cudaMemcpy(&h, s->status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) st = ODIS_ERR_CUDA;
            else if (h & (1 << ODIS_ERR_TIMEOUT)) st = ODIS_ERR_TIMEOUT;
            if (!s->use_tc) {          // the operand copies (4 B per Legendre value each) are not kept
                cudaDeviceSynchronize();
                shtc_destroy(s->tc);
                s->tc = nullptr;
            }
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(eta);
    cudaMemset(s->usg, 0, (s->precision == ODIS_FP32 ? sizeof(float) : sizeof(double)) * s->Np);
    if (cudaDeviceSynchronize() != cudaSuccess) st = ODIS_ERR_CUDA;
    return st;
}

int sh_autotune(ShLoading* s)
{
    if (s->precision == ODIS_FP64) return autotune_t<double>(s);
    if (s->precision == ODIS_DF64) return autotune_t<df64>(s);
    return autotune_t<float>(s);
}

bool sh_dense_candidate(const ShLoading* s) { return s && !s->use_tc && !s->zforced && s->Z && s->zw_cand > 0; }

void sh_set_dense(ShLoading* s, bool on)
{
    if (!sh_dense_candidate(s)) return;
    s->zw = on ? s->zw_cand : 0;
    s->zc = on ? s->zc_cand : 1;
    if (!on) {                                         // the factored synthesis is kept: free Z
        cudaDeviceSynchronize();
        cudaFree(s->Z);
        s->Z = nullptr;
        s->zw_cand = 0;
    }
}

void sh_try_dense(ShLoading* s, bool on)
{
    if (!sh_dense_candidate(s)) return;
    s->zw = on ? s->zw_cand : 0;
    s->zc = on ? s->zc_cand : 1;
}

void sh_tuning(const ShLoading* s, int* tl, int* nchunk, int* lanes, int* cells, int* pre)
{
    if (tl) *tl = s->use_tc ? 0 : s->tl;
    if (nchunk) *nchunk = s->use_tc ? shtc_chunks(s->tc) : s->nchunk;
    if (lanes) *lanes = s->use_tc ? shtc_tiles_per_pass(s->tc) : (s->zw ? -s->zw : s->lanes);
    if (cells) *cells = s->use_tc ? 0 : (s->zw ? s->zc : s->cells);
    if (pre) *pre = s->use_tc ? 0 : (s->pre ? 1 : 0);
}

template <class T>
static void enqueue_t(ShLoading* s, const void* eta, cudaStream_t st)
{
    if constexpr (std::is_same<T, float>::value) {
        if (s->use_tc) {
            shtc_analysis(s->tc, (const float*)eta, st);
            k_sh_fold<float><<<(s->K + 3) / 4, 128, 0, st>>>(shtc_partials(s->tc), s->K, shtc_chunks(s->tc), s->t);
            k_sh_coef<float><<<s->K, 32, 0, st>>>(s->t, s->K, s->FGinv, (float*)s->coef);
            shtc_pack(s->tc, (const float*)s->coef, st);
            shtc_synth(s->tc, (float*)s->usg, st);
            return;
        }
    }
    launch_analysis<T>(s, s->tl, s->tiles, s->ntiles, s->nchunk, s->pre, eta, st);   // partials and their fold
    if (s->zw) {
        launch_synth_z<T>(s, s->zw, s->zc, st);
        return;
    }
    pdl_launch(k_sh_coef<T>, s->K, 32, 0, st, s->t, s->K, s->FGinv, (T*)s->coef);
    launch_synth<T>(s, s->lanes, s->cells, st);
}

void sh_enqueue(ShLoading* s, const void* eta, cudaStream_t st)
{
    if (s->precision == ODIS_FP64) enqueue_t<double>(s, eta, st);
    else if (s->precision == ODIS_DF64) enqueue_t<df64>(s, eta, st);
    else enqueue_t<float>(s, eta, st);
}

int sh_kernels_per_step(const ShLoading* s)
{
    if (!s) return 0;
    if (s->use_tc) return shtc_kernels_per_step();
    return ((s->half || s->pre) ? 4 : 3) - (s->zw ? 1 : 0);
}

void sh_layout(const ShLoading* s, int* half, int* cells, long long* basis_bytes)
{
    const size_t esz = s->precision == ODIS_FP32 ? 4 : 8;
    if (half) *half = s->half ? 1 : 0;
    if (cells) *cells = s->bn();
    if (basis_bytes) *basis_bytes = (long long)((size_t)(s->MP + 2 * (s->L + 1)) * s->bn() * esz);
}

}  // namespace odis
