// Spherical-harmonic self-gravity / loading kernels (see odis_sh.cuh).
//
// Layout: Y is stored [K][Np] (one harmonic per row, cells contiguous), so the
// analysis (t_k = sum_i Y_ki eta_i) streams each row with coalesced loads and
// the synthesis (usg_i = sum_k Y_ki c_k) reads one coalesced column slice per
// k.  The normalised Legendre functions are evaluated in FP64 on the host
// (three-term recurrences of the fully normalised functions, Holmes &
// Featherstone 2002) and the Gram matrix Y^T Y is inverted in FP64 (Cholesky);
// the FP32-state variant stores Y in FP32 and accumulates in FP64.
#include "odis_sh.cuh"
#include "odis_df64.cuh"

#include <cmath>
#include <cstring>
#include <vector>

namespace odis {

namespace {

constexpr double kPi = 3.1415926535897932384626433832795028841971693993751058;
constexpr int kShThreads = 256;
constexpr int kSynthThreads = 128;

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

// column of harmonic (l, m, cos|sin): l^2 for m=0, l^2 + 2m-1 (cos), l^2 + 2m (sin)
inline int sh_col(int l, int m, int is_sin) { return l * l + (m == 0 ? 0 : 2 * m - 1 + is_sin); }

__device__ __forceinline__ double warp_sum_d(double x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    return x;
}

// Accumulator type of the transforms: FP64 for the FP64 method, FP32 inside a
// thread for the FP32-state variant (block and global sums are FP64 in both).
template <class T> struct Acc { using type = double; };
template <> struct Acc<float> { using type = float; };

// t[k] = sum_i Y[k][i] eta[i]: one block per harmonic, four independent
// accumulators per thread, FP64 block sum in a fixed order.
template <class T>
__global__ void __launch_bounds__(kShThreads) k_sh_analysis(const T* __restrict__ Y, const T* __restrict__ eta, int N,
                                                            int Np, double* __restrict__ t)
{
    using A = typename Acc<T>::type;
    __shared__ double red[kShThreads / 32];
    const int k = blockIdx.x;
    const T* row = Y + (size_t)k * Np;
    A a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    int i = threadIdx.x;
    for (; i + 3 * kShThreads < N; i += 4 * kShThreads) {
        a0 = fma((A)row[i], (A)eta[i], a0);
        a1 = fma((A)row[i + kShThreads], (A)eta[i + kShThreads], a1);
        a2 = fma((A)row[i + 2 * kShThreads], (A)eta[i + 2 * kShThreads], a2);
        a3 = fma((A)row[i + 3 * kShThreads], (A)eta[i + 3 * kShThreads], a3);
    }
    for (; i < N; i += kShThreads) a0 = fma((A)row[i], (A)eta[i], a0);
    double acc = (double)((a0 + a1) + (a2 + a3));
    acc = warp_sum_d(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double s = threadIdx.x < kShThreads / 32 ? red[threadIdx.x] : 0.0;
        s = warp_sum_d(s);
        if (threadIdx.x == 0) t[k] = s;
    }
}

// c = (F G^-1) t: one warp per coefficient
__global__ void __launch_bounds__(32) k_sh_coef(const double* __restrict__ t, int K, const double* __restrict__ FGinv,
                                                double* __restrict__ coef)
{
    const int a = blockIdx.x;
    const double* row = FGinv + (size_t)a * K;
    double s = 0.0;
    for (int b = threadIdx.x; b < K; b += 32) s = fma(row[b], t[b], s);
    s = warp_sum_d(s);
    if (threadIdx.x == 0) coef[a] = s;
}

// usg[i] = sum_{k >= 4} Y[k][i] c[k]  (c is zero below degree 2)
template <class T>
__global__ void __launch_bounds__(kSynthThreads) k_sh_synth(const T* __restrict__ Y, const double* __restrict__ coef,
                                                            int N, int Np, int K, T* __restrict__ usg)
{
    using A = typename Acc<T>::type;
    extern __shared__ double c_sh[];
    A* c = reinterpret_cast<A*>(c_sh);
    for (int k = threadIdx.x; k < K; k += kSynthThreads) c[k] = (A)coef[k];
    __syncthreads();
    const int i = blockIdx.x * kSynthThreads + threadIdx.x;
    if (i >= N) return;
    A a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    int k = 4;
    for (; k + 3 < K; k += 4) {
        a0 = fma((A)Y[(size_t)k * Np + i], c[k], a0);
        a1 = fma((A)Y[(size_t)(k + 1) * Np + i], c[k + 1], a1);
        a2 = fma((A)Y[(size_t)(k + 2) * Np + i], c[k + 2], a2);
        a3 = fma((A)Y[(size_t)(k + 3) * Np + i], c[k + 3], a3);
    }
    for (; k < K; k++) a0 = fma((A)Y[(size_t)k * Np + i], c[k], a0);
    usg[i] = (T)((a0 + a1) + (a2 + a3));
}

// double-float forms of the two transforms (ODIS_DF64 method)
__global__ void __launch_bounds__(kShThreads) k_sh_analysis_df(const df64* __restrict__ Y, const df64* __restrict__ eta,
                                                               int N, int Np, double* __restrict__ t)
{
    __shared__ df64 red[kShThreads / 32];
    const int k = blockIdx.x;
    const df64* row = Y + (size_t)k * Np;
    df64 a0 = df_make(0.f, 0.f), a1 = a0, a2 = a0, a3 = a0;
    int i = threadIdx.x;
    for (; i + 3 * kShThreads < N; i += 4 * kShThreads) {
        a0 = df_fma(row[i], eta[i], a0);
        a1 = df_fma(row[i + kShThreads], eta[i + kShThreads], a1);
        a2 = df_fma(row[i + 2 * kShThreads], eta[i + 2 * kShThreads], a2);
        a3 = df_fma(row[i + 3 * kShThreads], eta[i + 3 * kShThreads], a3);
    }
    for (; i < N; i += kShThreads) a0 = df_fma(row[i], eta[i], a0);
    df64 acc = df_add(df_add(a0, a1), df_add(a2, a3));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc = df_add(acc, df_shfl_down(acc, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        df64 s = threadIdx.x < kShThreads / 32 ? red[threadIdx.x] : df_make(0.f, 0.f);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s = df_add(s, df_shfl_down(s, o));
        if (threadIdx.x == 0) t[k] = df_to_double(s);
    }
}

__global__ void __launch_bounds__(kSynthThreads) k_sh_synth_df(const df64* __restrict__ Y, const double* __restrict__ coef,
                                                               int N, int Np, int K, df64* __restrict__ usg)
{
    extern __shared__ df64 cdf[];
    for (int k = threadIdx.x; k < K; k += kSynthThreads) cdf[k] = df_from_double(coef[k]);
    __syncthreads();
    const int i = blockIdx.x * kSynthThreads + threadIdx.x;
    if (i >= N) return;
    df64 a0 = df_make(0.f, 0.f), a1 = a0, a2 = a0, a3 = a0;
    int k = 4;
    for (; k + 3 < K; k += 4) {
        a0 = df_fma(Y[(size_t)k * Np + i], cdf[k], a0);
        a1 = df_fma(Y[(size_t)(k + 1) * Np + i], cdf[k + 1], a1);
        a2 = df_fma(Y[(size_t)(k + 2) * Np + i], cdf[k + 2], a2);
        a3 = df_fma(Y[(size_t)(k + 3) * Np + i], cdf[k + 3], a3);
    }
    for (; k < K; k++) a0 = df_fma(Y[(size_t)k * Np + i], cdf[k], a0);
    usg[i] = df_add(df_add(a0, a1), df_add(a2, a3));
}

}  // namespace

struct ShLoading {
    int L = 0, K = 0, N = 0, Np = 0, precision = ODIS_FP64;
    double* Y64 = nullptr;
    float* Y32 = nullptr;
    double* FGinv = nullptr;
    double* t = nullptr;
    double* coef = nullptr;
    double* usg64 = nullptr;
    float* usg32 = nullptr;
    df64* Ydf = nullptr;
    df64* usgdf = nullptr;
};

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

int sh_create(ShLoading** out, const Mesh& m, int L, const double* factors, int precision, int Np)
{
    *out = nullptr;
    const int K = (L + 1) * (L + 1);
    if (L < 2 || m.N < K) return ODIS_ERR_ARG;
    std::vector<double> Y;
    sh_basis_host(m, L, Y);
    // Gram matrix Y^T Y (FP64), inverted
    std::vector<double> G((size_t)K * K, 0.0);
#pragma omp parallel for schedule(dynamic)
    for (int a = 0; a < K; a++)
        for (int b = 0; b <= a; b++) {
            double s = 0.0;
            for (int i = 0; i < m.N; i++) s += Y[(size_t)i * K + a] * Y[(size_t)i * K + b];
            G[(size_t)a * K + b] = s;
            G[(size_t)b * K + a] = s;
        }
    if (chol_inverse(G, K) != ODIS_OK) return ODIS_ERR_ARG;
    // fold the per-degree factors (zero below degree 2)
    for (int l = 0; l <= L; l++)
        for (int a = l * l; a < (l + 1) * (l + 1); a++) {
            const double f = l >= 2 ? factors[l] : 0.0;
            for (int b = 0; b < K; b++) G[(size_t)a * K + b] *= f;
        }
    ShLoading* s = new ShLoading;
    s->L = L; s->K = K; s->N = m.N; s->Np = Np; s->precision = precision;
    std::vector<double> Yt((size_t)K * Np, 0.0);
    for (int i = 0; i < m.N; i++)
        for (int k = 0; k < K; k++) Yt[(size_t)k * Np + i] = Y[(size_t)i * K + k];
    bool ok = true;
    auto up = [&](void** d, const void* h, size_t bytes) {
        if (cudaMalloc(d, bytes) != cudaSuccess) { ok = false; *d = nullptr; return; }
        if (h) cudaMemcpy(*d, h, bytes, cudaMemcpyHostToDevice);
        else cudaMemset(*d, 0, bytes);
    };
    if (precision == ODIS_FP64) {
        up((void**)&s->Y64, Yt.data(), sizeof(double) * Yt.size());
        up((void**)&s->usg64, nullptr, sizeof(double) * Np);
    } else if (precision == ODIS_DF64) {
        std::vector<df64> Yd(Yt.size());
        for (size_t q = 0; q < Yt.size(); q++) Yd[q] = df_from_double(Yt[q]);
        up((void**)&s->Ydf, Yd.data(), sizeof(df64) * Yd.size());
        up((void**)&s->usgdf, nullptr, sizeof(df64) * Np);
    } else {
        std::vector<float> Yf(Yt.begin(), Yt.end());
        up((void**)&s->Y32, Yf.data(), sizeof(float) * Yf.size());
        up((void**)&s->usg32, nullptr, sizeof(float) * Np);
    }
    up((void**)&s->FGinv, G.data(), sizeof(double) * G.size());
    up((void**)&s->t, nullptr, sizeof(double) * K);
    up((void**)&s->coef, nullptr, sizeof(double) * K);
    if (!ok) { sh_destroy(s); return ODIS_ERR_NOMEM; }
    *out = s;
    return ODIS_OK;
}

void sh_destroy(ShLoading* s)
{
    if (!s) return;
    cudaFree(s->Y64); cudaFree(s->Y32); cudaFree(s->FGinv); cudaFree(s->t); cudaFree(s->coef);
    cudaFree(s->usg64); cudaFree(s->usg32); cudaFree(s->Ydf); cudaFree(s->usgdf);
    delete s;
}

const double* sh_usg64(ShLoading* s) { return s ? s->usg64 : nullptr; }
const float* sh_usg32(ShLoading* s) { return s ? s->usg32 : nullptr; }
const float2* sh_usgdf(ShLoading* s) { return s ? s->usgdf : nullptr; }

void sh_enqueue(ShLoading* s, const void* eta, cudaStream_t st)
{
    const int sb = (s->N + kSynthThreads - 1) / kSynthThreads;
    if (s->precision == ODIS_FP64) {
        k_sh_analysis<double><<<s->K, kShThreads, 0, st>>>(s->Y64, (const double*)eta, s->N, s->Np, s->t);
        k_sh_coef<<<s->K, 32, 0, st>>>(s->t, s->K, s->FGinv, s->coef);
        k_sh_synth<double><<<sb, kSynthThreads, sizeof(double) * s->K, st>>>(s->Y64, s->coef, s->N, s->Np, s->K, s->usg64);
    } else if (s->precision == ODIS_DF64) {
        k_sh_analysis_df<<<s->K, kShThreads, 0, st>>>(s->Ydf, (const df64*)eta, s->N, s->Np, s->t);
        k_sh_coef<<<s->K, 32, 0, st>>>(s->t, s->K, s->FGinv, s->coef);
        k_sh_synth_df<<<sb, kSynthThreads, sizeof(df64) * s->K, st>>>(s->Ydf, s->coef, s->N, s->Np, s->K, s->usgdf);
    } else {
        k_sh_analysis<float><<<s->K, kShThreads, 0, st>>>(s->Y32, (const float*)eta, s->N, s->Np, s->t);
        k_sh_coef<<<s->K, 32, 0, st>>>(s->t, s->K, s->FGinv, s->coef);
        k_sh_synth<float><<<sb, kSynthThreads, sizeof(float) * s->K, st>>>(s->Y32, s->coef, s->N, s->Np, s->K, s->usg32);
    }
}

}  // namespace odis
