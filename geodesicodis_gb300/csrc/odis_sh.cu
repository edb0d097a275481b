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

#include <cmath>
#include <cstring>
#include <vector>

namespace odis {

namespace {

constexpr double kPi = 3.1415926535897932384626433832795028841971693993751058;
constexpr int kChunk = 2048;          // cells per analysis block
constexpr int kShThreads = 256;

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

// t_partial[k][chunk] = sum over the chunk's cells of Y[k][i] eta[i]
template <class T>
__global__ void __launch_bounds__(kShThreads) k_sh_analysis(const T* __restrict__ Y, const T* __restrict__ eta, int N,
                                                            int Np, int nchunk, double* __restrict__ part)
{
    __shared__ double red[kShThreads / 32];
    const int k = blockIdx.y, ch = blockIdx.x;
    const T* row = Y + (size_t)k * Np;
    const int i0 = ch * kChunk, i1 = min(N, i0 + kChunk);
    double acc = 0.0;
    for (int i = i0 + threadIdx.x; i < i1; i += kShThreads) acc = fma((double)row[i], (double)eta[i], acc);
    acc = warp_sum_d(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double s = threadIdx.x < kShThreads / 32 ? red[threadIdx.x] : 0.0;
        s = warp_sum_d(s);
        if (threadIdx.x == 0) part[(size_t)k * nchunk + ch] = s;
    }
}

// c = F Ginv t, one block; t_k folded from the chunk partials in order
__global__ void __launch_bounds__(kShThreads) k_sh_solve(const double* __restrict__ part, int nchunk, int K,
                                                         const double* __restrict__ FGinv, double* __restrict__ coef)
{
    extern __shared__ double t[];
    for (int k = threadIdx.x; k < K; k += kShThreads) {
        double s = 0.0;
        for (int ch = 0; ch < nchunk; ch++) s += part[(size_t)k * nchunk + ch];
        t[k] = s;
    }
    __syncthreads();
    for (int a = threadIdx.x; a < K; a += kShThreads) {
        const double* row = FGinv + (size_t)a * K;
        double s = 0.0;
        for (int b = 0; b < K; b++) s = fma(row[b], t[b], s);
        coef[a] = s;
    }
}

// usg[i] = sum_k Y[k][i] c[k]   (harmonics l >= 2 only; c is zero below)
template <class T>
__global__ void __launch_bounds__(kShThreads) k_sh_synth(const T* __restrict__ Y, const double* __restrict__ coef,
                                                         int N, int Np, int K, T* __restrict__ usg)
{
    extern __shared__ double c[];
    for (int k = threadIdx.x; k < K; k += kShThreads) c[k] = coef[k];
    __syncthreads();
    const int i = blockIdx.x * kShThreads + threadIdx.x;
    if (i >= N) return;
    double s = 0.0;
    for (int k = 4; k < K; k++) s = fma((double)Y[(size_t)k * Np + i], c[k], s);
    usg[i] = (T)s;
}

}  // namespace

struct ShLoading {
    int L = 0, K = 0, N = 0, Np = 0, nchunk = 0, precision = ODIS_FP64;
    double* Y64 = nullptr;
    float* Y32 = nullptr;
    double* FGinv = nullptr;
    double* part = nullptr;
    double* coef = nullptr;
    double* usg64 = nullptr;
    float* usg32 = nullptr;
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
    s->nchunk = (m.N + kChunk - 1) / kChunk;
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
    } else {
        std::vector<float> Yf(Yt.begin(), Yt.end());
        up((void**)&s->Y32, Yf.data(), sizeof(float) * Yf.size());
        up((void**)&s->usg32, nullptr, sizeof(float) * Np);
    }
    up((void**)&s->FGinv, G.data(), sizeof(double) * G.size());
    up((void**)&s->part, nullptr, sizeof(double) * (size_t)K * s->nchunk);
    up((void**)&s->coef, nullptr, sizeof(double) * K);
    if (!ok) { sh_destroy(s); return ODIS_ERR_NOMEM; }
    *out = s;
    return ODIS_OK;
}

void sh_destroy(ShLoading* s)
{
    if (!s) return;
    cudaFree(s->Y64); cudaFree(s->Y32); cudaFree(s->FGinv); cudaFree(s->part); cudaFree(s->coef);
    cudaFree(s->usg64); cudaFree(s->usg32);
    delete s;
}

const double* sh_usg64(ShLoading* s) { return s ? s->usg64 : nullptr; }
const float* sh_usg32(ShLoading* s) { return s ? s->usg32 : nullptr; }

void sh_enqueue(ShLoading* s, const void* eta, cudaStream_t st)
{
    dim3 ga(s->nchunk, s->K);
    const size_t smem = sizeof(double) * s->K;
    const int sb = (s->N + kShThreads - 1) / kShThreads;
    if (s->precision == ODIS_FP64) {
        k_sh_analysis<double><<<ga, kShThreads, 0, st>>>(s->Y64, (const double*)eta, s->N, s->Np, s->nchunk, s->part);
        k_sh_solve<<<1, kShThreads, smem, st>>>(s->part, s->nchunk, s->K, s->FGinv, s->coef);
        k_sh_synth<double><<<sb, kShThreads, smem, st>>>(s->Y64, s->coef, s->N, s->Np, s->K, s->usg64);
    } else {
        k_sh_analysis<float><<<ga, kShThreads, 0, st>>>(s->Y32, (const float*)eta, s->N, s->Np, s->nchunk, s->part);
        k_sh_solve<<<1, kShThreads, smem, st>>>(s->part, s->nchunk, s->K, s->FGinv, s->coef);
        k_sh_synth<float><<<sb, kShThreads, smem, st>>>(s->Y32, s->coef, s->N, s->Np, s->K, s->usg32);
    }
}

}  // namespace odis
