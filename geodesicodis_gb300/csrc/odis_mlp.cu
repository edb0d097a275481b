// Warm-start surrogate network: a small MLP trained and evaluated by this
// library's own kernels (no reference counterpart).
//
// Layers: n_in -> width (GELU) -> ... -> width (GELU) -> n_mix * n_out (linear),
// then y = sum_k mix[k] * R_k with per-sample mixing weights (n_mix = 0: y = R).
// For the tidal response the mixing weights are the forcing amplitudes
// (eccentricity, obliquity): the linear LTE response is exactly linear in them,
// so the network only has to learn the response per unit forcing.
//
// Arithmetic: FP32 master weights; every GEMM rounds its operands to BF16 and
// accumulates in FP32 on the tensor cores (mma.sync m16n8k16); biases, GELU,
// the loss and Adam are FP32.  Loss = sum_i w_i * ||y_i - t_i||^2 / n
// (w_i: per-sample weights, e.g. 1 / ||t_i||^2 for a relative error).
#include "../../include/odis_gpu.h"

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

namespace odis {
namespace {

constexpr int kBM = 64, kBN = 64, kBK = 32, kPad = 8;
constexpr int kGemmThreads = 128;

__device__ __forceinline__ uint32_t lds32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, const uint32_t* b)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z)
{
    return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// C[m][n] = sum_k A(m, k) B(k, n) (+ bias[n]) with A(m, k) = A[m * sam + k * sak] and
// B(k, n) = B[k * sbk + n * sbn] (FP32 in memory, BF16 in the MMA).  mode 0:
// C = acc (+bias); mode 1: Z = acc + bias, H = GELU(Z).  Row stride of C/Z/H: ldc.
__global__ void __launch_bounds__(kGemmThreads) k_gemm(const float* __restrict__ A, long sam, long sak,
                                                       const float* __restrict__ B, long sbk, long sbn,
                                                       const float* __restrict__ bias, float* __restrict__ C,
                                                       float* __restrict__ H, int ldc, int M, int N, int K, int mode)
{
    __shared__ __align__(16) __nv_bfloat16 As[kBM][kBK + kPad];
    __shared__ __align__(16) __nv_bfloat16 Bs[kBN][kBK + kPad];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp >> 1, wn = warp & 1, g = lane >> 2, t = lane & 3;
    const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int r = 0; r < 4; r++) acc[i][j][r] = 0.f;
    for (int k0 = 0; k0 < K; k0 += kBK) {
        for (int idx = tid; idx < kBM * kBK; idx += kGemmThreads) {
            const int m = idx / kBK, k = idx % kBK;
            const int gm = m0 + m, gk = k0 + k;
            const float a = (gm < M && gk < K) ? A[gm * sam + gk * sak] : 0.f;
            As[m][k] = __float2bfloat16_rn(a);
        }
        for (int idx = tid; idx < kBN * kBK; idx += kGemmThreads) {
            const int n = idx / kBK, k = idx % kBK;
            const int gn = n0 + n, gk = k0 + k;
            const float b = (gn < N && gk < K) ? B[gk * sbk + gn * sbn] : 0.f;
            Bs[n][k] = __float2bfloat16_rn(b);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kBK; kk += 16) {
            uint32_t af[2][4], bf[4][2];
#pragma unroll
            for (int i = 0; i < 2; i++) {
                const int r0 = wm * 32 + i * 16;
                af[i][0] = lds32(&As[r0 + g][kk + 2 * t]);
                af[i][1] = lds32(&As[r0 + g + 8][kk + 2 * t]);
                af[i][2] = lds32(&As[r0 + g][kk + 2 * t + 8]);
                af[i][3] = lds32(&As[r0 + g + 8][kk + 2 * t + 8]);
            }
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int c0 = wn * 32 + j * 8;
                bf[j][0] = lds32(&Bs[c0 + g][kk + 2 * t]);
                bf[j][1] = lds32(&Bs[c0 + g][kk + 2 * t + 8]);
            }
#pragma unroll
            for (int i = 0; i < 2; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) mma_bf16(acc[i][j], af[i], bf[j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const int m = m0 + wm * 32 + i * 16 + g + (r >= 2 ? 8 : 0);
                const int n = n0 + wn * 32 + j * 8 + 2 * t + (r & 1);
                if (m >= M || n >= N) continue;
                float z = acc[i][j][r] + (bias ? bias[n] : 0.f);
                C[(long)m * ldc + n] = z;
                if (mode == 1) H[(long)m * ldc + n] = gelu(z);
            }
}

// dZ = dH * GELU'(Z)
__global__ void k_gelu_back(const float* __restrict__ dH, const float* __restrict__ Z, float* __restrict__ dZ, long n)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dZ[i] = dH[i] * gelu_grad(Z[i]);
}

// gb[n] = sum_m dZ[m][n] (fixed order: deterministic)
__global__ void k_colsum(const float* __restrict__ dZ, float* __restrict__ gb, int M, int N)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.f;
    for (int m = 0; m < M; m++) s += dZ[(long)m * N + n];
    gb[n] = s;
}

// mixing head: y[i][o] = sum_k mix[i][k] R[i][k * n_out + o]
__global__ void k_mix(const float* __restrict__ R, const float* __restrict__ mix, float* __restrict__ y, int n, int n_out,
                      int n_mix)
{
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)n * n_out) return;
    const int i = (int)(idx / n_out), o = (int)(idx % n_out);
    float s = 0.f;
    for (int k = 0; k < n_mix; k++) s += mix[(long)i * n_mix + k] * R[(long)i * n_mix * n_out + (long)k * n_out + o];
    y[idx] = s;
}

// dR[i][k * n_out + o] = mix[i][k] dy[i][o]
__global__ void k_mix_back(const float* __restrict__ dy, const float* __restrict__ mix, float* __restrict__ dR, int n,
                           int n_out, int n_mix)
{
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)n * n_mix * n_out) return;
    const int i = (int)(idx / ((long)n_mix * n_out));
    const int rem = (int)(idx % ((long)n_mix * n_out));
    const int k = rem / n_out, o = rem % n_out;
    dR[idx] = mix[(long)i * n_mix + k] * dy[(long)i * n_out + o];
}

// dy = 2 w_i (y - t) / n; per-block partial sums of w_i ||y_i - t_i||^2 / n (FP64)
__global__ void k_loss(const float* __restrict__ y, const float* __restrict__ t, const float* __restrict__ w,
                       float* __restrict__ dy, double* __restrict__ part, int n, int n_out)
{
    __shared__ double s[256];
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0;
    if (idx < (long)n * n_out) {
        const int i = (int)(idx / n_out);
        const float wi = w ? w[i] : 1.f;
        const float d = y[idx] - t[idx];
        dy[idx] = 2.f * wi * d / (float)n;
        l = (double)wi * (double)d * (double)d / n;
    }
    s[threadIdx.x] = l;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       long n, float lr, float b1, float b2, float eps, float c1, float c2)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void k_gather_rows(const float* __restrict__ src, const int* __restrict__ idx, float* __restrict__ dst, int n,
                              int width)
{
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (long)n * width) return;
    const int i = (int)(k / width), c = (int)(k % width);
    dst[k] = src[(long)idx[i] * width + c];
}

unsigned blocks(long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace
}  // namespace odis

using namespace odis;

struct odis_mlp {
    int n_in = 0, width = 0, depth = 0, n_out = 0, n_mix = 0;
    std::vector<int> dim;              // layer widths: dim[0] = n_in ... dim[L] = last layer outputs
    std::vector<long> woff, boff;      // offsets of W_l [dim l+1][dim l] and b_l in the flat parameter vector
    long n_params = 0;
    float* p = nullptr;                // parameters (FP32 master)
    float* grad = nullptr;
    float* am = nullptr;               // Adam moments
    float* av = nullptr;
    long step = 0;
    int cap = 0;                       // batch rows the work buffers hold
    std::vector<float*> Z, Hh, dZ;     // per layer [cap][dim l+1]
    float* X = nullptr;                // [cap][n_in]
    float* MIX = nullptr;              // [cap][n_mix]
    float* T = nullptr;                // [cap][n_out]
    float* W = nullptr;                // [cap]
    float* Y = nullptr;                // [cap][n_out]
    float* dY = nullptr;
    float* dH = nullptr;               // [cap][max dim]
    double* part = nullptr;
    int part_n = 0;
    cudaStream_t s = nullptr;
    ~odis_mlp() {
        cudaFree(p); cudaFree(grad); cudaFree(am); cudaFree(av);
        for (float* x : Z) cudaFree(x);
        for (float* x : Hh) cudaFree(x);
        for (float* x : dZ) cudaFree(x);
        cudaFree(X); cudaFree(MIX); cudaFree(T); cudaFree(W); cudaFree(Y); cudaFree(dY); cudaFree(dH); cudaFree(part);
        if (s) cudaStreamDestroy(s);
    }
};

#define ODIS_MCK(call)                                 \
    do {                                               \
        cudaError_t _e = (call);                       \
        if (_e != cudaSuccess) return ODIS_ERR_CUDA;   \
    } while (0)

static int layers(const odis_mlp* m) { return (int)m->dim.size() - 1; }

static int ensure_cap(odis_mlp* m, int n)
{
    if (n <= m->cap) return ODIS_OK;
    for (float* x : m->Z) cudaFree(x);
    for (float* x : m->Hh) cudaFree(x);
    for (float* x : m->dZ) cudaFree(x);
    cudaFree(m->X); cudaFree(m->MIX); cudaFree(m->T); cudaFree(m->W); cudaFree(m->Y); cudaFree(m->dY); cudaFree(m->dH);
    cudaFree(m->part);
    const int L = layers(m);
    m->Z.assign(L, nullptr);
    m->Hh.assign(L, nullptr);
    m->dZ.assign(L, nullptr);
    int maxd = 0;
    for (int d : m->dim) maxd = std::max(maxd, d);
    m->cap = 0;
    for (int l = 0; l < L; l++) {
        ODIS_MCK(cudaMalloc(&m->Z[l], sizeof(float) * (size_t)n * m->dim[l + 1]));
        ODIS_MCK(cudaMalloc(&m->Hh[l], sizeof(float) * (size_t)n * m->dim[l + 1]));
        ODIS_MCK(cudaMalloc(&m->dZ[l], sizeof(float) * (size_t)n * m->dim[l + 1]));
    }
    ODIS_MCK(cudaMalloc(&m->X, sizeof(float) * (size_t)n * m->n_in));
    ODIS_MCK(cudaMalloc(&m->MIX, sizeof(float) * (size_t)n * std::max(m->n_mix, 1)));
    ODIS_MCK(cudaMalloc(&m->T, sizeof(float) * (size_t)n * m->n_out));
    ODIS_MCK(cudaMalloc(&m->W, sizeof(float) * (size_t)n));
    ODIS_MCK(cudaMalloc(&m->Y, sizeof(float) * (size_t)n * m->n_out));
    ODIS_MCK(cudaMalloc(&m->dY, sizeof(float) * (size_t)n * m->n_out));
    ODIS_MCK(cudaMalloc(&m->dH, sizeof(float) * (size_t)n * maxd));
    m->part_n = (int)blocks((long)n * std::max(m->n_out, maxd), 256);
    ODIS_MCK(cudaMalloc(&m->part, sizeof(double) * m->part_n));
    m->cap = n;
    return ODIS_OK;
}

static void gemm(cudaStream_t s, const float* A, long sam, long sak, const float* B, long sbk, long sbn, const float* bias,
                 float* C, float* H, int ldc, int M, int N, int K, int mode)
{
    dim3 grid((N + kBN - 1) / kBN, (M + kBM - 1) / kBM);
    k_gemm<<<grid, kGemmThreads, 0, s>>>(A, sam, sak, B, sbk, sbn, bias, C, H, ldc, M, N, K, mode);
}

// forward pass of n rows already in m->X (and m->MIX); the output is in m->Y
static void forward(odis_mlp* m, int n)
{
    const int L = layers(m);
    const float* in = m->X;
    for (int l = 0; l < L; l++) {
        const int din = m->dim[l], dout = m->dim[l + 1];
        const float* Wl = m->p + m->woff[l];
        const float* bl = m->p + m->boff[l];
        // Z = in W^T + b : A = in [n][din], B(k, j) = W[j][k]
        gemm(m->s, in, din, 1, Wl, 1, din, bl, m->Z[l], m->Hh[l], dout, n, dout, din, l + 1 < L ? 1 : 0);
        in = m->Hh[l];
    }
    const float* R = m->Z[L - 1];
    if (m->n_mix > 0) k_mix<<<blocks((long)n * m->n_out, 256), 256, 0, m->s>>>(R, m->MIX, m->Y, n, m->n_out, m->n_mix);
    else cudaMemcpyAsync(m->Y, R, sizeof(float) * (size_t)n * m->n_out, cudaMemcpyDeviceToDevice, m->s);
}

// loss and gradient of n rows (X, MIX, T, W in the work buffers) into m->grad; returns the loss
static int backward(odis_mlp* m, int n, double* loss)
{
    const int L = layers(m);
    const long ny = (long)n * m->n_out;
    const unsigned nb = blocks(ny, 256);
    k_loss<<<nb, 256, 0, m->s>>>(m->Y, m->T, m->W, m->dY, m->part, n, m->n_out);
    // dR of the last layer
    float* dR = m->dZ[L - 1];
    if (m->n_mix > 0)
        k_mix_back<<<blocks((long)n * m->n_mix * m->n_out, 256), 256, 0, m->s>>>(m->dY, m->MIX, dR, n, m->n_out, m->n_mix);
    else cudaMemcpyAsync(dR, m->dY, sizeof(float) * ny, cudaMemcpyDeviceToDevice, m->s);
    for (int l = L - 1; l >= 0; l--) {
        const int din = m->dim[l], dout = m->dim[l + 1];
        const float* in = l == 0 ? m->X : m->Hh[l - 1];
        float* gW = m->grad + m->woff[l];
        float* gb = m->grad + m->boff[l];
        // gW[j][k] = sum_i dZ[i][j] in[i][k]: A(j, i) = dZ[i][j], B(i, k) = in[i][k]
        gemm(m->s, m->dZ[l], 1, dout, in, din, 1, nullptr, gW, nullptr, din, dout, din, n, 0);
        k_colsum<<<blocks(dout, 128), 128, 0, m->s>>>(m->dZ[l], gb, n, dout);
        if (l > 0) {
            // dH[i][k] = sum_j dZ[i][j] W[j][k]
            const float* Wl = m->p + m->woff[l];
            gemm(m->s, m->dZ[l], dout, 1, Wl, din, 1, nullptr, m->dH, nullptr, din, n, din, dout, 0);
            k_gelu_back<<<blocks((long)n * din, 256), 256, 0, m->s>>>(m->dH, m->Z[l - 1], m->dZ[l - 1], (long)n * din);
        }
    }
    if (loss) {
        std::vector<double> h(nb);
        ODIS_MCK(cudaMemcpyAsync(h.data(), m->part, sizeof(double) * nb, cudaMemcpyDeviceToHost, m->s));
        ODIS_MCK(cudaStreamSynchronize(m->s));
        double sum = 0.0;
        for (double x : h) sum += x;
        *loss = sum;
    }
    return ODIS_OK;
}

extern "C" odis_status odis_mlp_create(int n_in, int width, int depth, int n_out, int n_mix, unsigned long long seed,
                                       odis_mlp** out)
{
    if (!out || n_in <= 0 || width <= 0 || depth < 0 || n_out <= 0 || n_mix < 0) return ODIS_ERR_ARG;
    *out = nullptr;
    std::unique_ptr<odis_mlp> m(new (std::nothrow) odis_mlp);
    if (!m) return ODIS_ERR_NOMEM;
    m->n_in = n_in;
    m->width = width;
    m->depth = depth;
    m->n_out = n_out;
    m->n_mix = n_mix;
    m->dim.push_back(n_in);
    for (int l = 0; l < depth; l++) m->dim.push_back(width);
    m->dim.push_back(n_out * std::max(n_mix, 1));
    const int L = layers(m.get());
    long off = 0;
    for (int l = 0; l < L; l++) {
        m->woff.push_back(off);
        off += (long)m->dim[l + 1] * m->dim[l];
        m->boff.push_back(off);
        off += m->dim[l + 1];
    }
    m->n_params = off;
    // weights and biases uniform in +-1/sqrt(fan_in); splitmix64 stream from `seed`
    std::vector<float> h(off, 0.f);
    uint64_t x = seed;
    auto next = [&]() {
        uint64_t z = (x += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l < L; l++) {
        const double a = 1.0 / std::sqrt((double)m->dim[l]);
        for (long k = 0; k < (long)m->dim[l + 1] * m->dim[l]; k++) h[m->woff[l] + k] = (float)((2.0 * next() - 1.0) * a);
        for (long k = 0; k < m->dim[l + 1]; k++) h[m->boff[l] + k] = (float)((2.0 * next() - 1.0) * a);
    }
    ODIS_MCK(cudaStreamCreateWithFlags(&m->s, cudaStreamNonBlocking));
    ODIS_MCK(cudaMalloc(&m->p, sizeof(float) * off));
    ODIS_MCK(cudaMalloc(&m->grad, sizeof(float) * off));
    ODIS_MCK(cudaMalloc(&m->am, sizeof(float) * off));
    ODIS_MCK(cudaMalloc(&m->av, sizeof(float) * off));
    ODIS_MCK(cudaMemcpy(m->p, h.data(), sizeof(float) * off, cudaMemcpyHostToDevice));
    ODIS_MCK(cudaMemset(m->grad, 0, sizeof(float) * off));
    ODIS_MCK(cudaMemset(m->am, 0, sizeof(float) * off));
    ODIS_MCK(cudaMemset(m->av, 0, sizeof(float) * off));
    *out = m.release();
    return ODIS_OK;
}

extern "C" void odis_mlp_destroy(odis_mlp* m)
{
    if (!m) return;
    cudaStreamSynchronize(m->s);
    delete m;
}

extern "C" odis_status odis_mlp_num_params(const odis_mlp* m, long long* n)
{
    if (!m || !n) return ODIS_ERR_ARG;
    *n = m->n_params;
    return ODIS_OK;
}

extern "C" odis_status odis_mlp_get_params(odis_mlp* m, float* out)
{
    if (!m || !out) return ODIS_ERR_ARG;
    ODIS_MCK(cudaStreamSynchronize(m->s));
    ODIS_MCK(cudaMemcpy(out, m->p, sizeof(float) * m->n_params, cudaMemcpyDeviceToHost));
    return ODIS_OK;
}

extern "C" odis_status odis_mlp_set_params(odis_mlp* m, const float* in)
{
    if (!m || !in) return ODIS_ERR_ARG;
    ODIS_MCK(cudaStreamSynchronize(m->s));
    ODIS_MCK(cudaMemcpy(m->p, in, sizeof(float) * m->n_params, cudaMemcpyHostToDevice));
    m->step = 0;
    ODIS_MCK(cudaMemset(m->am, 0, sizeof(float) * m->n_params));
    ODIS_MCK(cudaMemset(m->av, 0, sizeof(float) * m->n_params));
    return ODIS_OK;
}

static int upload_rows(odis_mlp* m, const float* x, const float* mix, const float* t, const float* w, int n)
{
    ODIS_MCK(cudaMemcpyAsync(m->X, x, sizeof(float) * (size_t)n * m->n_in, cudaMemcpyHostToDevice, m->s));
    if (m->n_mix > 0) {
        if (!mix) return ODIS_ERR_ARG;
        ODIS_MCK(cudaMemcpyAsync(m->MIX, mix, sizeof(float) * (size_t)n * m->n_mix, cudaMemcpyHostToDevice, m->s));
    }
    if (t) ODIS_MCK(cudaMemcpyAsync(m->T, t, sizeof(float) * (size_t)n * m->n_out, cudaMemcpyHostToDevice, m->s));
    if (t) {
        if (w) ODIS_MCK(cudaMemcpyAsync(m->W, w, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, m->s));
        else {
            std::vector<float> one(n, 1.f);
            ODIS_MCK(cudaMemcpyAsync(m->W, one.data(), sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, m->s));
            ODIS_MCK(cudaStreamSynchronize(m->s));
        }
    }
    return ODIS_OK;
}

extern "C" odis_status odis_mlp_predict(odis_mlp* m, const float* x, const float* mix, int n, float* y)
{
    if (!m || !x || !y || n <= 0) return ODIS_ERR_ARG;
    const int chunk = 4096;
    int st = ensure_cap(m, std::min(n, chunk));
    if (st != ODIS_OK) return st;
    for (int i0 = 0; i0 < n; i0 += chunk) {
        const int k = std::min(chunk, n - i0);
        st = upload_rows(m, x + (size_t)i0 * m->n_in, mix ? mix + (size_t)i0 * m->n_mix : nullptr, nullptr, nullptr, k);
        if (st != ODIS_OK) return st;
        forward(m, k);
        ODIS_MCK(cudaMemcpyAsync(y + (size_t)i0 * m->n_out, m->Y, sizeof(float) * (size_t)k * m->n_out,
                                 cudaMemcpyDeviceToHost, m->s));
    }
    ODIS_MCK(cudaStreamSynchronize(m->s));
    ODIS_MCK(cudaGetLastError());
    return ODIS_OK;
}

extern "C" odis_status odis_mlp_gradient(odis_mlp* m, const float* x, const float* mix, const float* t, const float* w,
                                         int n, double* loss, float* grad)
{
    if (!m || !x || !t || n <= 0) return ODIS_ERR_ARG;
    int st = ensure_cap(m, n);
    if (st != ODIS_OK) return st;
    st = upload_rows(m, x, mix, t, w, n);
    if (st != ODIS_OK) return st;
    forward(m, n);
    st = backward(m, n, loss);
    if (st != ODIS_OK) return st;
    if (grad) ODIS_MCK(cudaMemcpyAsync(grad, m->grad, sizeof(float) * m->n_params, cudaMemcpyDeviceToHost, m->s));
    ODIS_MCK(cudaStreamSynchronize(m->s));
    ODIS_MCK(cudaGetLastError());
    return ODIS_OK;
}

// Adam (beta1 0.9, beta2 0.999, eps 1e-8) over minibatches of a shuffled copy of
// the data set, learning rate lr * (0.5 + 0.5 cos(pi * epoch / epochs)).
extern "C" odis_status odis_mlp_train(odis_mlp* m, const float* x, const float* mix, const float* t, const float* w, int n,
                                      int epochs, int batch, float lr, unsigned long long seed, double* loss_per_epoch)
{
    if (!m || !x || !t || n <= 0 || epochs <= 0 || batch <= 0) return ODIS_ERR_ARG;
    batch = std::min(batch, n);
    int st = ensure_cap(m, batch);
    if (st != ODIS_OK) return st;
    float *dx = nullptr, *dmix = nullptr, *dt = nullptr, *dw = nullptr;
    int* didx = nullptr;
    auto done = [&](int r) { cudaFree(dx); cudaFree(dmix); cudaFree(dt); cudaFree(dw); cudaFree(didx); return r; };
    if (cudaMalloc(&dx, sizeof(float) * (size_t)n * m->n_in) != cudaSuccess ||
        cudaMalloc(&dmix, sizeof(float) * (size_t)n * std::max(m->n_mix, 1)) != cudaSuccess ||
        cudaMalloc(&dt, sizeof(float) * (size_t)n * m->n_out) != cudaSuccess ||
        cudaMalloc(&dw, sizeof(float) * (size_t)n) != cudaSuccess || cudaMalloc(&didx, sizeof(int) * (size_t)n) != cudaSuccess)
        return done(ODIS_ERR_NOMEM);
    std::vector<float> ones;
    if (!w) ones.assign(n, 1.f);
    if (cudaMemcpy(dx, x, sizeof(float) * (size_t)n * m->n_in, cudaMemcpyHostToDevice) != cudaSuccess ||
        (m->n_mix > 0 && (!mix || cudaMemcpy(dmix, mix, sizeof(float) * (size_t)n * m->n_mix, cudaMemcpyHostToDevice) != cudaSuccess)) ||
        cudaMemcpy(dt, t, sizeof(float) * (size_t)n * m->n_out, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dw, w ? w : ones.data(), sizeof(float) * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess)
        return done(ODIS_ERR_CUDA);
    std::vector<int> perm(n);
    uint64_t rs = seed ^ 0x5DEECE66Dull;
    auto rnd = [&]() { rs ^= rs << 13; rs ^= rs >> 7; rs ^= rs << 17; return rs; };
    for (int e = 0; e < epochs; e++) {
        for (int i = 0; i < n; i++) perm[i] = i;
        for (int i = n - 1; i > 0; i--) std::swap(perm[i], perm[(int)(rnd() % (uint64_t)(i + 1))]);
        if (cudaMemcpyAsync(didx, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, m->s) != cudaSuccess) return done(ODIS_ERR_CUDA);
        const float lr_e = lr * (0.5f + 0.5f * (float)std::cos(3.14159265358979 * e / epochs));
        double eloss = 0.0;
        int nbatch = 0;
        for (int i0 = 0; i0 + batch <= n; i0 += batch) {       // whole minibatches only
            k_gather_rows<<<blocks((long)batch * m->n_in, 256), 256, 0, m->s>>>(dx, didx + i0, m->X, batch, m->n_in);
            if (m->n_mix > 0)
                k_gather_rows<<<blocks((long)batch * m->n_mix, 256), 256, 0, m->s>>>(dmix, didx + i0, m->MIX, batch, m->n_mix);
            k_gather_rows<<<blocks((long)batch * m->n_out, 256), 256, 0, m->s>>>(dt, didx + i0, m->T, batch, m->n_out);
            k_gather_rows<<<blocks(batch, 256), 256, 0, m->s>>>(dw, didx + i0, m->W, batch, 1);
            forward(m, batch);
            double l = 0.0;
            st = backward(m, batch, loss_per_epoch ? &l : nullptr);
            if (st != ODIS_OK) return done(st);
            m->step++;
            const float c1 = 1.f - std::pow(0.9f, (float)m->step), c2 = 1.f - std::pow(0.999f, (float)m->step);
            k_adam<<<blocks(m->n_params, 256), 256, 0, m->s>>>(m->p, m->grad, m->am, m->av, m->n_params, lr_e, 0.9f, 0.999f,
                                                              1e-8f, c1, c2);
            eloss += l;
            nbatch++;
        }
        if (loss_per_epoch) loss_per_epoch[e] = nbatch ? eloss / nbatch : 0.0;
    }
    if (cudaStreamSynchronize(m->s) != cudaSuccess || cudaGetLastError() != cudaSuccess) return done(ODIS_ERR_CUDA);
    return done(ODIS_OK);
}
