// Learned warm start: a small MLP (n_in -> H -> H -> n_out, GELU) that proposes
// starting angles for the optimiser, trained and run by the kernels in this file.
// Weights are stored in BF16 for the forward and backward products (FP32 master
// copies and Adam moments), every product accumulates in FP32, the loss is the mean
// squared error on standardised targets.  No counterpart in the reference.
//
// The products are small (batch <= a few thousand rows, widths <= 512): they are
// latency-bound, so they run as tiled FP32 FMA kernels (64 x 64 output tile per CTA,
// 4 x 4 per thread, K staged through shared memory) rather than on the tensor cores.
#include "../../include/aegpu.h"

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace {

constexpr int kTM = 64, kTN = 64, kTK = 32, kGemmThreads = 256;

enum Epilogue { kPlain = 0, kBiasGelu = 1, kBias = 2, kGeluGrad = 3 };

template <typename T>
__device__ __forceinline__ float ldf(const T *p);
template <>
__device__ __forceinline__ float ldf<float>(const float *p)
{
    return *p;
}
template <>
__device__ __forceinline__ float ldf<__nv_bfloat16>(const __nv_bfloat16 *p)
{
    return __bfloat162float(*p);
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z)
{
    return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

__device__ __forceinline__ float epilogue(float v, int64_t o, int n, const float *__restrict__ bias,
                                          float *__restrict__ Z, int epi)
{
    if (epi == kBias || epi == kBiasGelu) v += bias[n];
    if (epi == kBiasGelu) {
        Z[o] = v;
        v = gelu(v);
    } else if (epi == kGeluGrad) {
        v *= gelu_grad(Z[o]);
    }
    return v;
}

// C[m][n] = sum_k A(m,k) B(k,n), A(m,k) = A[m*a_rs + k*a_cs], B(k,n) = B[k*b_rs + n*b_cs],
// then the epilogue:
//   kPlain:    C = acc
//   kBias:     C = acc + bias[n]
//   kBiasGelu: Z = acc + bias[n] (pre-activation, stored), C = gelu(Z)
//   kGeluGrad: C = acc * gelu'(Z[m][n])  (Z read)
// Split K (gridDim.z > 1, for products with few output tiles): CTA z sums k in
// [z * kz, (z + 1) * kz) and writes its raw partial to C + z * M * N (a workspace);
// k_gemm_reduce adds the partials in z order and applies the epilogue.  The tile loads
// walk the operand's unit-stride dimension fastest, so they coalesce; the next K tile's
// loads are issued into registers before the current tile's products, so their latency
// overlaps the arithmetic.
template <typename TB>
__global__ void __launch_bounds__(kGemmThreads) k_gemm(const float *__restrict__ A, int64_t a_rs, int64_t a_cs,
                                                       const TB *__restrict__ B, int64_t b_rs, int64_t b_cs,
                                                       float *__restrict__ C, int M, int N, int K, int kz,
                                                       const float *__restrict__ bias, float *__restrict__ Z, int epi)
{
    constexpr int LA = kTK * kTM / kGemmThreads, LB = kTK * kTN / kGemmThreads;
    __shared__ float As[kTK][kTM + 1];
    __shared__ float Bs[kTK][kTN + 1];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.y * kTM, n0 = blockIdx.x * kTN;
    const int kb = blockIdx.z * kz, ke = kb + kz < K ? kb + kz : K;
    const bool a_k_fast = a_cs == 1, b_k_fast = b_rs == 1;
    float ra[LA], rb[LB];
    auto load = [&](int k0) {
#pragma unroll
        for (int t = 0; t < LA; ++t) {
            const int i = threadIdx.x + t * kGemmThreads;
            const int kk = a_k_fast ? i % kTK : i / kTM, mm = a_k_fast ? i / kTK : i % kTM;
            const int m = m0 + mm, k = k0 + kk;
            ra[t] = (m < M && k < ke) ? A[(int64_t)m * a_rs + (int64_t)k * a_cs] : 0.0f;
        }
#pragma unroll
        for (int t = 0; t < LB; ++t) {
            const int i = threadIdx.x + t * kGemmThreads;
            const int kk = b_k_fast ? i % kTK : i / kTN, nn = b_k_fast ? i / kTK : i % kTN;
            const int n = n0 + nn, k = k0 + kk;
            rb[t] = (n < N && k < ke) ? ldf(B + (int64_t)k * b_rs + (int64_t)n * b_cs) : 0.0f;
        }
    };
    float acc[4][4] = {};
    if (kb < ke) load(kb);
    for (int k0 = kb; k0 < ke; k0 += kTK) {
#pragma unroll
        for (int t = 0; t < LA; ++t) {
            const int i = threadIdx.x + t * kGemmThreads;
            As[a_k_fast ? i % kTK : i / kTM][a_k_fast ? i / kTK : i % kTM] = ra[t];
        }
#pragma unroll
        for (int t = 0; t < LB; ++t) {
            const int i = threadIdx.x + t * kGemmThreads;
            Bs[b_k_fast ? i % kTK : i / kTN][b_k_fast ? i / kTK : i % kTN] = rb[t];
        }
        __syncthreads();
        if (k0 + kTK < ke) load(k0 + kTK);
#pragma unroll
        for (int kk = 0; kk < kTK; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
    const bool split = gridDim.z > 1;
    float *Cz = C + (split ? (int64_t)blockIdx.z * M * N : 0);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int m = m0 + ty + 16 * i, n = n0 + tx + 16 * j;
            if (m >= M || n >= N) continue;
            const int64_t o = (int64_t)m * N + n;
            Cz[o] = split ? acc[i][j] : epilogue(acc[i][j], o, n, bias, Z, epi);
        }
}

// C = epilogue(sum over z of the split-K partials ws[z][M][N]), z in order.
__global__ void k_gemm_reduce(const float *__restrict__ ws, int ksplit, int M, int N, float *__restrict__ C,
                              const float *__restrict__ bias, float *__restrict__ Z, int epi)
{
    const int64_t MN = (int64_t)M * N;
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < MN; o += (int64_t)gridDim.x * blockDim.x) {
        float v = 0.0f;
        for (int z = 0; z < ksplit; ++z) v += ws[z * MN + o];
        C[o] = epilogue(v, o, (int)(o % N), bias, Z, epi);
    }
}

// column sums: out[n] = sum_m X[m][n] (bias gradients).  A CTA of 8 warps per 32
// columns: warp w sums rows w, w + 8, ... of column lane (coalesced), then the eight
// warp sums are added in warp order (fixed summation order).
constexpr int kColsumWarps = 8;
__global__ void k_colsum(const float *__restrict__ X, int M, int N, float *__restrict__ out)
{
    __shared__ float part[kColsumWarps][33];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int n = blockIdx.x * 32 + lane;
    float s = 0;
    if (n < N)
        for (int m = w; m < M; m += kColsumWarps) s += X[(int64_t)m * N + n];
    part[w][lane] = s;
    __syncthreads();
    if (w == 0 && n < N) {
        float t = 0;
        for (int k = 0; k < kColsumWarps; ++k) t += part[k][lane];
        out[n] = t;
    }
}

// rows of X (indexed through idx, nullable) standardised into Xn
__global__ void k_standardise(const float *__restrict__ X, const int *__restrict__ idx, int rows, int cols,
                              const float *__restrict__ mean, const float *__restrict__ inv_scale,
                              float *__restrict__ Xn)
{
    const int64_t total = (int64_t)rows * cols;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(i / cols), c = (int)(i % cols);
        const int src = idx ? idx[r] : r;
        Xn[i] = (X[(int64_t)src * cols + c] - mean[c]) * inv_scale[c];
    }
}

// dY = 2 (Y - T') / (rows * cols) with T' the standardised targets; per-row squared
// error sums into rowloss
__global__ void k_mse(const float *__restrict__ Y, const float *__restrict__ T, const int *__restrict__ idx, int rows,
                      int cols, const float *__restrict__ mean, const float *__restrict__ inv_scale,
                      float *__restrict__ dY, float *__restrict__ rowloss)
{
    // one warp per row: lanes take columns lane, lane + 32, ... (coalesced), the row's
    // squared error meets in a fixed butterfly
    const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (r >= rows) return;
    const int src = idx ? idx[r] : r;
    const float w = 2.0f / ((float)rows * (float)cols);
    float s = 0;
    for (int c = lane; c < cols; c += 32) {
        const float d = Y[(int64_t)r * cols + c] - (T[(int64_t)src * cols + c] - mean[c]) * inv_scale[c];
        s += d * d;
        dY[(int64_t)r * cols + c] = w * d;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) rowloss[r] = s;
}

// Y = Yn * scale + mean (outputs back to angle units)
__global__ void k_unstandardise(float *__restrict__ Y, int rows, int cols, const float *__restrict__ mean,
                                const float *__restrict__ scale)
{
    const int64_t total = (int64_t)rows * cols;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % cols);
        Y[i] = Y[i] * scale[c] + mean[c];
    }
}

// Adam (Kingma & Ba 2015, Algorithm 1) on the FP32 master weights, refreshing the
// BF16 copies used by the products.  Weight tensors only have BF16 copies (wq != null
// for them); biases stay FP32.  c12 = the step's bias corrections (1 - b1^t, 1 - b2^t),
// read from device memory so that a captured step serves every t.
__global__ void k_adam(float *__restrict__ w, __nv_bfloat16 *__restrict__ wq, const float *__restrict__ g,
                       float *__restrict__ m, float *__restrict__ v, int64_t n, float lr, float b1, float b2, float eps,
                       const float *__restrict__ c12)
{
    const float c1 = c12[0], c2 = c12[1];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        w[i] = wi;
        if (wq) wq[i] = __float2bfloat16_rn(wi);
    }
}

__global__ void k_to_bf16(const float *__restrict__ w, __nv_bfloat16 *__restrict__ wq, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        wq[i] = __float2bfloat16_rn(w[i]);
}

uint64_t splitmix64(uint64_t &s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
double uniform01(uint64_t &s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

}  // namespace

// Parameters, all in one FP32 array (and its gradient / Adam moments):
// W1[H][n_in], b1[H], W2[H][H], b2[H], W3[n_out][H], b3[n_out].
struct aegpu_mlp {
    int n_in = 0, H = 0, n_out = 0;
    int64_t off[7] = {};  // offsets of W1 b1 W2 b2 W3 b3, end
    float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
    __nv_bfloat16 *wq = nullptr;  // BF16 copies, same offsets
    float *scal = nullptr;        // in_mean[n_in], in_inv[n_in], out_mean[n_out], out_scale[n_out], out_inv[n_out]
    int64_t adam_t = 0;
    cudaStream_t stream = nullptr;
    std::vector<void *> allocs;
    std::string err;
    // activations for up to cap rows
    int cap = 0;
    float *X0 = nullptr, *Z1 = nullptr, *A1 = nullptr, *Z2 = nullptr, *A2 = nullptr, *Y = nullptr;
    float *dY = nullptr, *dA = nullptr, *dZ = nullptr, *rowloss = nullptr;
    float *ws = nullptr;  // split-K partial products
    int *idx = nullptr;

    ~aegpu_mlp()
    {
        for (void *p : allocs) cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
    }
    template <typename T>
    T *alloc(size_t n)
    {
        void *p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        allocs.push_back(p);
        return (T *)p;
    }
    void free_ptr(void *p)
    {
        if (!p) return;
        auto it = std::find(allocs.begin(), allocs.end(), p);
        if (it != allocs.end()) allocs.erase(it);
        cudaFree(p);
    }
    int64_t nparams() const { return off[6]; }
    const float *in_mean() const { return scal; }
    const float *in_inv() const { return scal + n_in; }
    const float *out_mean() const { return scal + 2 * n_in; }
    const float *out_scale() const { return scal + 2 * n_in + n_out; }
    const float *out_inv() const { return scal + 2 * n_in + 2 * n_out; }
    bool reserve(int rows)
    {
        if (rows <= cap) return true;
        for (void *p : {(void *)X0, (void *)Z1, (void *)A1, (void *)Z2, (void *)A2, (void *)Y, (void *)dY, (void *)dA,
                        (void *)dZ, (void *)rowloss, (void *)idx})
            free_ptr(p);
        const size_t r = rows;
        X0 = alloc<float>(r * n_in);
        Z1 = alloc<float>(r * H);
        A1 = alloc<float>(r * H);
        Z2 = alloc<float>(r * H);
        A2 = alloc<float>(r * H);
        Y = alloc<float>(r * n_out);
        dY = alloc<float>(r * n_out);
        dA = alloc<float>(r * H);
        dZ = alloc<float>(r * H);
        rowloss = alloc<float>(r);
        idx = alloc<int>(r);
        cap = rows;
        return X0 && Z1 && A1 && Z2 && A2 && Y && dY && dA && dZ && rowloss && idx;
    }
    int fail(int code, const std::string &m)
    {
        err = m;
        return code;
    }
    int check(const char *where)
    {
        cudaError_t rc = cudaGetLastError();
        if (rc != cudaSuccess) return fail(AEGPU_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(rc));
        return AEGPU_OK;
    }
};

namespace {

// Products with fewer than 128 output tiles split K over up to kMaxSplit CTAs per tile
// (at least 64 k per CTA), so that more SMs share the latency-bound K loop.
constexpr int kMaxSplit = 8;
constexpr int64_t kSplitWorkspace = (int64_t)kMaxSplit * 64 * kTM * kTN;

template <typename TB>
void gemm(cudaStream_t s, float *ws, const float *A, int64_t a_rs, int64_t a_cs, const TB *B, int64_t b_rs,
          int64_t b_cs, float *C, int M, int N, int K, const float *bias, float *Z, int epi)
{
    dim3 grid((N + kTN - 1) / kTN, (M + kTM - 1) / kTM);
    const int tiles = grid.x * grid.y;
    int split = 1;
    if (tiles < 128 && ws)
        while (split < kMaxSplit && K / (split * 2) >= 64 && (int64_t)split * 2 * M * N <= kSplitWorkspace) split *= 2;
    const int kz = (K + split - 1) / split;
    grid.z = split;
    k_gemm<TB><<<grid, kGemmThreads, 0, s>>>(A, a_rs, a_cs, B, b_rs, b_cs, split > 1 ? ws : C, M, N, K, kz, bias, Z,
                                             epi);
    if (split > 1) {
        const int64_t MN = (int64_t)M * N;
        k_gemm_reduce<<<(int)std::min<int64_t>((MN + 255) / 256, 1024), 256, 0, s>>>(ws, split, M, N, C, bias, Z, epi);
    }
}

// forward of `rows` standardised input rows already in X0; output (standardised) in Y
void forward(aegpu_mlp *m, int rows)
{
    const int H = m->H, ni = m->n_in, no = m->n_out;
    const __nv_bfloat16 *W1 = m->wq + m->off[0], *W2 = m->wq + m->off[2], *W3 = m->wq + m->off[4];
    const float *b1 = m->w + m->off[1], *b2 = m->w + m->off[3], *b3 = m->w + m->off[5];
    // Z = X W^T + b: B(k,n) = W[n][k]
    gemm(m->stream, m->ws, m->X0, ni, 1, W1, 1, ni, m->A1, rows, H, ni, b1, m->Z1, kBiasGelu);
    gemm(m->stream, m->ws, m->A1, H, 1, W2, 1, H, m->A2, rows, H, H, b2, m->Z2, kBiasGelu);
    gemm(m->stream, m->ws, m->A2, H, 1, W3, 1, H, m->Y, rows, no, H, b3, nullptr, kBias);
}

// gradients of the loss (dY already in m->dY) into m->g
void backward(aegpu_mlp *m, int rows)
{
    const int H = m->H, ni = m->n_in, no = m->n_out;
    const __nv_bfloat16 *W2 = m->wq + m->off[2], *W3 = m->wq + m->off[4];
    float *g = m->g;
    cudaStream_t s = m->stream;
    // layer 3: dW3[o][k] = sum_b dY[b][o] A2[b][k]; db3; dA2 = dY W3 (gelu' of Z2 fused)
    gemm(s, m->ws, m->dY, 1, no, m->A2, H, 1, g + m->off[4], no, H, rows, nullptr, nullptr, kPlain);
    k_colsum<<<(no + 31) / 32, 32 * kColsumWarps, 0, s>>>(m->dY, rows, no, g + m->off[5]);
    gemm(s, m->ws, m->dY, no, 1, W3, H, 1, m->dZ, rows, H, no, nullptr, m->Z2, kGeluGrad);
    // layer 2
    gemm(s, m->ws, m->dZ, 1, H, m->A1, H, 1, g + m->off[2], H, H, rows, nullptr, nullptr, kPlain);
    k_colsum<<<(H + 31) / 32, 32 * kColsumWarps, 0, s>>>(m->dZ, rows, H, g + m->off[3]);
    gemm(s, m->ws, m->dZ, H, 1, W2, H, 1, m->dA, rows, H, H, nullptr, m->Z1, kGeluGrad);
    // layer 1 (no input gradient needed)
    gemm(s, m->ws, m->dA, 1, H, m->X0, ni, 1, g + m->off[0], H, ni, rows, nullptr, nullptr, kPlain);
    k_colsum<<<(H + 31) / 32, 32 * kColsumWarps, 0, s>>>(m->dA, rows, H, g + m->off[1]);
}

}  // namespace

extern "C" {

int aegpu_mlp_create(aegpu_mlp **out, int n_in, int n_hidden, int n_out, uint64_t seed)
{
    if (!out || n_in < 1 || n_hidden < 1 || n_out < 1) return AEGPU_ERR_ARG;
    *out = nullptr;
    auto *m = new aegpu_mlp();
    m->n_in = n_in;
    m->H = n_hidden;
    m->n_out = n_out;
    const int64_t sizes[6] = {(int64_t)n_hidden * n_in, n_hidden, (int64_t)n_hidden * n_hidden, n_hidden,
                              (int64_t)n_out * n_hidden, n_out};
    m->off[0] = 0;
    for (int i = 0; i < 6; ++i) m->off[i + 1] = m->off[i] + sizes[i];
    const int64_t n = m->nparams();
    if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete m;
        return AEGPU_ERR_CUDA;
    }
    m->w = m->alloc<float>(n);
    m->g = m->alloc<float>(n);
    m->m = m->alloc<float>(n);
    m->v = m->alloc<float>(n);
    m->wq = m->alloc<__nv_bfloat16>(n);
    m->scal = m->alloc<float>(2 * n_in + 3 * n_out);
    m->ws = m->alloc<float>(kSplitWorkspace);
    if (!m->w || !m->g || !m->m || !m->v || !m->wq || !m->scal || !m->ws) {
        delete m;
        return AEGPU_ERR_NOMEM;
    }
    // U(-1/sqrt(fan_in), 1/sqrt(fan_in)) for weights and biases; identity scaling
    std::vector<float> w(n);
    uint64_t s = seed;
    const int fan[6] = {n_in, n_in, n_hidden, n_hidden, n_hidden, n_hidden};
    for (int t = 0; t < 6; ++t) {
        const double a = 1.0 / std::sqrt((double)fan[t]);
        for (int64_t i = m->off[t]; i < m->off[t + 1]; ++i) w[i] = (float)((2.0 * uniform01(s) - 1.0) * a);
    }
    std::vector<float> sc(2 * n_in + 3 * n_out, 0.0f);
    std::fill(sc.begin() + n_in, sc.begin() + 2 * n_in, 1.0f);
    std::fill(sc.begin() + 2 * n_in + n_out, sc.end(), 1.0f);
    cudaMemcpy(m->w, w.data(), n * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(m->scal, sc.data(), sc.size() * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemset(m->m, 0, n * sizeof(float));
    cudaMemset(m->v, 0, n * sizeof(float));
    k_to_bf16<<<256, 256, 0, m->stream>>>(m->w, m->wq, n);
    if (cudaStreamSynchronize(m->stream) != cudaSuccess || m->check("mlp_create")) {
        cudaGetLastError();
        delete m;
        return AEGPU_ERR_CUDA;
    }
    *out = m;
    return AEGPU_OK;
}

void aegpu_mlp_destroy(aegpu_mlp *m) { delete m; }

const char *aegpu_mlp_last_error(const aegpu_mlp *m) { return m ? m->err.c_str() : "null model"; }

int64_t aegpu_mlp_num_params(const aegpu_mlp *m) { return m ? m->nparams() : -1; }

int aegpu_mlp_set_scaling(aegpu_mlp *m, const float *in_mean, const float *in_scale, const float *out_mean,
                          const float *out_scale)
{
    if (!m || !in_mean || !in_scale || !out_mean || !out_scale) return AEGPU_ERR_ARG;
    std::vector<float> sc(2 * m->n_in + 3 * m->n_out);
    for (int i = 0; i < m->n_in; ++i) {
        if (!(in_scale[i] > 0)) return m->fail(AEGPU_ERR_ARG, "input scales must be positive");
        sc[i] = in_mean[i];
        sc[m->n_in + i] = 1.0f / in_scale[i];
    }
    for (int i = 0; i < m->n_out; ++i) {
        if (!(out_scale[i] > 0)) return m->fail(AEGPU_ERR_ARG, "output scales must be positive");
        sc[2 * m->n_in + i] = out_mean[i];
        sc[2 * m->n_in + m->n_out + i] = out_scale[i];
        sc[2 * m->n_in + 2 * m->n_out + i] = 1.0f / out_scale[i];
    }
    cudaMemcpy(m->scal, sc.data(), sc.size() * sizeof(float), cudaMemcpyHostToDevice);
    return m->check("mlp_set_scaling");
}

int aegpu_mlp_get_params(aegpu_mlp *m, float *params)
{
    if (!m || !params) return AEGPU_ERR_ARG;
    cudaMemcpy(params, m->w, m->nparams() * sizeof(float), cudaMemcpyDeviceToHost);
    return m->check("mlp_get_params");
}

int aegpu_mlp_set_params(aegpu_mlp *m, const float *params)
{
    if (!m || !params) return AEGPU_ERR_ARG;
    cudaMemcpy(m->w, params, m->nparams() * sizeof(float), cudaMemcpyHostToDevice);
    k_to_bf16<<<256, 256, 0, m->stream>>>(m->w, m->wq, m->nparams());
    cudaStreamSynchronize(m->stream);
    return m->check("mlp_set_params");
}

// Predictions (angle units) for n input rows, device pointers, on `stream`'s order
// (the model's stream when NULL); nothing synchronised.
int aegpu_mlp_predict_dev(aegpu_mlp *m, const float *X_dev, int n, float *Y_dev, void *stream)
{
    if (!m || !X_dev || !Y_dev || n < 1) return AEGPU_ERR_ARG;
    if (!m->reserve(n)) return m->fail(AEGPU_ERR_NOMEM, "activation allocation failed");
    cudaStream_t saved = m->stream;
    if (stream) m->stream = (cudaStream_t)stream;
    k_standardise<<<256, 256, 0, m->stream>>>(X_dev, nullptr, n, m->n_in, m->in_mean(), m->in_inv(), m->X0);
    forward(m, n);
    cudaMemcpyAsync(Y_dev, m->Y, (size_t)n * m->n_out * sizeof(float), cudaMemcpyDeviceToDevice, m->stream);
    k_unstandardise<<<256, 256, 0, m->stream>>>(Y_dev, n, m->n_out, m->out_mean(), m->out_scale());
    m->stream = saved;
    return m->check("mlp_predict");
}

int aegpu_mlp_predict(aegpu_mlp *m, const float *X, int n, float *Y)
{
    if (!m || !X || !Y || n < 1) return AEGPU_ERR_ARG;
    float *dx = m->alloc<float>((size_t)n * m->n_in), *dy = m->alloc<float>((size_t)n * m->n_out);
    if (!dx || !dy) {
        m->free_ptr(dx);
        m->free_ptr(dy);
        return m->fail(AEGPU_ERR_NOMEM, "prediction buffers");
    }
    cudaMemcpyAsync(dx, X, (size_t)n * m->n_in * sizeof(float), cudaMemcpyHostToDevice, m->stream);
    int rc = aegpu_mlp_predict_dev(m, dx, n, dy, nullptr);
    if (!rc) {
        cudaMemcpyAsync(Y, dy, (size_t)n * m->n_out * sizeof(float), cudaMemcpyDeviceToHost, m->stream);
        if (cudaStreamSynchronize(m->stream) != cudaSuccess) rc = m->check("mlp_predict");
    }
    m->free_ptr(dx);
    m->free_ptr(dy);
    return rc;
}

// Loss and parameter gradients at the current weights over n rows (host arrays):
// the mean squared error on standardised targets, gradients in the layout of
// aegpu_mlp_get_params.
int aegpu_mlp_loss_grad(aegpu_mlp *m, const float *X, const float *T, int n, float *loss, float *grads)
{
    if (!m || !X || !T || n < 1) return AEGPU_ERR_ARG;
    if (!m->reserve(n)) return m->fail(AEGPU_ERR_NOMEM, "activation allocation failed");
    float *dx = m->alloc<float>((size_t)n * m->n_in), *dt = m->alloc<float>((size_t)n * m->n_out);
    if (!dx || !dt) {
        m->free_ptr(dx);
        m->free_ptr(dt);
        return m->fail(AEGPU_ERR_NOMEM, "loss buffers");
    }
    cudaStream_t s = m->stream;
    cudaMemcpyAsync(dx, X, (size_t)n * m->n_in * sizeof(float), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dt, T, (size_t)n * m->n_out * sizeof(float), cudaMemcpyHostToDevice, s);
    k_standardise<<<256, 256, 0, s>>>(dx, nullptr, n, m->n_in, m->in_mean(), m->in_inv(), m->X0);
    forward(m, n);
    k_mse<<<(n + 7) / 8, 256, 0, s>>>(m->Y, dt, nullptr, n, m->n_out, m->out_mean(), m->out_inv(), m->dY,
                                          m->rowloss);
    backward(m, n);
    std::vector<float> rl(n);
    cudaMemcpyAsync(rl.data(), m->rowloss, n * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (grads) cudaMemcpyAsync(grads, m->g, m->nparams() * sizeof(float), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    int rc = m->check("mlp_loss_grad");
    double L = 0;
    for (float x : rl) L += x;
    if (loss) *loss = (float)(L / ((double)n * m->n_out));
    m->free_ptr(dx);
    m->free_ptr(dt);
    return rc;
}

// Adam training on n rows (host arrays) for `epochs` passes in shuffled minibatches
// of `batch` rows (seeded).  epoch_loss[epochs] (nullable) receives each epoch's
// mean minibatch loss.
int aegpu_mlp_train(aegpu_mlp *m, const float *X, const float *T, int n, int epochs, int batch, float lr,
                    uint64_t seed, float *epoch_loss)
{
    if (!m || !X || !T || n < 1 || epochs < 0 || batch < 1 || !(lr > 0)) return AEGPU_ERR_ARG;
    batch = std::min(batch, n);
    if (!m->reserve(batch)) return m->fail(AEGPU_ERR_NOMEM, "activation allocation failed");
    float *dx = m->alloc<float>((size_t)n * m->n_in), *dt = m->alloc<float>((size_t)n * m->n_out);
    int *didx = m->alloc<int>((size_t)epochs * n + 1);
    float *dloss = m->alloc<float>((size_t)std::max(1, epochs) * ((n + batch - 1) / batch) * batch);
    if (!dx || !dt || !didx || !dloss) {
        m->free_ptr(dx);
        m->free_ptr(dt);
        m->free_ptr(didx);
        m->free_ptr(dloss);
        return m->fail(AEGPU_ERR_NOMEM, "training buffers");
    }
    cudaStream_t s = m->stream;
    cudaMemcpyAsync(dx, X, (size_t)n * m->n_in * sizeof(float), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dt, T, (size_t)n * m->n_out * sizeof(float), cudaMemcpyHostToDevice, s);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const int nbat = (n + batch - 1) / batch;
    // every epoch's permutation (Fisher-Yates on a seeded generator) and every step's
    // Adam bias corrections up front
    std::vector<int> perm((size_t)epochs * n);
    uint64_t rs = seed;
    for (int ep = 0; ep < epochs; ++ep) {
        int *p = perm.data() + (size_t)ep * n;
        for (int i = 0; i < n; ++i) p[i] = i;
        for (int i = n - 1; i > 0; --i) std::swap(p[i], p[(int)(splitmix64(rs) % (uint64_t)(i + 1))]);
    }
    std::vector<float> coef((size_t)2 * nbat * epochs);
    for (size_t k = 0; k < (size_t)nbat * epochs; ++k) {
        const int64_t t = m->adam_t + 1 + (int64_t)k;
        coef[2 * k] = 1.0f - std::pow(b1, (float)t);
        coef[2 * k + 1] = 1.0f - std::pow(b2, (float)t);
    }
    // one epoch's steps are captured once as a CUDA graph over fixed buffers (the
    // epoch's permutation, bias corrections and minibatch losses) and replayed per epoch
    int *ep_idx = m->alloc<int>(n);
    float *dcoef = m->alloc<float>(coef.size() + 2), *ep_coef = m->alloc<float>((size_t)2 * nbat);
    float *ep_loss = m->alloc<float>((size_t)nbat * batch);
    auto release = [&]() {
        for (void *p : {(void *)dx, (void *)dt, (void *)didx, (void *)dloss, (void *)ep_idx, (void *)dcoef,
                        (void *)ep_coef, (void *)ep_loss})
            m->free_ptr(p);
    };
    if (!ep_idx || !dcoef || !ep_coef || !ep_loss) {
        release();
        return m->fail(AEGPU_ERR_NOMEM, "training buffers");
    }
    if (epochs) {
        cudaMemcpyAsync(didx, perm.data(), perm.size() * sizeof(int), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(dcoef, coef.data(), coef.size() * sizeof(float), cudaMemcpyHostToDevice, s);
    }
    const int64_t cnt = m->nparams();
    auto epoch = [&]() {
        for (int bi = 0; bi < nbat; ++bi) {
            const int r0 = bi * batch, rows = std::min(batch, n - r0);
            const int *idx = ep_idx + r0;
            k_standardise<<<256, 256, 0, s>>>(dx, idx, rows, m->n_in, m->in_mean(), m->in_inv(), m->X0);
            forward(m, rows);
            k_mse<<<(rows + 7) / 8, 256, 0, s>>>(m->Y, dt, idx, rows, m->n_out, m->out_mean(), m->out_inv(), m->dY,
                                                     ep_loss + (size_t)bi * batch);
            backward(m, rows);
            // every weight and bias in one launch (the parameters are contiguous); the BF16
            // copies of the biases are written too but never read (biases stay FP32)
            k_adam<<<std::min<int64_t>((cnt + 255) / 256, 1024), 256, 0, s>>>(m->w, m->wq, m->g, m->m, m->v, cnt, lr, b1,
                                                                              b2, eps, ep_coef + 2 * bi);
        }
    };
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int rc = AEGPU_OK;
    if (epochs) {
        if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            rc = m->check("mlp_train capture");
        } else {
            epoch();
            const cudaError_t ce = cudaStreamEndCapture(s, &graph);
            if (ce != cudaSuccess || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess)
                rc = m->check("mlp_train capture");
        }
    }
    for (int ep = 0; ep < epochs && rc == AEGPU_OK; ++ep) {
        cudaMemcpyAsync(ep_idx, didx + (size_t)ep * n, (size_t)n * sizeof(int), cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(ep_coef, dcoef + (size_t)2 * nbat * ep, (size_t)2 * nbat * sizeof(float),
                        cudaMemcpyDeviceToDevice, s);
        if (cudaGraphLaunch(exec, s) != cudaSuccess) rc = m->check("mlp_train graph launch");
        cudaMemcpyAsync(dloss + (size_t)ep * nbat * batch, ep_loss, (size_t)nbat * batch * sizeof(float),
                        cudaMemcpyDeviceToDevice, s);
    }
    m->adam_t += (int64_t)nbat * epochs;
    const int64_t lpos = (int64_t)nbat * batch * epochs;
    if (rc == AEGPU_OK && epoch_loss && epochs) {
        std::vector<float> l(lpos);
        cudaMemcpyAsync(l.data(), dloss, lpos * sizeof(float), cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        for (int ep = 0; ep < epochs; ++ep) {
            double sum = 0;
            for (int bi = 0; bi < nbat; ++bi) {
                const int rows = std::min(batch, n - bi * batch);
                const float *p = l.data() + ((size_t)ep * nbat + bi) * batch;
                double bs = 0;
                for (int r = 0; r < rows; ++r) bs += p[r];
                sum += bs / ((double)rows * m->n_out);
            }
            epoch_loss[ep] = (float)(sum / nbat);
        }
    }
    cudaStreamSynchronize(s);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (rc == AEGPU_OK) rc = m->check("mlp_train");
    release();
    return rc;
}

}  // extern "C"
