// Dense FP64 contractions of the Hessian and properties passes: an upper-triangle Gram
// matrix over very long columns, transposed and plain matrix-vector products against
// a column basis, and dot products.  All hand-written for sm_103a on the FP64 pipe.
//
// On GB300 the FP64 pipe issues about 2 DFMA per SM per clock (0.63 T DFMA/s measured),
// so these kernels are bound by the number of DFMAs they issue, not by HBM: the Gram
// kernel issues exactly one DFMA per (i <= j) pair per row, rounded up to 4 x 4
// micro-tiles, instead of the full 64 x 64 tiles of a blocked GEMM.
//
// Determinism: every sum is split into per-CTA partial sums over fixed row ranges and
// finished by one fixed-order pass, so a repeated call is bit-identical.
#include "dense.h"

#include "../../include/aegpu.h"

#include <algorithm>

namespace ae {
namespace {

constexpr int kGramPanel = 64;    // columns per panel: 16 micro-tiles of 4
constexpr int kGramThreads = 256;
constexpr int kGramSlab = 32;     // doubles of every column staged per step (32 real / 16 complex rows)
constexpr int kGemvThreads = 256;
constexpr int kGemvGroup = 8;     // columns reduced together by gemv_t

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Panel pair p (enumerated column by column over the upper triangle) -> (I, J), I <= J.
__device__ __forceinline__ void pair_of(int p, int &I, int &J)
{
    J = 0;
    while ((J + 1) * (J + 2) / 2 <= p) ++J;
    I = p - J * (J + 1) / 2;
}

// Partial Gram sums of one panel pair over one chunk of rows.
// grid.x = panel pair, grid.y = row chunk.  Thread t owns a 4 x 4 micro-tile (ib, jb):
// on a diagonal pair the 136 micro-tiles with ib <= jb, on an off-diagonal pair all
// 256.  A slab of kGramSlab doubles of each of the pair's 2 x 64 columns is staged in
// shared memory (row-major, padded rows); the next slab is loaded into registers while
// the current one is multiplied.
template <int W>
__global__ void __launch_bounds__(kGramThreads) k_gram(const double *__restrict__ A, int64_t lda,
                                                      const double *__restrict__ B, int64_t ldb, int64_t nrows, int V,
                                                      int npairs, int64_t slabs_per_chunk, double *__restrict__ partial)
{
    constexpr int LD = W * (kGramPanel + 1);   // padded smem row (doubles)
    constexpr int RS = kGramSlab / W;          // rows per slab
    constexpr int PER = kGramPanel * kGramSlab / kGramThreads;  // doubles each thread stages per matrix
    __shared__ double As[RS * LD], Bs[RS * LD];
    const int t = threadIdx.x;
    int I, J;
    pair_of(blockIdx.x, I, J);
    const int c0 = I * kGramPanel, c1 = J * kGramPanel;
    int ib, jb;
    bool act;
    if (I == J) {
        jb = 0;
        while ((jb + 1) * (jb + 2) / 2 <= t) ++jb;
        ib = t - jb * (jb + 1) / 2;
        act = t < 136;
    } else {
        ib = t & 15;
        jb = t >> 4;
        act = true;
    }
    act = act && c0 + ib * 4 < V && c1 + jb * 4 < V;
    const int64_t nel = nrows * W;               // doubles per column
    const int64_t nslabs = (nel + kGramSlab - 1) / kGramSlab;
    const int64_t s0 = (int64_t)blockIdx.y * slabs_per_chunk;
    const int64_t s1 = s0 + slabs_per_chunk < nslabs ? s0 + slabs_per_chunk : nslabs;

    double pa[PER], pb[PER];
    auto load = [&](int64_t slab) {
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int idx = t + q * kGramThreads, c = idx / kGramSlab, o = idx % kGramSlab;
            const int64_t e = slab * kGramSlab + o;
            pa[q] = (c0 + c < V && e < nel) ? A[(int64_t)(c0 + c) * lda + e] : 0.0;
            pb[q] = (c1 + c < V && e < nel) ? B[(int64_t)(c1 + c) * ldb + e] : 0.0;
        }
    };
    double acc[16 * W];
#pragma unroll
    for (int k = 0; k < 16 * W; ++k) acc[k] = 0.0;
    if (s0 < s1) load(s0);
    for (int64_t slab = s0; slab < s1; ++slab) {
        __syncthreads();
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int idx = t + q * kGramThreads, c = idx / kGramSlab, o = idx % kGramSlab;
            As[(o / W) * LD + c * W + (o % W)] = pa[q];
            Bs[(o / W) * LD + c * W + (o % W)] = pb[q];
        }
        __syncthreads();
        if (slab + 1 < s1) load(slab + 1);
        if (!act) continue;
#pragma unroll 4
        for (int r = 0; r < RS; ++r) {
            const double *ar = As + r * LD + ib * 4 * W, *br = Bs + r * LD + jb * 4 * W;
            double a[4 * W], b[4 * W];
#pragma unroll
            for (int k = 0; k < 4 * W; ++k) {
                a[k] = ar[k];
                b[k] = br[k];
            }
            if (W == 1) {
#pragma unroll
                for (int x = 0; x < 4; ++x)
#pragma unroll
                    for (int y = 0; y < 4; ++y) acc[x * 4 + y] = fma(a[x], b[y], acc[x * 4 + y]);
            } else {
                // Re(conj(a) b) = ar br + ai bi, Im(conj(a) b) = ar bi - ai br
#pragma unroll
                for (int x = 0; x < 4; ++x)
#pragma unroll
                    for (int y = 0; y < 4; ++y) {
                        const double xr = a[2 * x], xi = a[2 * x + 1], yr = b[2 * y], yi = b[2 * y + 1];
                        acc[x * 4 + y] = fma(xi, yi, fma(xr, yr, acc[x * 4 + y]));
                        acc[16 + x * 4 + y] = fma(-xi, yr, fma(xr, yi, acc[16 + x * 4 + y]));
                    }
            }
        }
    }
    if (!act) return;
    double *out = partial + ((int64_t)blockIdx.y * npairs + blockIdx.x) * W * kGramPanel * kGramPanel;
#pragma unroll
    for (int w = 0; w < W; ++w)
#pragma unroll
        for (int x = 0; x < 4; ++x)
#pragma unroll
            for (int y = 0; y < 4; ++y)
                out[w * kGramPanel * kGramPanel + (ib * 4 + x) + (jb * 4 + y) * kGramPanel] = acc[w * 16 + x * 4 + y];
}

// C[i + j ldc] = alpha * sum over chunks (fixed order) of the partials, i <= j < V.
__global__ void k_gram_finish(const double *__restrict__ partial, int nchunks, int npairs, int V, int W, double alpha,
                              double *__restrict__ Cre, double *__restrict__ Cim, int ldc)
{
    constexpr int PP = kGramPanel * kGramPanel;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)npairs * W * PP) return;
    const int p = (int)(idx / (W * PP)), rem = (int)(idx % (W * PP)), w = rem / PP, e = rem % PP;
    int I, J;
    pair_of(p, I, J);
    const int i = I * kGramPanel + e % kGramPanel, j = J * kGramPanel + e / kGramPanel;
    if (j >= V || i > j) return;
    double s = 0.0;
    for (int c = 0; c < nchunks; ++c) s += partial[((int64_t)c * npairs + p) * W * PP + (int64_t)w * PP + e];
    (w ? Cim : Cre)[i + (int64_t)j * ldc] = alpha * s;
}

struct GramShape {
    int npairs, nchunks;
    int64_t slabs_per_chunk;
};

GramShape gram_shape(int V, int W, int64_t nrows, int sm_count)
{
    const int np = (V + kGramPanel - 1) / kGramPanel;
    GramShape g;
    g.npairs = np * (np + 1) / 2;
    const int64_t nslabs = std::max<int64_t>(1, (nrows * W + kGramSlab - 1) / kGramSlab);
    // about 4 CTAs per SM over all pairs (at least one chunk per pair)
    const int64_t want = std::max<int64_t>(1, (int64_t)sm_count * 4 / g.npairs);
    g.slabs_per_chunk = (nslabs + std::min(nslabs, want) - 1) / std::min(nslabs, want);
    g.nchunks = (int)((nslabs + g.slabs_per_chunk - 1) / g.slabs_per_chunk);
    return g;
}

// Partial sums of y = A^T x: CTA (b, g) covers rows [b * rows_per, (b + 1) * rows_per)
// of the eight columns of group g = blockIdx.y and writes partial[b * k + j] for them.
// Each thread walks its rows with a stride of the CTA size, so a CTA streams a long
// contiguous stretch of every column (the loads of several rows are in flight per
// thread), and the eight sums meet in one block reduction at the end.
__global__ void __launch_bounds__(kGemvThreads) k_gemv_t(const double *__restrict__ A, int64_t lda, int64_t n, int k,
                                                         const double *__restrict__ x, int64_t rows_per,
                                                         double *__restrict__ partial, const int *flag)
{
    if (flag && !*flag) return;
    __shared__ double red[kGemvGroup][kGemvThreads / 32];
    const int64_t r0 = (int64_t)blockIdx.x * rows_per, r1 = r0 + rows_per < n ? r0 + rows_per : n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j0 = blockIdx.y * kGemvGroup;
    const int nj = k - j0 < kGemvGroup ? k - j0 : kGemvGroup;
    double acc[kGemvGroup];
#pragma unroll
    for (int q = 0; q < kGemvGroup; ++q) acc[q] = 0.0;
    const double *Aj = A + (int64_t)j0 * lda;
#pragma unroll 2
    for (int64_t r = r0 + threadIdx.x; r < r1; r += kGemvThreads) {
        const double xr = x[r];
#pragma unroll
        for (int q = 0; q < kGemvGroup; ++q)
            if (q < nj) acc[q] = fma(Aj[r + (int64_t)q * lda], xr, acc[q]);
    }
#pragma unroll
    for (int q = 0; q < kGemvGroup; ++q) {
        const double v = warp_sum(acc[q]);
        if (lane == 0) red[q][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < nj) {
        double s = 0.0;
        for (int w = 0; w < kGemvThreads / 32; ++w) s += red[threadIdx.x][w];
        partial[(int64_t)blockIdx.x * k + j0 + threadIdx.x] = s;
    }
}

// y[j] = alpha * sum of the m chunks' partials: one warp per column, lane l adding the
// partials l, l + 32, ... and the lanes combined by a fixed butterfly.
__global__ void k_gemv_t_finish(const double *__restrict__ partial, int m, int k, double alpha, double *__restrict__ y,
                                const int *flag)
{
    if (flag && !*flag) return;
    const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (j >= k) return;
    double s = 0.0;
    for (int b = lane; b < m; b += 32) s += partial[(int64_t)b * k + j];
    s = warp_sum(s);
    if (lane == 0) y[j] = alpha * s;
}

// y[r] = beta y[r] + alpha sum_j A[r + j lda] c[j]; the coefficients are staged in
// shared memory, two accumulators (even / odd j) per row.
__global__ void __launch_bounds__(kGemvThreads) k_gemv_n(const double *__restrict__ A, int64_t lda, int64_t n, int k,
                                                         const double *__restrict__ c, double alpha, double beta,
                                                         double *__restrict__ y, const int *flag)
{
    if (flag && !*flag) return;
    extern __shared__ double cs[];
    for (int j = threadIdx.x; j < k; j += blockDim.x) cs[j] = c[j];
    __syncthreads();
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        double s0 = 0.0, s1 = 0.0;
        int j = 0;
        for (; j + 1 < k; j += 2) {
            s0 = fma(A[r + (int64_t)j * lda], cs[j], s0);
            s1 = fma(A[r + (int64_t)(j + 1) * lda], cs[j + 1], s1);
        }
        if (j < k) s0 = fma(A[r + (int64_t)j * lda], cs[j], s0);
        const double v = alpha * (s0 + s1);
        y[r] = beta == 0.0 ? v : fma(beta, y[r], v);
    }
}

__device__ __forceinline__ double block_sum(double v, double *red)
{
    v = warp_sum(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
    return s;
}

// Per-CTA partial sums of sum_r a[r inc] b[r inc] (grid-stride share of the CTA).
__global__ void k_dot_part(const double *__restrict__ a, const double *__restrict__ b, int64_t n, int64_t inc,
                           double *__restrict__ part, const int *flag_in)
{
    __shared__ double red[32];
    if (flag_in && !*flag_in) return;
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s = fma(a[i * inc], b[i * inc], s);
    s = block_sum(s, red);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// *out = sum of m partials (or its square root).  With `coef` (k values), also
// *flag = (*out < f * sqrt(*out^2 + sum coef^2)): after w -= V c with orthonormal V,
// the norm before the subtraction is sqrt(|w|^2 + |c|^2).
__global__ void k_dot_fin(const double *__restrict__ part, int m, double *out, int take_sqrt, const double *coef,
                          int k, double f, int *flag, const int *flag_in)
{
    __shared__ double red[32];
    if (flag_in && !*flag_in) return;
    double s = 0.0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) s += part[i];
    s = block_sum(s, red);
    double c2 = 0.0;
    if (flag) {
        for (int i = threadIdx.x; i < k; i += blockDim.x) c2 = fma(coef[i], coef[i], c2);
        c2 = block_sum(c2, red);
    }
    if (threadIdx.x == 0) {
        const double v = take_sqrt ? sqrt(fmax(s, 0.0)) : s;
        *out = v;
        if (flag) *flag = v < f * sqrt(v * v + c2);
    }
}

// Per-CTA partial sums of sum_r conj(a_r) b_r (complex, interleaved): part[2 b], part[2 b + 1].
__global__ void k_dotc_part(const double *__restrict__ a, const double *__restrict__ b, int64_t n,
                            double *__restrict__ part)
{
    __shared__ double red[32];
    double re = 0.0, im = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 x = reinterpret_cast<const double2 *>(a)[i], y = reinterpret_cast<const double2 *>(b)[i];
        re = fma(x.y, y.y, fma(x.x, y.x, re));
        im = fma(-x.y, y.x, fma(x.x, y.y, im));
    }
    re = block_sum(re, red);
    im = block_sum(im, red);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = re;
        part[2 * blockIdx.x + 1] = im;
    }
}

__global__ void k_dotc_fin(const double *__restrict__ part, int m, double *out)
{
    __shared__ double red[32];
    double re = 0.0, im = 0.0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        re += part[2 * i];
        im += part[2 * i + 1];
    }
    re = block_sum(re, red);
    im = block_sum(im, red);
    if (threadIdx.x == 0) {
        out[0] = re;
        out[1] = im;
    }
}

__global__ void k_axpby(double *__restrict__ y, const double *__restrict__ x, int64_t n, double alpha, double beta,
                        const double *inv)
{
    const double f = inv ? (*inv > 1e-300 ? 1.0 / *inv : 0.0) : 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (inv)
            y[i] *= f;
        else if (alpha == 0.0)
            y[i] = beta * x[i];
        else
            y[i] = beta == 0.0 ? alpha * y[i] : fma(beta, x[i], alpha * y[i]);
    }
}

int vec_grid(int64_t n, int sm_count)
{
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sm_count * 8));
}

}  // namespace

int64_t gram_scratch_doubles(int V, int W, int64_t nrows, int sm_count)
{
    const GramShape g = gram_shape(V, W, nrows, sm_count);
    return (int64_t)g.nchunks * g.npairs * W * kGramPanel * kGramPanel;
}

int gram_upper(const double *A, int64_t lda, const double *B, int64_t ldb, int64_t nrows, int W, int V, double alpha,
               double *Cre, double *Cim, int ldc, double *scratch, int sm_count, cudaStream_t s)
{
    if (V < 1) return 0;
    const GramShape g = gram_shape(V, W, nrows, sm_count);
    const dim3 grid(g.npairs, g.nchunks);
    if (W == 1)
        k_gram<1><<<grid, kGramThreads, 0, s>>>(A, lda, B, ldb, nrows, V, g.npairs, g.slabs_per_chunk, scratch);
    else
        k_gram<2><<<grid, kGramThreads, 0, s>>>(A, lda, B, ldb, nrows, V, g.npairs, g.slabs_per_chunk, scratch);
    const int64_t nout = (int64_t)g.npairs * W * kGramPanel * kGramPanel;
    k_gram_finish<<<(int)((nout + 255) / 256), 256, 0, s>>>(scratch, g.nchunks, g.npairs, V, W, alpha, Cre, Cim, ldc);
    return 2;
}

int64_t gemv_scratch_doubles(int k, int sm_count) { return (int64_t)sm_count * 8 * std::max(k, 2); }

int gemv_t(const double *A, int64_t lda, int64_t n, int k, const double *x, double alpha, double *y, double *scratch,
           int sm_count, cudaStream_t s, const int *flag)
{
    if (k < 1) return 0;
    // about 8 CTAs per SM over all column groups, each chunk at least 8 rows per thread
    const int groups = (k + kGemvGroup - 1) / kGemvGroup;
    const int m = (int)std::max<int64_t>(1, std::min<int64_t>(std::max<int64_t>(1, (int64_t)sm_count * 8 / groups),
                                                              (n + 8 * kGemvThreads - 1) / (8 * kGemvThreads)));
    const int64_t rows_per = (n + m - 1) / m;
    k_gemv_t<<<dim3(m, groups), kGemvThreads, 0, s>>>(A, lda, n, k, x, rows_per, scratch, flag);
    k_gemv_t_finish<<<(k + 7) / 8, 256, 0, s>>>(scratch, m, k, alpha, y, flag);
    return 2;
}

int gemv_n(const double *A, int64_t lda, int64_t n, int k, const double *c, double alpha, double beta, double *y,
           cudaStream_t s, const int *flag)
{
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((n + kGemvThreads - 1) / kGemvThreads, 152 * 8));
    k_gemv_n<<<grid, kGemvThreads, (size_t)std::max(k, 1) * sizeof(double), s>>>(A, lda, n, k, c, alpha, beta, y, flag);
    return 1;
}

int dot(const double *a, const double *b, int64_t n, int64_t inc, double *out, int take_sqrt, double *scratch,
        int sm_count, cudaStream_t s, const double *coef, int ncoef, double cmp_factor, int *flag, const int *flag_in)
{
    const int m = vec_grid(n, sm_count);
    k_dot_part<<<m, 256, 0, s>>>(a, b, n, inc, scratch, flag_in);
    k_dot_fin<<<1, 256, 0, s>>>(scratch, m, out, take_sqrt, coef, ncoef, cmp_factor, flag, flag_in);
    return 2;
}

int dotc(const double *a, const double *b, int64_t n, double *out, double *scratch, int sm_count, cudaStream_t s)
{
    const int m = vec_grid(n, sm_count);
    k_dotc_part<<<m, 256, 0, s>>>(a, b, n, scratch);
    k_dotc_fin<<<1, 256, 0, s>>>(scratch, m, out);
    return 2;
}

int axpby(double *y, const double *x, int64_t n, double alpha, double beta, const double *inv, cudaStream_t s)
{
    k_axpby<<<vec_grid(n, 152), 256, 0, s>>>(y, x, n, alpha, beta, inv);
    return 1;
}

}  // namespace ae

extern "C" int aegpu_gram_upper_dev(const double *A, int64_t lda, const double *B, int64_t ldb, int64_t nrows, int W, int V,
                                    double alpha, double *Cre, double *Cim, int ldc, void *stream)
{
    if (!A || !B || !Cre || nrows < 0 || (W != 1 && W != 2) || (W == 2 && !Cim) || V < 1 || ldc < V ||
        lda < nrows * W || ldb < nrows * W)
        return AEGPU_ERR_ARG;
    int dev = 0, sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return AEGPU_ERR_CUDA;
    }
    cudaStream_t s = (cudaStream_t)stream;
    double *scratch = nullptr;
    if (cudaMallocAsync(&scratch, (size_t)ae::gram_scratch_doubles(V, W, nrows, sm) * sizeof(double), s) != cudaSuccess) {
        cudaGetLastError();
        return AEGPU_ERR_NOMEM;
    }
    ae::gram_upper(A, lda, B, ldb, nrows, W, V, alpha, Cre, Cim, ldc, scratch, sm, s);
    cudaFreeAsync(scratch, s);
    return cudaGetLastError() == cudaSuccess ? AEGPU_OK : AEGPU_ERR_CUDA;
}
