// Dense FP64 contractions of the Hessian and properties passes (device side).
//
// Replaces the library BLAS calls those passes used to make: the Gram matrices
// 2 T_C^T (H T_C) and T_C^T T_C of the Hessian (fusedevolve.cpp:2633-2650,
// tupsquantities.cpp:386-389), the projected row <proj|T_C> (fusedevolve.cpp:
// 3053-3062), the subspace matrices <psi_i|H|psi_j>, <psi_i|psi_j> (tupsquantities.cpp:
// 1600-1700), and the Lanczos basis products of the lowest-eigenpair search.
// Every routine enqueues kernels on `s` and reduces in a fixed order (per-CTA partial
// sums, then one fixed-order pass), so repeated calls give bit-identical results.
// Vectors are "rows" of W doubles (W = 1 real, 2 complex re/im interleaved); matrices
// are column-major with column c at A + c * lda (lda in doubles).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ae {

// Scratch (doubles) that gram_upper needs for V columns over nrows rows of W doubles.
int64_t gram_scratch_doubles(int V, int W, int64_t nrows, int sm_count);
// Upper triangle (i <= j < V) of C = alpha * A^H B: Cre[i + j * ldc] = alpha * Re sum_r
// conj(A[r][i]) B[r][j], and for W = 2 Cim likewise with the imaginary part (Cim may be
// null for W = 1).  Entries below the diagonal are not written.  Returns launches.
int gram_upper(const double *A, int64_t lda, const double *B, int64_t ldb, int64_t nrows, int W, int V, double alpha,
               double *Cre, double *Cim, int ldc, double *scratch, int sm_count, cudaStream_t s);

// Scratch (doubles) of gemv_t / dot for k columns.
int64_t gemv_scratch_doubles(int k, int sm_count);
// y[j] = alpha * sum_{r < n} A[r + j * lda] x[r] for j < k (real entries).  When `flag`
// is non-null the kernels do nothing unless *flag != 0 (conditional second pass).
int gemv_t(const double *A, int64_t lda, int64_t n, int k, const double *x, double alpha, double *y, double *scratch,
           int sm_count, cudaStream_t s, const int *flag = nullptr);
// y[r] = beta * y[r] + alpha * sum_{j < k} A[r + j * lda] c[j] for r < n (c on the device).
int gemv_n(const double *A, int64_t lda, int64_t n, int k, const double *c, double alpha, double beta, double *y,
           cudaStream_t s, const int *flag = nullptr);
// *out = sum_r a[r * inc] b[r * inc] over n terms (or its square root when take_sqrt).
// With `flag` (nullable), also *flag = (result < cmp_factor * sqrt(result^2 + sum of the
// ncoef squares of coef)).  With `flag_in` (nullable), nothing happens unless *flag_in != 0.
int dot(const double *a, const double *b, int64_t n, int64_t inc, double *out, int take_sqrt, double *scratch,
        int sm_count, cudaStream_t s, const double *coef = nullptr, int ncoef = 0, double cmp_factor = 0.0,
        int *flag = nullptr, const int *flag_in = nullptr);
// out[0] + i out[1] = sum_r conj(a_r) b_r over n complex entries (re, im interleaved).
int dotc(const double *a, const double *b, int64_t n, double *out, double *scratch, int sm_count, cudaStream_t s);
// y[r] = alpha * y[r] + beta * x[r] (alpha = 0: y = beta * x, whatever y held); with
// `inv` non-null, y[r] = y[r] / *inv (0 when *inv vanishes).
int axpby(double *y, const double *x, int64_t n, double alpha, double beta, const double *inv, cudaStream_t s);

}  // namespace ae
