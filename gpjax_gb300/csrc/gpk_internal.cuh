// Internal (C++) interfaces between the translation units of libgpk.
#pragma once
#include "gpk_common.cuh"

namespace gpk {

enum Tri { TRI_NONE = 0, TRI_LOWER = 1, TRI_UPPER = 2 };

// One NT GEMM problem: C[i, j] = alpha * sum_c A[i, c] * B[j, c] + beta * C[i, j]
// with A [M, K] and B [N, K] row-major.  A triangular flag zeroes the operand
// outside its triangle element-wise (in the problem's local coordinates), so
// the memory there is never read.  c_lower restricts work and stores to
// i >= j.  Ct (optional) receives the transposed result.  Batches of
// identically shaped problems are described by element strides.
template <typename T>
struct GemmProb {
  const T* A;
  const T* B;
  T* C;
  T* Ct;
  int64_t lda, ldb, ldc, ldct;
  int64_t sA, sB, sC, sCt;  // per-batch element strides
  int M, N, K;
  int a_tri, b_tri, c_lower;
  T alpha, beta;
};

// Block sizes of the SIMT paths (diagonal blocks of the factorisation).
template <typename T> struct Blk;
template <> struct Blk<double> { static constexpr int NB = 64; };
template <> struct Blk<float> { static constexpr int NB = 128; };

template <typename T>
cudaError_t gemm_nt(const GemmProb<T>& p, int batch, cudaStream_t s);

// Lower Cholesky in place (row-major, lda).  logdiag[n] (may be null)
// receives log(L_ii) in float64; info gets the first failing order.
// dtrack (may be null): float64 copy of diag(A) that is kept up to date
// through the factorisation and supplies the pivots, so the diagonal never
// accumulates rounding of the working precision.  zero_upper clears the
// strict upper triangle outside the diagonal blocks first.
template <typename T>
cudaError_t potrf_lower(T* A, int64_t lda, int n, double* logdiag, int* info, double* dtrack,
                        bool zero_upper, cudaStream_t s);

// M = L^-1 (lower, row-major) and V = L^-T (upper, row-major) from the factor L.
// scratch: n*n/2 elements of T.
template <typename T>
cudaError_t trtri_lower(const T* L, int64_t ldl, int n, T* M, int64_t ldm, T* V, int64_t ldv,
                        T* scratch, cudaStream_t s);

// y = op(Tri) x in float64 accumulation, Tri [n, n] row-major;
// lower: y_i = sum_{c<=i} Tri[i,c] x_c ; upper: y_i = sum_{c>=i} Tri[i,c] x_c.
// if accumulate: y += alpha * result, else y = alpha * result.
template <typename T>
cudaError_t gemv_tri(const T* Tri, int64_t ld, int n, bool lower, const double* x, double* y,
                     double alpha, bool accumulate, cudaStream_t s);

// Dense row-major GEMV y[i] = sum_j A[i, j] x[j], float64 accumulation.
template <typename T>
cudaError_t gemv_dense(const T* A, int64_t ld, int rows, int cols, const double* x, double* y,
                       cudaStream_t s);

// xs[i, k] = x[i, k] / l_k as T (row-major, ld = d)
template <typename T>
cudaError_t scale_inputs(const double* x, int64_t ldx, int n, int d, const double* theta, int n_ls,
                         T* xs, cudaStream_t s);

// Gram/cross-covariance from scaled inputs.  mode 0: out = K(xs, ys) full;
// mode 1: lower triangle of (K(xs, xs) + jitter I) + obs_stddev^2 I with zeros
// above the diagonal; mode 2: the same without the noise term.
template <typename T, typename TO>
cudaError_t cross_cov_scaled(int kind, int n, int m, int d, const T* xs, const T* ys,
                             const double* theta, int n_ls, int mode, double diag_add, TO* out,
                             int64_t ldo, cudaStream_t s);

// Fused W = V V^T (lower tiles) + gradient reduction.  gpart receives
// lauum_grad_tiles(n, T) * (d + 2) float64 per-tile partial sums
// [d lengthscale terms, variance term, noise term] of
//   sum_{i>=j} f_ij (alpha_i alpha_j - W_ij) dK_ij,  f = 1 on, 2 off the diagonal,
// with dK/dl_k carried as c1 * ((x_ik - x_jk)/l_k)^2 (unit variance).
template <typename T>
cudaError_t lauum_grad(int kind, const T* V, int64_t ldv, int n, int d, const T* xs,
                       const double* theta, int n_ls, const double* alpha, double* gpart,
                       cudaStream_t s);
template <typename T>
int lauum_grad_tiles(int n);

// r = diff - (K(xs, xs) + (jitter + obs_stddev^2) I) alpha, K regenerated in T,
// float64 accumulation; rpart holds residual_scratch_doubles(n) doubles.
template <typename T>
cudaError_t residual(int kind, int n, int d, const T* xs, const double* theta, int n_ls,
                     double jitter, const double* diff, const double* alpha, double* r,
                     double* rpart, cudaStream_t s);
size_t residual_scratch_doubles(int n);
// Scratch (doubles) of the multi-block MLL finalisation.
size_t mll_finalize_scratch_doubles(int d);

// dtrack[i] = (k(x_i, x_i) + jitter) + obs_stddev^2 in float64.
cudaError_t sigma_diag_init(int kind, int n, const double* theta, int n_ls, double jitter,
                            double* dtrack, cudaStream_t s);

}  // namespace gpk
