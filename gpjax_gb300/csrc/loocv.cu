// Leave-one-out predictive log-probability of a conjugate GP and its gradient.
//
// Reference: conjugate_loocv (gpjax/objectives.py:110-178):
//   Sigma = K + (obs_var + jitter) I, alpha = Sigma^-1 (y - m), W = Sigma^-1,
//   mu_i = y_i - alpha_i / W_ii, sigma_i^2 = 1 / W_ii,
//   loocv = sum_i log N(y_i; mu_i, sigma_i^2)
//         = sum_i [-1/2 log 2pi + 1/2 log W_ii - 1/2 alpha_i^2 / W_ii].
// The reference differentiates through jnp.linalg.inv; here the cotangent of
// Sigma is formed in closed form.  With a_i = 1/(2 W_ii) + alpha_i^2 / (2 W_ii^2),
// b_i = alpha_i / W_ii and u = W b,
//   d loocv = sum_kl G_kl dSigma_kl,  G = -W diag(a) W + (u alpha^T + alpha u^T) / 2,
//   d loocv / d mean = sum_i u_i,
// so the kernel-hyperparameter gradient is the cross-covariance VJP of G and the
// noise gradient 2 obs_stddev tr(G).  Everything is float64: Sigma's Cholesky
// factor, its triangular inverse, W = L^-T L^-1 and W diag(a) W as SIMT GEMMs,
// alpha refined once against a float64 residual.
#include <climits>
#include "gpk_internal.cuh"

extern "C" size_t gpk_cross_covariance_vjp_workspace_bytes(int64_t n, int64_t m, int d);
extern "C" gpk_status gpk_cross_covariance_vjp(int kind, int64_t n, int64_t m, int d,
                                               const double* x, int64_t ldx, const double* y,
                                               int64_t ldy, const double* theta, int n_ls,
                                               const double* G, int64_t ldg, double* grad_theta,
                                               double* grad_x, double* grad_y, void* workspace,
                                               size_t workspace_bytes, cudaStream_t stream);

namespace gpk {
namespace {

struct LoocvBuffers {
  int64_t ld;
  double *A, *M, *V, *W, *scratch, *xs;
  double *diff, *z, *alpha, *r, *logdiag, *dtrack, *rpart, *a, *sa, *b, *u, *red, *gth;
  void* vjp_ws;
  size_t vjp_bytes;
};

size_t loocv_layout(int64_t n, int d, void* ws, LoocvBuffers& b) {
  char* base = static_cast<char*>(ws);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    off = (off + 255) & ~size_t(255);
    char* p = base ? base + off : nullptr;
    off += bytes;
    return p;
  };
  b.ld = ((n + 63) / 64) * 64;
  const size_t nn = (size_t)n * b.ld * 8;
  b.A = (double*)take(nn);  // Sigma, its factor, later the cotangent G
  b.M = (double*)take(nn);  // L^-1, later P = W diag(sqrt a)
  b.V = (double*)take(nn);  // L^-T
  b.W = (double*)take(nn);  // Sigma^-1
  b.scratch = (double*)take(((size_t)n * n / 2 + 64) * 8);
  b.xs = (double*)take((size_t)n * d * 8);
  double** vecs[] = {&b.diff, &b.z, &b.alpha, &b.r, &b.logdiag, &b.dtrack, &b.a, &b.sa, &b.b, &b.u};
  for (double** v : vecs) *v = (double*)take((size_t)n * 8);
  b.rpart = (double*)take(residual_scratch_doubles((int)n) * 8);
  b.red = (double*)take(8 * 8);
  b.gth = (double*)take((size_t)(GPK_MAX_D + 8) * 8);
  b.vjp_bytes = gpk_cross_covariance_vjp_workspace_bytes(n, n, d);
  b.vjp_ws = take(b.vjp_bytes);
  return off + 256;
}

__global__ void loocv_init_kernel(int* info, double* red) {
  *info = INT_MAX;
  for (int k = 0; k < 8; ++k) red[k] = 0.0;
}

__global__ void loocv_diff_kernel(int n, const double* __restrict__ y,
                                  const double* __restrict__ theta, int n_ls,
                                  double* __restrict__ diff) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) diff[i] = y[i] - theta[n_ls + 2];
}

// Per point: a_i, sqrt(a_i), b_i and the summed log-probabilities (red[0]).
__global__ void loocv_point_kernel(int n, const double* __restrict__ W, int64_t ldw,
                                   const double* __restrict__ alpha, double* __restrict__ a,
                                   double* __restrict__ sa, double* __restrict__ b,
                                   double* __restrict__ red) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double term = 0.0;
  if (i < n) {
    const double w = W[(int64_t)i * ldw + i], al = alpha[i];
    const double ai = 0.5 / w + 0.5 * al * al / (w * w);
    a[i] = ai;
    sa[i] = sqrt(ai);
    b[i] = al / w;
    term = -0.5 * log(2.0 * 3.141592653589793) + 0.5 * log(w) - 0.5 * al * al / w;
  }
  block_atomic_add(&red[0], term);
}

// P[i, j] = W[i, j] sqrt(a_j)
__global__ void loocv_scale_cols_kernel(int n, const double* __restrict__ W, int64_t ld,
                                        const double* __restrict__ sa, double* __restrict__ P) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)n * n) return;
  const int i = (int)(e / n), j = (int)(e % n);
  P[(int64_t)i * ld + j] = W[(int64_t)i * ld + j] * sa[j];
}

// G = -(P P^T, lower triangle in G) + (u alpha^T + alpha u^T) / 2, made
// symmetric; red[1] += tr(G), red[2] += sum u
__global__ void loocv_cotangent_kernel(int n, double* __restrict__ G, int64_t ld,
                                       const double* __restrict__ u,
                                       const double* __restrict__ alpha,
                                       double* __restrict__ red) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double tr = 0.0, us = 0.0;
  if (e < (int64_t)n * n) {
    const int i = (int)(e / n), j = (int)(e % n);
    if (j <= i) {
      const double g = -G[(int64_t)i * ld + j] + 0.5 * (u[i] * alpha[j] + alpha[i] * u[j]);
      G[(int64_t)i * ld + j] = g;
      if (i == j) {
        tr = g;
        us = u[i];
      }
    }
  }
  block_atomic_add(&red[1], tr);
  block_atomic_add(&red[2], us);
}

__global__ void loocv_mirror_kernel(int n, double* __restrict__ G, int64_t ld) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)n * n) return;
  const int i = (int)(e / n), j = (int)(e % n);
  if (j > i) G[(int64_t)i * ld + j] = G[(int64_t)j * ld + i];
}

__global__ void loocv_finalize_kernel(int n_ls, const double* __restrict__ theta,
                                      const double* __restrict__ red,
                                      const double* __restrict__ gth, int want_grad,
                                      int* __restrict__ info, double* __restrict__ out,
                                      double* __restrict__ out_grad) {
  int inf = *info;
  if (inf == INT_MAX) inf = 0;
  *info = inf;
  const double nan = __longlong_as_double(0x7ff8000000000000ULL);
  *out = inf ? nan : red[0];
  if (!want_grad) return;
  for (int k = 0; k <= n_ls; ++k) out_grad[k] = inf ? nan : gth[k];  // lengthscales, variance
  out_grad[n_ls + 1] = inf ? nan : 2.0 * theta[n_ls + 1] * red[1];  // obs_stddev
  out_grad[n_ls + 2] = inf ? nan : red[2];                          // constant mean
}

}  // namespace
}  // namespace gpk

using namespace gpk;

extern "C" size_t gpk_conjugate_loocv_workspace_bytes(int64_t n, int d) {
  if (n < 0 || d < 1 || d > GPK_MAX_D) return 0;
  LoocvBuffers b;
  return loocv_layout(n, d, nullptr, b);
}

extern "C" gpk_status gpk_conjugate_loocv(int kind, int64_t n, int d, const double* x,
                                          int64_t ldx, const double* y, const double* theta,
                                          int n_ls, double jitter, int want_grad,
                                          double* out_loocv, double* out_grad, int* info,
                                          void* workspace, size_t workspace_bytes,
                                          cudaStream_t s) {
  if (kind < GPK_RBF || kind > GPK_RATIONAL_QUADRATIC) return GPK_ERR_BAD_ARG;
  if (n < 1 || n > (1 << 16) || d < 1 || d > GPK_MAX_D || ldx < d) return GPK_ERR_BAD_ARG;
  if (n_ls != 1 && n_ls != d) return GPK_ERR_BAD_ARG;
  if (!x || !y || !theta || !out_loocv || !info || (want_grad && !out_grad) || !workspace)
    return GPK_ERR_BAD_ARG;
  if (workspace_bytes < gpk_conjugate_loocv_workspace_bytes(n, d)) return GPK_ERR_WORKSPACE;
  const int nn = (int)n;
  LoocvBuffers b;
  loocv_layout(n, d, workspace, b);
  const int64_t ld = b.ld;
  const int g1 = (int)cdiv(nn, 256), g2 = (int)cdiv((int64_t)nn * nn, 256);
  loocv_init_kernel<<<1, 1, 0, s>>>(info, b.red);
  GPK_LAUNCH_CHECK();
  GPK_CUDA_TRY(scale_inputs<double>(x, ldx, nn, d, theta, n_ls, b.xs, s));
  loocv_diff_kernel<<<g1, 256, 0, s>>>(nn, y, theta, n_ls, b.diff);
  GPK_LAUNCH_CHECK();
  // Sigma = K + (jitter + obs_stddev^2) I (objectives.py:160-165), its factor and inverse
  GPK_CUDA_TRY(cross_cov_scaled<double, double>(kind, nn, nn, d, b.xs, b.xs, theta, n_ls, 1,
                                                jitter, b.A, ld, s));
  GPK_CUDA_TRY(sigma_diag_init(kind, nn, theta, n_ls, jitter, b.dtrack, s));
  GPK_CUDA_TRY(potrf_lower<double>(b.A, ld, nn, b.logdiag, info, b.dtrack, false, s));
  GPK_CUDA_TRY(trtri_lower<double>(b.A, ld, nn, b.M, ld, b.V, ld, b.scratch, s));
  // alpha = Sigma^-1 (y - m) (objectives.py:167), refined once
  GPK_CUDA_TRY(gemv_tri<double>(b.M, ld, nn, true, b.diff, b.z, 1.0, false, s));
  GPK_CUDA_TRY(gemv_tri<double>(b.V, ld, nn, false, b.z, b.alpha, 1.0, false, s));
  GPK_CUDA_TRY(residual<double>(kind, nn, d, b.xs, theta, n_ls, jitter, b.diff, b.alpha, b.r,
                                b.rpart, s));
  GPK_CUDA_TRY(gemv_tri<double>(b.M, ld, nn, true, b.r, b.z, 1.0, false, s));
  GPK_CUDA_TRY(gemv_tri<double>(b.V, ld, nn, false, b.z, b.alpha, 1.0, true, s));
  // W = Sigma^-1 = L^-T L^-1 = V V^T (objectives.py:168)
  {
    GemmProb<double> p{};
    p.A = b.V;
    p.B = b.V;
    p.C = b.W;
    p.lda = p.ldb = p.ldc = ld;
    p.M = p.N = p.K = nn;
    p.a_tri = p.b_tri = TRI_UPPER;
    p.alpha = 1.0;
    p.beta = 0.0;
    GPK_CUDA_TRY(gemm_nt<double>(p, 1, s));
  }
  loocv_point_kernel<<<g1, 256, 0, s>>>(nn, b.W, ld, b.alpha, b.a, b.sa, b.b, b.red);
  GPK_LAUNCH_CHECK();
  if (want_grad) {
    GPK_CUDA_TRY(gemv_dense<double>(b.W, ld, nn, nn, b.b, b.u, s));  // u = W b
    loocv_scale_cols_kernel<<<g2, 256, 0, s>>>(nn, b.W, ld, b.sa, b.M);
    GPK_LAUNCH_CHECK();
    GemmProb<double> p{};  // lower triangle of P P^T = W diag(a) W into A
    p.A = b.M;
    p.B = b.M;
    p.C = b.A;
    p.lda = p.ldb = p.ldc = ld;
    p.M = p.N = p.K = nn;
    p.c_lower = 1;
    p.alpha = 1.0;
    p.beta = 0.0;
    GPK_CUDA_TRY(gemm_nt<double>(p, 1, s));
    loocv_cotangent_kernel<<<g2, 256, 0, s>>>(nn, b.A, ld, b.u, b.alpha, b.red);
    GPK_LAUNCH_CHECK();
    loocv_mirror_kernel<<<g2, 256, 0, s>>>(nn, b.A, ld);
    GPK_LAUNCH_CHECK();
    const gpk_status st = gpk_cross_covariance_vjp(kind, n, n, d, x, ldx, x, ldx, theta, n_ls,
                                                   b.A, ld, b.gth, nullptr, nullptr, b.vjp_ws,
                                                   b.vjp_bytes, s);
    if (st != GPK_OK) return st;
  }
  loocv_finalize_kernel<<<1, 1, 0, s>>>(n_ls, theta, b.red, b.gth, want_grad, info, out_loocv,
                                        out_grad);
  GPK_LAUNCH_CHECK();
  return GPK_OK;
}
