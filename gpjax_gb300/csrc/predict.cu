// ConjugatePosterior.predict (gpjax/gps.py:443-526):
//   Sigma = (K(x, x) + I*jitter) + I*obs_stddev^2 = L L^T
//   mean  = m(t) + (L^-1 Kxt)^T L^-1 (y - m(x))
//   cov   = K(t, t) - (L^-1 Kxt)^T (L^-1 Kxt) + I*prior_jitter
// Q^T = Ktx M^T is one NT GEMM against the triangular inverse M = L^-1; the
// mean is formed as Ktx alpha with the same refined alpha as the marginal
// likelihood, the variance as k(t, t) - |Q^T row|^2 + prior_jitter, and the
// full covariance only when requested (the reference always forms it).
#include <algorithm>
#include <climits>
#include "gpk_internal.cuh"

namespace gpk {

// mixed_tc.cu: mean and variance on the tensor-core factorisation
bool mll_tc_supported(int d);
size_t predict_tc_workspace_bytes(int64_t n, int64_t t, int d);
gpk_status predict_run_tc(int kind, int n, int t, int d, const double* x, int64_t ldx,
                          const double* y, const double* xt, int64_t ldxt, const double* theta,
                          int n_ls, double jitter, double prior_jitter, double* mean, double* var,
                          int* info, void* ws, cudaStream_t s);

namespace {

struct Arena {
  char* base;
  size_t off = 0;
  explicit Arena(void* b) : base(static_cast<char*>(b)) {}
  template <typename U>
  U* take(size_t count) {
    off = (off + 255) & ~size_t(255);
    U* p = base ? reinterpret_cast<U*>(base + off) : nullptr;
    off += count * sizeof(U);
    return p;
  }
};

inline int64_t pad_ld(int64_t n) { return ((n + 63) / 64) * 64; }

template <typename T>
struct PredBuffers {
  int64_t ld, ldt;
  T *A, *M, *V, *scratch, *xs, *ts, *Ktx, *QT, *QQ;
  double *tsd, *diff, *z, *alpha, *r, *rpart, *logdiag, *dtrack;
};

template <typename T>
size_t pred_layout(int64_t n, int64_t t, int d, bool want_cov, void* ws, PredBuffers<T>& b) {
  Arena a(ws);
  b.ld = pad_ld(n);
  b.ldt = pad_ld(t);
  b.A = a.take<T>((size_t)n * b.ld);
  b.M = a.take<T>((size_t)n * b.ld);
  b.V = a.take<T>((size_t)n * b.ld);
  b.scratch = a.take<T>((size_t)n * n / 2 + 64);
  b.xs = a.take<T>((size_t)n * d);
  b.ts = a.take<T>((size_t)t * d);
  b.Ktx = a.take<T>((size_t)t * b.ld);
  b.QT = a.take<T>((size_t)t * b.ld);
  b.QQ = want_cov ? a.take<T>((size_t)t * b.ldt) : nullptr;
  b.tsd = a.take<double>((size_t)t * d);
  b.diff = a.take<double>(n);
  b.z = a.take<double>(n);
  b.alpha = a.take<double>(n);
  b.r = a.take<double>(n);
  b.logdiag = a.take<double>(n);
  b.dtrack = a.take<double>(n);
  b.rpart = a.take<double>(residual_scratch_doubles((int)n));
  return a.off + 256;
}

__global__ void pred_init_kernel(int* info) { *info = INT_MAX; }

__global__ void pred_diff_kernel(int n, const double* __restrict__ y,
                                 const double* __restrict__ theta, int n_ls,
                                 double* __restrict__ diff) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) diff[i] = y[i] - theta[n_ls + 2];
}

// mean_a = c + (Ktx alpha)_a ; var_a = k(t_a, t_a) - |QT_a|^2 + prior_jitter
template <typename T>
__global__ void pred_mean_var_kernel(int n, int t, const T* __restrict__ Ktx,
                                     const T* __restrict__ QT, int64_t ld,
                                     const double* __restrict__ alpha,
                                     const double* __restrict__ theta, int n_ls, int kind,
                                     double prior_jitter, const int* __restrict__ info,
                                     double* __restrict__ mean, double* __restrict__ var) {
  const int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (a >= t) return;
  double sm = 0.0, sq = 0.0;
  const T* kr = Ktx + (int64_t)a * ld;
  const T* qr = QT + (int64_t)a * ld;
  for (int i = lane; i < n; i += 32) {
    sm += (double)kr[i] * alpha[i];
    const double q = (double)qr[i];
    sq += q * q;
  }
  sm = warp_sum(sm);
  sq = warp_sum(sq);
  if (lane == 0) {
    const double nan = __longlong_as_double(0x7ff8000000000000ULL);
    const bool bad = *info != 0 && *info != INT_MAX;
    const double kaa = kval<double>(kind, 0.0, theta[n_ls], kshape<double>(kind, theta, n_ls));
    mean[a] = bad ? nan : theta[n_ls + 2] + sm;
    var[a] = bad ? nan : (kaa - sq) + prior_jitter;
  }
}

// cov = K(t, t) - QQ (lower tile product mirrored) + prior_jitter I, float64 out
template <typename T>
__global__ void pred_cov_kernel(int t, int d, int kind, const double* __restrict__ tsd,
                                const T* __restrict__ QQ, int64_t ldq,
                                const double* __restrict__ theta, int n_ls, double prior_jitter,
                                const int* __restrict__ info, double* __restrict__ cov,
                                int64_t ldc) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)t * t) return;
  const int a = (int)(e / t), b = (int)(e % t);
  const int hi = a > b ? a : b, lo = a > b ? b : a;
  double sq = 0.0;
  for (int k = 0; k < d; ++k) {
    const double df = tsd[(int64_t)a * d + k] - tsd[(int64_t)b * d + k];
    sq = fma(df, df, sq);
  }
  const double kab = kval<double>(kind, sq, theta[n_ls], kshape<double>(kind, theta, n_ls));
  double v = kab - (double)QQ[(int64_t)hi * ldq + lo];
  if (a == b) v += prior_jitter;
  const bool bad = *info != 0 && *info != INT_MAX;
  cov[(int64_t)a * ldc + b] = bad ? __longlong_as_double(0x7ff8000000000000ULL) : v;
}

__global__ void pred_finish_info(int* info) {
  if (*info == INT_MAX) *info = 0;
}

template <typename T>
gpk_status predict_run(int kind, int n, int t, int d, const double* x, int64_t ldx,
                       const double* y, const double* xt, int64_t ldxt, const double* theta,
                       int n_ls, double jitter, double prior_jitter, int refine, double* mean,
                       double* var, double* cov, int64_t ldcov, int* info, void* ws,
                       cudaStream_t s) {
  PredBuffers<T> b;
  pred_layout<T>(n, t, d, cov != nullptr, ws, b);
  pred_init_kernel<<<1, 1, 0, s>>>(info);
  GPK_LAUNCH_CHECK();
  GPK_CUDA_TRY(scale_inputs<T>(x, ldx, n, d, theta, n_ls, b.xs, s));
  GPK_CUDA_TRY(scale_inputs<T>(xt, ldxt, t, d, theta, n_ls, b.ts, s));
  GPK_CUDA_TRY(scale_inputs<double>(xt, ldxt, t, d, theta, n_ls, b.tsd, s));
  pred_diff_kernel<<<(int)cdiv(n, 256), 256, 0, s>>>(n, y, theta, n_ls, b.diff);
  GPK_LAUNCH_CHECK();
  GPK_CUDA_TRY(cross_cov_scaled<T, T>(kind, n, n, d, b.xs, b.xs, theta, n_ls, 1, jitter, b.A,
                                      b.ld, s));
  GPK_CUDA_TRY(sigma_diag_init(kind, n, theta, n_ls, jitter, b.dtrack, s));
  GPK_CUDA_TRY(potrf_lower<T>(b.A, b.ld, n, b.logdiag, info, b.dtrack, false, s));
  GPK_CUDA_TRY(trtri_lower<T>(b.A, b.ld, n, b.M, b.ld, b.V, b.ld, b.scratch, s));
  GPK_CUDA_TRY(gemv_tri<T>(b.M, b.ld, n, true, b.diff, b.z, 1.0, false, s));
  GPK_CUDA_TRY(gemv_tri<T>(b.V, b.ld, n, false, b.z, b.alpha, 1.0, false, s));
  for (int it = 0; it < refine; ++it) {
    GPK_CUDA_TRY(residual<T>(kind, n, d, b.xs, theta, n_ls, jitter, b.diff, b.alpha, b.r, b.rpart,
                             s));
    GPK_CUDA_TRY(gemv_tri<T>(b.M, b.ld, n, true, b.r, b.z, 1.0, false, s));
    GPK_CUDA_TRY(gemv_tri<T>(b.V, b.ld, n, false, b.z, b.alpha, 1.0, true, s));
  }
  GPK_CUDA_TRY(cross_cov_scaled<T, T>(kind, t, n, d, b.ts, b.xs, theta, n_ls, 0, 0.0, b.Ktx,
                                      b.ld, s));
  GemmProb<T> p{};  // QT[a, i] = sum_c Ktx[a, c] M[i, c]
  p.A = b.Ktx;
  p.lda = b.ld;
  p.M = t;
  p.B = b.M;
  p.ldb = b.ld;
  p.b_tri = TRI_LOWER;
  p.N = n;
  p.K = n;
  p.C = b.QT;
  p.ldc = b.ld;
  p.alpha = T(1);
  p.beta = T(0);
  GPK_CUDA_TRY(gemm_nt<T>(p, 1, s));
  pred_mean_var_kernel<T><<<(int)cdiv((int64_t)t * 32, 256), 256, 0, s>>>(
      n, t, b.Ktx, b.QT, b.ld, b.alpha, theta, n_ls, kind, prior_jitter, info, mean, var);
  GPK_LAUNCH_CHECK();
  if (cov) {
    GemmProb<T> q{};  // QQ = QT QT^T (lower)
    q.A = b.QT;
    q.lda = b.ld;
    q.B = b.QT;
    q.ldb = b.ld;
    q.M = t;
    q.N = t;
    q.K = n;
    q.c_lower = 1;
    q.C = b.QQ;
    q.ldc = b.ldt;
    q.alpha = T(1);
    q.beta = T(0);
    GPK_CUDA_TRY(gemm_nt<T>(q, 1, s));
    pred_cov_kernel<T><<<(int)cdiv((int64_t)t * t, 256), 256, 0, s>>>(
        t, d, kind, b.tsd, b.QQ, b.ldt, theta, n_ls, prior_jitter, info, cov, ldcov);
    GPK_LAUNCH_CHECK();
  }
  pred_finish_info<<<1, 1, 0, s>>>(info);
  GPK_LAUNCH_CHECK();
  return GPK_OK;
}

}  // namespace
}  // namespace gpk

using namespace gpk;

extern "C" size_t gpk_predict_workspace_bytes(int64_t n, int64_t t, int d, int precision) {
  if (n <= 0 || t <= 0 || d <= 0) return 256;
  if (precision == GPK_PREC_FP64) {
    PredBuffers<double> b;
    return pred_layout<double>(n, t, d, true, nullptr, b);
  }
  PredBuffers<float> b;
  const size_t simt = pred_layout<float>(n, t, d, true, nullptr, b);
  // mean and variance only: the tensor-core factorisation and Q^T product
  return mll_tc_supported(d) ? std::max(simt, predict_tc_workspace_bytes(n, t, d)) : simt;
}

extern "C" gpk_status gpk_predict(int kind, int64_t n, int64_t t, int d, const double* x,
                                  int64_t ldx, const double* y, const double* xt, int64_t ldxt,
                                  const double* theta, int n_ls, double jitter,
                                  double prior_jitter, int precision, double* mean, double* var,
                                  double* cov, int64_t ldcov, int* info, void* workspace,
                                  size_t workspace_bytes, cudaStream_t stream) {
  if (kind < GPK_RBF || kind > GPK_RATIONAL_QUADRATIC) return GPK_ERR_BAD_ARG;
  if (n <= 0 || t < 0 || n > (1 << 20) || t > (1 << 20)) return GPK_ERR_BAD_ARG;
  if (d <= 0 || d > GPK_MAX_D || ldx < d || ldxt < d || !(n_ls == 1 || n_ls == d))
    return GPK_ERR_BAD_ARG;
  if (precision != GPK_PREC_FP64 && precision != GPK_PREC_MIXED) return GPK_ERR_BAD_ARG;
  if (t == 0) return GPK_OK;
  if (!x || !y || !xt || !theta || !mean || !var || !info || !workspace) return GPK_ERR_BAD_ARG;
  if (cov && ldcov < t) return GPK_ERR_BAD_ARG;
  if (workspace_bytes < gpk_predict_workspace_bytes(n, t, d, precision)) return GPK_ERR_WORKSPACE;
  if (precision == GPK_PREC_FP64)
    return predict_run<double>(kind, (int)n, (int)t, d, x, ldx, y, xt, ldxt, theta, n_ls, jitter,
                               prior_jitter, 1, mean, var, cov, ldcov, info, workspace, stream);
  if (!cov && mll_tc_supported(d))
    return predict_run_tc(kind, (int)n, (int)t, d, x, ldx, y, xt, ldxt, theta, n_ls, jitter,
                          prior_jitter, mean, var, info, workspace, stream);
  return predict_run<float>(kind, (int)n, (int)t, d, x, ldx, y, xt, ldxt, theta, n_ls, jitter,
                            prior_jitter, 2, mean, var, cov, ldcov, info, workspace, stream);
}
