// Gram and cross-covariance tiles generated from the inputs.
//
// Reference: DenseKernelComputation._cross_covariance builds
// K[i, j] = k(x_i, y_j) with a vmap of a vmap over the pointwise kernel
// (gpjax/kernels/computations/dense.py:32-36); gram() is cross_covariance(x, x)
// (computations/base.py:56-72).  Each pointwise kernel divides both inputs by
// the lengthscale before taking the squared distance
// (kernels/stationary/rbf.py:41-43, matern32.py:46-47, matern52.py:45-46).
// Here the inputs are scaled once (xs = x / l), then each CTA stages a
// 64-row panel of each side in shared memory and every thread produces a
// column strip of the output tile.
#include "gpk_internal.cuh"

namespace gpk {

template <typename T>
__global__ void scale_inputs_kernel(const double* __restrict__ x, int64_t ldx, int n, int d,
                                    const double* __restrict__ theta, int n_ls, T* __restrict__ xs) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)n * d) return;
  const int i = (int)(e / d), k = (int)(e % d);
  const double l = theta[n_ls == 1 ? 0 : k];
  xs[e] = (T)(x[(int64_t)i * ldx + k] / l);
}

template <typename T>
cudaError_t scale_inputs(const double* x, int64_t ldx, int n, int d, const double* theta, int n_ls,
                         T* xs, cudaStream_t s) {
  const int64_t total = (int64_t)n * d;
  if (total == 0) return cudaSuccess;
  scale_inputs_kernel<T><<<(int)cdiv(total, 256), 256, 0, s>>>(x, ldx, n, d, theta, n_ls, xs);
  return launch_status();
}

constexpr int GT = 64;  // output tile edge

template <typename T, typename TO>
__global__ void __launch_bounds__(256)
    cross_cov_kernel(int kind, int n, int m, int d, const T* __restrict__ xs,
                     const T* __restrict__ ys, const double* __restrict__ theta, int n_ls, int mode,
                     double jitter, TO* __restrict__ out, int64_t ldo) {
  __shared__ T sx[GT][GPK_MAX_D + 1];
  __shared__ T sy[GT][GPK_MAX_D + 1];
  const int i0 = blockIdx.y * GT, j0 = blockIdx.x * GT;
  const T s2 = (T)theta[n_ls];
  const double sd = theta[n_ls + 1];
  if (mode >= 1 && j0 > i0 + GT - 1) {
    // strictly-upper tile of the factorisation input: zeros
    for (int e = threadIdx.x; e < GT * GT; e += blockDim.x) {
      int r = e / GT, c = e % GT;
      if (i0 + r < n && j0 + c < m) out[(int64_t)(i0 + r) * ldo + j0 + c] = TO(0);
    }
    return;
  }
  for (int e = threadIdx.x; e < GT * d; e += blockDim.x) {
    int r = e / d, k = e % d;
    sx[r][k] = (i0 + r < n) ? xs[(int64_t)(i0 + r) * d + k] : T(0);
    sy[r][k] = (j0 + r < m) ? ys[(int64_t)(j0 + r) * d + k] : T(0);
  }
  __syncthreads();
  const int c = threadIdx.x % GT;
  const int rbase = threadIdx.x / GT;  // 0..3
  const int gj = j0 + c;
  if (gj >= m) return;
  T yv[GPK_MAX_D];
#pragma unroll
  for (int k = 0; k < GPK_MAX_D; ++k) yv[k] = (k < d) ? sy[c][k] : T(0);
  for (int r = rbase; r < GT; r += 4) {
    const int gi = i0 + r;
    if (gi >= n) break;
    TO v;
    if (mode >= 1 && gj > gi) {
      v = TO(0);
    } else {
      T sq = T(0);
#pragma unroll
      for (int k = 0; k < GPK_MAX_D; ++k) {
        if (k < d) {
          T df = sx[r][k] - yv[k];
          sq = fma(df, df, sq);
        }
      }
      T kv = kval<T>(kind, sq, s2, kshape<T>(kind, theta, n_ls));
      if (mode == 1 && gi == gj) {
        // (K + I*jitter) + I*obs_stddev^2 (objectives.py:100-103)
        double dv = ((double)kv + jitter) + sd * sd;
        v = (TO)dv;
      } else if (mode == 2 && gi == gj) {
        v = (TO)((double)kv + jitter);  // K + I*jitter (objectives.py:353-354)
      } else {
        v = (TO)kv;
      }
    }
    out[(int64_t)gi * ldo + gj] = v;
  }
}

template <typename T, typename TO>
cudaError_t cross_cov_scaled(int kind, int n, int m, int d, const T* xs, const T* ys,
                             const double* theta, int n_ls, int mode, double jitter, TO* out,
                             int64_t ldo, cudaStream_t s) {
  if (n <= 0 || m <= 0) return cudaSuccess;
  if (d > GPK_MAX_D) return cudaErrorInvalidValue;
  dim3 grid((unsigned)cdiv(m, GT), (unsigned)cdiv(n, GT));
  cross_cov_kernel<T, TO><<<grid, 256, 0, s>>>(kind, n, m, d, xs, ys, theta, n_ls, mode, jitter,
                                               out, ldo);
  return launch_status();
}

__global__ void sigma_diag_kernel(int kind, int n, const double* __restrict__ theta, int n_ls,
                                  double jitter, double* __restrict__ dtrack) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double sd = theta[n_ls + 1];
  dtrack[i] = (kval<double>(kind, 0.0, theta[n_ls], kshape<double>(kind, theta, n_ls)) + jitter) + sd * sd;
}

cudaError_t sigma_diag_init(int kind, int n, const double* theta, int n_ls, double jitter,
                            double* dtrack, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  sigma_diag_kernel<<<(int)cdiv(n, 256), 256, 0, s>>>(kind, n, theta, n_ls, jitter, dtrack);
  return launch_status();
}

template cudaError_t scale_inputs<double>(const double*, int64_t, int, int, const double*, int,
                                          double*, cudaStream_t);
template cudaError_t scale_inputs<float>(const double*, int64_t, int, int, const double*, int,
                                         float*, cudaStream_t);
template cudaError_t cross_cov_scaled<double, double>(int, int, int, int, const double*,
                                                      const double*, const double*, int, int,
                                                      double, double*, int64_t, cudaStream_t);
template cudaError_t cross_cov_scaled<float, float>(int, int, int, int, const float*, const float*,
                                                    const double*, int, int, double, float*,
                                                    int64_t, cudaStream_t);

}  // namespace gpk

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using namespace gpk;

// The public Gram / cross-covariance calls take no workspace: each output
// element scales its two input rows by the lengthscales on the fly, exactly
// as the reference's pointwise kernels do.
template <typename T>
__global__ void cross_cov_raw_kernel(int kind, int n, int m, int d, const double* __restrict__ x,
                                     int64_t ldx, const double* __restrict__ y, int64_t ldy,
                                     const double* __restrict__ theta, int n_ls, int diag_only,
                                     T* __restrict__ out, int64_t ldo) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t total = diag_only ? (int64_t)n : (int64_t)n * m;
  if (e >= total) return;
  const int i = diag_only ? (int)e : (int)(e / m);
  const int j = diag_only ? (int)e : (int)(e % m);
  T sq = T(0);
  for (int k = 0; k < d; ++k) {
    const double l = theta[n_ls == 1 ? 0 : k];
    T df = (T)(x[(int64_t)i * ldx + k] / l) - (T)(y[(int64_t)j * ldy + k] / l);
    sq = fma(df, df, sq);
  }
  T v = kval<T>(kind, sq, (T)theta[n_ls], kshape<T>(kind, theta, n_ls));
  if (diag_only)
    out[i] = v;
  else
    out[(int64_t)i * ldo + j] = v;
}

static bool valid_common(int kind, int64_t n, int d, int n_ls) {
  if (kind < GPK_RBF || kind > GPK_RATIONAL_QUADRATIC) return false;
  if (n < 0 || d <= 0 || d > GPK_MAX_D) return false;
  if (!(n_ls == 1 || n_ls == d)) return false;
  if (n > (int64_t)1 << 30) return false;
  return true;
}

extern "C" gpk_status gpk_cross_covariance(int kind, int64_t n, int64_t m, int d, const double* x,
                                           int64_t ldx, const double* y, int64_t ldy,
                                           const double* theta, int n_ls, int out_dtype, void* out,
                                           int64_t ldo, cudaStream_t stream) {
  if (!valid_common(kind, n, d, n_ls) || m < 0 || ldx < d || ldy < d || ldo < m)
    return GPK_ERR_BAD_ARG;
  if (n == 0 || m == 0) return GPK_OK;
  if (!x || !y || !theta || !out) return GPK_ERR_BAD_ARG;
  const int64_t total = n * m;
  const int blocks = (int)cdiv(total, 256);
  if (out_dtype == GPK_F64)
    cross_cov_raw_kernel<double><<<blocks, 256, 0, stream>>>(kind, (int)n, (int)m, d, x, ldx, y,
                                                             ldy, theta, n_ls, 0, (double*)out, ldo);
  else if (out_dtype == GPK_F32)
    cross_cov_raw_kernel<float><<<blocks, 256, 0, stream>>>(kind, (int)n, (int)m, d, x, ldx, y, ldy,
                                                            theta, n_ls, 0, (float*)out, ldo);
  else
    return GPK_ERR_BAD_ARG;
  GPK_LAUNCH_CHECK();
  return GPK_OK;
}

extern "C" gpk_status gpk_gram(int kind, int64_t n, int d, const double* x, int64_t ldx,
                               const double* theta, int n_ls, int out_dtype, void* out,
                               int64_t ldo, cudaStream_t stream) {
  return gpk_cross_covariance(kind, n, n, d, x, ldx, x, ldx, theta, n_ls, out_dtype, out, ldo,
                              stream);
}

extern "C" gpk_status gpk_diagonal(int kind, int64_t n, int d, const double* x, int64_t ldx,
                                   const double* theta, int n_ls, double* out,
                                   cudaStream_t stream) {
  if (!valid_common(kind, n, d, n_ls) || ldx < d) return GPK_ERR_BAD_ARG;
  if (n == 0) return GPK_OK;
  if (!x || !theta || !out) return GPK_ERR_BAD_ARG;
  cross_cov_raw_kernel<double><<<(int)cdiv(n, 256), 256, 0, stream>>>(
      kind, (int)n, (int)n, d, x, ldx, x, ldx, theta, n_ls, 1, out, 1);
  GPK_LAUNCH_CHECK();
  return GPK_OK;
}

// ---------------------------------------------------------------------------
// Cotangent of the cross-covariance: given G = dL/dK for K = K(x, y),
//   d theta: sum_ij G_ij dK_ij/dl_k, sum_ij G_ij dK_ij/d variance
//   d x_i = sum_j G_ij dk(x_i, y_j)/dx_i,  d y_j = sum_i G_ij dk(x_i, y_j)/dy_j
// (the reverse-mode derivative of DenseKernelComputation.cross_covariance,
// gpjax/kernels/computations/dense.py:32-36).  One block per row (theta and
// d x partials) and one per column (d y); partials summed in a fixed order.
// ---------------------------------------------------------------------------
namespace gpk {
namespace {

constexpr int VJP_DMAX = GPK_MAX_D;

__global__ void __launch_bounds__(256)
    vjp_rows_kernel(int kind, int n, int m, int d, const double* __restrict__ x, int64_t ldx,
                    const double* __restrict__ y, int64_t ldy, const double* __restrict__ theta,
                    int n_ls, const double* __restrict__ G, int64_t ldg, int by_col,
                    double* __restrict__ parts) {
  // by_col == 0: block = row i of G, loop over columns; by_col == 1: block = column j
  const int r = blockIdx.x;
  const int nr = by_col ? m : n, nc = by_col ? n : m;
  if (r >= nr) return;
  __shared__ double red[8][2 * VJP_DMAX + 1];
  double pr[VJP_DMAX];
  for (int k = 0; k < d; ++k) {
    const double l = theta[n_ls == 1 ? 0 : k];
    pr[k] = by_col ? y[(int64_t)r * ldy + k] / l : x[(int64_t)r * ldx + k] / l;
  }
  double al[VJP_DMAX], az[VJP_DMAX], av = 0.0;
  for (int k = 0; k < d; ++k) al[k] = az[k] = 0.0;
  for (int c = threadIdx.x; c < nc; c += blockDim.x) {
    const double g = by_col ? G[(int64_t)c * ldg + r] : G[(int64_t)r * ldg + c];
    double df[VJP_DMAX], sq = 0.0;
    for (int k = 0; k < d; ++k) {
      const double l = theta[n_ls == 1 ? 0 : k];
      const double o = by_col ? x[(int64_t)c * ldx + k] / l : y[(int64_t)c * ldy + k] / l;
      df[k] = by_col ? (o - pr[k]) : (pr[k] - o);  // always (x_i - y_j) / l
      sq += df[k] * df[k];
    }
    double k1, c1;
    kval_dcoef<double>(kind, sq, 1.0, k1, c1, kshape<double>(kind, theta, n_ls));
    av += g * k1;
    for (int k = 0; k < d; ++k) {
      al[k] += g * c1 * df[k] * df[k];
      az[k] += g * c1 * df[k];
    }
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  for (int k = 0; k < 2 * d + 1; ++k) {
    double v = (k < d) ? al[k] : (k < 2 * d ? az[k - d] : av);
    v = warp_sum(v);
    if (l == 0) red[w][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < 2 * d + 1) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red[q][threadIdx.x];
    parts[(int64_t)r * (2 * d + 1) + threadIdx.x] = t;
  }
}

__global__ void vjp_finalize_kernel(int n, int m, int d, const double* __restrict__ theta,
                                    int n_ls, const double* __restrict__ rparts,
                                    const double* __restrict__ cparts,
                                    double* __restrict__ gtheta, double* __restrict__ gx,
                                    double* __restrict__ gy) {
  const double s2 = theta[n_ls];
  const int tid = threadIdx.x;
  // theta: one thread per slot, rows summed in order
  if (tid <= d) {
    double t = 0.0;
    const int slot = tid < d ? tid : 2 * d;
    for (int i = 0; i < n; ++i) t += rparts[(int64_t)i * (2 * d + 1) + slot];
    if (tid < d) {
      if (n_ls == 1) {
        // summed below by thread 0 after a barrier
      } else {
        gtheta[tid] = s2 * t / theta[tid];
      }
    } else {
      gtheta[n_ls] = t;
    }
    if (n_ls == 1 && tid < d) gtheta[n_ls + 3 + tid] = t;  // scratch slots past the output
  }
  __syncthreads();
  if (n_ls == 1 && tid == 0) {
    double a = 0.0;
    for (int k = 0; k < d; ++k) a += gtheta[n_ls + 3 + k];
    gtheta[0] = s2 * a / theta[0];
  }
  if (tid == 0) {
    gtheta[n_ls + 1] = 0.0;
    gtheta[n_ls + 2] = 0.0;
  }
  for (int e = tid; gx && e < n * d; e += blockDim.x) {
    const int i = e / d, k = e % d;
    gx[e] = -s2 * rparts[(int64_t)i * (2 * d + 1) + d + k] / theta[n_ls == 1 ? 0 : k];
  }
  for (int e = tid; gy && e < m * d; e += blockDim.x) {
    const int j = e / d, k = e % d;
    gy[e] = s2 * cparts[(int64_t)j * (2 * d + 1) + d + k] / theta[n_ls == 1 ? 0 : k];
  }
}

}  // namespace
}  // namespace gpk

extern "C" size_t gpk_cross_covariance_vjp_workspace_bytes(int64_t n, int64_t m, int d) {
  if (n < 0 || m < 0 || d <= 0) return 256;
  return (size_t)(n + m) * (2 * d + 1) * sizeof(double) + (size_t)(d + 8) * sizeof(double) + 512;
}

extern "C" gpk_status gpk_cross_covariance_vjp(int kind, int64_t n, int64_t m, int d,
                                               const double* x, int64_t ldx, const double* y,
                                               int64_t ldy, const double* theta, int n_ls,
                                               const double* G, int64_t ldg, double* grad_theta,
                                               double* grad_x, double* grad_y, void* workspace,
                                               size_t workspace_bytes, cudaStream_t stream) {
  if (!valid_common(kind, n, d, n_ls) || m < 0 || m > (int64_t)1 << 30 || ldx < d || ldy < d ||
      ldg < m)
    return GPK_ERR_BAD_ARG;
  if (!theta || !grad_theta || !workspace) return GPK_ERR_BAD_ARG;
  if (workspace_bytes < gpk_cross_covariance_vjp_workspace_bytes(n, m, d)) return GPK_ERR_WORKSPACE;
  if ((n > 0 && m > 0) && (!x || !y || !G)) return GPK_ERR_BAD_ARG;
  double* rparts = static_cast<double*>(workspace);
  double* cparts = rparts + (size_t)n * (2 * d + 1);
  // grad_theta needs d scratch slots past its n_ls + 3 outputs in the isotropic
  // case: they live in the workspace tail and are copied back by the kernel
  double* gth = (n_ls == 1) ? cparts + (size_t)m * (2 * d + 1) : grad_theta;
  if (n > 0 && m > 0) {
    vjp_rows_kernel<<<(int)n, 256, 0, stream>>>(kind, (int)n, (int)m, d, x, ldx, y, ldy, theta,
                                                n_ls, G, ldg, 0, rparts);
    GPK_LAUNCH_CHECK();
    if (grad_y) {
      vjp_rows_kernel<<<(int)m, 256, 0, stream>>>(kind, (int)n, (int)m, d, x, ldx, y, ldy, theta,
                                                  n_ls, G, ldg, 1, cparts);
      GPK_LAUNCH_CHECK();
    }
  }
  vjp_finalize_kernel<<<1, 256, 0, stream>>>((int)n, (int)m, d, theta, n_ls, rparts, cparts, gth,
                                             grad_x, grad_y);
  GPK_LAUNCH_CHECK();
  if (gth != grad_theta) GPK_CUDA_TRY(cudaMemcpyAsync(grad_theta, gth, (size_t)(n_ls + 3) * 8,
                                                      cudaMemcpyDeviceToDevice, stream));
  return GPK_OK;
}
