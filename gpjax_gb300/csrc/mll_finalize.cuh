// Compensated block reductions and the MLL / gradient assembly from the
// reduced sums, shared by the single-instance finalisation (mll.cu) and the
// persistent batched kernel (batched.cu).
#pragma once
#include <climits>
#include "gpk_common.cuh"

namespace gpk {

template <typename F>
__device__ void block_ksum_pair(int lo, int hi, F f, double& out_sum, double& out_c) {
  __shared__ double s_sum[32], s_c[32];
  double sum = 0.0, c = 0.0;
  for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const double v = f(i);
    const double t = sum + v;
    c += (fabs(sum) >= fabs(v)) ? (sum - t) + v : (v - t) + sum;
    sum = t;
  }
  // combine the (sum, c) pairs: warp then block, compensating each addition
  for (int o = 16; o > 0; o >>= 1) {
    const double os = __shfl_xor_sync(0xffffffffu, sum, o);
    const double oc = __shfl_xor_sync(0xffffffffu, c, o);
    const double t = sum + os;
    c += oc + ((fabs(sum) >= fabs(os)) ? (sum - t) + os : (os - t) + sum);
    sum = t;
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) {
    s_sum[w] = sum;
    s_c[w] = c;
  }
  __syncthreads();
  double tot = 0.0, tc = 0.0;
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    for (int k = 0; k < nw; ++k) {
      const double v = s_sum[k];
      const double t = tot + v;
      tc += s_c[k] + ((fabs(tot) >= fabs(v)) ? (tot - t) + v : (v - t) + tot);
      tot = t;
    }
  }
  __syncthreads();
  out_sum = tot;
  out_c = tc;
}

template <typename F>
__device__ double block_ksum(int n, F f) {
  double s, c;
  block_ksum_pair(0, n, f, s, c);
  return s + c;  // valid on thread 0
}

// MLL and gradient from the reduced sums (thread 0).
__device__ inline void finalize_outputs(int n, int d, const double* __restrict__ theta, int n_ls,
                                 double jitter, double logdet, double quad, double asum,
                                 const double* sg, int want_grad, int* __restrict__ info,
                                 double* __restrict__ out_mll, double* __restrict__ out_grad) {
  int inf = *info;
  if (inf == INT_MAX) inf = 0;
  *info = inf;
  const double nan = __longlong_as_double(0x7ff8000000000000ULL);
  const double mll = -0.5 * ((double)n * log(2.0 * 3.141592653589793) + logdet + quad);
  *out_mll = inf ? nan : mll;
  if (!want_grad) return;
  const double s2 = theta[n_ls];
  const double sd = theta[n_ls + 1];
  if (n_ls == 1) {
    double a = 0.0;
    for (int k = 0; k < d; ++k) a += sg[k];
    out_grad[0] = inf ? nan : 0.5 * s2 * a / theta[0];
  } else {
    for (int k = 0; k < d; ++k) out_grad[k] = inf ? nan : 0.5 * s2 * sg[k] / theta[k];
  }
  // d/d variance: 1/2 sum (alpha alpha^T - W) o K / s2.  With Sigma = K + s I
  // (s = jitter + obs_stddev^2), W = Sigma^-1 and Sigma alpha = diff this is
  // exactly 1/2 (diff^T alpha - n - s (alpha^T alpha - tr W)) / s2, which needs
  // only the refined alpha and the noise sum instead of n^2 cancelling terms.
  const double snoise = jitter + sd * sd;
  const double gvar = (s2 > 0.0) ? 0.5 * (quad - (double)n - snoise * sg[d + 1]) / s2
                                 : 0.5 * sg[d];
  out_grad[n_ls] = inf ? nan : gvar;
  out_grad[n_ls + 1] = inf ? nan : sd * sg[d + 1];
  out_grad[n_ls + 2] = inf ? nan : asum;
}

}  // namespace gpk
