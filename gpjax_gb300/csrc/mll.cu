// Exact-GP marginal log-likelihood with its adjoint, plus the dense
// linear-algebra entry points of the C ABI.
//
// Reference op sequence (gpjax/objectives.py:93-107):
//   obs_noise = obs_stddev^2 ; mx = constant
//   Sigma = (K(x, x) + I*jitter) + I*obs_noise
//   mll = -1/2 (n log 2pi + logdet(Sigma) + diff^T solve(Sigma, diff))
// where logdet and solve are two LU factorisations (linalg/operations.py:
// 111,164).  Here one Cholesky factor L serves both: log|Sigma| = 2 sum log L_ii
// and alpha = Sigma^-1 diff = V (M diff) with M = L^-1, V = M^T, refined
// against residuals accumulated in float64.  The gradient is the fused
// inverse-product/kernel-derivative reduction of adjoint.cu.
#include "mll_finalize.cuh"
#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <mutex>
#include <vector>
#include "gpk_internal.cuh"

namespace gpk {

static std::atomic<long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

// Optional phase events (benchmark instrumentation), see gpk_set_profile_events.
static cudaEvent_t g_prof_events[8];
static int g_prof_count = 0;
void prof_mark(int k, cudaStream_t s) {
  if (k < g_prof_count && g_prof_events[k]) cudaEventRecord(g_prof_events[k], s);
}

// mixed_tc.cu
size_t mll_tc_workspace_bytes(int64_t n, int d);
bool mll_tc_supported(int d);
struct TcPredict;
gpk_status mll_run_tc(int kind, int n, int d, const double* x, int64_t ldx, const double* y,
                      const double* theta, int n_ls, double jitter, int refine, int want_grad,
                      double* out_mll, double* out_grad, int* info, void* ws, cudaStream_t s,
                      const TcPredict* pred = nullptr);

// Carves caller-provided workspace into 256-byte aligned regions.
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
struct MllBuffers {
  int64_t ld;
  T *A, *M, *V, *scratch, *xs;
  double *diff, *z, *alpha, *r, *logdiag, *rpart, *gpart, *dtrack, *fin;
};

template <typename T>
static size_t mll_layout(int64_t n, int d, void* ws, MllBuffers<T>& b) {
  Arena a(ws);
  b.ld = pad_ld(n);
  const size_t nn = (size_t)n * b.ld;
  b.A = a.take<T>(nn);
  b.M = a.take<T>(nn);
  b.V = a.take<T>(nn);
  b.scratch = a.take<T>((size_t)n * n / 2 + 64);
  b.xs = a.take<T>((size_t)n * d);
  b.diff = a.take<double>(n);
  b.z = a.take<double>(n);
  b.alpha = a.take<double>(n);
  b.r = a.take<double>(n);
  b.logdiag = a.take<double>(n);
  b.dtrack = a.take<double>(n);
  b.rpart = a.take<double>(residual_scratch_doubles((int)n));
  b.gpart = a.take<double>((size_t)lauum_grad_tiles<T>((int)n) * (d + 2));
  b.fin = a.take<double>(mll_finalize_scratch_doubles(d));
  return a.off + 256;
}

__global__ void init_info_kernel(int* info) { *info = INT_MAX; }

__global__ void diff_kernel(int n, const double* __restrict__ y, const double* __restrict__ theta,
                            int n_ls, double* __restrict__ diff) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) diff[i] = y[i] - theta[n_ls + 2];
}

__global__ void axpy_kernel(int n, const double* __restrict__ x, double* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] += x[i];
}

// Neumaier-compensated block sum of f(i) over lo <= i < hi (one block); the
// result and its compensation term are valid on thread 0.
__global__ void __launch_bounds__(256)
    mll_finalize_kernel(int n, int d, const double* __restrict__ theta, int n_ls,
                        const double* __restrict__ logdiag, const double* __restrict__ diff,
                        const double* __restrict__ alpha, const double* __restrict__ gpart,
                        int ntiles, int want_grad, double jitter, int* __restrict__ info,
                        double* __restrict__ out_mll, double* __restrict__ out_grad) {
  const double logdet = 2.0 * block_ksum(n, [&](int i) { return logdiag[i]; });
  const double quad = block_ksum(n, [&](int i) { return diff[i] * alpha[i]; });
  const double asum = block_ksum(n, [&](int i) { return alpha[i]; });
  const int slots = d + 2;
  __shared__ double sg[GPK_MAX_D + 2];
  if (want_grad) {
    // one warp per slot, tiles summed in a fixed strided order
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    for (int s = w; s < slots; s += blockDim.x >> 5) {
      double acc = 0.0;
      for (int t = l; t < ntiles; t += 32) acc += gpart[(int64_t)t * slots + s];
      acc = warp_sum(acc);
      if (l == 0) sg[s] = acc;
    }
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  finalize_outputs(n, d, theta, n_ls, jitter, logdet, quad, asum, sg, want_grad, info, out_mll,
                   out_grad);
}

// The fixed partition of the finalisation sums over FIN_BLOCKS blocks: per
// block the compensated (sum, c) pairs of logdiag, diff * alpha and alpha over
// its index range and the gradient slots over its tile range.
constexpr int FIN_BLOCKS = 64;
__global__ void __launch_bounds__(256)
    mll_finalize_partial_kernel(int n, int d, const double* __restrict__ logdiag,
                                const double* __restrict__ diff, const double* __restrict__ alpha,
                                const double* __restrict__ gpart, int ntiles, int want_grad,
                                double* __restrict__ part) {
  const int b = blockIdx.x, stride = 6 + d + 2;
  const int lo = (int)((int64_t)n * b / FIN_BLOCKS), hi = (int)((int64_t)n * (b + 1) / FIN_BLOCKS);
  double v[6];
  block_ksum_pair(lo, hi, [&](int i) { return logdiag[i]; }, v[0], v[1]);
  block_ksum_pair(lo, hi, [&](int i) { return diff[i] * alpha[i]; }, v[2], v[3]);
  block_ksum_pair(lo, hi, [&](int i) { return alpha[i]; }, v[4], v[5]);
  if (threadIdx.x == 0)
    for (int k = 0; k < 6; ++k) part[(int64_t)b * stride + k] = v[k];
  if (want_grad) {
    const int tlo = (int)((int64_t)ntiles * b / FIN_BLOCKS);
    const int thi = (int)((int64_t)ntiles * (b + 1) / FIN_BLOCKS);
    const int slots = d + 2, w = threadIdx.x >> 5, l = threadIdx.x & 31;
    for (int sl = w; sl < slots; sl += blockDim.x >> 5) {
      double acc = 0.0;
      for (int t = tlo + l; t < thi; t += 32) acc += gpart[(int64_t)t * slots + sl];
      acc = warp_sum(acc);
      if (l == 0) part[(int64_t)b * stride + 6 + sl] = acc;
    }
  }
}

__global__ void mll_finalize_combine_kernel(int n, int d, const double* __restrict__ theta,
                                            int n_ls, const double* __restrict__ part,
                                            int want_grad, double jitter, int* __restrict__ info,
                                            double* __restrict__ out_mll,
                                            double* __restrict__ out_grad) {
  if (threadIdx.x != 0) return;
  const int stride = 6 + d + 2;
  double tot[3], comp[3];
  for (int q = 0; q < 3; ++q) {
    tot[q] = 0.0;
    comp[q] = 0.0;
    for (int b = 0; b < FIN_BLOCKS; ++b) {
      const double v = part[(int64_t)b * stride + 2 * q];
      const double t = tot[q] + v;
      comp[q] += part[(int64_t)b * stride + 2 * q + 1] +
                 ((fabs(tot[q]) >= fabs(v)) ? (tot[q] - t) + v : (v - t) + tot[q]);
      tot[q] = t;
    }
  }
  double sg[GPK_MAX_D + 2];
  for (int sl = 0; sl < d + 2; ++sl) {
    double acc = 0.0;
    if (want_grad)
      for (int b = 0; b < FIN_BLOCKS; ++b) acc += part[(int64_t)b * stride + 6 + sl];
    sg[sl] = acc;
  }
  finalize_outputs(n, d, theta, n_ls, jitter, 2.0 * (tot[0] + comp[0]), tot[1] + comp[1],
                   tot[2] + comp[2], sg, want_grad, info, out_mll, out_grad);
}

size_t mll_finalize_scratch_doubles(int d) { return (size_t)FIN_BLOCKS * (6 + d + 2); }

cudaError_t mll_finalize_launch(int n, int d, const double* theta, int n_ls, const double* logdiag,
                                const double* diff, const double* alpha, const double* gpart,
                                int ntiles, int want_grad, double jitter, int* info,
                                double* out_mll, double* out_grad, cudaStream_t s,
                                double* scratch) {
  if (!scratch) {
    mll_finalize_kernel<<<1, 256, 0, s>>>(n, d, theta, n_ls, logdiag, diff, alpha, gpart, ntiles,
                                          want_grad, jitter, info, out_mll, out_grad);
    return launch_status();
  }
  mll_finalize_partial_kernel<<<FIN_BLOCKS, 256, 0, s>>>(n, d, logdiag, diff, alpha, gpart, ntiles,
                                                         want_grad, scratch);
  cudaError_t e = launch_status();
  if (e != cudaSuccess) return e;
  mll_finalize_combine_kernel<<<1, 32, 0, s>>>(n, d, theta, n_ls, scratch, want_grad, jitter, info,
                                               out_mll, out_grad);
  return launch_status();
}

__global__ void finish_info_kernel(int* info) {
  if (*info == INT_MAX) *info = 0;
}

__global__ void zero_outputs_kernel(double* out_mll, double* out_grad, int ng, int* info) {
  if (out_mll) *out_mll = 0.0;
  if (out_grad)
    for (int k = 0; k < ng; ++k) out_grad[k] = 0.0;
  if (info) *info = 0;
}

template <typename T>
static gpk_status mll_run(int kind, int n, int d, const double* x, int64_t ldx, const double* y,
                          const double* theta, int n_ls, double jitter, int refine, int want_grad,
                          double* out_mll, double* out_grad, int* info, void* ws,
                          cudaStream_t s) {
  MllBuffers<T> b;
  mll_layout<T>(n, d, ws, b);
  prof_mark(0, s);
  init_info_kernel<<<1, 1, 0, s>>>(info);
  GPK_LAUNCH_CHECK();
  GPK_CUDA_TRY(scale_inputs<T>(x, ldx, n, d, theta, n_ls, b.xs, s));
  diff_kernel<<<(int)cdiv(n, 256), 256, 0, s>>>(n, y, theta, n_ls, b.diff);
  GPK_LAUNCH_CHECK();
  GPK_CUDA_TRY(cross_cov_scaled<T, T>(kind, n, n, d, b.xs, b.xs, theta, n_ls, 1, jitter, b.A,
                                      b.ld, s));
  GPK_CUDA_TRY(sigma_diag_init(kind, n, theta, n_ls, jitter, b.dtrack, s));
  prof_mark(1, s);
  GPK_CUDA_TRY(potrf_lower<T>(b.A, b.ld, n, b.logdiag, info, b.dtrack, false, s));
  prof_mark(2, s);
  GPK_CUDA_TRY(trtri_lower<T>(b.A, b.ld, n, b.M, b.ld, b.V, b.ld, b.scratch, s));
  prof_mark(3, s);
  GPK_CUDA_TRY(gemv_tri<T>(b.M, b.ld, n, true, b.diff, b.z, 1.0, false, s));
  GPK_CUDA_TRY(gemv_tri<T>(b.V, b.ld, n, false, b.z, b.alpha, 1.0, false, s));
  for (int it = 0; it < refine; ++it) {
    GPK_CUDA_TRY(residual<T>(kind, n, d, b.xs, theta, n_ls, jitter, b.diff, b.alpha, b.r, b.rpart,
                             s));
    GPK_CUDA_TRY(gemv_tri<T>(b.M, b.ld, n, true, b.r, b.z, 1.0, false, s));
    GPK_CUDA_TRY(gemv_tri<T>(b.V, b.ld, n, false, b.z, b.alpha, 1.0, true, s));
  }
  prof_mark(4, s);
  if (want_grad)
    GPK_CUDA_TRY(lauum_grad<T>(kind, b.V, b.ld, n, d, b.xs, theta, n_ls, b.alpha, b.gpart, s));
  prof_mark(5, s);
  GPK_CUDA_TRY(mll_finalize_launch(n, d, theta, n_ls, b.logdiag, b.diff, b.alpha, b.gpart,
                                   lauum_grad_tiles<T>(n), want_grad, jitter, info, out_mll,
                                   out_grad, s, b.fin));
  prof_mark(6, s);
  return GPK_OK;
}

}  // namespace gpk

using namespace gpk;

extern "C" int gpk_version(void) { return 100; }

extern "C" long long gpk_launch_count(void) { return g_launches.load(); }

extern "C" void gpk_set_profile_events(void* const* events, int count) {
  g_prof_count = 0;
  if (!events || count <= 0) return;
  const int m = count < 8 ? count : 8;
  for (int k = 0; k < m; ++k) g_prof_events[k] = static_cast<cudaEvent_t>(events[k]);
  g_prof_count = m;
}

extern "C" const char* gpk_status_string(int status) {
  switch (status) {
    case GPK_OK: return "ok";
    case GPK_ERR_BAD_ARG: return "invalid argument";
    case GPK_ERR_NOT_PD: return "matrix is not positive definite";
    case GPK_ERR_WORKSPACE: return "workspace too small";
    case GPK_ERR_CUDA: return "CUDA error";
    case GPK_ERR_TIMEOUT: return "device wait timed out";
    case GPK_ERR_UNSUPPORTED: return "unsupported configuration";
    default: return "unknown status";
  }
}

static bool mll_args_ok(int kind, int64_t n, int d, int64_t ldx, int n_ls, int precision) {
  if (kind < GPK_RBF || kind > GPK_RATIONAL_QUADRATIC) return false;
  if (n < 0 || n > (1 << 20)) return false;
  if (d <= 0 || d > GPK_MAX_D || ldx < d) return false;
  if (!(n_ls == 1 || n_ls == d)) return false;
  if (precision != GPK_PREC_FP64 && precision != GPK_PREC_MIXED) return false;
  return true;
}

extern "C" size_t gpk_conjugate_mll_workspace_bytes(int64_t n, int d, int precision) {
  if (n <= 0 || d <= 0) return 256;
  if (precision == GPK_PREC_FP64) {
    MllBuffers<double> b;
    return mll_layout<double>(n, d, nullptr, b);
  }
  if (mll_tc_supported(d)) return mll_tc_workspace_bytes(n, d);
  MllBuffers<float> b;
  return mll_layout<float>(n, d, nullptr, b);
}

extern "C" gpk_status gpk_conjugate_mll(int kind, int64_t n, int d, const double* x, int64_t ldx,
                                        const double* y, const double* theta, int n_ls,
                                        double jitter, int precision, int want_grad,
                                        double* out_mll, double* out_grad, int* info,
                                        void* workspace, size_t workspace_bytes,
                                        cudaStream_t stream) {
  if (!mll_args_ok(kind, n, d, ldx, n_ls, precision)) return GPK_ERR_BAD_ARG;
  if (!out_mll || !info || !theta || (want_grad && !out_grad)) return GPK_ERR_BAD_ARG;
  if (n == 0) {
    zero_outputs_kernel<<<1, 1, 0, stream>>>(out_mll, want_grad ? out_grad : nullptr, n_ls + 3,
                                             info);
    GPK_LAUNCH_CHECK();
    return GPK_OK;
  }
  if (!x || !y || !workspace) return GPK_ERR_BAD_ARG;
  if (workspace_bytes < gpk_conjugate_mll_workspace_bytes(n, d, precision))
    return GPK_ERR_WORKSPACE;
  if (precision == GPK_PREC_FP64)
    return mll_run<double>(kind, (int)n, d, x, ldx, y, theta, n_ls, jitter, 1, want_grad, out_mll,
                           out_grad, info, workspace, stream);
  if (mll_tc_supported(d))
    return mll_run_tc(kind, (int)n, d, x, ldx, y, theta, n_ls, jitter, 2, want_grad, out_mll,
                      out_grad, info, workspace, stream);
  return mll_run<float>(kind, (int)n, d, x, ldx, y, theta, n_ls, jitter, 2, want_grad, out_mll,
                        out_grad, info, workspace, stream);
}

// ---------------------------------------------------------------------------
// Batched MLL + gradient: independent GPs of different sizes in one call, each
// in the float32 form (SIMT), spread over a few internal streams that fork
// from and join back into the caller's stream.
// ---------------------------------------------------------------------------
namespace {
constexpr int kBatchStreams = 64;
struct BatchCtx {
  cudaStream_t s[kBatchStreams] = {};
  cudaEvent_t fork = nullptr;
  cudaEvent_t join[kBatchStreams] = {};
};
std::mutex g_batch_mu;
BatchCtx g_batch[64];

cudaError_t batch_ctx(BatchCtx** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  BatchCtx& c = g_batch[dev];
  if (!c.fork) {
    e = cudaEventCreateWithFlags(&c.fork, cudaEventDisableTiming);
    for (int k = 0; k < kBatchStreams && e == cudaSuccess; ++k) {
      e = cudaStreamCreateWithFlags(&c.s[k], cudaStreamNonBlocking);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c.join[k], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) return e;
  }
  *out = &c;
  return cudaSuccess;
}

// Per-instance workspace offsets (256-byte aligned); returns the total.
size_t batch_offsets(int count, const int64_t* n, const int* d, size_t* off) {
  size_t tot = 0;
  for (int i = 0; i < count; ++i) {
    MllBuffers<float> b;
    const size_t w = (mll_layout<float>(n[i], d[i], nullptr, b) + 255) & ~size_t(255);
    if (off) off[i] = tot;
    tot += w;
  }
  return tot + 256;
}
}  // namespace

extern "C" size_t gpk_conjugate_mll_batched_workspace_bytes(int count, const int64_t* n,
                                                            const int* d) {
  if (count <= 0 || !n || !d) return 256;
  for (int i = 0; i < count; ++i)
    if (n[i] <= 0 || d[i] <= 0) return 256;
  return batch_offsets(count, n, d, nullptr);
}

extern "C" gpk_status gpk_conjugate_mll_batched(
    int count, const int* kind, const int64_t* n, const int* d, const double* const* x,
    const int64_t* ldx, const double* const* y, const double* const* theta, const int* n_ls,
    double jitter, int want_grad, double* const* out_mll, double* const* out_grad, int* info,
    void* workspace, size_t workspace_bytes, cudaStream_t stream) {
  if (count < 0) return GPK_ERR_BAD_ARG;
  if (count == 0) return GPK_OK;
  if (!kind || !n || !d || !x || !ldx || !y || !theta || !n_ls || !out_mll || !info ||
      (want_grad && !out_grad) || !workspace)
    return GPK_ERR_BAD_ARG;
  for (int i = 0; i < count; ++i) {
    if (n[i] <= 0 || !mll_args_ok(kind[i], n[i], d[i], ldx[i], n_ls[i], GPK_PREC_MIXED))
      return GPK_ERR_BAD_ARG;
    if (!x[i] || !y[i] || !theta[i] || !out_mll[i] || (want_grad && !out_grad[i]))
      return GPK_ERR_BAD_ARG;
  }
  std::vector<size_t> off(count);
  if (workspace_bytes < batch_offsets(count, n, d, off.data())) return GPK_ERR_WORKSPACE;
  // largest first, each onto the least loaded stream (cost ~ n^3)
  std::vector<int> order(count);
  for (int i = 0; i < count; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int a, int b) { return n[a] > n[b]; });
  std::lock_guard<std::mutex> lock(g_batch_mu);
  BatchCtx* bc = nullptr;
  GPK_CUDA_TRY(batch_ctx(&bc));
  GPK_CUDA_TRY(cudaEventRecord(bc->fork, stream));
  for (int k = 0; k < kBatchStreams; ++k) GPK_CUDA_TRY(cudaStreamWaitEvent(bc->s[k], bc->fork, 0));
  double load[kBatchStreams] = {};
  for (int i : order) {
    int k = 0;
    for (int q = 1; q < kBatchStreams; ++q)
      if (load[q] < load[k]) k = q;
    load[k] += (double)n[i] * (double)n[i] * (double)n[i];
    const gpk_status st =
        mll_run<float>(kind[i], (int)n[i], d[i], x[i], ldx[i], y[i], theta[i], n_ls[i], jitter, 2,
                       want_grad, out_mll[i], want_grad ? out_grad[i] : nullptr, info + i,
                       static_cast<char*>(workspace) + off[i], bc->s[k]);
    if (st != GPK_OK) return st;
  }
  for (int k = 0; k < kBatchStreams; ++k) {
    GPK_CUDA_TRY(cudaEventRecord(bc->join[k], bc->s[k]));
    GPK_CUDA_TRY(cudaStreamWaitEvent(stream, bc->join[k], 0));
  }
  return GPK_OK;
}

extern "C" gpk_status gpk_lower_cholesky(int64_t n, int dtype, void* A, int64_t lda,
                                         double* logdiag, int* info, cudaStream_t stream) {
  if (n < 0 || n > (1 << 20) || lda < n || !info) return GPK_ERR_BAD_ARG;
  if (dtype != GPK_F64 && dtype != GPK_F32) return GPK_ERR_BAD_ARG;  // before any device work
  if (n == 0) {
    zero_outputs_kernel<<<1, 1, 0, stream>>>(nullptr, nullptr, 0, info);
    GPK_LAUNCH_CHECK();
    return GPK_OK;
  }
  if (!A) return GPK_ERR_BAD_ARG;
  init_info_kernel<<<1, 1, 0, stream>>>(info);
  GPK_LAUNCH_CHECK();
  if (dtype == GPK_F64)
    GPK_CUDA_TRY(potrf_lower<double>((double*)A, lda, (int)n, logdiag, info, nullptr, true, stream));
  else if (dtype == GPK_F32)
    GPK_CUDA_TRY(potrf_lower<float>((float*)A, lda, (int)n, logdiag, info, nullptr, true, stream));
  else
    return GPK_ERR_BAD_ARG;
  finish_info_kernel<<<1, 1, 0, stream>>>(info);
  GPK_LAUNCH_CHECK();
  return GPK_OK;
}

// ---------------------------------------------------------------------------
// Triangular solve L X = B through the triangular inverse:
// X^T = B^T M^T, one NT GEMM with the transposed store landing in B.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void transpose_kernel(int rows, int cols, const T* __restrict__ src, int64_t lds,
                                 T* __restrict__ dst, int64_t ldd) {
  __shared__ T tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int r = by + k, c = bx + threadIdx.x;
    tile[k][threadIdx.x] = (r < rows && c < cols) ? src[(int64_t)r * lds + c] : T(0);
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int r = bx + k, c = by + threadIdx.x;  // dst is cols x rows
    if (r < cols && c < rows) dst[(int64_t)r * ldd + c] = tile[threadIdx.x][k];
  }
}

template <typename T>
static size_t solve_layout(int64_t n, int64_t nrhs, bool upper, void* ws, T** M, T** V, T** scr,
                           T** BT, T** LT, int64_t* ld) {
  Arena a(ws);
  *ld = pad_ld(n);
  *M = a.take<T>((size_t)n * *ld);
  *V = a.take<T>((size_t)n * *ld);
  *scr = a.take<T>((size_t)n * n / 2 + 64);
  *BT = a.take<T>((size_t)nrhs * *ld);
  *LT = upper ? a.take<T>((size_t)n * *ld) : nullptr;  // lower copy U^T of an upper input
  return a.off + 256;
}

static size_t solve_ws(int64_t n, int64_t nrhs, int dtype, bool upper) {
  int64_t ld;
  if (dtype == GPK_F64) {
    double *M, *V, *S, *B, *LT;
    return solve_layout<double>(n, nrhs, upper, nullptr, &M, &V, &S, &B, &LT, &ld);
  }
  float *M, *V, *S, *B, *LT;
  return solve_layout<float>(n, nrhs, upper, nullptr, &M, &V, &S, &B, &LT, &ld);
}

extern "C" size_t gpk_solve_triangular_workspace_bytes(int64_t n, int64_t nrhs, int dtype) {
  return solve_ws(n, nrhs, dtype, false);
}

extern "C" size_t gpk_solve_triangular_ex_workspace_bytes(int64_t n, int64_t nrhs, int dtype,
                                                          int upper) {
  return solve_ws(n, nrhs, dtype, upper != 0);
}

// op(T) X = B in place.  A lower input L gives M = L^-1 and V = L^-T by the
// triangular inverse; an upper input U is first copied to the lower L = U^T,
// so that U^-1 = L^-T (V) and U^-T = L^-1 (M).  X^T = B^T op^T, one NT GEMM
// whose transposed output lands in B.
template <typename T>
static gpk_status solve_run(int n, int nrhs, const T* L, int64_t lda, bool upper, bool trans,
                            T* B, int64_t ldb, void* ws, cudaStream_t s) {
  T *M, *V, *scr, *BT, *LT;
  int64_t ld;
  solve_layout<T>(n, nrhs, upper, ws, &M, &V, &scr, &BT, &LT, &ld);
  dim3 tb(32, 8);
  if (upper) {
    transpose_kernel<T><<<dim3((unsigned)cdiv(n, 32), (unsigned)cdiv(n, 32)), tb, 0, s>>>(
        n, n, L, lda, LT, ld);
    GPK_LAUNCH_CHECK();
    L = LT;
    lda = ld;
  }
  GPK_CUDA_TRY(trtri_lower<T>(L, lda, n, M, ld, V, ld, scr, s));
  // lower: T^-1 = M, T^-T = V ; upper (T = L^T): T^-1 = V, T^-T = M
  const bool use_v = upper != trans;
  transpose_kernel<T><<<dim3((unsigned)cdiv(nrhs, 32), (unsigned)cdiv(n, 32)), tb, 0, s>>>(
      n, nrhs, B, ldb, BT, ld);
  GPK_LAUNCH_CHECK();
  GemmProb<T> p{};
  p.A = BT;
  p.lda = ld;
  p.M = nrhs;
  p.B = use_v ? V : M;
  p.ldb = ld;
  p.b_tri = use_v ? TRI_UPPER : TRI_LOWER;
  p.N = n;
  p.K = n;
  p.C = nullptr;
  p.Ct = B;
  p.ldct = ldb;
  p.alpha = T(1);
  p.beta = T(0);
  GPK_CUDA_TRY(gemm_nt<T>(p, 1, s));
  return GPK_OK;
}

static gpk_status solve_dispatch(int64_t n, int64_t nrhs, int dtype, bool upper, bool trans,
                                 const void* L, int64_t lda, void* B, int64_t ldb,
                                 void* workspace, size_t workspace_bytes, cudaStream_t stream) {
  if (n < 0 || nrhs < 0 || n > (1 << 20) || lda < n || ldb < nrhs) return GPK_ERR_BAD_ARG;
  if (dtype != GPK_F64 && dtype != GPK_F32) return GPK_ERR_BAD_ARG;
  if (n == 0 || nrhs == 0) return GPK_OK;
  if (!L || !B || !workspace) return GPK_ERR_BAD_ARG;
  if (workspace_bytes < solve_ws(n, nrhs, dtype, upper)) return GPK_ERR_WORKSPACE;
  if (dtype == GPK_F64)
    return solve_run<double>((int)n, (int)nrhs, (const double*)L, lda, upper, trans, (double*)B,
                             ldb, workspace, stream);
  return solve_run<float>((int)n, (int)nrhs, (const float*)L, lda, upper, trans, (float*)B, ldb,
                          workspace, stream);
}

extern "C" gpk_status gpk_solve_triangular(int64_t n, int64_t nrhs, int dtype, const void* L,
                                           int64_t lda, void* B, int64_t ldb, void* workspace,
                                           size_t workspace_bytes, cudaStream_t stream) {
  return solve_dispatch(n, nrhs, dtype, false, false, L, lda, B, ldb, workspace, workspace_bytes,
                        stream);
}

extern "C" gpk_status gpk_solve_triangular_ex(int64_t n, int64_t nrhs, int dtype, int upper,
                                              int trans, const void* T, int64_t ldt, void* B,
                                              int64_t ldb, void* workspace,
                                              size_t workspace_bytes, cudaStream_t stream) {
  return solve_dispatch(n, nrhs, dtype, upper != 0, trans != 0, T, ldt, B, ldb, workspace,
                        workspace_bytes, stream);
}

// ---------------------------------------------------------------------------
// float64 GEMM C = alpha op(A) op(B) + beta C (row-major), on the library's
// NT kernel: operands that are not already in NT form are transposed into the
// workspace first.
// ---------------------------------------------------------------------------
static size_t gemm64_layout(int64_t M, int64_t N, int64_t K, int transa, int transb, void* ws,
                            double** At, double** Bt, int64_t* lda_t, int64_t* ldb_t) {
  Arena a(ws);
  *lda_t = pad_ld(K);
  *ldb_t = pad_ld(K);
  *At = transa ? a.take<double>((size_t)M * *lda_t) : nullptr;  // op(A) = A^T: A^T copy [M, K]
  *Bt = transb ? nullptr : a.take<double>((size_t)N * *ldb_t);  // op(B) = B: B^T copy [N, K]
  return a.off + 256;
}

extern "C" size_t gpk_gemm_f64_workspace_bytes(int transa, int transb, int64_t M, int64_t N,
                                               int64_t K) {
  double *a, *b;
  int64_t la, lb;
  return gemm64_layout(M, N, K, transa, transb, nullptr, &a, &b, &la, &lb);
}

extern "C" gpk_status gpk_gemm_f64(int transa, int transb, int64_t M, int64_t N, int64_t K,
                                   double alpha, const double* A, int64_t lda, const double* B,
                                   int64_t ldb, double beta, double* C, int64_t ldc,
                                   void* workspace, size_t workspace_bytes, cudaStream_t s) {
  if (M < 0 || N < 0 || K < 0 || M > (1 << 24) || N > (1 << 24) || K > (1 << 24))
    return GPK_ERR_BAD_ARG;
  if (lda < (transa ? M : K) || ldb < (transb ? K : N) || ldc < N) return GPK_ERR_BAD_ARG;
  if (M == 0 || N == 0) return GPK_OK;
  if (!A || !B || !C || !workspace) return GPK_ERR_BAD_ARG;
  if (workspace_bytes < gpk_gemm_f64_workspace_bytes(transa, transb, M, N, K))
    return GPK_ERR_WORKSPACE;
  double *At, *Bt;
  int64_t la, lb;
  gemm64_layout(M, N, K, transa, transb, workspace, &At, &Bt, &la, &lb);
  dim3 tb(32, 8);
  const double* An = A;
  int64_t ldan = lda;
  if (transa) {  // A stored [K, M]
    transpose_kernel<double><<<dim3((unsigned)cdiv(M, 32), (unsigned)cdiv(K, 32)), tb, 0, s>>>(
        (int)K, (int)M, A, lda, At, la);
    GPK_LAUNCH_CHECK();
    An = At;
    ldan = la;
  }
  const double* Bn = B;
  int64_t ldbn = ldb;
  if (!transb) {  // B stored [K, N]
    transpose_kernel<double><<<dim3((unsigned)cdiv(N, 32), (unsigned)cdiv(K, 32)), tb, 0, s>>>(
        (int)K, (int)N, B, ldb, Bt, lb);
    GPK_LAUNCH_CHECK();
    Bn = Bt;
    ldbn = lb;
  }
  GemmProb<double> p{};
  p.A = An;
  p.lda = ldan;
  p.B = Bn;
  p.ldb = ldbn;
  p.C = C;
  p.ldc = ldc;
  p.M = (int)M;
  p.N = (int)N;
  p.K = (int)K;
  p.alpha = alpha;
  p.beta = beta;
  GPK_CUDA_TRY(gemm_nt<double>(p, 1, s));
  return GPK_OK;
}

template <typename T>
__global__ void __launch_bounds__(256)
    logdet_tri_kernel(int n, const T* __restrict__ L, int64_t lda, double* out) {
  const double v = block_ksum(n, [&](int i) { return log((double)L[(int64_t)i * lda + i]); });
  if (threadIdx.x == 0) *out = v;
}

extern "C" gpk_status gpk_logdet_triangular(int64_t n, int dtype, const void* L, int64_t lda,
                                            double* out, cudaStream_t stream) {
  if (n < 0 || lda < n || !out || (n > 0 && !L)) return GPK_ERR_BAD_ARG;
  if (dtype == GPK_F64)
    logdet_tri_kernel<double><<<1, 256, 0, stream>>>((int)n, (const double*)L, lda, out);
  else if (dtype == GPK_F32)
    logdet_tri_kernel<float><<<1, 256, 0, stream>>>((int)n, (const float*)L, lda, out);
  else
    return GPK_ERR_BAD_ARG;
  GPK_LAUNCH_CHECK();
  return GPK_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free float64 marginal log-likelihood for small problems.
//
// Callers that cannot allocate device memory (host frameworks that hand a
// custom call no workspace; embedded or real-time hosts that forbid
// allocation after start-up) use this entry point instead of
// gpk_conjugate_mll: its scratch is a file-scope device array, so the call
// allocates nothing.  The array holds kNoallocBytes (8 MiB), enough for
// n <= kNoallocMaxN (512, reported by gpk_conjugate_mll_noalloc_max_n()) at
// every d the library accepts (d <= GPK_MAX_D); every GPU that loads the
// library keeps it until the process exits.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoallocBytes = (size_t)8 << 20;  // 8 MiB
constexpr int kNoallocMaxN = 512;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

// Device address of g_noalloc_scratch per device.  In host code the array's
// name is only a host-side stand-in, so the address comes from
// cudaGetSymbolAddress, taken once per device with that device current.  The
// cache is keyed by device ordinal, i.e. the runtime's primary context.
static void* g_noalloc_ptr[kMaxDevices];
static std::mutex g_noalloc_mutex;

gpk_status noalloc_scratch(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GPK_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return GPK_ERR_CUDA;
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return GPK_OK;
}

}  // namespace

extern "C" size_t gpk_conjugate_mll_noalloc_max_n(void) { return kNoallocMaxN; }

extern "C" gpk_status gpk_conjugate_mll_noalloc(int kind, int64_t n, int d, const double* x,
                                                int64_t ldx, const double* y,
                                                const double* theta, int n_ls, double jitter,
                                                int want_grad, double* out_mll,
                                                double* out_grad, int* info,
                                                cudaStream_t stream) {
  if (!mll_args_ok(kind, n, d, ldx, n_ls, GPK_PREC_FP64)) return GPK_ERR_BAD_ARG;
  // sizes beyond the static scratch are refused, never truncated (d is bounded
  // by GPK_MAX_D above, like every entry point of the library)
  if (n > kNoallocMaxN) return GPK_ERR_UNSUPPORTED;
  if (!out_mll || !info || !theta || (want_grad && !out_grad)) return GPK_ERR_BAD_ARG;
  if (n == 0) {
    zero_outputs_kernel<<<1, 1, 0, stream>>>(out_mll, want_grad ? out_grad : nullptr, n_ls + 3,
                                             info);
    GPK_LAUNCH_CHECK();
    return GPK_OK;
  }
  if (!x || !y) return GPK_ERR_BAD_ARG;
  MllBuffers<double> b;
  if (mll_layout<double>(n, d, nullptr, b) > kNoallocBytes) return GPK_ERR_UNSUPPORTED;
  void* ws = nullptr;
  const gpk_status st = noalloc_scratch(&ws);
  if (st != GPK_OK) return st;
  // Every region of the layout is written before it is read within one
  // call (Gram, factor, inverse, solves, per-tile partials), so nothing left
  // by an earlier call has to be cleared.
  return mll_run<double>(kind, (int)n, d, x, ldx, y, theta, n_ls, jitter, 1, want_grad, out_mll,
                         out_grad, info, ws, stream);
}
