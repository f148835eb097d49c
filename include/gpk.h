/*
 * gpk.h -- C ABI of the GB300 (sm_103a) exact/sparse Gaussian-process library.
 *
 * Plain C types only: device pointers, sizes, a CUDA stream.  Every device
 * buffer is owned by the caller (torch tensors, XLA buffers under jax.ffi);
 * the library never allocates.  Scratch memory comes from the caller through
 * the matching *_workspace_bytes() query.  All calls are asynchronous on the
 * given stream and do not synchronise the host.
 *
 * Hyperparameters live on the device as a float64 vector
 *     theta = [ lengthscale[0..n_ls), variance, obs_stddev, mean_constant ]
 * with n_ls = 1 (isotropic) or d (ARD), in the reference's constrained
 * coordinates (kernels/stationary/base.py:54-95, likelihoods.py:129-152,
 * mean_functions.py:131-153).  Gradients use the same layout.
 *
 * Errors: a gpk_status is returned for argument/launch errors.  A factorised
 * matrix that is not positive definite is reported on the device through
 * *info (0 = ok, k > 0 = the leading minor of order k is not positive
 * definite, LAPACK convention); outputs are then NaN, which is what the
 * reference's jnp.linalg.cholesky produces (linalg/operations.py:54-55).
 */
#ifndef GPK_H_
#define GPK_H_

#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  GPK_OK = 0,
  GPK_ERR_BAD_ARG = 1,
  GPK_ERR_NOT_PD = 2,
  GPK_ERR_WORKSPACE = 3,
  GPK_ERR_CUDA = 4,
  GPK_ERR_TIMEOUT = 5,
  GPK_ERR_UNSUPPORTED = 6
} gpk_status;

/* stationary kernels: kernels/stationary/{rbf,matern32,matern52,matern12,
 * rational_quadratic}.py.  GPK_RATIONAL_QUADRATIC reads its alpha from one
 * more theta slot, theta[n_ls + 3] (after the mean constant); gradients keep
 * the n_ls + 3 layout (alpha is a fixed constant of the reference's kernel,
 * rational_quadratic.py:64). */
typedef enum {
  GPK_RBF = 0,
  GPK_MATERN32 = 1,
  GPK_MATERN52 = 2,
  GPK_MATERN12 = 3,
  GPK_RATIONAL_QUADRATIC = 4
} gpk_kernel_kind;

typedef enum { GPK_F64 = 0, GPK_F32 = 1 } gpk_dtype;

/* GPK_PREC_FP64: every step in float64.
 * GPK_PREC_MIXED: float32 Gram, tensor-core factorisation, inversion and
 * adjoint with float32 accumulation -- split-TF32 products, and split-float16
 * products on power-of-two row-scaled operand copies for the large ones (the
 * same 11-bit significand split) -- float64 residual refinement of
 * alpha = Sigma^-1 (y - m), float64 log-det and gradient accumulation. */
typedef enum { GPK_PREC_FP64 = 0, GPK_PREC_MIXED = 1 } gpk_precision;

/* Library version as major*10000 + minor*100 + patch. */
int gpk_version(void);

/* Human-readable name of a status code (static string). */
const char* gpk_status_string(int status);

/* Instrumentation (no counterpart in the reference).
 * gpk_launch_count: kernel launches issued by the library since it was loaded.
 * gpk_set_profile_events: when given >= 7 cudaEvent_t handles, each
 * gpk_conjugate_mll call records them on its stream at its phase boundaries
 * (float64 form: 0 start, 1 Gram built, 2 Cholesky done, 3 triangular inverse
 * done, 4 alpha solved and refined, 5 adjoint done, 6 end; mixed form: 0 start,
 * 1 Gram built, 2 factor and inverse done, 3 alpha solved and refined,
 * 4 adjoint done, 5 internal streams joined, 6 end); NULL disables.
 * Process-global and not thread-safe: meant for benchmarks. */
long long gpk_launch_count(void);
void gpk_set_profile_events(void* const* events, int count);

/* ---------------------------------------------------------------------------
 * Kernel computations
 * Replaces AbstractKernelComputation.cross_covariance / gram / diagonal
 * (gpjax/kernels/computations/base.py:56-109) and
 * DenseKernelComputation._cross_covariance (computations/dense.py:32-36).
 * x [n, d] and y [m, d] are row-major float64 with leading dims ldx, ldy;
 * out [n, m] is row-major with leading dim ldo in out_dtype.
 * ------------------------------------------------------------------------- */
gpk_status gpk_cross_covariance(int kind, int64_t n, int64_t m, int d,
                                const double* x, int64_t ldx,
                                const double* y, int64_t ldy,
                                const double* theta, int n_ls,
                                int out_dtype, void* out, int64_t ldo,
                                cudaStream_t stream);

/* Full-square Gram K(x, x) (computations/base.py:56-72). */
gpk_status gpk_gram(int kind, int64_t n, int d, const double* x, int64_t ldx,
                    const double* theta, int n_ls, int out_dtype, void* out,
                    int64_t ldo, cudaStream_t stream);

/* Reverse-mode derivative of gpk_cross_covariance: given the cotangent
 * G [n, m] (float64, leading dim ldg) of K(x, y), writes grad_theta
 * [n_ls + 3] (lengthscales, variance; the obs_stddev and mean slots are 0)
 * and, when non-NULL, grad_x [n, d] and grad_y [m, d].  Counterpart of JAX
 * differentiating DenseKernelComputation.cross_covariance
 * (computations/dense.py:32-36).  workspace: gpk_cross_covariance_vjp_workspace_bytes. */
size_t gpk_cross_covariance_vjp_workspace_bytes(int64_t n, int64_t m, int d);
gpk_status gpk_cross_covariance_vjp(int kind, int64_t n, int64_t m, int d,
                                    const double* x, int64_t ldx,
                                    const double* y, int64_t ldy,
                                    const double* theta, int n_ls,
                                    const double* G, int64_t ldg,
                                    double* grad_theta, double* grad_x, double* grad_y,
                                    void* workspace, size_t workspace_bytes,
                                    cudaStream_t stream);

/* diag k(x_i, x_i) as float64 [n] (computations/base.py:95-109). */
gpk_status gpk_diagonal(int kind, int64_t n, int d, const double* x, int64_t ldx,
                        const double* theta, int n_ls, double* out,
                        cudaStream_t stream);

/* ---------------------------------------------------------------------------
 * Linear algebra on dense row-major matrices
 * ------------------------------------------------------------------------- */
/* In-place lower Cholesky of the SPD matrix A [n, n] (only the lower triangle
 * is read; the strict upper triangle is zeroed on return).
 * Replaces lower_cholesky's Dense branch (linalg/operations.py:54-55).
 * logdiag (optional, float64 [n]) receives log L_ii. */
gpk_status gpk_lower_cholesky(int64_t n, int dtype, void* A, int64_t lda,
                              double* logdiag, int* info, cudaStream_t stream);

/* Solves L X = B in place for lower-triangular L [n, n] and B [n, nrhs]
 * (row-major, ldb >= nrhs).  Replaces solve's Triangular branch
 * (linalg/operations.py:105-107, jsp.linalg.solve_triangular lower=True).
 * workspace: gpk_solve_triangular_workspace_bytes(). */
size_t gpk_solve_triangular_workspace_bytes(int64_t n, int64_t nrhs, int dtype);
gpk_status gpk_solve_triangular(int64_t n, int64_t nrhs, int dtype,
                                const void* L, int64_t lda, void* B, int64_t ldb,
                                void* workspace, size_t workspace_bytes,
                                cudaStream_t stream);

/* op(T) X = B in place for a triangular T [n, n] that is lower (upper = 0)
 * or upper (upper = 1), op(T) = T (trans = 0) or T^T (trans = 1); B [n, nrhs]
 * row-major.  The Triangular branch of solve with the lower / trans flags of
 * jax.scipy.linalg.solve_triangular (linalg/operations.py:105-107;
 * variational_families.py:839-852 solves against L^T).  workspace:
 * gpk_solve_triangular_ex_workspace_bytes(n, nrhs, dtype, upper). */
size_t gpk_solve_triangular_ex_workspace_bytes(int64_t n, int64_t nrhs, int dtype, int upper);
gpk_status gpk_solve_triangular_ex(int64_t n, int64_t nrhs, int dtype, int upper, int trans,
                                   const void* T, int64_t ldt, void* B, int64_t ldb,
                                   void* workspace, size_t workspace_bytes, cudaStream_t stream);

/* float64 C = alpha op(A) op(B) + beta C, row-major, op(A) [M, K], op(B)
 * [K, N]: the dense products of the reference's predict paths (jnp.matmul at
 * gps.py:520-522, variational_families.py:830-861).  workspace:
 * gpk_gemm_f64_workspace_bytes (transposed operand copies, 256 bytes when
 * none is needed). */
size_t gpk_gemm_f64_workspace_bytes(int transa, int transb, int64_t M, int64_t N, int64_t K);
gpk_status gpk_gemm_f64(int transa, int transb, int64_t M, int64_t N, int64_t K, double alpha,
                        const double* A, int64_t lda, const double* B, int64_t ldb, double beta,
                        double* C, int64_t ldc, void* workspace, size_t workspace_bytes,
                        cudaStream_t stream);

/* sum_i log L_ii in float64 (compensated), the Triangular branch of logdet
 * (linalg/operations.py:142-144); out is one device double. */
gpk_status gpk_logdet_triangular(int64_t n, int dtype, const void* L, int64_t lda,
                                 double* out, cudaStream_t stream);

/* ---------------------------------------------------------------------------
 * Objectives
 * ------------------------------------------------------------------------- */
/* Exact-GP marginal log-likelihood and its gradient
 * (conjugate_mll, gpjax/objectives.py:36-107, through
 * GaussianDistribution.log_prob, gpjax/distributions.py:115-134).
 *   Sigma = K(x, x) + I*jitter + I*obs_stddev^2, diff = y - mean_constant,
 *   mll   = -1/2 (n log 2pi + log|Sigma| + diff^T Sigma^-1 diff).
 * x [n, d] float64 row-major, y [n] float64; out_mll: 1 device double;
 * out_grad (if want_grad): device double [n_ls + 3] in theta's layout;
 * info: device int (0 or first non-PD order).  jitter is posterior.prior.jitter. */
size_t gpk_conjugate_mll_workspace_bytes(int64_t n, int d, int precision);
gpk_status gpk_conjugate_mll(int kind, int64_t n, int d,
                             const double* x, int64_t ldx, const double* y,
                             const double* theta, int n_ls, double jitter,
                             int precision, int want_grad,
                             double* out_mll, double* out_grad, int* info,
                             void* workspace, size_t workspace_bytes,
                             cudaStream_t stream);

/* Leave-one-out predictive log-probability and its gradient, float64
 * (conjugate_loocv, gpjax/objectives.py:110-178):
 *   loocv = sum_i log N(y_i; y_i - alpha_i / W_ii, 1 / W_ii),
 *   alpha = Sigma^-1 (y - mean_constant), W = Sigma^-1,
 *   Sigma = K(x, x) + (obs_stddev^2 + jitter) I.
 * Arguments as gpk_conjugate_mll (theta layout, info); out_loocv: 1 device
 * double; out_grad (if want_grad): device double [n_ls + 3].
 * n <= 65536.  workspace: gpk_conjugate_loocv_workspace_bytes (about 4 n^2
 * doubles: Sigma's factor, its inverse, Sigma^-1 and the cotangent). */
size_t gpk_conjugate_loocv_workspace_bytes(int64_t n, int d);
gpk_status gpk_conjugate_loocv(int kind, int64_t n, int d, const double* x, int64_t ldx,
                               const double* y, const double* theta, int n_ls, double jitter,
                               int want_grad, double* out_loocv, double* out_grad, int* info,
                               void* workspace, size_t workspace_bytes, cudaStream_t stream);

/* Allocation-free variant of gpk_conjugate_mll, float64 form only.
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory -- host frameworks that pass a custom call no workspace, hosts that
 * forbid allocation after start-up -- the scratch is a static device array
 * of 8 MiB inside the library, which bounds the problem to
 * n <= gpk_conjugate_mll_noalloc_max_n() (512); a larger n returns
 * GPK_ERR_UNSUPPORTED.  d is bounded as everywhere in the library (d <= 32,
 * GPK_ERR_BAD_ARG beyond).  Every GPU that loads the library holds the array
 * until the process exits.  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress) and keeps it for that device
 * ordinal.  Only the runtime's primary
 * context is supported: after cudaDeviceReset, or with another context
 * current, the kept address is stale.  All calls share the one array: calls
 * that overlap on the GPU (different streams, or different host threads on the
 * same device) race; serialise them.  Arguments and results are those of
 * gpk_conjugate_mll. */
size_t gpk_conjugate_mll_noalloc_max_n(void);
gpk_status gpk_conjugate_mll_noalloc(int kind, int64_t n, int d,
                                     const double* x, int64_t ldx, const double* y,
                                     const double* theta, int n_ls, double jitter,
                                     int want_grad, double* out_mll, double* out_grad,
                                     int* info, cudaStream_t stream);

/* SGPR collapsed ELBO and its gradient (collapsed_elbo,
 * gpjax/objectives.py:321-416), including d/dZ for the inducing inputs.
 * z [m, d] float64; out_grad: theta layout [n_ls + 3]; out_grad_z [m, d]. */
size_t gpk_collapsed_elbo_workspace_bytes(int64_t n, int64_t m, int d, int precision);
gpk_status gpk_collapsed_elbo(int kind, int64_t n, int64_t m, int d,
                              const double* x, int64_t ldx, const double* y,
                              const double* z, int64_t ldz,
                              const double* theta, int n_ls, double jitter,
                              int precision, int want_grad,
                              double* out_elbo, double* out_grad, double* out_grad_z,
                              int* info, void* workspace, size_t workspace_bytes,
                              cudaStream_t stream);

/* Data-parallel collapsed ELBO: each rank passes its own rows of x and y
 * (n_local of n_total), the same z and theta, and a callback that sums a
 * float64 region of its workspace over the ranks, in place, ordered on
 * `stream` (an NCCL or gloo all-reduce; 0 on success).  The library calls it
 * with the byte offset of the region inside `workspace` at two points: after
 * the rank-local statistics (P = Phi Phi^T [m x ldm], c = Phi d and Phi 1 [2m],
 * (d^T d, 1^T d) [2]) and, with want_grad, after the rank-local gradient sums
 * (theta part [d + 1], z part [m x d]); the m x m algebra in between and after
 * is replicated.  Every rank gets the full-data ELBO and gradients
 * (objectives.py:321-416 over all n_total rows).  workspace:
 * gpk_collapsed_elbo_workspace_bytes(n_local, m, d, precision).  No
 * counterpart in the reference, which runs on one device. */
typedef int (*gpk_allreduce_fn)(void* user, size_t byte_offset, int64_t count,
                                cudaStream_t stream);
gpk_status gpk_collapsed_elbo_sharded(int kind, int64_t n_local, int64_t n_total, int64_t m, int d,
                                      const double* x, int64_t ldx, const double* y,
                                      const double* z, int64_t ldz, const double* theta, int n_ls,
                                      double jitter, int precision, int want_grad,
                                      double* out_elbo, double* out_grad, double* out_grad_z,
                                      int* info, void* workspace, size_t workspace_bytes,
                                      cudaStream_t stream, gpk_allreduce_fn allreduce, void* user);

/* ---------------------------------------------------------------------------
 * Batched MLL + gradient over independent GPs of different sizes (no single
 * reference counterpart: the reference evaluates conjugate_mll
 * (gpjax/objectives.py:36-107) per model, e.g. under jax.vmap for equal
 * shapes).  Instance i has kind[i], n[i], d[i] and device pointers x[i]
 * ([n, d], ldx[i]), y[i], theta[i] (layout as gpk_conjugate_mll, n_ls[i]
 * lengthscales); out_mll[i] (1 double), out_grad[i] (n_ls[i] + 3 doubles)
 * and info[i] (device int array [count]) receive the results.  The host
 * arrays are read during the call only.  Float32 compute (SIMT), instances
 * spread over internal streams joined back into `stream`; workspace from
 * gpk_conjugate_mll_batched_workspace_bytes.
 * ------------------------------------------------------------------------- */
size_t gpk_conjugate_mll_batched_workspace_bytes(int count, const int64_t* n, const int* d);
gpk_status gpk_conjugate_mll_batched(int count, const int* kind, const int64_t* n, const int* d,
                                     const double* const* x, const int64_t* ldx,
                                     const double* const* y, const double* const* theta,
                                     const int* n_ls, double jitter, int want_grad,
                                     double* const* out_mll, double* const* out_grad, int* info,
                                     void* workspace, size_t workspace_bytes,
                                     cudaStream_t stream);

/* ---------------------------------------------------------------------------
 * Persistent batched MLL + gradient through a plan (no single counterpart:
 * conjugate_mll, gpjax/objectives.py:36-107, and jax.value_and_grad of it per
 * instance, as the reference would vmap or loop over independent GPs).
 * gpk_batch_plan_create records the instances (same arguments and result
 * locations as gpk_conjugate_mll_batched; the device arrays are read at each
 * execution, so their contents may change between executions), sorts them
 * by n (largest first) into a device queue and, when autotune != 0, times the
 * tile configurations on the plan's own instances for every n_pad not yet
 * tuned on this device and keeps the fastest of those that fail the fewest
 * of the trial's instances (results kept for the process).  It allocates a few
 * bytes per instance of device memory and synchronises the device: call it
 * outside stream capture.  gpk_batch_plan_execute zeroes the queue head and
 * launches ONE persistent kernel (one CTA per SM pulls instances from the
 * queue and runs each to completion), so an execution can be captured in a
 * CUDA graph.  Float32 compute with float64 pivots, float-float refinement of
 * alpha and float64 sums.  n <= 4096, d <= 16 (else GPK_ERR_UNSUPPORTED).
 * gpk_batch_plan_config returns the configuration chosen for instances of
 * size n (0: K slices of 16 on the CUDA cores, 1: of 32, 2: K slices of 32 on
 * the tcgen05 tensor cores in split TF32) or -1; gpk_batch_plan_config_count
 * gives the number of configurations.  gpk_batch_plan_force_config runs every
 * instance of later executions with configuration cfg (-1: the tuned ones
 * again); GPK_ERR_BAD_ARG outside [-1, count).
 * ------------------------------------------------------------------------- */
typedef struct gpk_batch_plan_s* gpk_batch_plan;
gpk_status gpk_batch_plan_create(int count, const int* kind, const int64_t* n, const int* d,
                                 const double* const* x, const int64_t* ldx,
                                 const double* const* y, const double* const* theta,
                                 const int* n_ls, double jitter, int want_grad,
                                 double* const* out_mll, double* const* out_grad, int* info,
                                 int autotune, gpk_batch_plan* plan);
size_t gpk_batch_plan_workspace_bytes(gpk_batch_plan plan);
int gpk_batch_plan_config(gpk_batch_plan plan, int64_t n);
int gpk_batch_plan_config_count(void);
gpk_status gpk_batch_plan_force_config(gpk_batch_plan plan, int cfg);
/* Self-test of the bounded waits of the tensor-core configuration: with
 * cycles > 0, the first MMA wait of every CTA in later executions also waits
 * up to `cycles` SM clocks on a barrier that nothing arrives on, records that
 * it ran out, and the instances that CTA runs report info = -1 with NaN
 * outputs (the MMAs themselves are still waited for).  0 turns it off;
 * GPK_ERR_BAD_ARG for a null plan or cycles outside [0, 4e9]. */
gpk_status gpk_batch_plan_selftest_stall(gpk_batch_plan plan, long long cycles);
gpk_status gpk_batch_plan_execute(gpk_batch_plan plan, void* workspace, size_t workspace_bytes,
                                  cudaStream_t stream);
gpk_status gpk_batch_plan_destroy(gpk_batch_plan plan);

/* ---------------------------------------------------------------------------
 * Prediction: ConjugatePosterior.predict (gpjax/gps.py:443-526).
 * mean [t] and var [t] float64 (var = diag of the predictive covariance,
 * GaussianDistribution.variance, distributions.py:79-81); cov [t, t] float64
 * row-major only when cov != NULL.  jitter is the posterior's (added to Kxx),
 * prior_jitter the prior's (added to the predictive covariance).
 * ------------------------------------------------------------------------- */
size_t gpk_predict_workspace_bytes(int64_t n, int64_t t, int d, int precision);
gpk_status gpk_predict(int kind, int64_t n, int64_t t, int d,
                       const double* x, int64_t ldx, const double* y,
                       const double* xt, int64_t ldxt,
                       const double* theta, int n_ls,
                       double jitter, double prior_jitter, int precision,
                       double* mean, double* var, double* cov, int64_t ldcov,
                       int* info, void* workspace, size_t workspace_bytes,
                       cudaStream_t stream);

/* ---------------------------------------------------------------------------
 * Split-TF32 tensor-core GEMM (no counterpart in the reference; the building
 * block of the mixed form).  C = beta*C + alpha * A B^T with A [M, K],
 * B [N, K], C [M, N] float32 row-major, computed on tcgen05 as
 * A_lo B_hi + A_hi B_lo + A_hi B_hi with float32 accumulation.  lower_only
 * (M == N) updates only i >= j.  err_flag (optional device int) is set to 1
 * if a device-side wait timed out.  workspace: gpk_gemm_tf32x3_workspace_bytes.
 * ------------------------------------------------------------------------- */
size_t gpk_gemm_tf32x3_workspace_bytes(int64_t M, int64_t N, int64_t K);
gpk_status gpk_gemm_tf32x3(int64_t M, int64_t N, int64_t K, float alpha,
                           const float* A, int64_t lda, const float* B, int64_t ldb,
                           float beta, float* C, int64_t ldc, int lower_only,
                           int* err_flag, void* workspace, size_t workspace_bytes,
                           cudaStream_t stream);

/* Self-test of the bounded device waits (no counterpart in the reference).
 * Launches one small tensor-core GEMM whose MMA thread waits on a barrier that
 * nothing arrives at, with a ~10 ms limit: the wait runs out and the kernel
 * sets *err_flag (device int) to 1 and returns, leaving the context usable --
 * the path every mbarrier wait of the library takes after its ~2 s bound.
 * workspace: gpk_selftest_wait_timeout_workspace_bytes(). */
size_t gpk_selftest_wait_timeout_workspace_bytes(void);
gpk_status gpk_selftest_wait_timeout(int* err_flag, void* workspace, size_t workspace_bytes,
                                     cudaStream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* GPK_H_ */
