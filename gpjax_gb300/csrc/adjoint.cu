// Adjoint of the exact-GP marginal log-likelihood.
//
//   d mll / d theta = 1/2 tr((alpha alpha^T - Sigma^-1) dSigma/dtheta),
//   alpha = Sigma^-1 (y - m).
//
// The reference obtains this by JAX reverse-mode through slogdet and solve
// (gpjax/objectives.py:100-107 -> distributions.py:132-134 ->
// linalg/operations.py:111,164) and the vmap'd pointwise kernel
// (computations/dense.py:35).  Here Sigma^-1 = V V^T with V = L^-T is formed
// tile by tile (the LAUUM product) and never stored: each lower tile of
// Sigma^-1 is reduced at once against dK/dtheta, whose entries are
// regenerated in registers from the scaled inputs.  Per-tile partial sums
// go to a workspace array that a single block reduces in a fixed order, so
// the gradient is deterministic.
#include "simt_tile.cuh"

namespace gpk {

// Number of float64 partial sums written per tile: d lengthscale terms,
// the variance term and the noise term.
__host__ __device__ inline int grad_slots(int d) { return d + 2; }

template <typename T, int DMAX>
__global__ void __launch_bounds__((GemmCfg<T>::BM / GemmCfg<T>::TM) * (GemmCfg<T>::BN / GemmCfg<T>::TN))
    lauum_grad_kernel(int kind, const T* __restrict__ V, int64_t ldv, int n, int d,
                      const T* __restrict__ xs, const double* __restrict__ alpha,
                      double* __restrict__ gpart, const double* __restrict__ kaptr) {
  constexpr int BM = GemmCfg<T>::BM, BN = GemmCfg<T>::BN, BK = GemmCfg<T>::BK;
  constexpr int TM = GemmCfg<T>::TM, TN = GemmCfg<T>::TN;
  constexpr int NTX = BN / TN, NTY = BM / TM, NT = NTX * NTY;
  constexpr int WLD = BN + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // main-loop staging and the W tile share the front of shared memory
  SimtSmem<T>& sm = *reinterpret_cast<SimtSmem<T>*>(smem_raw);
  T* Ws = reinterpret_cast<T*>(smem_raw);
  constexpr size_t front = sizeof(SimtSmem<T>) > sizeof(T) * BM * WLD ? sizeof(SimtSmem<T>)
                                                                       : sizeof(T) * BM * WLD;
  T* sxi = reinterpret_cast<T*>(smem_raw + ((front + 15) & ~size_t(15)));
  T* sxj = sxi + BM * DMAX;
  T* sai = sxj + BN * DMAX;
  T* saj = sai + BM;
  double* rbuf = reinterpret_cast<double*>(
      (reinterpret_cast<uintptr_t>(saj + BN) + 15) & ~static_cast<uintptr_t>(15));

  const int t = blockIdx.x;
  int I, J;
  tri_index(t, I, J);
  const int i0 = I * BM, j0 = J * BN;
  int klo, khi;
  tile_krange<BM, BN, BK>(n, TRI_UPPER, TRI_UPPER, i0, j0, klo, khi);
  T acc[TM][TN];
#pragma unroll
  for (int a = 0; a < TM; ++a)
#pragma unroll
    for (int b = 0; b < TN; ++b) acc[a][b] = T(0);
  simt_tile_mma<T>(V, ldv, n, TRI_UPPER, V, ldv, n, TRI_UPPER, i0, j0, klo, khi, sm, acc);
  // (simt_tile_mma ends with a barrier, so the staging area can be reused)
  const int tx = threadIdx.x % NTX, ty = threadIdx.x / NTX;
#pragma unroll
  for (int a = 0; a < TM; ++a)
#pragma unroll
    for (int b = 0; b < TN; ++b) Ws[(ty + a * NTY) * WLD + tx + b * NTX] = acc[a][b];
  for (int e = threadIdx.x; e < BM * DMAX; e += NT) {
    int r = e / DMAX, k = e % DMAX;
    sxi[e] = (i0 + r < n && k < d) ? xs[(int64_t)(i0 + r) * d + k] : T(0);
  }
  for (int e = threadIdx.x; e < BN * DMAX; e += NT) {
    int r = e / DMAX, k = e % DMAX;
    sxj[e] = (j0 + r < n && k < d) ? xs[(int64_t)(j0 + r) * d + k] : T(0);
  }
  for (int e = threadIdx.x; e < BM; e += NT) sai[e] = (i0 + e < n) ? (T)alpha[i0 + e] : T(0);
  for (int e = threadIdx.x; e < BN; e += NT) saj[e] = (j0 + e < n) ? (T)alpha[j0 + e] : T(0);
  __syncthreads();

  const T ka = kaptr ? (T)*kaptr : T(1);  // kernel shape parameter (rational quadratic)
  // float64 accumulators: the terms cancel heavily (the variance and noise
  // sums are differences of O(n) quantities), so per-thread sums stay exact
  // to float64 while each term is formed in T
  double gl[DMAX];
#pragma unroll
  for (int k = 0; k < DMAX; ++k) gl[k] = 0.0;
  double gvar = 0.0, gnoise = 0.0;
  // consecutive threads take consecutive columns of one row
#pragma unroll 1
  for (int e = threadIdx.x; e < BM * BN; e += NT) {
    const int r = e / BN, c = e % BN;
    const int gi = i0 + r, gj = j0 + c;
    if (gi >= n || gj >= n || gj > gi) continue;
    const T w = Ws[r * WLD + c];
    const T ai = sai[r];
    const T f = (gi == gj) ? T(1) : T(2);
    const T coef = f * (ai * saj[c] - w);
    T dsq[DMAX];
    T sq = T(0);
#pragma unroll
    for (int k = 0; k < DMAX; ++k) {
      const T df = sxi[r * DMAX + k] - sxj[c * DMAX + k];
      dsq[k] = df * df;
      sq += dsq[k];
    }
    T k1, c1;
    kval_dcoef<T>(kind, sq, T(1), k1, c1, ka);
    gvar += (double)(coef * k1);
    const T cc = coef * c1;
#pragma unroll
    for (int k = 0; k < DMAX; ++k) gl[k] += (double)(cc * dsq[k]);
    if (gi == gj) gnoise += (double)ai * (double)ai - (double)w;
  }
  // block reduction in float64, fixed order
  const int slots = grad_slots(d);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int NW = NT / 32;
#pragma unroll
  for (int k = 0; k < DMAX; ++k) {
    if (k < d) {
      const double dv = warp_sum(gl[k]);
      if (lane == 0) rbuf[k * NW + warp] = dv;
    }
  }
  {
    const double dv = warp_sum(gvar);
    if (lane == 0) rbuf[d * NW + warp] = dv;
    const double dn = warp_sum(gnoise);
    if (lane == 0) rbuf[(d + 1) * NW + warp] = dn;
  }
  __syncthreads();
  for (int s = threadIdx.x; s < slots; s += NT) {
    double tot = 0.0;
    for (int w = 0; w < NW; ++w) tot += rbuf[s * NW + w];
    gpart[(int64_t)t * slots + s] = tot;
  }
}

template <typename T, int DMAX>
static cudaError_t launch_lauum_grad(int kind, const T* V, int64_t ldv, int n, int d, const T* xs,
                                     const double* alpha, double* gpart, const double* kaptr,
                                     cudaStream_t s) {
  constexpr int BM = GemmCfg<T>::BM, BN = GemmCfg<T>::BN;
  constexpr int NT = (GemmCfg<T>::BM / GemmCfg<T>::TM) * (GemmCfg<T>::BN / GemmCfg<T>::TN);
  const int tiles_m = (n + BM - 1) / BM;
  const int tiles = tiles_m * (tiles_m + 1) / 2;
  const size_t front = sizeof(SimtSmem<T>) > sizeof(T) * BM * (BN + 1) ? sizeof(SimtSmem<T>)
                                                                          : sizeof(T) * BM * (BN + 1);
  const size_t smem = ((front + 15) & ~size_t(15)) + (size_t)(BM + BN) * DMAX * sizeof(T) +
                      (size_t)(BM + BN) * sizeof(T) + 16 +
                      (size_t)(GPK_MAX_D + 2) * (NT / 32) * sizeof(double);
  cudaFuncSetAttribute(lauum_grad_kernel<T, DMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem);
  lauum_grad_kernel<T, DMAX><<<tiles, NT, smem, s>>>(kind, V, ldv, n, d, xs, alpha, gpart,
                                                     kaptr);
  return launch_status();
}

template <typename T>
int lauum_grad_tiles(int n) {
  const int tm = (n + GemmCfg<T>::BM - 1) / GemmCfg<T>::BM;
  return tm * (tm + 1) / 2;
}
template int lauum_grad_tiles<double>(int);
template int lauum_grad_tiles<float>(int);

template <typename T>
cudaError_t lauum_grad(int kind, const T* V, int64_t ldv, int n, int d, const T* xs,
                       const double* theta, int n_ls, const double* alpha, double* gpart,
                       cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const double* ka = kind == GPK_RATIONAL_QUADRATIC ? theta + n_ls + 3 : nullptr;
  if (d <= 8) return launch_lauum_grad<T, 8>(kind, V, ldv, n, d, xs, alpha, gpart, ka, s);
  if (d <= 16) return launch_lauum_grad<T, 16>(kind, V, ldv, n, d, xs, alpha, gpart, ka, s);
  if (d <= 32) return launch_lauum_grad<T, 32>(kind, V, ldv, n, d, xs, alpha, gpart, ka, s);
  return cudaErrorInvalidValue;
}

// ---------------------------------------------------------------------------
// Residual r = diff - (K + diag_add I) alpha with K regenerated from the
// scaled inputs in T; per-chunk partial sums (RES_CHUNK columns) in T are
// accumulated in float64.  Column chunks are spread over gridDim.y and their
// partials written to rpart[y][n]; residual_finish sums them in fixed order.
// ---------------------------------------------------------------------------
constexpr int RES_ROWS = 128;
constexpr int RES_COLS = 128;
constexpr int RES_SPLIT = 16;

template <typename T, int DMAX>
__global__ void __launch_bounds__(RES_ROWS)
    residual_kernel(int kind, int n, int d, const T* __restrict__ xs,
                    const double* __restrict__ theta, int n_ls, const double* __restrict__ alpha,
                    double* __restrict__ rpart) {
  __shared__ T sx[RES_COLS][DMAX + 1];
  __shared__ T sa[RES_COLS];
  const int i = blockIdx.x * RES_ROWS + threadIdx.x;
  const T s2 = (T)theta[n_ls];
  T xi[DMAX];
#pragma unroll
  for (int k = 0; k < DMAX; ++k) xi[k] = (i < n && k < d) ? xs[(int64_t)i * d + k] : T(0);
  const int per = (n + RES_SPLIT - 1) / RES_SPLIT;
  const int cbeg = blockIdx.y * per, cend = min(n, cbeg + per);
  double accd = 0.0;
  for (int c0 = cbeg; c0 < cend; c0 += RES_COLS) {
    __syncthreads();
    for (int e = threadIdx.x; e < RES_COLS * d; e += RES_ROWS) {
      int r = e / d, k = e % d;
      sx[r][k] = (c0 + r < cend) ? xs[(int64_t)(c0 + r) * d + k] : T(0);
    }
    for (int e = threadIdx.x; e < RES_COLS; e += RES_ROWS)
      sa[e] = (c0 + e < cend) ? (T)alpha[c0 + e] : T(0);
    __syncthreads();
    const int cnt = min(RES_COLS, cend - c0);
    T part = T(0);
    for (int c = 0; c < cnt; ++c) {
      T sq = T(0);
#pragma unroll
      for (int k = 0; k < DMAX; ++k) {
        if (k < d) {
          T df = xi[k] - sx[c][k];
          sq = fma(df, df, sq);
        }
      }
      part = fma(kval<T>(kind, sq, s2, kshape<T>(kind, theta, n_ls)), sa[c], part);
    }
    accd += (double)part;
  }
  if (i < n) rpart[(int64_t)blockIdx.y * n + i] = accd;
}

__global__ void residual_finish_kernel(int n, const double* __restrict__ theta, int n_ls,
                                       double jitter, const double* __restrict__ diff,
                                       const double* __restrict__ alpha,
                                       const double* __restrict__ rpart, double* __restrict__ r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double sd = theta[n_ls + 1];
  double s = 0.0;
  for (int y = 0; y < RES_SPLIT; ++y) s += rpart[(int64_t)y * n + i];
  s += (jitter + sd * sd) * alpha[i];
  r[i] = diff[i] - s;
}

size_t residual_scratch_doubles(int n) { return (size_t)RES_SPLIT * n; }

template <typename T>
cudaError_t residual(int kind, int n, int d, const T* xs, const double* theta, int n_ls,
                     double jitter, const double* diff, const double* alpha, double* r,
                     double* rpart, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  dim3 grid((unsigned)cdiv(n, RES_ROWS), RES_SPLIT);
  if (d <= 8)
    residual_kernel<T, 8><<<grid, RES_ROWS, 0, s>>>(kind, n, d, xs, theta, n_ls, alpha, rpart);
  else if (d <= 16)
    residual_kernel<T, 16><<<grid, RES_ROWS, 0, s>>>(kind, n, d, xs, theta, n_ls, alpha, rpart);
  else if (d <= 32)
    residual_kernel<T, 32><<<grid, RES_ROWS, 0, s>>>(kind, n, d, xs, theta, n_ls, alpha, rpart);
  else
    return cudaErrorInvalidValue;
  cudaError_t e = launch_status();
  if (e != cudaSuccess) return e;
  residual_finish_kernel<<<(int)cdiv(n, 256), 256, 0, s>>>(n, theta, n_ls, jitter, diff, alpha,
                                                           rpart, r);
  return launch_status();
}

template cudaError_t lauum_grad<double>(int, const double*, int64_t, int, int, const double*,
                                        const double*, int, const double*, double*, cudaStream_t);
template cudaError_t lauum_grad<float>(int, const float*, int64_t, int, int, const float*,
                                       const double*, int, const double*, double*, cudaStream_t);
template cudaError_t residual<double>(int, int, int, const double*, const double*, int, double,
                                      const double*, const double*, double*, double*,
                                      cudaStream_t);
template cudaError_t residual<float>(int, int, int, const float*, const double*, int, double,
                                     const double*, const double*, double*, double*, cudaStream_t);

}  // namespace gpk
