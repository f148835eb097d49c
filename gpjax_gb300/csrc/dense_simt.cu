// CUDA-core (SIMT) dense linear algebra for the float64 form and for the
// parts of the mixed form that stay off the tensor cores: a batched NT GEMM
// with triangular operand masks, the blocked right-looking Cholesky
// (diagonal block in shared memory, row-substitution panel solve, SYRK
// trailing update), the recursive triangular inverse and triangular GEMVs.
//
// The reference reaches the same arithmetic through XLA: jnp.linalg.cholesky
// (gpjax/linalg/operations.py:54-55), jsp.linalg.solve_triangular
// (operations.py:105-107) and the LU of jnp.linalg.solve / slogdet
// (operations.py:109-111,163-165).
#include "simt_tile.cuh"

namespace gpk {

// ---------------------------------------------------------------------------
// Batched NT GEMM, register-tiled.
// ---------------------------------------------------------------------------
template <typename T, typename Cfg>
__global__ void __launch_bounds__((Cfg::BM / Cfg::TM) * (Cfg::BN / Cfg::TN))
    gemm_nt_kernel(GemmProb<T> p) {
  constexpr int BM = Cfg::BM, BN = Cfg::BN, BK = Cfg::BK;
  constexpr int TM = Cfg::TM, TN = Cfg::TN;
  constexpr int NTX = BN / TN, NTY = BM / TM;
  const int z = blockIdx.z;
  const T* A = p.A + (int64_t)z * p.sA;
  const T* B = p.B + (int64_t)z * p.sB;
  T* C = p.C ? p.C + (int64_t)z * p.sC : nullptr;
  T* Ct = p.Ct ? p.Ct + (int64_t)z * p.sCt : nullptr;

  const int tilesM = (p.M + BM - 1) / BM, tilesN = (p.N + BN - 1) / BN;
  int I, J;
  const int t = blockIdx.x;
  if (p.c_lower) {
    if (t >= tilesM * (tilesM + 1) / 2) return;
    tri_index(t, I, J);
  } else {
    if (t >= tilesM * tilesN) return;
    I = t / tilesN;
    J = t % tilesN;
  }
  const int i0 = I * BM, j0 = J * BN;
  int klo, khi;
  tile_krange<BM, BN, BK>(p.K, p.a_tri, p.b_tri, i0, j0, klo, khi);

  __shared__ SimtSmem<T, Cfg> sm;
  T acc[TM][TN];
#pragma unroll
  for (int a = 0; a < TM; ++a)
#pragma unroll
    for (int b = 0; b < TN; ++b) acc[a][b] = T(0);
  simt_tile_mma<T, Cfg>(A, p.lda, p.M, p.a_tri, B, p.ldb, p.N, p.b_tri, i0, j0, klo, khi, sm,
                        acc);

  const int tx = threadIdx.x % NTX, ty = threadIdx.x / NTX;
#pragma unroll
  for (int a = 0; a < TM; ++a) {
    const int gi = i0 + ty + a * NTY;
    if (gi >= p.M) continue;
#pragma unroll
    for (int b = 0; b < TN; ++b) {
      const int gj = j0 + tx + b * NTX;
      if (gj >= p.N) continue;
      if (p.c_lower && gj > gi) continue;
      T v = p.alpha * acc[a][b];
      if (C) {
        if (p.beta != T(0)) v += p.beta * C[(int64_t)gi * p.ldc + gj];
        C[(int64_t)gi * p.ldc + gj] = v;
      }
      if (Ct) Ct[(int64_t)gj * p.ldct + gi] = v;
    }
  }
}

template <typename T, typename Cfg>
static int gemm_tiles(const GemmProb<T>& p) {
  const int tilesM = (p.M + Cfg::BM - 1) / Cfg::BM, tilesN = (p.N + Cfg::BN - 1) / Cfg::BN;
  return p.c_lower ? tilesM * (tilesM + 1) / 2 : tilesM * tilesN;
}

template <typename T, typename Cfg>
static cudaError_t gemm_nt_cfg(const GemmProb<T>& p, int batch, cudaStream_t s) {
  constexpr int NT = (Cfg::BM / Cfg::TM) * (Cfg::BN / Cfg::TN);
  dim3 grid(gemm_tiles<T, Cfg>(p), 1, batch);
  gemm_nt_kernel<T, Cfg><<<grid, NT, 0, s>>>(p);
  return launch_status();
}

constexpr int SIMT_SMALL_BELOW = 152;  // CTAs of the full-size grid (one wave)

template <typename T>
cudaError_t gemm_nt(const GemmProb<T>& p, int batch, cudaStream_t s) {
  if (p.M <= 0 || p.N <= 0 || batch <= 0) return cudaSuccess;
  // float64 only: the float32 form runs many independent GPs side by side
  // (batched MLL), where total work rather than one launch's latency counts
  if (sizeof(T) == 8 && (int64_t)gemm_tiles<T, GemmCfg<T>>(p) * batch < SIMT_SMALL_BELOW)
    return gemm_nt_cfg<T, GemmCfgSmall<T>>(p, batch, s);
  return gemm_nt_cfg<T, GemmCfg<T>>(p, batch, s);
}

// ---------------------------------------------------------------------------
// Diagonal-block Cholesky: one CTA factors the nb x nb block at (k0, k0) in
// shared memory (unblocked right-looking, two barriers per column).  Each
// pivot's square root and reciprocal are taken once, by the thread that
// finishes that diagonal entry (float64 square roots and divisions are slow
// on this part: one per thread per column dominated the block).
// ---------------------------------------------------------------------------
template <typename T, int NB>
__global__ void __launch_bounds__(512) potrf_diag_kernel(T* A, int64_t lda, int n, int k0,
                                                         double* logdiag, int* info,
                                                         const double* __restrict__ dtrack) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int LD = NB + 1;
  double* Dd = reinterpret_cast<double*>(smem_raw);  // float64 diagonal of the block
  double* Pv = Dd + NB;                              // float64 pivots
  T* S = reinterpret_cast<T*>(Pv + NB);
  T* col = S + NB * LD;
  T* dl = col + NB;   // L[j, j]
  T* rl = dl + NB;    // 1 / L[j, j]
  const int nb = min(NB, n - k0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    int i = e / nb, j = e % nb;
    if (j <= i) S[i * LD + j] = A[(int64_t)(k0 + i) * lda + k0 + j];
  }
  // NaN when the pivot is negative, as in the reference; float64 square
  // root only when the factor itself is float64
  auto pivot = [&](int j) {
    const double pivd = Dd[j];
    const T ljj = sizeof(T) == 8 ? (T)sqrt(pivd) : (T)sqrtf((float)pivd);
    Pv[j] = pivd;
    dl[j] = ljj;
    rl[j] = T(1) / ljj;
  };
  for (int i = threadIdx.x; i < nb; i += blockDim.x)
    Dd[i] = dtrack ? dtrack[k0 + i] : (double)A[(int64_t)(k0 + i) * lda + k0 + i];
  __syncthreads();
  if (threadIdx.x == 0 && nb > 0) pivot(0);
  __syncthreads();
  for (int j = 0; j < nb; ++j) {
    const T rj = rl[j];
    for (int i = j + 1 + threadIdx.x; i < nb; i += blockDim.x) {
      T v = S[i * LD + j] * rj;
      S[i * LD + j] = v;
      col[i] = v;
    }
    __syncthreads();
    for (int i = j + 1 + warp; i < nb; i += nwarps) {
      const T ci = col[i];
      for (int k = j + 1 + lane; k < i; k += 32) S[i * LD + k] -= ci * col[k];
    }
    for (int i = j + 1 + threadIdx.x; i < nb; i += blockDim.x) {
      const double c = (double)col[i];
      Dd[i] -= c * c;
      if (i == j + 1) pivot(i);  // Dd[j + 1] is final after this column
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    if (logdiag) logdiag[k0 + i] = 0.5 * log(Pv[i]);
    if (!(Pv[i] > 0.0)) atomicMin(info, k0 + i + 1);
  }
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    int i = e / nb, j = e % nb;
    T v = (j < i) ? S[i * LD + j] : (j == i ? dl[i] : T(0));
    A[(int64_t)(k0 + i) * lda + k0 + j] = v;
  }
}

// dtrack[r] -= sum_k P[r, k]^2 in float64 for the rows below the panel.
template <typename T>
__global__ void diag_track_kernel(const T* __restrict__ A, int64_t lda, int n, int r0, int k0,
                                  int nb, double* __restrict__ dtrack) {
  const int r = r0 + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= n) return;
  const T* row = A + (int64_t)r * lda + k0;
  double s = 0.0;
  for (int c = lane; c < nb; c += 32) {
    const double v = (double)row[c];
    s += v * v;
  }
  s = warp_sum(s);
  if (lane == 0) dtrack[r] -= s;
}

// Zeroes the strict upper triangle outside the diagonal blocks of width nb.
template <typename T>
__global__ void zero_upper_kernel(T* A, int64_t lda, int n, int nb) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)n * n) return;
  const int i = (int)(e / n), j = (int)(e % n);
  if (j > i && (j / nb) != (i / nb)) A[(int64_t)i * lda + j] = T(0);
}

// Panel solve, float32 form: one thread per row, 128 rows per CTA, L_kk and
// the rows staged in shared memory (the float32 form serves the batched MLL,
// where many solves run side by side).
template <typename T, int NB>
__global__ void __launch_bounds__(128) trsm_rows_thread_kernel(T* A, int64_t lda, int n, int k0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int LD = NB + 1;
  T* Ls = reinterpret_cast<T*>(smem_raw);
  T* Xs = Ls + NB * LD;
  T* rinv = Xs + 128 * LD;
  const int nb = min(NB, n - k0);
  const int r0 = k0 + nb + blockIdx.x * 128;
  const int rows = min(128, n - r0);
  if (rows <= 0) return;
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    int i = e / nb, j = e % nb;
    Ls[i * LD + j] = (j <= i) ? A[(int64_t)(k0 + i) * lda + k0 + j] : T(0);
  }
  for (int e = threadIdx.x; e < rows * nb; e += blockDim.x) {
    int r = e / nb, c = e % nb;
    Xs[r * LD + c] = A[(int64_t)(r0 + r) * lda + k0 + c];
  }
  __syncthreads();
  for (int j = threadIdx.x; j < nb; j += blockDim.x) rinv[j] = T(1) / Ls[j * LD + j];
  __syncthreads();
  if (threadIdx.x < rows) {
    T* x = Xs + threadIdx.x * LD;
    for (int j = 0; j < nb; ++j) {
      T s0 = x[j], s1 = T(0), s2 = T(0), s3 = T(0);
      const T* lj = Ls + j * LD;
      int k = 0;
      for (; k + 4 <= j; k += 4) {
        s0 -= x[k] * lj[k];
        s1 -= x[k + 1] * lj[k + 1];
        s2 -= x[k + 2] * lj[k + 2];
        s3 -= x[k + 3] * lj[k + 3];
      }
      for (; k < j; ++k) s0 -= x[k] * lj[k];
      x[j] = ((s0 + s1) + (s2 + s3)) * rinv[j];
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < rows * nb; e += blockDim.x) {
    int r = e / nb, c = e % nb;
    A[(int64_t)(r0 + r) * lda + k0 + c] = Xs[r * LD + c];
  }
}

// Panel solve, float64 form: TRSM_ROWS rows per CTA (so that a short panel
// still spreads over many SMs: float64 throughput per SM is low), eliminated
// column by column by all threads: after column j is final, every later
// column c of every row takes x[c] -= (x[j] / L[j, j]) L[c, j].  The columns
// stay unscaled until the end (one barrier per column).
constexpr int TRSM_ROWS = 32;
template <typename T, int NB>
__global__ void __launch_bounds__(256) trsm_rows_kernel(T* A, int64_t lda, int n, int k0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int LD = NB + 1;
  T* Ls = reinterpret_cast<T*>(smem_raw);
  T* Xs = Ls + NB * LD;
  T* rinv = Xs + TRSM_ROWS * LD;
  const int nb = min(NB, n - k0);
  const int r0 = k0 + nb + blockIdx.x * TRSM_ROWS;
  const int rows = min(TRSM_ROWS, n - r0);
  if (rows <= 0) return;
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    int i = e / nb, j = e % nb;
    Ls[i * LD + j] = (j <= i) ? A[(int64_t)(k0 + i) * lda + k0 + j] : T(0);
  }
  for (int e = threadIdx.x; e < rows * nb; e += blockDim.x) {
    int r = e / nb, c = e % nb;
    Xs[r * LD + c] = A[(int64_t)(r0 + r) * lda + k0 + c];
  }
  __syncthreads();
  for (int j = threadIdx.x; j < nb; j += blockDim.x) rinv[j] = T(1) / Ls[j * LD + j];
  __syncthreads();
  for (int j = 0; j + 1 < nb; ++j) {
    const int w = nb - 1 - j;  // columns j+1 .. nb-1
    const T rj = rinv[j];
    for (int e = threadIdx.x; e < rows * w; e += blockDim.x) {
      const int r = e / w, c = j + 1 + e % w;
      Xs[r * LD + c] -= (Xs[r * LD + j] * rj) * Ls[c * LD + j];
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < rows * nb; e += blockDim.x) {
    int r = e / nb, c = e % nb;
    A[(int64_t)(r0 + r) * lda + k0 + c] = Xs[r * LD + c] * rinv[c];
  }
}

template <typename T>
cudaError_t potrf_lower(T* A, int64_t lda, int n, double* logdiag, int* info, double* dtrack,
                        bool zero_upper, cudaStream_t s) {
  constexpr int NB = Blk<T>::NB;
  const size_t smem_diag = (size_t)(NB * (NB + 1) + 3 * NB) * sizeof(T) + 2 * NB * sizeof(double);
  constexpr bool f64 = sizeof(T) == 8;
  const size_t smem_trsm =
      (size_t)(NB * (NB + 1) + (f64 ? TRSM_ROWS : 128) * (NB + 1) + NB) * sizeof(T);
  cudaFuncSetAttribute(potrf_diag_kernel<T, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem_diag);
  if (f64)
    cudaFuncSetAttribute(trsm_rows_kernel<T, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem_trsm);
  else
    cudaFuncSetAttribute(trsm_rows_thread_kernel<T, NB>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_trsm);
  if (zero_upper && n > NB) {
    zero_upper_kernel<T><<<(int)cdiv((int64_t)n * n, 256), 256, 0, s>>>(A, lda, n, NB);
    cudaError_t e0 = launch_status();
    if (e0 != cudaSuccess) return e0;
  }
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int nb = min(NB, n - k0);
    potrf_diag_kernel<T, NB><<<1, 512, smem_diag, s>>>(A, lda, n, k0, logdiag, info, dtrack);
    cudaError_t e = launch_status();
    if (e != cudaSuccess) return e;
    const int rest = n - k0 - nb;
    if (rest <= 0) break;
    if (f64)
      trsm_rows_kernel<T, NB><<<(rest + TRSM_ROWS - 1) / TRSM_ROWS, 256, smem_trsm, s>>>(A, lda, n,
                                                                                       k0);
    else
      trsm_rows_thread_kernel<T, NB><<<(rest + 127) / 128, 128, smem_trsm, s>>>(A, lda, n, k0);
    e = launch_status();
    if (e != cudaSuccess) return e;
    if (dtrack) {
      diag_track_kernel<T><<<(int)cdiv((int64_t)rest * 32, 256), 256, 0, s>>>(A, lda, n, k0 + nb,
                                                                           k0, nb, dtrack);
      e = launch_status();
      if (e != cudaSuccess) return e;
    }
    GemmProb<T> p{};
    p.A = A + (int64_t)(k0 + nb) * lda + k0;
    p.B = p.A;
    p.C = A + (int64_t)(k0 + nb) * lda + k0 + nb;
    p.lda = p.ldb = p.ldc = lda;
    p.M = p.N = rest;
    p.K = nb;
    p.c_lower = 1;
    p.alpha = T(-1);
    p.beta = T(1);
    e = gemm_nt<T>(p, 1, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// ---------------------------------------------------------------------------
// Triangular inverse.  Leaves: every nb x nb diagonal block inverted by
// column-parallel forward substitution (one CTA per block).  Then pairs of
// sibling blocks are merged level by level:
//   [L11 0; L21 L22]^-1 = [M11 0; -M22 L21 M11, M22]
// as two batched NT GEMMs per level.  M (lower) and V = M^T (upper) are both
// kept row-major so that every product reads K-contiguous operands.
// ---------------------------------------------------------------------------
template <typename T, int NB>
__global__ void __launch_bounds__(NB) trtri_diag_kernel(const T* L, int64_t ldl, int n, T* M,
                                                        int64_t ldm, T* V, int64_t ldv) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int LD = NB + 1;
  T* Ls = reinterpret_cast<T*>(smem_raw);
  T* Ms = Ls + NB * LD;
  T* ri = Ms + NB * LD;  // 1 / L[i, i], one division per row
  const int k0 = blockIdx.x * NB;
  const int nb = min(NB, n - k0);
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    int i = e / nb, j = e % nb;
    Ls[i * LD + j] = (j <= i) ? L[(int64_t)(k0 + i) * ldl + k0 + j] : T(0);
  }
  __syncthreads();
  if (threadIdx.x < nb) ri[threadIdx.x] = T(1) / Ls[threadIdx.x * LD + threadIdx.x];
  __syncthreads();
  const int c = threadIdx.x;
  if (c < nb) {
    for (int i = 0; i < c; ++i) Ms[i * LD + c] = T(0);
    Ms[c * LD + c] = ri[c];
    for (int i = c + 1; i < nb; ++i) {
      T s0 = T(0), s1 = T(0);
      const T* li = Ls + i * LD;
      int k = c;
      for (; k + 2 <= i; k += 2) {
        s0 += li[k] * Ms[k * LD + c];
        s1 += li[k + 1] * Ms[(k + 1) * LD + c];
      }
      if (k < i) s0 += li[k] * Ms[k * LD + c];
      Ms[i * LD + c] = -(s0 + s1) * ri[i];
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    int i = e / nb, j = e % nb;
    M[(int64_t)(k0 + i) * ldm + k0 + j] = Ms[i * LD + j];
    V[(int64_t)(k0 + i) * ldv + k0 + j] = Ms[j * LD + i];
  }
}

template <typename T>
static cudaError_t trtri_merge(const T* L, int64_t ldl, T* M, int64_t ldm, T* V, int64_t ldv,
                               T* scratch, int o, int b, int b2, int count, cudaStream_t s) {
  // count pairs starting at offset o, each [b | b2], pair stride 2b.
  const int64_t step = 2 * (int64_t)b;
  GemmProb<T> p{};
  // T_p^T = (L21 M11)^T ; T[i,j] = sum_c L21[i,c] V11[j,c]
  p.A = L + (int64_t)(o + b) * ldl + o;
  p.lda = ldl;
  p.sA = step * ldl + step;
  p.B = V + (int64_t)o * ldv + o;
  p.ldb = ldv;
  p.sB = step * ldv + step;
  p.b_tri = TRI_UPPER;
  p.C = nullptr;
  p.Ct = scratch;
  p.ldct = b2;
  p.sCt = (int64_t)b * b;
  p.M = b2;
  p.N = b;
  p.K = b;
  p.alpha = T(1);
  p.beta = T(0);
  cudaError_t e = gemm_nt<T>(p, count, s);
  if (e != cudaSuccess) return e;
  // M21 = -M22 T ; M21[i,j] = sum_c M22[i,c] TT[j,c]; also V12 = M21^T
  GemmProb<T> q{};
  q.A = M + (int64_t)(o + b) * ldm + o + b;
  q.lda = ldm;
  q.sA = step * ldm + step;
  q.a_tri = TRI_LOWER;
  q.B = scratch;
  q.ldb = b2;
  q.sB = (int64_t)b * b;
  q.C = M + (int64_t)(o + b) * ldm + o;
  q.ldc = ldm;
  q.sC = step * ldm + step;
  q.Ct = V + (int64_t)o * ldv + o + b;
  q.ldct = ldv;
  q.sCt = step * ldv + step;
  q.M = b2;
  q.N = b;
  q.K = b2;
  q.alpha = T(-1);
  q.beta = T(0);
  return gemm_nt<T>(q, count, s);
}

template <typename T>
cudaError_t trtri_lower(const T* L, int64_t ldl, int n, T* M, int64_t ldm, T* V, int64_t ldv,
                        T* scratch, cudaStream_t s) {
  constexpr int NB = Blk<T>::NB;
  const size_t smem = (size_t)(2 * NB * (NB + 1) + NB) * sizeof(T);
  cudaFuncSetAttribute(trtri_diag_kernel<T, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem);
  const int nblk = (n + NB - 1) / NB;
  trtri_diag_kernel<T, NB><<<nblk, NB, smem, s>>>(L, ldl, n, M, ldm, V, ldv);
  cudaError_t e = launch_status();
  if (e != cudaSuccess) return e;
  for (int b = NB; b < n; b *= 2) {
    // pairs at offsets p*2b whose second block starts before n
    const int npairs = (int)((n - b + 2 * (int64_t)b - 1) / (2 * (int64_t)b));
    int full = 0;
    for (int q = 0; q < npairs; ++q)
      if ((int64_t)q * 2 * b + 2 * b <= n) ++full;
    if (full > 0) {
      e = trtri_merge<T>(L, ldl, M, ldm, V, ldv, scratch, 0, b, b, full, s);
      if (e != cudaSuccess) return e;
    }
    if (full < npairs) {
      const int o = full * 2 * b;
      const int b2 = n - o - b;
      e = trtri_merge<T>(L, ldl, M, ldm, V, ldv, scratch + (int64_t)full * b * b, o, b, b2, 1, s);
      if (e != cudaSuccess) return e;
    }
  }
  return cudaSuccess;
}

// ---------------------------------------------------------------------------
// GEMVs, float64 accumulation; one warp per row.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void gemv_tri_kernel(const T* __restrict__ A, int64_t ld, int n, int lower,
                                const double* __restrict__ x, double* __restrict__ y,
                                double alpha, int accumulate) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= n) return;
  const int i = warp;
  const int c0 = lower ? 0 : i, c1 = lower ? i + 1 : n;
  const T* row = A + (int64_t)i * ld;
  double s = 0.0;
  for (int c = c0 + lane; c < c1; c += 32) s += (double)row[c] * x[c];
  s = warp_sum(s);
  if (lane == 0) y[i] = accumulate ? y[i] + alpha * s : alpha * s;
}

template <typename T>
cudaError_t gemv_tri(const T* Tri, int64_t ld, int n, bool lower, const double* x, double* y,
                     double alpha, bool accumulate, cudaStream_t s) {
  const int threads = 256;
  const int blocks = (int)cdiv((int64_t)n * 32, threads);
  gemv_tri_kernel<T><<<blocks, threads, 0, s>>>(Tri, ld, n, lower ? 1 : 0, x, y, alpha,
                                                accumulate ? 1 : 0);
  return launch_status();
}

template <typename T>
__global__ void gemv_dense_kernel(const T* __restrict__ A, int64_t ld, int rows, int cols,
                                  const double* __restrict__ x, double* __restrict__ y) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= rows) return;
  const T* row = A + (int64_t)warp * ld;
  double s = 0.0;
  for (int c = lane; c < cols; c += 32) s += (double)row[c] * x[c];
  s = warp_sum(s);
  if (lane == 0) y[warp] = s;
}

template <typename T>
cudaError_t gemv_dense(const T* A, int64_t ld, int rows, int cols, const double* x, double* y,
                       cudaStream_t s) {
  const int threads = 256;
  const int blocks = (int)cdiv((int64_t)rows * 32, threads);
  gemv_dense_kernel<T><<<blocks, threads, 0, s>>>(A, ld, rows, cols, x, y);
  return launch_status();
}

#define GPK_INST(T)                                                                             \
  template cudaError_t gemm_nt<T>(const GemmProb<T>&, int, cudaStream_t);                       \
  template cudaError_t potrf_lower<T>(T*, int64_t, int, double*, int*, double*, bool,          \
                                      cudaStream_t);                                            \
  template cudaError_t trtri_lower<T>(const T*, int64_t, int, T*, int64_t, T*, int64_t, T*,     \
                                      cudaStream_t);                                            \
  template cudaError_t gemv_tri<T>(const T*, int64_t, int, bool, const double*, double*, double, \
                                   bool, cudaStream_t);                                         \
  template cudaError_t gemv_dense<T>(const T*, int64_t, int, int, const double*, double*,      \
                                     cudaStream_t);
GPK_INST(double)
GPK_INST(float)
#undef GPK_INST

}  // namespace gpk
