// Mixed-precision exact-GP marginal log-likelihood and gradient on tcgen05.
//
// Same quantity as mll.cu (gpjax/objectives.py:93-107, its adjoint as in
// adjoint.cu) with the three O(n^3) phases on the tensor cores in split-TF32:
//
//   chol_inv(A):  [L11, M11] = chol_inv(A11)
//                 L21  = A21 M11^T          (triangular solve as a product)
//                 A22 -= L21 L21^T          (trailing update)
//                 [L22, M22] = chol_inv(A22)
//                 M21  = -M22 (L21 M11)     (inverse of the factor)
//   W = M^T M  tile by tile, reduced at once against dK/dtheta (adjoint).
//
// Every product is one split-TF32 NT GEMM (tc_gemm.cu) reading K-contiguous
// operands: L (rows), M = L^-1 and V = M^T are each kept row-major as TF32
// hi/lo pairs.  Recursion leaves are 128 x 128 diagonal blocks factored and
// inverted by one CTA in float32, with pivots from a float64 diagonal track
// (decremented by every L21 product; carried as float-float pairs inside the
// leaf).  n is padded to a multiple of
// 128 with an identity block, which leaves the factor, the inverse, the
// log-determinant and alpha of the original system unchanged.
#include <climits>
#include "tc_gemm.cuh"

namespace gpk {
namespace {

constexpr int LEAF = 128;
constexpr int LEAF_NT = 512;  // threads of the leaf kernel

constexpr int LEAF_LD = LEAF + 1;   // S / Ms row stride: odd, so column walks are conflict-free
constexpr int LEAF_PB = 32;         // panel width
constexpr int LEAF_PTLD = LEAF + 4; // k-major panel copy: 16-byte rows
constexpr int LEAF_LTLD = LEAF_PB + 4;

__device__ __forceinline__ float tf32_rna_f(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// (hi, lo) -= c * c, exact to ~2^-48 of the result: the product error comes
// from one FMA, the sum error from TwoSum, then a renormalisation.  The _rn
// intrinsics keep the compiler from contracting the steps into FMAs.
__device__ __forceinline__ void ff_sub_sq(float& hi, float& lo, float c) {
  const float p = __fmul_rn(c, c);
  const float pe = fmaf(c, c, -p);
  const float s1 = __fsub_rn(hi, p);
  const float bb = __fsub_rn(s1, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s1, bb)), __fsub_rn(-p, bb));
  const float l2 = __fadd_rn(__fsub_rn(lo, pe), err);
  const float h2 = __fadd_rn(s1, l2);
  lo = __fsub_rn(l2, __fsub_rn(h2, s1));
  hi = h2;
}

// One CTA: Cholesky of the 128 x 128 diagonal block at (o, o) by 32-wide
// panels (a warp-level register factor of the diagonal block, row substitution
// below it, a rank-32 trailing update), pivots from the float64 diagonal track
// carried as float-float pairs; the inverse from the four 32 x 32 diagonal
// inverses and two doubling merges.  Writes the M (hi/lo) and V = M^T (hi/lo)
// diagonal blocks and half the log of each pivot.
__global__ void __launch_bounds__(LEAF_NT)
    leaf_chol_inv_kernel(const float* __restrict__ A, int64_t lda, int o,
                         const double* __restrict__ dtrack, double* __restrict__ logdiag,
                         int* __restrict__ info, float* __restrict__ Mh, float* __restrict__ Ml,
                         float* __restrict__ Vh, float* __restrict__ Vl, int64_t ldm) {
  constexpr int N = LEAF, LD = LEAF_LD, NT = LEAF_NT, PB = LEAF_PB;
  static_assert(N == 128 && NT == 512, "tile maps below assume a 128-wide leaf and 512 threads");
  extern __shared__ __align__(16) float leaf_smem[];
  float* Pt = leaf_smem;              // [PB][PTLD]  rows below the panel, k-major
  float* Lt = Pt + PB * LEAF_PTLD;    // [PB][LTLD]  diagonal block of the panel, transposed
  float* S = Lt + PB * LEAF_LTLD;     // [N][LD]     A -> L (strictly lower part)
  float* Ms = S + N * LD;             // [N][LD]     M = L^-1
  float* Tt = Ms + N * LD;            // [64 * 65]   merge products
  float* Dh = Tt + 64 * 65;           // float-float diagonal track
  float* Dlo = Dh + N;
  float* Ph = Dlo + N;                // float-float pivots
  float* Pl = Ph + N;
  float* Rl = Pl + N;                 // 1 / diag(L)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // ---- load the block (32 coalesced loads in flight per thread), zero M ----
  {
    float v[N * N / NT];
#pragma unroll
    for (int u = 0; u < N * N / NT; ++u) {
      const int e = tid + u * NT;
      v[u] = A[(int64_t)(o + e / N) * lda + o + e % N];
    }
#pragma unroll
    for (int u = 0; u < N * N / NT; ++u) {
      const int e = tid + u * NT;
      S[(e / N) * LD + e % N] = v[u];
    }
  }
  for (int e = tid; e < N * LD; e += NT) Ms[e] = 0.f;
  if (tid < N) {
    const double dv = dtrack[o + tid];
    const float hi = (float)dv;
    Dh[tid] = hi;
    Dlo[tid] = (float)(dv - (double)hi);
  }
  __syncthreads();

  // ---- blocked right-looking Cholesky, 32-wide panels ----
  for (int p = 0; p < N / PB; ++p) {
    const int c0 = p * PB;
    // P1: one warp factors the diagonal block in registers (lane = row).  The
    // pivot for the next column comes from a float32 candidate one FMA away,
    // while the float-float track is updated off that dependency chain.
    if (warp == 0) {
      const int row = c0 + lane;
      float r[PB];
#pragma unroll
      for (int k = 0; k < PB; ++k) r[k] = S[row * LD + c0 + k];
      float dh = Dh[row], dlo = Dlo[row];
      float pf = dh + dlo;
#pragma unroll
      for (int j = 0; j < PB; ++j) {
        const float piv = __shfl_sync(0xffffffffu, pf, j);
        const float rl = rsqrtf(piv);
        const float lij = r[j] * rl;  // meaningful for lane > j
        if (lane == j) {
          Ph[row] = dh;
          Pl[row] = dlo;
          Rl[row] = rl;
        }
        if (lane > j) {
          r[j] = lij;
          pf = fmaf(-lij, lij, dh) + dlo;
          ff_sub_sq(dh, dlo, lij);
        }
#pragma unroll
        for (int k = j + 1; k < PB; ++k) r[k] = fmaf(-lij, __shfl_sync(0xffffffffu, lij, k), r[k]);
      }
#pragma unroll
      for (int k = 0; k < PB; ++k) {
        if (k < lane) S[row * LD + c0 + k] = r[k];
        Lt[k * LEAF_LTLD + lane] = (k < lane) ? r[k] : 0.f;  // Lt[k][i] = L[i][k]
      }
    }
    __syncthreads();
    // P2: rows below the panel by substitution, one thread per row; one warp
    // meanwhile inverts the diagonal block (lane = column).
    const int r0 = c0 + PB, R = N - r0;
    if (tid < R) {
      const int row = r0 + tid;
      float a[PB], rl[PB];
#pragma unroll
      for (int k = 0; k < PB; ++k) a[k] = S[row * LD + c0 + k];
#pragma unroll
      for (int g = 0; g < PB / 4; ++g) {
        const float4 t = *reinterpret_cast<const float4*>(Rl + c0 + 4 * g);
        rl[4 * g] = t.x;
        rl[4 * g + 1] = t.y;
        rl[4 * g + 2] = t.z;
        rl[4 * g + 3] = t.w;
      }
#pragma unroll
      for (int m = 0; m < PB; ++m) {
        const float x = a[m] * rl[m];
        a[m] = x;
#pragma unroll
        for (int g = 0; g < PB / 4; ++g) {
          if (4 * g + 3 > m) {
            const float4 l = *reinterpret_cast<const float4*>(Lt + m * LEAF_LTLD + 4 * g);
            if (4 * g + 0 > m) a[4 * g + 0] = fmaf(-x, l.x, a[4 * g + 0]);
            if (4 * g + 1 > m) a[4 * g + 1] = fmaf(-x, l.y, a[4 * g + 1]);
            if (4 * g + 2 > m) a[4 * g + 2] = fmaf(-x, l.z, a[4 * g + 2]);
            a[4 * g + 3] = fmaf(-x, l.w, a[4 * g + 3]);
          }
        }
      }
#pragma unroll
      for (int k = 0; k < PB; ++k) {
        S[row * LD + c0 + k] = a[k];
        Pt[k * LEAF_PTLD + row] = a[k];
      }
    }
    if (warp == 8) {
      const int cc = lane;
      float mc[PB];
#pragma unroll
      for (int i = 0; i < PB; ++i) {
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int k = 0; k < i; ++k) {
          const float l = Lt[k * LEAF_LTLD + i];  // L[i][k], the same for every lane
          if (k & 1)
            s1 = fmaf(l, mc[k], s1);
          else
            s0 = fmaf(l, mc[k], s0);
        }
        const float rli = Rl[c0 + i];
        mc[i] = (i < cc) ? 0.f : ((i == cc) ? rli : -rli * (s0 + s1));
      }
#pragma unroll
      for (int i = 0; i < PB; ++i) Ms[(c0 + i) * LD + c0 + cc] = mc[i];
    }
    __syncthreads();
    // P3: rank-32 update of the strictly lower trailing part from the k-major
    // copy (4 x 4 tiles, float4 operands); the float-float diagonal track
    // loses the squares of the new rows on other threads.
    if (R > 0) {
      const int T = R / 4, ntiles = T * (T + 1) / 2;
      for (int t = tid; t < ntiles; t += NT) {
        int tr = (int)((sqrtf(8.f * (float)t + 1.f) - 1.f) * 0.5f);
        while (tr * (tr + 1) / 2 > t) --tr;
        while ((tr + 1) * (tr + 2) / 2 <= t) ++tr;
        const int tc = t - tr * (tr + 1) / 2;
        const int R0 = r0 + 4 * tr, C0 = r0 + 4 * tc;
        float acc[4][4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
#pragma unroll 8
        for (int k = 0; k < PB; ++k) {
          const float4 a4 = *reinterpret_cast<const float4*>(Pt + k * LEAF_PTLD + R0);
          const float4 b4 = *reinterpret_cast<const float4*>(Pt + k * LEAF_PTLD + C0);
          const float av[4] = {a4.x, a4.y, a4.z, a4.w}, bv[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
          for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(av[u], bv[v], acc[u][v]);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v)
            if (R0 + u > C0 + v) S[(R0 + u) * LD + C0 + v] -= acc[u][v];
      }
      if (tid >= NT - R) {
        const int row = r0 + tid - (NT - R);
        float dh = Dh[row], dlo = Dlo[row];
#pragma unroll
        for (int k = 0; k < PB; ++k) ff_sub_sq(dh, dlo, Pt[k * LEAF_PTLD + row]);
        Dh[row] = dh;
        Dlo[row] = dlo;
      }
      __syncthreads();
    }
  }
  if (tid < N) {
    const double pv = (double)Ph[tid] + (double)Pl[tid];
    logdiag[o + tid] = 0.5 * log(pv);
    if (!(pv > 0.0)) atomicMin(info, o + tid + 1);
  }
  // ---- off-diagonal blocks of M by doubling merges, M21 = -M22 (L21 M11):
  //      both 32-wide pairs in one pass, then the 64-wide one; 2 x 4 tiles ----
  for (int h = PB; h < N; h *= 2) {
    const int pairs = N / (2 * h), per = (h / 2) * (h / 4), tl = h + 1;
    for (int job = tid; job < pairs * per; job += NT) {
      const int pr = job / per, b = job % per, ob = pr * 2 * h;
      const int i2 = (b / (h / 4)) * 2, j4 = (b % (h / 4)) * 4;
      float* T = Tt + pr * h * tl;
      float a0[4] = {0.f, 0.f, 0.f, 0.f}, a1[4] = {0.f, 0.f, 0.f, 0.f};
      for (int c = j4; c < h; ++c) {  // M11[c][j] = 0 for c < j
        const float l0 = S[(ob + h + i2) * LD + ob + c], l1 = S[(ob + h + i2 + 1) * LD + ob + c];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float m = Ms[(ob + c) * LD + ob + j4 + q];
          a0[q] = fmaf(l0, m, a0[q]);
          a1[q] = fmaf(l1, m, a1[q]);
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        T[i2 * tl + j4 + q] = a0[q];
        T[(i2 + 1) * tl + j4 + q] = a1[q];
      }
    }
    __syncthreads();
    for (int job = tid; job < pairs * per; job += NT) {
      const int pr = job / per, b = job % per, ob = pr * 2 * h;
      const int i2 = (b / (h / 4)) * 2, j4 = (b % (h / 4)) * 4;
      const float* T = Tt + pr * h * tl;
      float a0[4] = {0.f, 0.f, 0.f, 0.f}, a1[4] = {0.f, 0.f, 0.f, 0.f};
      for (int c = 0; c <= i2 + 1; ++c) {  // M22[i][c] = 0 for c > i
        const float m0 = Ms[(ob + h + i2) * LD + ob + h + c];
        const float m1 = Ms[(ob + h + i2 + 1) * LD + ob + h + c];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float t = T[c * tl + j4 + q];
          a0[q] = fmaf(m0, t, a0[q]);
          a1[q] = fmaf(m1, t, a1[q]);
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        Ms[(ob + h + i2) * LD + ob + j4 + q] = -a0[q];
        Ms[(ob + h + i2 + 1) * LD + ob + j4 + q] = -a1[q];
      }
    }
    __syncthreads();
  }
  // ---- write M and V = M^T as TF32 hi/lo: one warp per 32 x 32 block,
  //      lane = column (coalesced rows, conflict-free shared reads) ----
  {
    const int bi = warp >> 2, bj = warp & 3;
    const int col = bj * PB + lane;
    for (int i = 0; i < PB; ++i) {
      const int row = bi * PB + i;
      const int64_t off = (int64_t)(o + row) * ldm + o + col;
      const float m = (bj <= bi) ? Ms[row * LD + col] : 0.f;
      const float mt = (bj >= bi) ? Ms[col * LD + row] : 0.f;
      const float hi = tf32_rna_f(m), hit = tf32_rna_f(mt);
      Mh[off] = hi;
      Ml[off] = tf32_rna_f(m - hi);
      Vh[off] = hit;
      Vl[off] = tf32_rna_f(mt - hit);
    }
  }
}

size_t leaf_smem_bytes() {
  return (size_t)(LEAF_PB * LEAF_PTLD + LEAF_PB * LEAF_LTLD + 2 * LEAF * LEAF_LD + 64 * 65 + 5 * LEAF) * 4;
}

// y = op(Th + Tl) x over a triangle, float64 accumulation, one warp per row.
__global__ void gemv_split_kernel(const float* __restrict__ Th, const float* __restrict__ Tl,
                                  int64_t ld, int n, int lower, const double* __restrict__ x,
                                  double* __restrict__ y, int accumulate) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  const int c0 = lower ? 0 : i, c1 = lower ? i + 1 : n;
  const float* rh = Th + (int64_t)i * ld;
  const float* rl = Tl + (int64_t)i * ld;
  // float32 products and per-lane sums (this applies the approximate inverse
  // inside the refinement loop, whose float64 residual sets the final
  // accuracy); float64 across lanes
  float s = 0.f;
  for (int c = c0 + lane; c < c1; c += 32) s = fmaf(rh[c] + rl[c], (float)x[c], s);
  double sd = warp_sum((double)s);
  if (lane == 0) y[i] = accumulate ? y[i] + sd : sd;
}

// Identity padding of the factorisation input and the float64 diagonal.
__global__ void pad_identity_kernel(float* A, int64_t lda, int n, int npad, double* dtrack,
                                    double* vec0, double* vec1) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int pad = npad - n;
  if (e >= (int64_t)pad * npad) return;
  const int i = n + (int)(e / npad), j = (int)(e % npad);
  if (j <= i) A[(int64_t)i * lda + j] = (i == j) ? 1.f : 0.f;
  if (j == 0) {
    dtrack[i] = 1.0;
    vec0[i] = 0.0;
    vec1[i] = 0.0;
  }
}

__global__ void tc_init_info(int* info, int* err) {
  *info = INT_MAX;
  *err = 0;
}

// a device-side wait that timed out turns into info = -1 (outputs NaN)
__global__ void tc_check_err(const int* err, int* info) {
  if (*err) *info = -1;
}

__global__ void tc_diff_kernel(int n, const double* __restrict__ y, const double* __restrict__ theta,
                               int n_ls, double* __restrict__ diff) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) diff[i] = y[i] - theta[n_ls + 2];
}

struct TcChol {
  float* A;
  int64_t ld;
  float *Lh, *Ll, *Mh, *Ml, *Vh, *Vl, *SAh, *SAl, *TTh, *TTl;
  int64_t ldsa;
  TcMap mL, mM, mV, mSA, mTT;
  double *dtrack, *logdiag;
  int *info, *err;
  cudaStream_t s;
};

cudaError_t chol_inv_rec(TcChol& c, int o, int sz) {
  if (sz == LEAF) {
    leaf_chol_inv_kernel<<<1, LEAF_NT, leaf_smem_bytes(), c.s>>>(c.A, c.ld, o, c.dtrack, c.logdiag,
                                                             c.info, c.Mh, c.Ml, c.Vh, c.Vl, c.ld);
    return launch_status();
  }
  const int h = ((sz / 2 + LEAF - 1) / LEAF) * LEAF;
  const int h2 = sz - h;
  cudaError_t e = chol_inv_rec(c, o, h);
  if (e != cudaSuccess) return e;
  // A21 -> split scratch
  e = tf32_split(c.A + (int64_t)(o + h) * c.ld + o, c.ld, h2, h, c.SAh, c.SAl, c.ldsa, c.s);
  if (e != cudaSuccess) return e;
  {  // L21 = A21 M11^T, float64 diagonal track of A22
    tc::TcParams p{};
    p.M = h2;
    p.N = h;
    p.K = h;
    p.b_row0 = o;
    p.b_col0 = o;
    p.b_tri = TRI_LOWER;
    p.c0 = c.Lh;
    p.c1 = c.Ll;
    p.ldc = c.ld;
    p.c_row0 = o + h;
    p.c_col0 = o;
    p.alpha = 1.f;
    p.dtrack = c.dtrack;
    p.err = c.err;
    e = tc_gemm_run(tc::MODE_STORE_SPLIT, c.mSA, c.mM, p, 1, c.s);
    if (e != cudaSuccess) return e;
  }
  {  // A22 -= L21 L21^T (lower tiles)
    tc::TcParams p{};
    p.M = h2;
    p.N = h2;
    p.K = h;
    p.a_row0 = o + h;
    p.a_col0 = o;
    p.b_row0 = o + h;
    p.b_col0 = o;
    p.c_lower = 1;
    p.c0 = c.A;
    p.ldc = c.ld;
    p.c_row0 = o + h;
    p.c_col0 = o + h;
    p.alpha = -1.f;
    p.err = c.err;
    e = tc_gemm_run(tc::MODE_ADD_F32, c.mL, c.mL, p, 1, c.s);
    if (e != cudaSuccess) return e;
  }
  e = chol_inv_rec(c, o + h, h2);
  if (e != cudaSuccess) return e;
  {  // T^T = (L21 M11)^T ; T[i, j] = sum_c L21[i, c] V11[j, c]
    tc::TcParams p{};
    p.M = h2;
    p.N = h;
    p.K = h;
    p.a_row0 = o + h;
    p.a_col0 = o;
    p.b_row0 = o;
    p.b_col0 = o;
    p.b_tri = TRI_UPPER;
    p.t0 = c.TTh;
    p.t1 = c.TTl;
    p.ldt = c.ldsa;
    p.alpha = 1.f;
    p.err = c.err;
    e = tc_gemm_run(tc::MODE_STORE_SPLIT, c.mL, c.mV, p, 1, c.s);
    if (e != cudaSuccess) return e;
  }
  {  // M21 = -M22 T ; M21[i, j] = sum_c M22[i, c] TT[j, c]; V12 = M21^T
    tc::TcParams p{};
    p.M = h2;
    p.N = h;
    p.K = h2;
    p.a_row0 = o + h;
    p.a_col0 = o + h;
    p.a_tri = TRI_LOWER;
    p.c0 = c.Mh;
    p.c1 = c.Ml;
    p.ldc = c.ld;
    p.c_row0 = o + h;
    p.c_col0 = o;
    p.t0 = c.Vh;
    p.t1 = c.Vl;
    p.ldt = c.ld;
    p.t_row0 = o;
    p.t_col0 = o + h;
    p.alpha = -1.f;
    p.err = c.err;
    e = tc_gemm_run(tc::MODE_STORE_SPLIT, c.mM, c.mTT, p, 1, c.s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

struct TcBuffers {
  int npad;
  int64_t ld, ldsa;
  float *A, *Lh, *Ll, *Mh, *Ml, *Vh, *Vl, *SAh, *SAl, *TTh, *TTl, *xs;
  double *diff, *z, *alpha, *r, *logdiag, *dtrack, *rpart, *gpart;
  int* err;
};

size_t tc_layout(int64_t n, int d, void* ws, TcBuffers& b) {
  char* base = static_cast<char*>(ws);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    off = (off + 1023) & ~size_t(1023);
    void* p = base ? base + off : nullptr;
    off += bytes;
    return p;
  };
  b.npad = (int)(((n + LEAF - 1) / LEAF) * LEAF);
  b.ld = b.npad;
  const int hmax = ((b.npad / 2 + LEAF - 1) / LEAF) * LEAF;
  b.ldsa = hmax > 0 ? hmax : LEAF;
  const size_t nn = (size_t)b.npad * b.ld * 4;
  const size_t hh = (size_t)b.ldsa * b.ldsa * 4;
  b.A = (float*)take(nn);
  b.Lh = (float*)take(nn);
  b.Ll = (float*)take(nn);
  b.Mh = (float*)take(nn);
  b.Ml = (float*)take(nn);
  b.Vh = (float*)take(nn);
  b.Vl = (float*)take(nn);
  b.SAh = (float*)take(hh);
  b.SAl = (float*)take(hh);
  b.TTh = (float*)take(hh);
  b.TTl = (float*)take(hh);
  b.xs = (float*)take((size_t)n * d * 4);
  b.diff = (double*)take((size_t)b.npad * 8);
  b.z = (double*)take((size_t)b.npad * 8);
  b.alpha = (double*)take((size_t)b.npad * 8);
  b.r = (double*)take((size_t)b.npad * 8);
  b.logdiag = (double*)take((size_t)b.npad * 8);
  b.dtrack = (double*)take((size_t)b.npad * 8);
  b.rpart = (double*)take(residual_scratch_doubles((int)n) * 8);
  const size_t tm = (size_t)b.npad / LEAF;
  b.gpart = (double*)take(tm * (tm + 1) / 2 * (d + 2) * 8);
  b.err = (int*)take(64);
  return off + 1024;
}

}  // namespace

// float64 finalisation shared with mll.cu
cudaError_t mll_finalize_launch(int n, int d, const double* theta, int n_ls, const double* logdiag,
                                const double* diff, const double* alpha, const double* gpart,
                                int ntiles, int want_grad, double jitter, int* info,
                                double* out_mll, double* out_grad, cudaStream_t s);
void prof_mark(int k, cudaStream_t s);

size_t mll_tc_workspace_bytes(int64_t n, int d) {
  TcBuffers b;
  return tc_layout(n, d, nullptr, b);
}

bool mll_tc_supported(int d) { return d <= tc::GRAD_DMAX; }

gpk_status mll_run_tc(int kind, int n, int d, const double* x, int64_t ldx, const double* y,
                      const double* theta, int n_ls, double jitter, int refine, int want_grad,
                      double* out_mll, double* out_grad, int* info, void* ws, cudaStream_t s) {
  TcBuffers b;
  tc_layout(n, d, ws, b);
  const int np = b.npad;
  prof_mark(0, s);
  tc_init_info<<<1, 1, 0, s>>>(info, b.err);
  GPK_LAUNCH_CHECK();
  GPK_CUDA_TRY(scale_inputs<float>(x, ldx, n, d, theta, n_ls, b.xs, s));
  tc_diff_kernel<<<(int)cdiv(n, 256), 256, 0, s>>>(n, y, theta, n_ls, b.diff);
  GPK_LAUNCH_CHECK();
  GPK_CUDA_TRY(cross_cov_scaled<float, float>(kind, n, n, d, b.xs, b.xs, theta, n_ls, 1, jitter,
                                              b.A, b.ld, s));
  GPK_CUDA_TRY(sigma_diag_init(kind, n, theta, n_ls, jitter, b.dtrack, s));
  if (np > n) {
    pad_identity_kernel<<<(int)cdiv((int64_t)(np - n) * np, 256), 256, 0, s>>>(
        b.A, b.ld, n, np, b.dtrack, b.diff, b.r);
    GPK_LAUNCH_CHECK();
  }
  prof_mark(1, s);
  TcChol c;
  c.A = b.A;
  c.ld = b.ld;
  c.Lh = b.Lh;
  c.Ll = b.Ll;
  c.Mh = b.Mh;
  c.Ml = b.Ml;
  c.Vh = b.Vh;
  c.Vl = b.Vl;
  c.SAh = b.SAh;
  c.SAl = b.SAl;
  c.TTh = b.TTh;
  c.TTl = b.TTl;
  c.ldsa = b.ldsa;
  c.dtrack = b.dtrack;
  c.logdiag = b.logdiag;
  c.info = info;
  c.err = b.err;
  c.s = s;
  if (!tc_make_map(&c.mL, b.Lh, b.Ll, np, np, b.ld) || !tc_make_map(&c.mM, b.Mh, b.Ml, np, np, b.ld) ||
      !tc_make_map(&c.mV, b.Vh, b.Vl, np, np, b.ld) ||
      !tc_make_map(&c.mSA, b.SAh, b.SAl, b.ldsa, b.ldsa, b.ldsa) ||
      !tc_make_map(&c.mTT, b.TTh, b.TTl, b.ldsa, b.ldsa, b.ldsa))
    return GPK_ERR_UNSUPPORTED;
  cudaFuncSetAttribute(leaf_chol_inv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)leaf_smem_bytes());
  GPK_CUDA_TRY(chol_inv_rec(c, 0, np));
  prof_mark(2, s);
  prof_mark(3, s);
  const int gb = (int)cdiv((int64_t)np * 32, 256);
  gemv_split_kernel<<<gb, 256, 0, s>>>(b.Mh, b.Ml, b.ld, np, 1, b.diff, b.z, 0);
  GPK_LAUNCH_CHECK();
  gemv_split_kernel<<<gb, 256, 0, s>>>(b.Vh, b.Vl, b.ld, np, 0, b.z, b.alpha, 0);
  GPK_LAUNCH_CHECK();
  for (int it = 0; it < refine; ++it) {
    GPK_CUDA_TRY(residual<float>(kind, n, d, b.xs, theta, n_ls, jitter, b.diff, b.alpha, b.r,
                                 b.rpart, s));
    gemv_split_kernel<<<gb, 256, 0, s>>>(b.Mh, b.Ml, b.ld, np, 1, b.r, b.z, 0);
    GPK_LAUNCH_CHECK();
    gemv_split_kernel<<<gb, 256, 0, s>>>(b.Vh, b.Vl, b.ld, np, 0, b.z, b.alpha, 1);
    GPK_LAUNCH_CHECK();
  }
  prof_mark(4, s);
  const int tm = np / LEAF;
  const int ntiles = tm * (tm + 1) / 2;
  if (want_grad) {
    tc::TcParams p{};
    p.M = np;
    p.N = np;
    p.K = np;
    p.a_tri = TRI_UPPER;
    p.b_tri = TRI_UPPER;
    p.c_lower = 1;
    p.n_true = n;
    p.d = d;
    p.kind = kind;
    p.xs = b.xs;
    p.avec = b.alpha;
    p.gpart = b.gpart;
    p.err = b.err;
    GPK_CUDA_TRY(tc_gemm_run(tc::MODE_GRAD, c.mV, c.mV, p, 1, s));
  }
  prof_mark(5, s);
  tc_check_err<<<1, 1, 0, s>>>(b.err, info);
  GPK_LAUNCH_CHECK();
  GPK_CUDA_TRY(mll_finalize_launch(n, d, theta, n_ls, b.logdiag, b.diff, b.alpha, b.gpart, ntiles,
                                   want_grad, jitter, info, out_mll, out_grad, s));
  prof_mark(6, s);
  return GPK_OK;
}

}  // namespace gpk
