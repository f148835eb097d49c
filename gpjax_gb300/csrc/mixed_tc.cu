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
// hi/lo pairs.  The products of the wide nodes (both halves >= 2048) and the
// adjoint run as split-float16 GEMMs instead, on float16 hi/lo copies of their
// operands scaled row by row by powers of two (the epilogues undo the scales
// exactly): the same 11-bit significand at twice the MMA rate.  Recursion leaves are 128 x 128 diagonal blocks factored and
// inverted by one CTA in float32, with pivots from a float64 diagonal track
// (decremented by every L21 product; carried as float-float pairs inside the
// leaf).  n is padded to a multiple of
// 128 with an identity block, which leaves the factor, the inverse, the
// log-determinant and alpha of the original system unchanged.
#include <climits>
#include <cuda_fp16.h>
#include <mutex>
#include "tc_gemm.cuh"
#include "simt_tile.cuh"
#include "leaf_chol.cuh"

namespace gpk {
namespace {

// M rows [r0, r0+nr) x columns [c0, c0+nc) to global as TF32 hi/lo (float4 rows)
__device__ __forceinline__ void leaf_put_m(const float* Ms, int r0, int nr, int c0, int nc, int o,
                                           int64_t ldm, float* Mh, float* Ml, int t, int nth) {
  const int q4 = nc / 4;
  for (int e = t; e < nr * q4; e += nth) {
    const int i = r0 + e / q4, c = c0 + 4 * (e % q4);
    const float4 m = *reinterpret_cast<const float4*>(Ms + i * LEAF_LDT + c);
    const float4 hi = make_float4(tf32_rna_f(m.x), tf32_rna_f(m.y), tf32_rna_f(m.z), tf32_rna_f(m.w));
    const float4 lo = make_float4(tf32_rna_f(m.x - hi.x), tf32_rna_f(m.y - hi.y),
                                  tf32_rna_f(m.z - hi.z), tf32_rna_f(m.w - hi.w));
    const int64_t off = (int64_t)(o + i) * ldm + o + c;
    *reinterpret_cast<float4*>(Mh + off) = hi;
    *reinterpret_cast<float4*>(Ml + off) = lo;
  }
}

// V = M^T rows [vr0, vr0+nvr) x columns [vc0, vc0+nvc): lane = V column
// (coalesced stores), float4 reads along M rows (conflict-free)
__device__ __forceinline__ void leaf_put_v(const float* Ms, int vr0, int nvr, int vc0, int nvc,
                                           int o, int64_t ldm, float* Vh, float* Vl, int t, int nth) {
  for (int e = t; e < (nvr / 4) * nvc; e += nth) {
    const int vc = vc0 + e % nvc, vr = vr0 + 4 * (e / nvc);
    const float4 m = *reinterpret_cast<const float4*>(Ms + vc * LEAF_LDT + vr);  // M[vc][vr..]
    const float mv[4] = {m.x, m.y, m.z, m.w};
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int64_t off = (int64_t)(o + vr + u) * ldm + o + vc;
      const float hi = tf32_rna_f(mv[u]);
      Vh[off] = hi;
      Vl[off] = tf32_rna_f(mv[u] - hi);
    }
  }
}


// Writes the leaf's M blocks as TF32 hi/lo pairs and the transposed blocks of
// V = M^T likewise; the zero blocks of M and V come from leaf_zero_kernel.
struct LeafOutSplit {
  float *Mh, *Ml, *Vh, *Vl;
  int64_t ldm;
  int o;
  __device__ void put_m(const float* Ms, int r0, int nr, int c0, int nc, int t, int nth) const {
    leaf_put_m(Ms, r0, nr, c0, nc, o, ldm, Mh, Ml, t, nth);
  }
  __device__ void put_v(const float* Ms, int r0, int nr, int c0, int nc, int t, int nth) const {
    leaf_put_v(Ms, r0, nr, c0, nc, o, ldm, Vh, Vl, t, nth);
  }
};

__global__ void __launch_bounds__(LEAF_NT)
    leaf_chol_inv_kernel(const float* __restrict__ A, int64_t lda, int o,
                         const double* __restrict__ dtrack, double* __restrict__ logdiag,
                         int* __restrict__ info, float* __restrict__ Mh, float* __restrict__ Ml,
                         float* __restrict__ Vh, float* __restrict__ Vl, int64_t ldm) {
  extern __shared__ __align__(16) float leaf_smem[];
  pdl_wait();
  pdl_trigger();
  leaf_chol_inv_body(A, lda, o, dtrack, logdiag, info, LeafOutSplit{Mh, Ml, Vh, Vl, ldm, o},
                     leaf_smem);
}


// Zeros of the outputs inside every 128 x 128 diagonal block: M above and
// V = M^T below the 32-wide diagonal blocks (the leaves write the rest).
__global__ void leaf_zero_kernel(float* Mh, float* Ml, float* Vh, float* Vl, int64_t ldm) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;  // (row, float4) of one block
  if (e >= LEAF * 24) return;
  const int o = blockIdx.y * LEAF, i = e / 24, q = e % 24, bi = i / LEAF_PB;
  const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
  if (q < 24 - 8 * bi) {
    const int64_t off = (int64_t)(o + i) * ldm + o + LEAF_PB * (bi + 1) + 4 * q;
    *reinterpret_cast<float4*>(Mh + off) = z;
    *reinterpret_cast<float4*>(Ml + off) = z;
  } else {
    const int64_t off = (int64_t)(o + i) * ldm + o + 4 * (q - (24 - 8 * bi));
    *reinterpret_cast<float4*>(Vh + off) = z;
    *reinterpret_cast<float4*>(Vl + off) = z;
  }
}

// Zeros of the first off-diagonal 128 x 128 blocks outside the triangles of M
// (lower: blocks (b, b + 1)) and V (upper: blocks (b + 1, b)).  A 256-wide
// GEMM tile over a triangular B operand (L21 reads M11, T^T reads V11) masks K
// per tile, so its rows in one 128-block read the neighbouring block on the
// wrong side of the diagonal; nothing else writes there, so without this the
// products would read whatever the workspace held.
__global__ void band_zero_kernel(float* Mh, float* Ml, float* Vh, float* Vl, int64_t ldm) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;  // (row, float4) of one block
  if (e >= LEAF * (LEAF / 4)) return;
  const int b = blockIdx.y, i = e / (LEAF / 4), c = 4 * (e % (LEAF / 4));
  const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
  const int64_t om = (int64_t)(b * LEAF + i) * ldm + (b + 1) * LEAF + c;   // M[b][b + 1]
  const int64_t ov = (int64_t)((b + 1) * LEAF + i) * ldm + b * LEAF + c;   // V[b + 1][b]
  *reinterpret_cast<float4*>(Mh + om) = z;
  *reinterpret_cast<float4*>(Ml + om) = z;
  *reinterpret_cast<float4*>(Vh + ov) = z;
  *reinterpret_cast<float4*>(Vl + ov) = z;
}


// x in float32 for the triangular GEMVs (a float64 -> float32 conversion per
// matrix element would run at this part's float64 rate)
__global__ void to_f32_kernel(int n, const double* __restrict__ x, float* __restrict__ xf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) xf[i] = (float)x[i];
}

// y = op(Th + Tl) x over a triangle, float64 accumulation, one warp per row.
// float32 products and per-lane sums (this applies the approximate inverse
// inside the refinement loop, whose float64 residual sets the final accuracy);
// float64 across lanes.  The 16-byte-aligned middle of each row is read as
// float4 (four rows of loads in flight per lane), the ragged ends as scalars.
__global__ void __launch_bounds__(256)
    gemv_split_kernel(const float* __restrict__ Th, const float* __restrict__ Tl, int64_t ld,
                      int n, int lower, const float* __restrict__ x, double* __restrict__ y,
                      int accumulate) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= n) return;
  const int i = lower ? n - 1 - w : w;  // longest rows first: no long tail in the last wave
  const int c0 = lower ? 0 : i, c1 = lower ? i + 1 : n;
  const float* rh = Th + (int64_t)i * ld;
  const float* rl = Tl + (int64_t)i * ld;
  const int a0 = (c0 + 3) & ~3, a1 = c1 & ~3;  // aligned middle [a0, a1) when a0 < a1
  float s0 = 0.f, s1 = 0.f;
  for (int c = c0 + lane; c < min(a0, c1); c += 32) s0 = fmaf(rh[c] + rl[c], x[c], s0);
#pragma unroll 4
  for (int c = a0 + 4 * lane; c < a1; c += 128) {
    const float4 h = *reinterpret_cast<const float4*>(rh + c);
    const float4 l = *reinterpret_cast<const float4*>(rl + c);
    const float4 xv = *reinterpret_cast<const float4*>(x + c);
    s0 = fmaf(h.x + l.x, xv.x, s0);
    s1 = fmaf(h.y + l.y, xv.y, s1);
    s0 = fmaf(h.z + l.z, xv.z, s0);
    s1 = fmaf(h.w + l.w, xv.w, s1);
  }
  for (int c = max(a0, a1) + lane; c < c1; c += 32) s1 = fmaf(rh[c] + rl[c], x[c], s1);
  const double sd = warp_sum((double)s0 + (double)s1);
  if (lane == 0) y[i] = accumulate ? y[i] + sd : sd;
}

// Identity padding of the factorisation input and the float64 diagonal.
__global__ void pad_identity_kernel(float* A, float* Ah, float* Al, int64_t lda, int n, int npad,
                                    double* dtrack, double* vec0, double* vec1) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int pad = npad - n;
  if (e >= (int64_t)pad * npad) return;
  const int i = n + (int)(e / npad), j = (int)(e % npad);
  if (j <= i) {
    const float v = (i == j) ? 1.f : 0.f;
    A[(int64_t)i * lda + j] = v;
    Ah[(int64_t)i * lda + j] = v;
    Al[(int64_t)i * lda + j] = 0.f;
  }
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

// Gram matrix of the factorisation, mirrored: the lower triangle gets
// Sigma = K + (jitter + obs_stddev^2) I (gpjax/objectives.py:100-103), with
// its TF32 hi/lo split in Ah/Al (the L21 products read their A operand from
// there), and the strict upper triangle the same kernel values, written once
// per lower tile and transposed through shared memory (both writes
// coalesced).  The factorisation only ever touches the lower triangle, so the
// upper one still holds Sigma for the residuals of the alpha refinement.
constexpr int SG_T = 64;
// One CTA per lower 64 x 64 tile (linear lower-tile index); D bounds the input
// dimension so that the distance loop unrolls and each thread keeps its
// column point in registers.
template <int D>
__global__ void __launch_bounds__(256)
    gram_mirror_kernel(int kind, int n, int d, const float* __restrict__ xs,
                       const double* __restrict__ theta, int n_ls, double jitter,
                       float* __restrict__ A, float* __restrict__ Ah, float* __restrict__ Al,
                       int64_t lda) {
  __shared__ float sx[SG_T][D + 1];
  __shared__ float st[SG_T][SG_T + 1];
  int I, J;
  tri_index(blockIdx.x, I, J);
  const int i0 = I * SG_T, j0 = J * SG_T;
  const float s2 = (float)theta[n_ls];
  const double sd = theta[n_ls + 1];
  for (int e = threadIdx.x; e < SG_T * D; e += blockDim.x) {
    const int r = e / D, k = e % D;
    sx[r][k] = (i0 + r < n && k < d) ? xs[(int64_t)(i0 + r) * d + k] : 0.f;
  }
  const int c = threadIdx.x % SG_T, gj = j0 + c;
  float yv[D];
#pragma unroll
  for (int k = 0; k < D; ++k) yv[k] = (gj < n && k < d) ? xs[(int64_t)gj * d + k] : 0.f;
  __syncthreads();
  for (int r = threadIdx.x / SG_T; r < SG_T; r += 256 / SG_T) {
    const int gi = i0 + r;
    float kv = 0.f;
    if (gi < n && gj < n && gj <= gi) {
      float sq = 0.f;
#pragma unroll
      for (int k = 0; k < D; ++k) {
        const float df = sx[r][k] - yv[k];
        sq = fmaf(df, df, sq);
      }
      kv = kval<float>(kind, sq, s2, kshape<float>(kind, theta, n_ls));
      const float vh = tf32_rna_f(kv);
      A[(int64_t)gi * lda + gj] = kv;
      Ah[(int64_t)gi * lda + gj] = vh;
      Al[(int64_t)gi * lda + gj] = tf32_rna_f(kv - vh);
    }
    st[r][c] = kv;
  }
  __syncthreads();
  if (I == J) {
    // the diagonal gets (K + jitter) + obs_stddev^2, summed in float64 once
    // per element (inside the loop above the float64 arithmetic of a select
    // ran for every element and made this kernel float64-pipe bound)
    if (threadIdx.x < SG_T && i0 + threadIdx.x < n) {
      const int gi = i0 + threadIdx.x;
      const float v = (float)(((double)st[threadIdx.x][threadIdx.x] + jitter) + sd * sd);
      const float vh = tf32_rna_f(v);
      A[(int64_t)gi * lda + gi] = v;
      Ah[(int64_t)gi * lda + gi] = vh;
      Al[(int64_t)gi * lda + gi] = tf32_rna_f(v - vh);
    }
    for (int e = threadIdx.x; e < SG_T * SG_T; e += blockDim.x) {
      const int rr = e / SG_T, cc = e % SG_T;  // element (i0 + cc, j0 + rr) -> (j0 + rr, i0 + cc)
      const int gi = i0 + cc, gjj = j0 + rr;
      if (gi < n && gjj < gi) A[(int64_t)gjj * lda + gi] = st[cc][rr];
    }
  } else {
    for (int e = threadIdx.x; e < SG_T * SG_T; e += blockDim.x) {
      const int rr = e / SG_T, cc = e % SG_T;
      const int gi = i0 + cc, gjj = j0 + rr;
      if (gi < n && gjj < n) A[(int64_t)gjj * lda + gi] = st[cc][rr];
    }
  }
}

// Partial products of the stored strict upper triangle U of Sigma with alpha,
// one 128 x 128 tile (I <= J) per CTA: row sums U alpha into rbuf[J][i],
// column sums U^T alpha into cbuf[I][j]; float32 inside the tile, combined in
// float64 by residual_upper_finish.
constexpr int RU_T = 128;
__global__ void __launch_bounds__(256)
    residual_upper_kernel(int n, const float* __restrict__ A, int64_t lda,
                          const double* __restrict__ alpha, double* __restrict__ rbuf,
                          double* __restrict__ cbuf) {
  __shared__ float sa_row[RU_T], sa_col[RU_T];
  __shared__ float cpart[8][RU_T];
  int J, I;
  tri_index(blockIdx.x, J, I);  // upper tile (I, J), I <= J
  const int i0 = I * RU_T, j0 = J * RU_T;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int e = threadIdx.x; e < RU_T; e += blockDim.x) {
    sa_row[e] = (i0 + e < n) ? (float)alpha[i0 + e] : 0.f;
    sa_col[e] = (j0 + e < n) ? (float)alpha[j0 + e] : 0.f;
  }
  __syncthreads();
  const int cb = 4 * lane;
  float colacc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 4
  for (int rr = 0; rr < RU_T / 8; ++rr) {
    const int r = warp * (RU_T / 8) + rr, gi = i0 + r;
    float u[4] = {0.f, 0.f, 0.f, 0.f};
    if (gi < n) {
      const int64_t base = (int64_t)gi * lda + j0 + cb;
      if (j0 + cb + 3 < n) {
        const float4 v = *reinterpret_cast<const float4*>(A + base);
        u[0] = v.x;
        u[1] = v.y;
        u[2] = v.z;
        u[3] = v.w;
      } else {
        for (int q = 0; q < 4; ++q)
          if (j0 + cb + q < n) u[q] = A[base + q];
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (I == J && j0 + cb + q <= gi) u[q] = 0.f;  // strict upper only
    }
    float rp = 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      rp = fmaf(u[q], sa_col[cb + q], rp);
      colacc[q] = fmaf(u[q], sa_row[r], colacc[q]);
    }
    for (int off = 16; off > 0; off >>= 1) rp += __shfl_xor_sync(0xffffffffu, rp, off);
    if (lane == 0 && gi < n) rbuf[(int64_t)J * n + gi] = (double)rp;
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) cpart[warp][cb + q] = colacc[q];
  __syncthreads();
  for (int c = threadIdx.x; c < RU_T; c += blockDim.x) {
    if (j0 + c >= n) continue;
    double tot = 0.0;
    for (int w = 0; w < 8; ++w) tot += (double)cpart[w][c];
    cbuf[(int64_t)I * n + j0 + c] = tot;
  }
}

// r = diff - Sigma alpha: the diagonal (k(0) as the Gram kernel computes it,
// plus jitter and noise) in float64, the off-diagonal partials summed in a
// fixed order.
__global__ void residual_upper_finish(int kind, int n, const double* __restrict__ theta, int n_ls,
                                      double jitter, const double* __restrict__ diff,
                                      const double* __restrict__ alpha,
                                      const double* __restrict__ rbuf,
                                      const double* __restrict__ cbuf, double* __restrict__ r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int T = (n + RU_T - 1) / RU_T, ti = i / RU_T;
  const double sd = theta[n_ls + 1];
  const double kdiag = (double)kval<float>(kind, 0.f, (float)theta[n_ls], kshape<float>(kind, theta, n_ls));
  double s = (kdiag + (jitter + sd * sd)) * alpha[i];
  for (int J = ti; J < T; ++J) s += rbuf[(int64_t)J * n + i];
  for (int I = 0; I <= ti; ++I) s += cbuf[(int64_t)I * n + i];
  r[i] = diff[i] - s;
}

// float16 row scaling: each row's largest magnitude lands in [2^13, 2^14)
constexpr int V16_TARGET_EXP = 14;

// Rows [0, rows) of the rows x cols block at (row0, col0) of a TF32 pair
// (hi + lo, leading dimension ld) to compact float16 hi/lo [rows][cols] with
// the power-of-two row scales of v16_convert_kernel (rinv[r] = 1 / scale).
// tri = TRI_LOWER / TRI_UPPER keeps the block's lower / upper triangle and
// writes zeros elsewhere (so nothing outside the operand reaches a scale or
// a product), TRI_NONE the whole row.  One warp per row; cols % 4 == 0,
// col0 % 4 == 0.
__global__ void __launch_bounds__(256)
    split16_block_kernel(const float* __restrict__ hi, const float* __restrict__ lo, int64_t ld,
                         int row0, int col0, int rows, int cols, int tri, __half* __restrict__ dh,
                         __half* __restrict__ dl, float* __restrict__ rinv) {
  const int r = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= rows) return;
  const int cb = tri == TRI_UPPER ? r : 0;
  const int ce = tri == TRI_LOWER ? min(cols, r + 1) : cols;  // exclusive
  const int64_t o = (int64_t)(row0 + r) * ld + col0;
  float mx = 0.f;
  for (int c = (cb & ~3) + lane * 4; c < ce; c += 128) {
    const float4 h = *reinterpret_cast<const float4*>(hi + o + c);
    const float4 l = *reinterpret_cast<const float4*>(lo + o + c);
    const float v[4] = {h.x + l.x, h.y + l.y, h.z + l.z, h.w + l.w};
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (c + k >= cb && c + k < ce) mx = fmaxf(mx, fabsf(v[k]));
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  int e = 0;
  if (mx > 0.f && isfinite(mx)) frexpf(mx, &e);
  e = max(e, -100);
  const float sc = ldexpf(1.f, V16_TARGET_EXP - e);
  const int64_t d0 = (int64_t)r * cols;
  for (int c = lane * 4; c < cols; c += 128) {
    float v[4] = {0.f, 0.f, 0.f, 0.f};
    if (c + 3 >= cb && c < ce) {
      const float4 h = *reinterpret_cast<const float4*>(hi + o + c);
      const float4 l = *reinterpret_cast<const float4*>(lo + o + c);
      const float w[4] = {h.x + l.x, h.y + l.y, h.z + l.z, h.w + l.w};
#pragma unroll
      for (int k = 0; k < 4; ++k) v[k] = (c + k >= cb && c + k < ce) ? w[k] * sc : 0.f;
    }
    __half hv[4], lv[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      hv[k] = __float2half_rn(v[k]);
      lv[k] = __float2half_rn(v[k] - __half2float(hv[k]));
    }
    *reinterpret_cast<uint2*>(dh + d0 + c) = make_uint2(
        (uint32_t)__half_as_ushort(hv[0]) | ((uint32_t)__half_as_ushort(hv[1]) << 16),
        (uint32_t)__half_as_ushort(hv[2]) | ((uint32_t)__half_as_ushort(hv[3]) << 16));
    *reinterpret_cast<uint2*>(dl + d0 + c) = make_uint2(
        (uint32_t)__half_as_ushort(lv[0]) | ((uint32_t)__half_as_ushort(lv[1]) << 16),
        (uint32_t)__half_as_ushort(lv[2]) | ((uint32_t)__half_as_ushort(lv[3]) << 16));
  }
  if (lane == 0) rinv[r] = ldexpf(1.f, e - V16_TARGET_EXP);
}

constexpr int kMaxDepth = 24;  // recursion depth bound (n_pad < 128 * 2^23)
// Nodes whose halves are both at least this wide run their four products as
// split-float16 GEMMs on float16 copies of the operands (the wide-tile range).
constexpr int F16_MIN = 2048;

// float16 operand copies of one depth's nodes (compact, row-scaled):
//   a: A21, later M22     m: M11, later T^T     l: L21     v: V11
// with their inverse row scales; each array holds up to cap elements.
struct F16Set {
  __half *ah, *al, *mh, *ml, *lh, *ll, *vh, *vl;
  float *ra, *rm, *rl, *rv;
};

cudaError_t to16(const float* hi, const float* lo, int64_t ld, int row0, int col0, int rows,
                 int cols, int tri, __half* dh, __half* dl, float* rinv, cudaStream_t s) {
  split16_block_kernel<<<(unsigned)cdiv((int64_t)rows * 32, 256), 256, 0, s>>>(
      hi, lo, ld, row0, col0, rows, cols, tri, dh, dl, rinv);
  return launch_status();
}

// Look-ahead in nodes whose right half is at least LA_MIN wide: only the rows
// of L21 and the block of A22 that the right child's left half needs (its first
// hq rows and columns) stay on the critical stream.  The other rows of L21 and
// the rest of the trailing update run on a per-depth look-ahead stream while
// that left half is factored; the right child waits for them before its L21.
// (Factor at n = 16384: without look-ahead 18.51 ms; with this bound at 1024
// 18.15, 2048 18.11, 4096 18.06.)
constexpr int LA_MIN = 4096;

// Per-depth look-ahead streams (priority between the critical stream and the
// side stream) and their events; created on first use and kept.
struct LookAhead {
  cudaStream_t s[kMaxDepth] = {};
  cudaEvent_t fork[kMaxDepth] = {}, fork2[kMaxDepth] = {}, mid[kMaxDepth] = {},
              done[kMaxDepth] = {};
};

cudaError_t la_streams(LookAhead& L, int depth) {
  if (L.s[depth]) return cudaSuccess;
  int least = 0, greatest = 0;
  cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
  for (cudaEvent_t* ev : {&L.fork[depth], &L.fork2[depth], &L.mid[depth], &L.done[depth]})
    if (e == cudaSuccess && !*ev) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
  // numerically lower is more urgent: one step below the critical stream
  const int prio = greatest < least ? greatest + 1 : greatest;
  if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&L.s[depth], cudaStreamNonBlocking, prio);
  return e;
}

struct TcChol {
  float* A;
  int64_t ld;
  float *Lh, *Ll, *Mh, *Ml, *Vh, *Vl, *Ah, *Al;
  TcMap mL, mM, mV, mA;  // mA: the TF32 split copy of the trailing matrix
  TcMap mTT[kMaxDepth];  // T^T scratch, one per depth: TT(node) lives until M21(node)
  float *TTh[kMaxDepth], *TTl[kMaxDepth];
  int64_t ldtt[kMaxDepth];
  double *dtrack, *logdiag;
  int *info, *err;
  cudaStream_t s;     // the factor's critical path
  cudaStream_t side;  // T^T = (L21 M11)^T products, overlapped with the right subtree
  cudaEvent_t efork, ejoin;
  bool prev_kernel;   // the last operation enqueued on s was a kernel launch (PDL allowed)
  F16Set f16[kMaxDepth];
  int nf16;           // depths [0, nf16) have float16 buffers
  LookAhead* la;      // null: no look-ahead
};

// A node of size sz at depth `depth`: [L11, M11] = chol_inv(A11) (left, size h),
// L21 = A21 M11^T, A22 -= L21 L21^T, [L22, M22] = chol_inv(A22) (right), and
// M21 = -M22 T with T = L21 M11.  T^T only needs L21 and the left child, so it
// runs on the side stream while the right subtree is factored; M21 waits for it.
// Nodes whose halves are at most this wide run T^T inline (factor at n =
// 16384 with the fork after the trailing update: 0 -> 18.8 ms, 128 -> 18.5,
// 512 -> 18.0; with the fork before it: 0 -> 20.9, 128 -> 20.7, 512 -> 20.1,
// 1024 -> 20.3, 4096 -> 21.0, measured before the float16 wide nodes).
constexpr int TT_INLINE_MAX = 512;
cudaError_t chol_inv_rec(TcChol& c, int o, int sz, int depth, cudaEvent_t join = nullptr) {
  if (sz == LEAF) {
    PdlAttr attr(c.prev_kernel);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(1);
    cfg.blockDim = dim3(LEAF_NT);
    cfg.dynamicSmemBytes = leaf_smem_bytes();
    cfg.stream = c.s;
    cfg.attrs = attr.a;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, leaf_chol_inv_kernel, (const float*)c.A, c.ld, o,
                       (const double*)c.dtrack, c.logdiag, c.info, c.Mh, c.Ml, c.Vh, c.Vl, c.ld);
    c.prev_kernel = true;
    return launch_status();
  }
  const int h = ((sz / 2 + LEAF - 1) / LEAF) * LEAF;
  const int h2 = sz - h;
  cudaError_t e = chol_inv_rec(c, o, h, depth + 1);
  if (e != cudaSuccess) return e;
  if (join) {  // the parent's look-ahead work on this node's A21 and A22
    e = cudaStreamWaitEvent(c.s, join, 0);
    c.prev_kernel = false;
    if (e != cudaSuccess) return e;
  }
  // wide nodes: split-float16 products on row-scaled float16 copies
  const bool f16 = h2 >= F16_MIN && depth < c.nf16;
  F16Set* f = f16 ? &c.f16[depth] : nullptr;
  TcMap fa, fm, fl, fv;  // float16 maps of this node's operand copies
  // look-ahead: rows [0, hq) of L21 and A22 are the right child's left half
  const bool la = c.la && h2 >= LA_MIN;
  const int hq = la ? ((h2 / 2 + LEAF - 1) / LEAF) * LEAF : h2;
  const int hb = h2 - hq;
  cudaStream_t ls = nullptr;
  if (la) {
    e = la_streams(*c.la, depth);
    if (e != cudaSuccess) return e;
    ls = c.la->s[depth];
  }
  if (f16) {
    e = to16(c.Mh, c.Ml, c.ld, o, o, h, h, TRI_LOWER, f->mh, f->ml, f->rm, c.s);
    if (e != cudaSuccess) return e;
    c.prev_kernel = true;
    if (!tc_make_map_f16(&fa, f->ah, f->al, h2, h, h) ||
        !tc_make_map_f16(&fm, f->mh, f->ml, h, h, h) ||
        !tc_make_map_f16(&fl, f->lh, f->ll, h2, h, h))
      return cudaErrorInvalidValue;
  }
  // L21 = A21 M11^T on rows [r0, r0 + rows), float64 diagonal track of A22
  auto l21 = [&](int r0, int rows, cudaStream_t st, bool pdl) -> cudaError_t {
    tc::TcParams p{};
    p.M = rows;
    p.N = h;
    p.K = h;
    p.a_row0 = o + h + r0;  // A21 in the split copy of the trailing matrix
    p.a_col0 = o;
    p.b_row0 = o;
    p.b_col0 = o;
    p.b_tri = TRI_LOWER;
    p.c0 = c.Lh;
    p.c1 = c.Ll;
    p.ldc = c.ld;
    p.c_row0 = o + h + r0;
    p.c_col0 = o;
    p.alpha = 1.f;
    p.dtrack = c.dtrack;
    p.err = c.err;
    if (!f16) return tc_gemm_run(tc::MODE_STORE_SPLIT, c.mA, c.mM, p, 1, st, pdl);
    const int64_t d0 = (int64_t)r0 * h;
    cudaError_t ee = to16(c.Ah, c.Al, c.ld, o + h + r0, o, rows, h, TRI_NONE, f->ah + d0,
                          f->al + d0, f->ra + r0, st);
    if (ee != cudaSuccess) return ee;
    p.a_row0 = r0;
    p.a_col0 = p.b_row0 = p.b_col0 = 0;
    p.force_shape = 4;
    p.ra = f->ra + r0;
    p.rb = f->rm;
    ee = tc_gemm_run(tc::MODE_STORE_SPLIT, fa, fm, p, 1, st, true);
    if (ee == cudaSuccess)
      ee = to16(c.Lh, c.Ll, c.ld, o + h + r0, o, rows, h, TRI_NONE, f->lh + d0, f->ll + d0,
                f->rl + r0, st);
    return ee;
  };
  // A22 -= L21 L21^T on rows [r0, r0 + rows) x columns [c0, c0 + cols) of A22
  // (lower tiles only when the block straddles the diagonal)
  auto update = [&](int r0, int rows, int c0, int cols, int lower, cudaStream_t st,
                    bool pdl) -> cudaError_t {
    tc::TcParams p{};
    p.M = rows;
    p.N = cols;
    p.K = h;
    p.a_row0 = o + h + r0;
    p.a_col0 = o;
    p.b_row0 = o + h + c0;
    p.b_col0 = o;
    p.c_lower = lower;
    p.c0 = c.A;
    p.s0 = c.Ah;  // TF32 split copy of the updated A22
    p.s1 = c.Al;
    p.ldc = c.ld;
    p.c_row0 = o + h + r0;
    p.c_col0 = o + h + c0;
    p.alpha = -1.f;
    p.err = c.err;
    if (!f16) return tc_gemm_run(tc::MODE_ADD_F32, c.mL, c.mL, p, 1, st, pdl);
    p.a_row0 = r0;
    p.b_row0 = c0;
    p.a_col0 = p.b_col0 = 0;
    p.force_shape = 4;
    p.ra = f->rl + r0;
    p.rb = f->rl + c0;
    return tc_gemm_run(tc::MODE_ADD_F32, fl, fl, p, 1, st, pdl);
  };
  if (la) {  // the rest of L21 on the look-ahead stream, beside its first rows
    e = cudaEventRecord(c.la->fork[depth], c.s);
    c.prev_kernel = false;
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ls, c.la->fork[depth], 0);
    if (e == cudaSuccess) e = l21(hq, hb, ls, false);
    if (e == cudaSuccess) e = cudaEventRecord(c.la->mid[depth], ls);
    if (e != cudaSuccess) return e;
  }
  e = l21(0, hq, c.s, c.prev_kernel);
  c.prev_kernel = true;
  if (e != cudaSuccess) return e;
  if (la) {  // the trailing update below the right child's left half, look-ahead stream
    e = cudaEventRecord(c.la->fork2[depth], c.s);
    c.prev_kernel = false;
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ls, c.la->fork2[depth], 0);
    if (e == cudaSuccess) e = update(hq, hb, 0, hq, 0, ls, false);
    if (e == cudaSuccess) e = update(hq, hb, hq, hb, 1, ls, true);
    if (e == cudaSuccess) e = cudaEventRecord(c.la->done[depth], ls);
    if (e != cudaSuccess) return e;
  }
  // T^T = (L21 M11)^T; T[i, j] = sum_c L21[i, c] V11[j, c].  Large nodes run it
  // on the side stream beside the trailing update and the right recursion;
  // small ones inline, where the fork and join events would cost the next
  // launches on the critical path their programmatic-dependent overlap.
  const bool tt_inline = h <= TT_INLINE_MAX;
  // T^T: inline before the trailing update, or on the side stream forked after
  // it (so that the update keeps its programmatic-dependent launch)
  auto tt = [&]() -> cudaError_t {
    if (!tt_inline) {
      cudaError_t ee = cudaEventRecord(c.efork, c.s);
      c.prev_kernel = false;
      if (ee == cudaSuccess) ee = cudaStreamWaitEvent(c.side, c.efork, 0);
      if (ee == cudaSuccess && la) ee = cudaStreamWaitEvent(c.side, c.la->mid[depth], 0);
      if (ee != cudaSuccess) return ee;
    }
    tc::TcParams p{};
    p.M = h2;
    p.N = h;
    p.K = h;
    p.a_row0 = o + h;
    p.a_col0 = o;
    p.b_row0 = o;
    p.b_col0 = o;
    p.b_tri = TRI_UPPER;
    p.t0 = c.TTh[depth];
    p.t1 = c.TTl[depth];
    p.ldt = c.ldtt[depth];
    p.alpha = 1.f;
    p.err = c.err;
    if (f16) {  // (never inline: h > TT_INLINE_MAX) V11 and T^T to float16 on the side
      e = to16(c.Vh, c.Vl, c.ld, o, o, h, h, TRI_UPPER, f->vh, f->vl, f->rv, c.side);
      if (e == cudaSuccess && !tc_make_map_f16(&fv, f->vh, f->vl, h, h, h))
        e = cudaErrorInvalidValue;
      if (e != cudaSuccess) return e;
      p.a_row0 = p.a_col0 = p.b_row0 = p.b_col0 = 0;
      p.force_shape = 4;
      p.ra = f->rl;
      p.rb = f->rv;
      e = tc_gemm_run(tc::MODE_STORE_SPLIT, fl, fv, p, 1, c.side);
      if (e == cudaSuccess)  // T^T (h x h2) into the M11 copy's storage, now free
        e = to16(c.TTh[depth], c.TTl[depth], c.ldtt[depth], 0, 0, h, h2, TRI_NONE, f->mh,
                 f->ml, f->rm, c.side);
      if (e == cudaSuccess) e = cudaEventRecord(c.ejoin, c.side);
    } else if (tt_inline) {
      e = tc_gemm_run(tc::MODE_STORE_SPLIT, c.mL, c.mV, p, 1, c.s, c.prev_kernel);
      c.prev_kernel = true;
    } else {
      e = tc_gemm_run(tc::MODE_STORE_SPLIT, c.mL, c.mV, p, 1, c.side);
      if (e == cudaSuccess) e = cudaEventRecord(c.ejoin, c.side);
    }
    return e;
  };
  if (tt_inline) {
    e = tt();
    if (e != cudaSuccess) return e;
  }
  // A22 -= L21 L21^T: the whole lower triangle, or with look-ahead its block
  // [0, hq) x [0, hq) only
  e = update(0, hq, 0, hq, 1, c.s, c.prev_kernel);
  c.prev_kernel = true;
  if (e != cudaSuccess) return e;
  if (!tt_inline) {
    e = tt();
    if (e != cudaSuccess) return e;
  }
  e = chol_inv_rec(c, o + h, h2, depth + 1, la ? c.la->done[depth] : nullptr);
  if (e != cudaSuccess) return e;
  if (f16) {  // M22 into the A21 copy's storage (free since L21)
    e = to16(c.Mh, c.Ml, c.ld, o + h, o + h, h2, h2, TRI_LOWER, f->ah, f->al, f->ra, c.s);
    if (e == cudaSuccess && (!tc_make_map_f16(&fa, f->ah, f->al, h2, h2, h2) ||
                             !tc_make_map_f16(&fm, f->mh, f->ml, h, h2, h2)))
      e = cudaErrorInvalidValue;
    if (e != cudaSuccess) return e;
    c.prev_kernel = true;
  }
  if (!tt_inline) {
    // the latest T^T on the side stream is this node's or a later one:
    // either way this node's is complete when it is
    e = cudaStreamWaitEvent(c.s, c.ejoin, 0);
    c.prev_kernel = false;
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
    if (f16) {
      p.a_row0 = p.a_col0 = p.b_row0 = p.b_col0 = 0;
      p.force_shape = 4;
      p.ra = f->ra;
      p.rb = f->rm;
      e = tc_gemm_run(tc::MODE_STORE_SPLIT, fa, fm, p, 1, c.s, c.prev_kernel);
    } else {
      e = tc_gemm_run(tc::MODE_STORE_SPLIT, c.mM, c.mTT[depth], p, 1, c.s, c.prev_kernel);
    }
    c.prev_kernel = true;
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// V (TF32 hi + lo, upper triangular) -> float16 hi/lo with a power-of-two
// scale per row that brings the row's largest magnitude into [2^13, 2^14):
// float16 then keeps an 11-bit significand for every entry down to ~2^-17 of
// the row maximum (smaller ones lose relative precision but not absolute), and
// the split pair carries ~22 bits like the TF32 split.  One warp per row; row r
// is converted from column 128 * (r / 128) on, the part the adjoint reads for
// outputs it keeps.  vscale[r] = 1 / scale (the epilogue's exact undo).
__global__ void __launch_bounds__(256)
    v16_convert_kernel(int np, const float* __restrict__ Vh, const float* __restrict__ Vl,
                       int64_t ld, __half* __restrict__ Hh, __half* __restrict__ Hl,
                       float* __restrict__ vscale) {
  const int r = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= np) return;
  const int c0 = (r / LEAF) * LEAF;
  const int64_t o = (int64_t)r * ld;
  float mx = 0.f;
  for (int c = c0 + lane * 4; c < np; c += 128) {
    const float4 h = *reinterpret_cast<const float4*>(Vh + o + c);
    const float4 l = *reinterpret_cast<const float4*>(Vl + o + c);
    mx = fmaxf(mx, fmaxf(fmaxf(fabsf(h.x + l.x), fabsf(h.y + l.y)),
                         fmaxf(fabsf(h.z + l.z), fabsf(h.w + l.w))));
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  int e = 0;
  if (mx > 0.f && isfinite(mx)) frexpf(mx, &e);  // mx = f * 2^e, f in [0.5, 1)
  e = max(e, -100);  // keeps both scales finite
  const float sc = ldexpf(1.f, V16_TARGET_EXP - e), inv = ldexpf(1.f, e - V16_TARGET_EXP);
  for (int c = c0 + lane * 4; c < np; c += 128) {
    const float4 h = *reinterpret_cast<const float4*>(Vh + o + c);
    const float4 l = *reinterpret_cast<const float4*>(Vl + o + c);
    const float v[4] = {(h.x + l.x) * sc, (h.y + l.y) * sc, (h.z + l.z) * sc, (h.w + l.w) * sc};
    __half hv[4], lv[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      hv[k] = __float2half_rn(v[k]);
      lv[k] = __float2half_rn(v[k] - __half2float(hv[k]));
    }
    *reinterpret_cast<uint2*>(Hh + o + c) = make_uint2(
        (uint32_t)__half_as_ushort(hv[0]) | ((uint32_t)__half_as_ushort(hv[1]) << 16),
        (uint32_t)__half_as_ushort(hv[2]) | ((uint32_t)__half_as_ushort(hv[3]) << 16));
    *reinterpret_cast<uint2*>(Hl + o + c) = make_uint2(
        (uint32_t)__half_as_ushort(lv[0]) | ((uint32_t)__half_as_ushort(lv[1]) << 16),
        (uint32_t)__half_as_ushort(lv[2]) | ((uint32_t)__half_as_ushort(lv[3]) << 16));
  }
  if (lane == 0) vscale[r] = inv;
}

struct TcBuffers {
  int npad;
  int64_t ld;
  float *A, *Ah, *Al, *Lh, *Ll, *Mh, *Ml, *Vh, *Vl, *xs, *vf;
  __half *V16h, *V16l;  // row-scaled float16 hi/lo of V (the adjoint's operand)
  float* vscale;        // inverse power-of-two row scales of V16
  float *TTh[kMaxDepth], *TTl[kMaxDepth];
  int64_t ldtt[kMaxDepth];
  int ndepth;
  F16Set f16[kMaxDepth];  // float16 operand copies of the wide nodes, per depth
  int nf16;
  double *diff, *z, *alpha, *r, *logdiag, *dtrack, *rpart, *gpart, *rbuf, *cbuf, *fin;
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
  const size_t nn = (size_t)b.npad * b.ld * 4;
  b.A = (float*)take(nn);
  b.Ah = (float*)take(nn);
  b.Al = (float*)take(nn);
  b.Lh = (float*)take(nn);
  b.Ll = (float*)take(nn);
  b.Mh = (float*)take(nn);
  b.Ml = (float*)take(nn);
  b.Vh = (float*)take(nn);
  b.Vl = (float*)take(nn);
  b.V16h = (__half*)take(nn / 2);
  b.V16l = (__half*)take(nn / 2);
  b.vscale = (float*)take((size_t)b.npad * 4);
  // T^T at depth k is at most s_{k+1} x s_{k+1}, s_0 = n_pad, s_{k+1} = ceil128(s_k / 2)
  b.ndepth = 0;
  for (int64_t sk = b.npad; sk > LEAF && b.ndepth < kMaxDepth; ++b.ndepth) {
    sk = ((sk / 2 + LEAF - 1) / LEAF) * LEAF;
    b.ldtt[b.ndepth] = sk;
    b.TTh[b.ndepth] = (float*)take((size_t)sk * sk * 4);
    b.TTl[b.ndepth] = (float*)take((size_t)sk * sk * 4);
  }
  // float16 copies for the depths whose nodes can have both halves >= F16_MIN:
  // a node of size s at depth k has halves at most h_k = ceil128(s_k / 2)
  b.nf16 = 0;
  for (int64_t sk = b.npad; b.nf16 < kMaxDepth; ++b.nf16) {
    const int64_t hk = ((sk / 2 + LEAF - 1) / LEAF) * LEAF;
    if (sk - hk < F16_MIN) break;
    const size_t cap = (size_t)hk * hk;
    F16Set& f = b.f16[b.nf16];
    f.ah = (__half*)take(cap * 2);
    f.al = (__half*)take(cap * 2);
    f.mh = (__half*)take(cap * 2);
    f.ml = (__half*)take(cap * 2);
    f.lh = (__half*)take(cap * 2);
    f.ll = (__half*)take(cap * 2);
    f.vh = (__half*)take(cap * 2);
    f.vl = (__half*)take(cap * 2);
    f.ra = (float*)take((size_t)hk * 4);
    f.rm = (float*)take((size_t)hk * 4);
    f.rl = (float*)take((size_t)hk * 4);
    f.rv = (float*)take((size_t)hk * 4);
    sk = hk;
  }
  b.xs = (float*)take((size_t)n * d * 4);
  b.vf = (float*)take((size_t)b.npad * 4);
  b.diff = (double*)take((size_t)b.npad * 8);
  b.z = (double*)take((size_t)b.npad * 8);
  b.alpha = (double*)take((size_t)b.npad * 8);
  b.r = (double*)take((size_t)b.npad * 8);
  b.logdiag = (double*)take((size_t)b.npad * 8);
  b.dtrack = (double*)take((size_t)b.npad * 8);
  b.rpart = (double*)take(residual_scratch_doubles((int)n) * 8);
  b.rbuf = (double*)take((size_t)(b.npad / LEAF) * n * 8);  // residual partials, by tile
  b.cbuf = (double*)take((size_t)(b.npad / LEAF) * n * 8);
  b.fin = (double*)take(mll_finalize_scratch_doubles(d) * 8);
  const size_t tm = (size_t)b.npad / LEAF;
  b.gpart = (double*)take(tm * (tm + 1) / 2 * (d + 2) * 8);  // one row per adjoint tile
  b.err = (int*)take(64);
  return off + 1024;
}

}  // namespace

// float64 finalisation shared with mll.cu
cudaError_t mll_finalize_launch(int n, int d, const double* theta, int n_ls, const double* logdiag,
                                const double* diff, const double* alpha, const double* gpart,
                                int ntiles, int want_grad, double jitter, int* info,
                                double* out_mll, double* out_grad, cudaStream_t s,
                                double* scratch);
void prof_mark(int k, cudaStream_t s);

namespace {
struct SideCtx {
  cudaStream_t hp = nullptr;    // highest priority: the critical path
  cudaStream_t side = nullptr;  // lowest priority: work that fills idle SMs
  cudaEvent_t estart = nullptr, efork = nullptr, ejoin = nullptr, edone = nullptr;
  LookAhead la;                 // the recursion's look-ahead streams
};
constexpr int kMaxDevices = 64;
std::mutex g_side_mu;
SideCtx g_side[kMaxDevices];

// Created once per device and kept: two non-blocking streams at the ends of
// the device's priority range (pending blocks of the high-priority stream are
// dispatched first as SMs free up, so overlapped work only fills what the
// critical path leaves idle) and the fork / join events (timing disabled).
cudaError_t side_ctx(SideCtx** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  SideCtx& sc = g_side[dev];
  if (!sc.side) {
    int least = 0, greatest = 0;
    e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&sc.hp, cudaStreamNonBlocking, greatest);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&sc.side, cudaStreamNonBlocking, least);
    for (cudaEvent_t* ev : {&sc.estart, &sc.efork, &sc.ejoin, &sc.edone})
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    if (e != cudaSuccess) return e;
  }
  *out = &sc;
  return cudaSuccess;
}
}  // namespace

// Predictive mean and variance on the factor of the mixed form
// (ConjugatePosterior.predict, gpjax/gps.py:443-526, without the full
// covariance): Ktx in TF32 hi/lo, Q^T = Ktx M^T as one split-TF32 GEMM whose
// epilogue only sums the squares of each row of Q^T (the float64 diagonal
// track, nothing stored), mean = m + Ktx alpha with the refined alpha.
struct TcPredict {
  int t;
  const double* xt;
  int64_t ldxt;
  double prior_jitter;
  double* mean;
  double* var;
  float *Kh, *Kl, *ts;  // [t_pad][np] x 2, [t][d]
  double* vacc;         // [t_pad]: minus the row sums of squares of Q^T
};

__global__ void pred_tc_info_kernel(int* info) {
  if (*info == INT_MAX) *info = 0;
}

size_t predict_tc_extra_bytes(int64_t np, int64_t t, int d) {
  const int64_t tp = ((t + LEAF - 1) / LEAF) * LEAF;
  return 2 * (size_t)tp * np * sizeof(float) + (size_t)t * d * sizeof(float) +
         (size_t)tp * sizeof(double) + 4 * 1024;
}

// Kh/Kl[i][k] = TF32 split of k(t_i, x_k) for i < t, k < n; zeros elsewhere
__global__ void __launch_bounds__(256)
    ktx_split_kernel(int kind, int t, int tp, int n, int np, int d, const float* __restrict__ ts,
                     const float* __restrict__ xs, const double* __restrict__ theta, int n_ls,
                     float* __restrict__ Kh, float* __restrict__ Kl) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)tp * np) return;
  const int i = (int)(e / np), k = (int)(e % np);
  float v = 0.f;
  if (i < t && k < n) {
    float sq = 0.f;
    for (int c = 0; c < d; ++c) {
      const float df = ts[(int64_t)i * d + c] - xs[(int64_t)k * d + c];
      sq = fmaf(df, df, sq);
    }
    v = kval<float>(kind, sq, (float)theta[n_ls], kshape<float>(kind, theta, n_ls));
  }
  const float hi = tf32_rna_f(v);
  Kh[e] = hi;
  Kl[e] = tf32_rna_f(v - hi);
}

// mean_i = m + sum_k Ktx[i][k] alpha_k (float64 sums), var_i = s2 + prior
// jitter - |Q^T row i|^2; NaN when the factorisation failed
__global__ void __launch_bounds__(256)
    pred_tc_finish_kernel(int t, int n, int np, const float* __restrict__ Kh,
                          const float* __restrict__ Kl, const double* __restrict__ alpha,
                          const double* __restrict__ vacc, const double* __restrict__ theta,
                          int n_ls, double prior_jitter, const int* __restrict__ info,
                          double* __restrict__ mean, double* __restrict__ var) {
  const int i = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= t) return;
  double s = 0.0;
  for (int k = lane; k < n; k += 32)
    s += ((double)Kh[(int64_t)i * np + k] + (double)Kl[(int64_t)i * np + k]) * alpha[k];
  s = warp_sum(s);
  if (lane == 0) {
    const bool bad = *info != 0 && *info != INT_MAX;
    const double nan = __longlong_as_double(0x7ff8000000000000ULL);
    mean[i] = bad ? nan : theta[n_ls + 2] + s;
    var[i] = bad ? nan : theta[n_ls] + prior_jitter + vacc[i];
  }
}

size_t mll_tc_workspace_bytes(int64_t n, int d) {
  TcBuffers b;
  return tc_layout(n, d, nullptr, b);
}

bool mll_tc_supported(int d) { return d <= tc::GRAD_DMAX; }

gpk_status mll_run_tc(int kind, int n, int d, const double* x, int64_t ldx, const double* y,
                      const double* theta, int n_ls, double jitter, int refine, int want_grad,
                      double* out_mll, double* out_grad, int* info, void* ws, cudaStream_t s,
                      const TcPredict* pred) {
  TcBuffers b;
  tc_layout(n, d, ws, b);
  const int np = b.npad;
  prof_mark(0, s);
  tc_init_info<<<1, 1, 0, s>>>(info, b.err);
  GPK_LAUNCH_CHECK();
  GPK_CUDA_TRY(scale_inputs<float>(x, ldx, n, d, theta, n_ls, b.xs, s));
  tc_diff_kernel<<<(int)cdiv(n, 256), 256, 0, s>>>(n, y, theta, n_ls, b.diff);
  GPK_LAUNCH_CHECK();
  {
    const int64_t tt = cdiv(n, SG_T);
    const unsigned grid = (unsigned)(tt * (tt + 1) / 2);  // lower tiles
    if (d <= 8)
      gram_mirror_kernel<8><<<grid, 256, 0, s>>>(kind, n, d, b.xs, theta, n_ls, jitter, b.A, b.Ah,
                                                 b.Al, b.ld);
    else if (d <= 16)
      gram_mirror_kernel<16><<<grid, 256, 0, s>>>(kind, n, d, b.xs, theta, n_ls, jitter, b.A,
                                                  b.Ah, b.Al, b.ld);
    else
      gram_mirror_kernel<GPK_MAX_D><<<grid, 256, 0, s>>>(kind, n, d, b.xs, theta, n_ls, jitter,
                                                         b.A, b.Ah, b.Al, b.ld);
    GPK_LAUNCH_CHECK();
  }
  GPK_CUDA_TRY(sigma_diag_init(kind, n, theta, n_ls, jitter, b.dtrack, s));
  if (np > n) {
    pad_identity_kernel<<<(int)cdiv((int64_t)(np - n) * np, 256), 256, 0, s>>>(
        b.A, b.Ah, b.Al, b.ld, n, np, b.dtrack, b.diff, b.r);
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
  c.Ah = b.Ah;
  c.Al = b.Al;
  c.dtrack = b.dtrack;
  c.logdiag = b.logdiag;
  c.info = info;
  c.err = b.err;
  if (!tc_make_map(&c.mL, b.Lh, b.Ll, np, np, b.ld) || !tc_make_map(&c.mM, b.Mh, b.Ml, np, np, b.ld) ||
      !tc_make_map(&c.mV, b.Vh, b.Vl, np, np, b.ld) ||
      !tc_make_map(&c.mA, b.Ah, b.Al, np, np, b.ld))
    return GPK_ERR_UNSUPPORTED;
  c.nf16 = b.nf16;
  for (int k = 0; k < b.nf16; ++k) c.f16[k] = b.f16[k];
  for (int k = 0; k < b.ndepth; ++k) {
    c.TTh[k] = b.TTh[k];
    c.TTl[k] = b.TTl[k];
    c.ldtt[k] = b.ldtt[k];
    if (!tc_make_map(&c.mTT[k], b.TTh[k], b.TTl[k], b.ldtt[k], b.ldtt[k], b.ldtt[k]))
      return GPK_ERR_UNSUPPORTED;
  }
  cudaFuncSetAttribute(leaf_chol_inv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)leaf_smem_bytes());
  // The factor, the alpha solve and the adjoint GEMM run on the library's
  // high-priority stream (hs), the T^T products of the recursion on its
  // low-priority side stream; both fork from and join back into the caller's
  // stream s.  The streams and events are per device; the host-side enqueue
  // of one evaluation holds them.
  std::lock_guard<std::mutex> lock(g_side_mu);
  SideCtx* sc = nullptr;
  GPK_CUDA_TRY(side_ctx(&sc));
  cudaStream_t hs = sc->hp;
  c.s = hs;
  c.side = sc->side;
  c.efork = sc->efork;
  c.ejoin = sc->ejoin;
  c.la = &sc->la;
  GPK_CUDA_TRY(cudaEventRecord(sc->estart, s));
  GPK_CUDA_TRY(cudaStreamWaitEvent(hs, sc->estart, 0));
  leaf_zero_kernel<<<dim3(cdiv(LEAF * 24, 256), np / LEAF), 256, 0, hs>>>(b.Mh, b.Ml, b.Vh, b.Vl,
                                                                           b.ld);
  GPK_LAUNCH_CHECK();
  if (np > LEAF) {
    band_zero_kernel<<<dim3(LEAF * (LEAF / 4) / 256, np / LEAF - 1), 256, 0, hs>>>(b.Mh, b.Ml, b.Vh,
                                                                                 b.Vl, b.ld);
  }
  GPK_LAUNCH_CHECK();
  c.prev_kernel = true;
  GPK_CUDA_TRY(chol_inv_rec(c, 0, np, 0));
  prof_mark(2, hs);
  // alpha = Sigma^-1 (y - m), refined against float64 residuals from the
  // mirrored upper triangle of the Gram matrix
  const int gb = (int)cdiv((int64_t)np * 32, 256), gv = (int)cdiv(np, 256);
  auto gemv = [&](const float* Th, const float* Tl, int lower, const double* x, double* y,
                  int accumulate) -> gpk_status {
    to_f32_kernel<<<gv, 256, 0, hs>>>(np, x, b.vf);
    GPK_LAUNCH_CHECK();
    gemv_split_kernel<<<gb, 256, 0, hs>>>(Th, Tl, b.ld, np, lower, b.vf, y, accumulate);
    GPK_LAUNCH_CHECK();
    return GPK_OK;
  };
  gpk_status st = gemv(b.Mh, b.Ml, 1, b.diff, b.z, 0);
  if (st == GPK_OK) st = gemv(b.Vh, b.Vl, 0, b.z, b.alpha, 0);
  if (st != GPK_OK) return st;
  for (int it = 0; it < refine; ++it) {
    const int tn = (int)cdiv(n, RU_T);
    residual_upper_kernel<<<tn * (tn + 1) / 2, 256, 0, hs>>>(n, b.A, b.ld, b.alpha, b.rbuf,
                                                             b.cbuf);
    GPK_LAUNCH_CHECK();
    residual_upper_finish<<<(int)cdiv(n, 256), 256, 0, hs>>>(kind, n, theta, n_ls, jitter,
                                                             b.diff, b.alpha, b.rbuf, b.cbuf,
                                                             b.r);
    GPK_LAUNCH_CHECK();
    st = gemv(b.Mh, b.Ml, 1, b.r, b.z, 0);
    if (st == GPK_OK) st = gemv(b.Vh, b.Vl, 0, b.z, b.alpha, 1);
    if (st != GPK_OK) return st;
  }
  prof_mark(3, hs);
  if (pred) {  // predictive mean and variance instead of the adjoint
    const int t = pred->t, tp = (int)(((int64_t)t + LEAF - 1) / LEAF * LEAF);
    GPK_CUDA_TRY(scale_inputs<float>(pred->xt, pred->ldxt, t, d, theta, n_ls, pred->ts, hs));
    ktx_split_kernel<<<(unsigned)cdiv((int64_t)tp * np, 256), 256, 0, hs>>>(
        kind, t, tp, n, np, d, pred->ts, b.xs, theta, n_ls, pred->Kh, pred->Kl);
    GPK_LAUNCH_CHECK();
    GPK_CUDA_TRY(cudaMemsetAsync(pred->vacc, 0, sizeof(double) * tp, hs));
    TcMap mK;
    if (!tc_make_map(&mK, pred->Kh, pred->Kl, tp, np, np)) return GPK_ERR_UNSUPPORTED;
    tc::TcParams pq{};  // Q^T[i, j] = sum_k Ktx[i, k] M[j, k], M[j, k] = 0 for k > j
    pq.M = tp;
    pq.N = np;
    pq.K = np;
    pq.b_tri = TRI_LOWER;
    pq.alpha = 1.f;
    pq.dtrack = pred->vacc;
    pq.err = b.err;
    GPK_CUDA_TRY(tc_gemm_run(tc::MODE_STORE_SPLIT, mK, c.mM, pq, 1, hs));
    GPK_CUDA_TRY(cudaEventRecord(sc->edone, hs));
    GPK_CUDA_TRY(cudaStreamWaitEvent(s, sc->edone, 0));
    tc_check_err<<<1, 1, 0, s>>>(b.err, info);
    GPK_LAUNCH_CHECK();
    pred_tc_finish_kernel<<<(unsigned)cdiv((int64_t)t * 32, 256), 256, 0, s>>>(
        t, n, np, pred->Kh, pred->Kl, b.alpha, pred->vacc, theta, n_ls, pred->prior_jitter, info,
        pred->mean, pred->var);
    GPK_LAUNCH_CHECK();
    pred_tc_info_kernel<<<1, 1, 0, s>>>(info);
    GPK_LAUNCH_CHECK();
    return GPK_OK;
  }
  // the adjoint: W = V V^T tiles contracted with (alpha alpha^T - W) x dK/dtheta
  // in the GEMM epilogue
  tc::TcParams pg{};
  pg.M = np;
  pg.N = np;
  pg.K = np;
  pg.a_tri = TRI_UPPER;
  pg.b_tri = TRI_UPPER;
  pg.c_lower = 1;
  pg.n_true = n;
  pg.d = d;
  pg.kind = kind;
  pg.kaptr = kind == GPK_RATIONAL_QUADRATIC ? theta + n_ls + 3 : nullptr;
  pg.xs = b.xs;
  pg.avec = b.alpha;
  pg.gpart = b.gpart;
  pg.err = b.err;
  // large problems with d <= 8 (the wide tile): float16 split of V, rows
  // scaled by powers of two (twice the MMA rate and half the operand bytes of
  // the TF32 split at the same 11-bit significand)
  const bool f16adj = np >= 2048 && d <= 8;
  TcMap mV16;
  if (f16adj) {
    pg.force_shape = 4;  // Tile shape 3
    pg.ra = pg.rb = b.vscale;
  }
  const int ntiles_adj = tc_gemm_tiles(tc::MODE_GRAD, pg);  // gpart rows of the adjoint
  if (want_grad && f16adj) {
    if (!tc_make_map_f16(&mV16, b.V16h, b.V16l, np, np, b.ld)) return GPK_ERR_CUDA;
    v16_convert_kernel<<<(unsigned)cdiv((int64_t)np * 32, 256), 256, 0, hs>>>(
        np, b.Vh, b.Vl, b.ld, b.V16h, b.V16l, b.vscale);
    GPK_LAUNCH_CHECK();
    GPK_CUDA_TRY(tc_gemm_run(tc::MODE_GRAD, mV16, mV16, pg, 1, hs, true));
  } else if (want_grad) {
    GPK_CUDA_TRY(tc_gemm_run(tc::MODE_GRAD, c.mV, c.mV, pg, 1, hs));
  }
  prof_mark(4, hs);
  prof_mark(5, hs);
  GPK_CUDA_TRY(cudaEventRecord(sc->edone, hs));
  GPK_CUDA_TRY(cudaStreamWaitEvent(s, sc->edone, 0));
  tc_check_err<<<1, 1, 0, s>>>(b.err, info);
  GPK_LAUNCH_CHECK();
  GPK_CUDA_TRY(mll_finalize_launch(n, d, theta, n_ls, b.logdiag, b.diff, b.alpha, b.gpart,
                                   want_grad ? ntiles_adj : 0, want_grad, jitter, info,
                                   out_mll, out_grad, s, b.fin));
  prof_mark(6, s);
  return GPK_OK;
}

size_t predict_tc_workspace_bytes(int64_t n, int64_t t, int d) {
  TcBuffers b;
  const size_t base = tc_layout(n, d, nullptr, b);
  return ((base + 1023) & ~size_t(1023)) + predict_tc_extra_bytes(b.npad, t, d);
}

gpk_status predict_run_tc(int kind, int n, int t, int d, const double* x, int64_t ldx,
                          const double* y, const double* xt, int64_t ldxt, const double* theta,
                          int n_ls, double jitter, double prior_jitter, double* mean, double* var,
                          int* info, void* ws, cudaStream_t s) {
  TcBuffers b;
  const size_t base = (tc_layout(n, d, nullptr, b) + 1023) & ~size_t(1023);
  const int64_t tp = ((int64_t)t + LEAF - 1) / LEAF * LEAF;
  char* p = static_cast<char*>(ws) + base;
  TcPredict pr{};
  pr.t = t;
  pr.xt = xt;
  pr.ldxt = ldxt;
  pr.prior_jitter = prior_jitter;
  pr.mean = mean;
  pr.var = var;
  pr.Kh = reinterpret_cast<float*>(p);
  pr.Kl = pr.Kh + tp * b.npad;
  pr.vacc = reinterpret_cast<double*>(pr.Kl + tp * b.npad);
  pr.ts = reinterpret_cast<float*>(pr.vacc + tp);
  return mll_run_tc(kind, n, d, x, ldx, y, theta, n_ls, jitter, 2, 0, nullptr, nullptr, info, ws,
                    s, &pr);
}

}  // namespace gpk
