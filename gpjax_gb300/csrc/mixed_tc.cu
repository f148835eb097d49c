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
// inverted by one CTA in float32 with float64 pivots (the float64 diagonal
// track is decremented by every L21 product).  n is padded to a multiple of
// 128 with an identity block, which leaves the factor, the inverse, the
// log-determinant and alpha of the original system unchanged.
#include <climits>
#include "tc_gemm.cuh"

namespace gpk {
namespace {

constexpr int LEAF = 128;

__device__ __forceinline__ float tf32_rna_f(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// One CTA: Cholesky of the 128 x 128 diagonal block at (o, o) with float64
// pivots from dtrack, then its inverse by 32-wide blocks and two doubling
// merges; writes M (hi/lo) and V = M^T (hi/lo) diagonal blocks.
__global__ void __launch_bounds__(512)
    leaf_chol_inv_kernel(const float* __restrict__ A, int64_t lda, int o,
                         const double* __restrict__ dtrack, double* __restrict__ logdiag,
                         int* __restrict__ info, float* __restrict__ Mh, float* __restrict__ Ml,
                         float* __restrict__ Vh, float* __restrict__ Vl, int64_t ldm) {
  constexpr int N = LEAF, LD = LEAF + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* Dd = reinterpret_cast<double*>(smem_raw);  // diagonal track (as float pairs below)
  double* Pv = Dd + N;                            // pivots (as float pairs below)
  float* S = reinterpret_cast<float*>(Pv + N);   // L
  float* Ms = S + N * LD;                         // L^-1
  float* Tt = Ms + N * LD;                        // panel / merge temporary, 96 x 33 >= 64 x 65
  float* col = Tt + 96 * 65;
  float* dl = col + N;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31, nwarps = nt >> 5;
  for (int e = tid; e < N * N; e += nt) {
    const int i = e / N, j = e % N;
    S[i * LD + j] = 0.f;
    Ms[i * LD + j] = 0.f;
  }
  __syncthreads();
  for (int e = tid; e < N * N; e += nt) {
    const int i = e / N, j = e % N;
    if (j < i) S[i * LD + j] = A[(int64_t)(o + i) * lda + o + j];
  }
  // float-float copy (hi + lo, ~48 bits) of the float64 diagonal track: the
  // pivot history keeps float64-class accuracy with float32 arithmetic only
  // (float64 throughput on this part is a small fraction of float32)
  float* Dh = reinterpret_cast<float*>(Dd);
  float* Dlo = Dh + N;
  float* Ph = reinterpret_cast<float*>(Pv);  // pivots as float-float pairs
  float* Pl = Ph + N;
  for (int i = tid; i < N; i += nt) {
    const double dv = dtrack[o + i];
    const float hi = (float)dv;
    Dh[i] = hi;
    Dlo[i] = (float)(dv - (double)hi);
  }
  __syncthreads();
  // ---- Cholesky by 32-wide panels: inside a panel each pivot step touches
  //      only the panel's columns (warps over rows, lanes over columns); the
  //      columns right of the panel get one rank-32 update per panel ----
  for (int c0 = 0; c0 < N; c0 += 32) {
    const int pend = c0 + 31;
    for (int j = c0; j <= pend; ++j) {
      const float ph = Dh[j], pl = Dlo[j];
      const float ljj = sqrtf(ph + pl);
      const float rl = 1.f / ljj;
      for (int i = j + 1 + tid; i < N; i += nt) {
        const float v = S[i * LD + j] * rl;
        S[i * LD + j] = v;
        col[i] = v;
      }
      if (tid == 0) {
        dl[j] = ljj;
        Ph[j] = ph;  // no float64 work inside the loop: every warp waits on this one
        Pl[j] = pl;
      }
      __syncthreads();
      const int k = j + 1 + lane;  // panel column updated by this lane
      if (k <= pend) {
        const float ck = col[k];
        for (int i = k + 1 + warp; i < N; i += nwarps) S[i * LD + k] = fmaf(-col[i], ck, S[i * LD + k]);
      }
      if (tid > j && tid < N) {
        // (Dh, Dlo) -= c^2 exactly to ~2^-48: product error by FMA, TwoSum,
        // then renormalisation
        const float c = col[tid];
        const float p = c * c, pe = fmaf(c, c, -p);
        const float a = Dh[tid];
        const float s1 = a - p, bb = s1 - a;
        const float err = (a - (s1 - bb)) + (-p - bb);
        const float lo = (Dlo[tid] - pe) + err;
        const float hi = s1 + lo;
        Dlo[tid] = lo - (hi - s1);
        Dh[tid] = hi;
      }
      __syncthreads();
    }
    // rank-32 update of the strictly lower part right of the panel
    const int r0 = pend + 1, nr = N - r0;
    if (nr > 1) {
      for (int e = tid; e < nr * nr; e += nt) {
        const int r = e / nr, q = e % nr;
        if (q >= r) continue;
        float sacc = 0.f;
#pragma unroll 8
        for (int c = c0; c <= pend; ++c) sacc = fmaf(S[(r0 + r) * LD + c], S[(r0 + q) * LD + c], sacc);
        S[(r0 + r) * LD + r0 + q] -= sacc;
      }
      __syncthreads();
    }
  }
  for (int i = tid; i < N; i += nt) {
    S[i * LD + i] = dl[i];
    const double pv = (double)Ph[i] + (double)Pl[i];
    logdiag[o + i] = 0.5 * log(pv);
    if (!(pv > 0.0)) atomicMin(info, o + i + 1);
  }
  __syncthreads();
  // ---- inverse: 32 x 32 diagonal blocks (lane = column, registers) ----
  if (warp < 4) {
    const int b0 = warp * 32, c = lane;
    float mc[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      float sacc = 0.f;
#pragma unroll
      for (int k = 0; k < i; ++k) sacc = fmaf(S[(b0 + i) * LD + b0 + k], mc[k], sacc);
      const float dii = S[(b0 + i) * LD + b0 + i];
      mc[i] = (i < c) ? 0.f : ((i == c) ? 1.f / dii : -sacc / dii);
    }
#pragma unroll
    for (int i = 0; i < 32; ++i) Ms[(b0 + i) * LD + b0 + c] = mc[i];
  }
  __syncthreads();
  // ---- doubling merges: M21 = -M22 (L21 M11) for half sizes 32 then 64,
  //      each thread computing a 2 x 4 output block ----
  for (int h = 32; h < N; h *= 2) {
    const int pairs = N / (2 * h);
    const int nblk = (h / 2) * (h / 4);  // 2 x 4 blocks per h x h product
    for (int pr = 0; pr < pairs; ++pr) {
      const int ob = pr * 2 * h;
      // T = L21 M11 (M11 lower: M11[c][j] = 0 for c < j)
      for (int bidx = tid; bidx < nblk; bidx += nt) {
        const int i2 = (bidx / (h / 4)) * 2, j4 = (bidx % (h / 4)) * 4;
        float a0[4] = {0.f, 0.f, 0.f, 0.f}, a1[4] = {0.f, 0.f, 0.f, 0.f};
        for (int c = j4; c < h; ++c) {
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
          Tt[i2 * 65 + j4 + q] = a0[q];
          Tt[(i2 + 1) * 65 + j4 + q] = a1[q];
        }
      }
      __syncthreads();
      // M21 = -M22 T (M22 lower: M22[i][c] = 0 for c > i)
      for (int bidx = tid; bidx < nblk; bidx += nt) {
        const int i2 = (bidx / (h / 4)) * 2, j4 = (bidx % (h / 4)) * 4;
        float a0[4] = {0.f, 0.f, 0.f, 0.f}, a1[4] = {0.f, 0.f, 0.f, 0.f};
        for (int c = 0; c <= i2 + 1; ++c) {
          const float m0 = Ms[(ob + h + i2) * LD + ob + h + c];  // zero when c > i2
          const float m1 = Ms[(ob + h + i2 + 1) * LD + ob + h + c];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const float t = Tt[c * 65 + j4 + q];
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
  }
  // ---- write M and V = M^T as TF32 hi/lo ----
  for (int e = tid; e < N * N; e += nt) {
    const int i = e / N, j = e % N;
    const float m = Ms[i * LD + j];
    const float hi = tf32_rna_f(m), lo = tf32_rna_f(m - hi);
    Mh[(int64_t)(o + i) * ldm + o + j] = hi;
    Ml[(int64_t)(o + i) * ldm + o + j] = lo;
    const float mt = Ms[j * LD + i];
    const float hit = tf32_rna_f(mt), lot = tf32_rna_f(mt - hit);
    Vh[(int64_t)(o + i) * ldm + o + j] = hit;
    Vl[(int64_t)(o + i) * ldm + o + j] = lot;
  }
}

size_t leaf_smem_bytes() {
  return 2 * LEAF * sizeof(double) + (size_t)(2 * LEAF * (LEAF + 1) + 96 * 65 + 2 * LEAF) * 4;
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
    leaf_chol_inv_kernel<<<1, 512, leaf_smem_bytes(), c.s>>>(c.A, c.ld, o, c.dtrack, c.logdiag,
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
