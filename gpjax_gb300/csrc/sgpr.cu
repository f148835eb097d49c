// SGPR collapsed evidence lower bound and its gradient
// (collapsed_elbo, gpjax/objectives.py:321-416).
//
// With K = Kzz + jitter I, Phi = Kzx, s = obs_stddev^2, d = y - m:
//   P = Phi Phi^T, c = Phi d, Su = K + P / s, gamma = Su^-1 c
//   2 ELBO = -n log(2 pi s) - (log|Su| - log|K|) - (d^T d / s - c^T gamma / s^2)
//            - (n sigma_f^2 / s - tr(K^-1 P) / s)
// which equals the reference's op sequence (log|B| = log|Su| - log|K| with
// B = I + A A^T, A = Lz^-1 Phi / sqrt(s); the quadratic term through the
// matrix inversion lemma).  The gradient is formed in closed form:
//   dF/dPhi = H Phi + gamma d^T / s^2,  H = (K^-1 - Su^-1) / s - gamma gamma^T / s^3
//   dF/dK   = 1/2 (K^-1 - Su^-1 - gamma gamma^T / s^2 - K^-1 P K^-1 / s)
// contracted against dK/dtheta, dK/dZ and dPhi/dtheta, dPhi/dZ regenerated
// from the scaled inputs; the reference differentiates the same sequence
// with JAX reverse mode.
//
// The m x n work has two forms.  Plain (float64): Phi, P, c and the fused
// H Phi adjoint on CUDA cores.  Mixed: Phi is generated once in float32 and
// stored as TF32 hi/lo pairs in both layouts (m x n for P, n x m for the
// adjoint); P = Phi Phi^T per n-chunk and G = H Phi run on the tensor cores
// (split-TF32 tcgen05 GEMM), with G reduced against dPhi/dtheta, dPhi/dZ in
// the GEMM epilogue; c = Phi d and Phi 1 are summed in float-float during
// generation.  The m x m algebra always runs in float64.  Reductions go
// through per-block partials summed in a fixed order.
#include <climits>
#include <mutex>
#include <type_traits>
#include "gpk_internal.cuh"
#include "tc_gemm.cuh"

namespace gpk {
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

constexpr int KCHUNK = 8192;    // P = sum over n-chunks of Phi_k Phi_k^T (float64 sum of chunks)
constexpr int AB = 64;          // fused adjoint tile
constexpr int ASPLIT = 64;      // column (n) split of the fused adjoint
constexpr int DMAXS = 16;       // input dimension limit of the SGPR path

inline int64_t pad64(int64_t n) { return ((n + 63) / 64) * 64; }

constexpr int PG_I = 64;    // Phi generation: inducing rows per block
constexpr int PG_X = 128;   // data columns per sub-tile
constexpr int PG_SUB = 4;   // sub-tiles per block
constexpr int CS_PARTS = 64;  // first-level partials of the column sums

// Tile parameters of the mixed-form adjoint GEMM (G = H Phi, M = m, N = n, K = m).
inline tc::TcParams sg_adj_params(int64_t n, int64_t m, int d) {
  tc::TcParams q{};
  q.M = (int)m;
  q.N = (int)n;
  q.K = (int)m;
  q.d = d;
  return q;
}

template <typename T>
struct SgprBuf {
  static constexpr bool kMixed = std::is_same<T, float>::value;
  int64_t ldn, ldm;
  int nchunks, nb, nxb, gtiles, gcols;
  T *zs, *xs, *Phi, *Pparts, *Ht;                 // Phi, Ht: plain form only
  float *Phh, *Phl, *PTh, *PTl, *Hh, *Hl;         // mixed form only
  double *zs64, *Kf, *Lz, *Mz, *Vz, *Kinv, *Su, *Mu, *Vu, *Suinv, *P64, *T1, *KPK, *GK, *scr;
  double *dv, *cv, *phi1, *gam, *gams, *pgam, *ldK, *ldU, *red, *thK, *dzK, *thP, *dzP;
  double *ddpart, *cpart, *colpart, *sth, *gzs, *ddds;
  int* err;
};

template <typename T>
size_t sgpr_layout(int64_t n, int64_t m, int d, void* ws, SgprBuf<T>& b) {
  constexpr bool mixed = SgprBuf<T>::kMixed;
  Arena a(ws);
  b.ldn = pad64(n);
  b.ldm = pad64(m);
  b.nchunks = (int)((n + KCHUNK - 1) / KCHUNK);
  b.nb = (int)((n + 255) / 256);
  // Phi generation blocks: the chunk-blocked P operand is written (zeros past
  // n) up to nchunks * KCHUNK columns
  b.nxb = mixed ? b.nchunks * (KCHUNK / (PG_X * PG_SUB))
                : (int)((n + PG_X * PG_SUB - 1) / (PG_X * PG_SUB));
  const tc::TcParams q = sg_adj_params(n, m, d);
  b.gtiles = mixed ? tc_gemm_tiles(tc::MODE_SGPR, q) : 0;
  b.gcols = mixed ? tc_gemm_col_tiles(tc::MODE_SGPR, q) : 0;
  const size_t mm = (size_t)m * b.ldm;
  b.zs = a.take<T>((size_t)m * d);
  b.xs = a.take<T>((size_t)n * d);
  b.Phi = mixed ? nullptr : a.take<T>((size_t)m * b.ldn);
  b.Pparts = a.take<T>((size_t)b.nchunks * m * m);
  b.Ht = mixed ? nullptr : a.take<T>(mm);
  b.Phh = b.Phl = b.PTh = b.PTl = b.Hh = b.Hl = nullptr;
  if (mixed) {
    // chunk-blocked: Phh[c][i][k] = hi(Phi[i][c * KCHUNK + k]), so that one
    // chunk of the P product reads one contiguous m x KCHUNK block
    b.Phh = a.take<float>((size_t)b.nchunks * m * KCHUNK);
    b.Phl = a.take<float>((size_t)b.nchunks * m * KCHUNK);
    b.PTh = a.take<float>((size_t)n * b.ldm);
    b.PTl = a.take<float>((size_t)n * b.ldm);
    b.Hh = a.take<float>(mm);
    b.Hl = a.take<float>(mm);
  }
  b.zs64 = a.take<double>((size_t)m * d);
  b.Kf = a.take<double>(mm);
  b.Lz = a.take<double>(mm);
  b.Mz = a.take<double>(mm);
  b.Vz = a.take<double>(mm);
  b.Kinv = a.take<double>(mm);
  b.Su = a.take<double>(mm);
  b.Mu = a.take<double>(mm);
  b.Vu = a.take<double>(mm);
  b.Suinv = a.take<double>(mm);
  b.P64 = a.take<double>(mm);
  b.T1 = a.take<double>(mm);
  b.KPK = a.take<double>(mm);
  b.GK = a.take<double>(mm);
  b.scr = a.take<double>((size_t)m * m / 2 + 64);
  b.dv = a.take<double>(n);
  b.cv = a.take<double>(2 * m);  // c, then Phi 1
  b.phi1 = b.cv ? b.cv + m : nullptr;
  b.gam = a.take<double>(m);
  b.gams = a.take<double>(m);
  b.pgam = a.take<double>(m);
  b.ldK = a.take<double>(m);
  b.ldU = a.take<double>(m);
  b.red = a.take<double>(64);
  b.thK = a.take<double>((size_t)m * (d + 1));
  b.dzK = a.take<double>((size_t)m * d);
  const int mt = (int)((m + AB - 1) / AB);
  if (mixed) {
    b.thP = a.take<double>((size_t)b.gtiles * (d + 1));
    b.dzP = a.take<double>((size_t)b.gcols * m * d);
    b.cpart = a.take<double>((size_t)b.nxb * 2 * m);
  } else {
    b.thP = a.take<double>((size_t)ASPLIT * mt * (d + 1));
    b.dzP = a.take<double>((size_t)ASPLIT * m * d);
    b.cpart = nullptr;
  }
  b.ddpart = a.take<double>((size_t)b.nb * 2);
  int64_t maxcols = 2 * m > (int64_t)m * d ? 2 * m : (int64_t)m * d;
  if (maxcols < 32) maxcols = 32;
  b.colpart = a.take<double>((size_t)CS_PARTS * maxcols);
  b.sth = a.take<double>(GPK_MAX_D + 2);
  b.gzs = a.take<double>((size_t)m * d);
  b.ddds = a.take<double>(2);
  b.err = a.take<int>(1);
  return a.off + 256;
}

// Column sums of a row-major double array a[rows][cols] in a fixed order:
// block (bx, by) sums rows [by * rchunk, (by + 1) * rchunk) of columns
// [32 bx, 32 bx + 32), eight warps striding over the rows.
__global__ void __launch_bounds__(256)
    colsum_part(const double* __restrict__ a, int64_t rows, int64_t cols, int64_t rchunk,
                double* __restrict__ part) {
  __shared__ double sh[8][33];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t c = (int64_t)blockIdx.x * 32 + lane;
  const int64_t r0 = (int64_t)blockIdx.y * rchunk;
  const int64_t r1 = r0 + rchunk < rows ? r0 + rchunk : rows;
  double s = 0.0;
  if (c < cols)
    for (int64_t r = r0 + w; r < r1; r += 8) s += a[r * cols + c];
  sh[w][lane] = s;
  __syncthreads();
  if (w == 0 && c < cols) {
    double t = 0.0;
#pragma unroll
    for (int q = 0; q < 8; ++q) t += sh[q][lane];
    part[(int64_t)blockIdx.y * cols + c] = t;
  }
}

__global__ void colsum_final(const double* __restrict__ part, int nparts, int64_t cols,
                             double* __restrict__ out, int accumulate) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  double t = 0.0;
  for (int q = 0; q < nparts; ++q) t += part[(int64_t)q * cols + c];
  out[c] = accumulate ? out[c] + t : t;
}

// out[c] (+)= sum_r a[r][c]; part holds CS_PARTS * cols doubles
cudaError_t colsum(const double* a, int64_t rows, int64_t cols, double* out, bool accumulate,
                   double* part, cudaStream_t s) {
  if (cols <= 0) return cudaSuccess;
  int nparts = 0;
  if (rows > 0) {
    const int64_t rchunk = (rows + CS_PARTS - 1) / CS_PARTS;
    nparts = (int)((rows + rchunk - 1) / rchunk);
    colsum_part<<<dim3((unsigned)cdiv(cols, 32), (unsigned)nparts), 256, 0, s>>>(a, rows, cols,
                                                                                rchunk, part);
    cudaError_t e = launch_status();
    if (e != cudaSuccess) return e;
  }
  colsum_final<<<(unsigned)cdiv(cols, 256), 256, 0, s>>>(part, nparts, cols, out,
                                                         accumulate ? 1 : 0);
  return launch_status();
}

// d = y - mean; block partials of d^T d and 1^T d (256 threads per block)
__global__ void __launch_bounds__(256)
    sg_init(int* info, int* err, const double* __restrict__ y, const double* __restrict__ theta,
            int n_ls, int n, double* __restrict__ dv, double* __restrict__ ddpart) {
  __shared__ double sh[2][8];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    *info = INT_MAX;
    *err = 0;
  }
  double v = 0.0;
  if (i < n) {
    v = y[i] - theta[n_ls + 2];
    dv[i] = v;
  }
  const double a = warp_sum(v * v), b = warp_sum(v);
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    sh[0][w] = a;
    sh[1][w] = b;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    double t = 0.0;
    for (int q = 0; q < 8; ++q) t += sh[threadIdx.x][q];
    ddpart[(int64_t)blockIdx.x * 2 + threadIdx.x] = t;
  }
}

// float-float accumulation: (hi, lo) += a, with the rounding error of the
// addition kept in lo (Knuth's two-sum); explicit _rn operations keep the
// compiler from contracting the error terms
__device__ __forceinline__ void ff_acc(float& hi, float& lo, float a) {
  const float s = __fadd_rn(hi, a);
  const float bb = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(a, bb));
  hi = s;
  lo = __fadd_rn(lo, err);
}

// Mixed form: Phi = K(Z, X) (float32) for PG_I inducing rows and PG_SUB
// sub-tiles of PG_X data columns, stored as TF32 hi/lo pairs chunk-blocked
// (Phh/Phl [c][i][k] for column c * KCHUNK + k, zeros past n: the P operand)
// and transposed (PTh/PTl, n x m, the adjoint operand); c = Phi d and Phi 1 of
// the block's columns summed in float-float (d split into float hi + lo) into
// cpart[block column][c (m) | Phi 1 (m)].  The grid covers npad columns (a
// multiple of KCHUNK; PG_X * PG_SUB divides KCHUNK).
template <int D>
__global__ void __launch_bounds__(256)
    sg_phi_gen(int kind, int m, int n, int64_t npad, int d, const float* __restrict__ zs,
               const float* __restrict__ xs, const double* __restrict__ theta, int n_ls,
               const double* __restrict__ dv, float* __restrict__ Phh, float* __restrict__ Phl,
               float* __restrict__ PTh, float* __restrict__ PTl, int64_t ldt,
               double* __restrict__ cpart) {
  static_assert(KCHUNK % (PG_X * PG_SUB) == 0, "generation blocks must not straddle chunks");
  __shared__ __align__(16) float tile[PG_I][PG_X + 1];
  __shared__ float sz[PG_I][D + 1];
  __shared__ float sxp[PG_X][D + 1];
  __shared__ float sdh[PG_X], sdl[PG_X];
  const int i0 = blockIdx.y * PG_I;
  const int64_t xb0 = (int64_t)blockIdx.x * PG_X * PG_SUB;
  const float s2 = (float)theta[n_ls];
  const int t = threadIdx.x;
  for (int e = t; e < PG_I * D; e += 256) {
    const int r = e / D, k = e % D;
    sz[r][k] = (i0 + r < m && k < d) ? zs[(int64_t)(i0 + r) * d + k] : 0.f;
  }
  const int bi = t & (PG_I - 1), bg = t >> 6;  // transposed pass: row bi, columns bg + 4 q
  float ch = 0.f, cl = 0.f, ph = 0.f, pl = 0.f;
  for (int sub = 0; sub < PG_SUB; ++sub) {
    const int64_t x0 = xb0 + (int64_t)sub * PG_X;
    if (x0 >= npad) break;
    __syncthreads();  // the previous sub-tile is consumed
    for (int e = t; e < PG_X * D; e += 256) {
      const int c = e / D, k = e % D;
      sxp[c][k] = (x0 + c < n && k < d) ? xs[(x0 + c) * d + k] : 0.f;
    }
    for (int c = t; c < PG_X; c += 256) {
      const double v = x0 + c < n ? dv[x0 + c] : 0.0;
      const float h = (float)v;
      sdh[c] = h;
      sdl[c] = (float)(v - (double)h);
    }
    __syncthreads();
    {  // chunk-blocked pass: column a, rows (t >> 7) + 2 r
      const int a = t & (PG_X - 1);
      const int64_t gx = x0 + a;
      const int64_t cbase = (gx / KCHUNK) * (int64_t)m * KCHUNK + gx % KCHUNK;
      float xr[D];
#pragma unroll
      for (int k = 0; k < D; ++k) xr[k] = sxp[a][k];
      for (int r = t >> 7; r < PG_I; r += 2) {
        float sq = 0.f;
#pragma unroll
        for (int k = 0; k < D; ++k) {
          const float df = sz[r][k] - xr[k];
          sq = fmaf(df, df, sq);
        }
        const float v = gx < n ? kval<float>(kind, sq, s2, kshape<float>(kind, theta, n_ls)) : 0.f;
        tile[r][a] = v;
        if (i0 + r < m) {
          const float h = tf32_round(v);
          Phh[cbase + (int64_t)(i0 + r) * KCHUNK] = h;
          Phl[cbase + (int64_t)(i0 + r) * KCHUNK] = tf32_round(v - h);
        }
      }
    }
    __syncthreads();
    if (i0 + bi < m) {  // transposed pass and the c / Phi 1 sums
      for (int c = bg; c < PG_X; c += 4) {
        const int64_t gx = x0 + c;
        if (gx >= n) break;
        const float v = tile[bi][c];
        const float h = tf32_round(v);
        PTh[gx * ldt + i0 + bi] = h;
        PTl[gx * ldt + i0 + bi] = tf32_round(v - h);
        const float p = __fmul_rn(v, sdh[c]);
        const float e = fmaf(v, sdh[c], -p);  // exact product error
        ff_acc(ch, cl, p);
        cl = __fadd_rn(cl, fmaf(v, sdl[c], e));
        ff_acc(ph, pl, v);
      }
    }
  }
  __syncthreads();
  double* red = reinterpret_cast<double*>(&tile[0][0]);  // [4][PG_I][2]
  red[(bg * PG_I + bi) * 2 + 0] = (double)ch + (double)cl;
  red[(bg * PG_I + bi) * 2 + 1] = (double)ph + (double)pl;
  __syncthreads();
  if (t < PG_I && i0 + t < m) {
    double c = 0.0, p = 0.0;
    for (int g = 0; g < 4; ++g) {
      c += red[(g * PG_I + t) * 2 + 0];
      p += red[(g * PG_I + t) * 2 + 1];
    }
    cpart[(int64_t)blockIdx.x * 2 * m + i0 + t] = c;
    cpart[(int64_t)blockIdx.x * 2 * m + m + i0 + t] = p;
  }
}

// c = Phi d and phi1 = Phi 1 (float64 accumulation), one warp per row of Phi
template <typename T>
__global__ void sg_phi_gemv(const T* __restrict__ Phi, int64_t ld, int m, int n,
                            const double* __restrict__ dv, double* __restrict__ cv,
                            double* __restrict__ phi1) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (i >= m) return;
  const T* row = Phi + (int64_t)i * ld;
  double s = 0.0, t = 0.0;
  for (int j = lane; j < n; j += 32) {
    const double p = (double)row[j];
    s += p * dv[j];
    t += p;
  }
  s = warp_sum(s);
  t = warp_sum(t);
  if (lane == 0) {
    cv[i] = s;
    phi1[i] = t;
  }
}

// P64 (full, symmetric) = sum of the lower triangles of the chunk partials;
// Su (lower) = K + P / s
template <typename T>
__global__ void sg_reduce_P(const T* __restrict__ parts, int nchunks, int m, int64_t ldm,
                            const double* __restrict__ Kf, const double* __restrict__ theta,
                            int n_ls, double jitter, double* __restrict__ P64,
                            double* __restrict__ Su) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)m * m) return;
  const int i = (int)(e / m), j = (int)(e % m);
  const int hi = i > j ? i : j, lo = i > j ? j : i;
  double s = 0.0;
  for (int c = 0; c < nchunks; ++c) s += (double)parts[(int64_t)c * m * m + (int64_t)hi * m + lo];
  P64[(int64_t)i * ldm + j] = s;
  const double sd = theta[n_ls + 1];
  // Su = (Kzz + jitter I) + P / s
  Su[(int64_t)i * ldm + j] = Kf[(int64_t)i * ldm + j] + (i == j ? jitter : 0.0) + s / (sd * sd);
}

// H (in T for the plain form; TF32 hi/lo Hh, Hl for the mixed form), GK
// (float64), gams = gamma / s^2 and the traces tr(K^-1 P), tr(Su^-1 P)
// (block partials)
template <typename T>
__global__ void sg_combine(int m, int64_t ldm, const double* __restrict__ Kinv,
                           const double* __restrict__ Suinv, const double* __restrict__ KPK,
                           const double* __restrict__ P64, const double* __restrict__ gam,
                           const double* __restrict__ theta, int n_ls, T* __restrict__ Ht,
                           float* __restrict__ Hh, float* __restrict__ Hl,
                           double* __restrict__ gams, double* __restrict__ GK,
                           double* __restrict__ red) {
  const double sd = theta[n_ls + 1], s = sd * sd;
  double tK = 0.0, tU = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
    gams[i] = gam[i] / (s * s);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < (int64_t)m * m;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / m), j = (int)(e % m);
    const int64_t o = (int64_t)i * ldm + j;
    const double ki = Kinv[o], ui = Suinv[o], gg = gam[i] * gam[j], p = P64[o];
    const double h = (ki - ui) / s - gg / (s * s * s);
    if (Hh) {
      const float hv = tf32_round((float)h);
      Hh[o] = hv;
      Hl[o] = tf32_round((float)(h - (double)hv));
    } else {
      Ht[o] = (T)h;
    }
    GK[o] = 0.5 * (ki - ui - gg / (s * s) - KPK[o] / s);
    tK += ki * p;
    tU += ui * p;
  }
  tK = warp_sum(tK);
  tU = warp_sum(tU);
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&red[0], tK);  // m^2 terms, float64; order-insensitive to ~1e-16 relative
    atomicAdd(&red[1], tU);
  }
}

// Kzz part of the gradient: one block per row i of GK (full square).
// thK[i] = [sum_j g c1 dsq_k (k < d), sum_j g k1]; dzK[i][k] = sum_j 2 g c1 (zs_ik - zs_jk)
__global__ void __launch_bounds__(256)
    sg_grad_kzz(int kind, int m, int d, int64_t ldm, const double* __restrict__ zs,
                const double* __restrict__ GK, double* __restrict__ thK,
                double* __restrict__ dzK, const double* __restrict__ theta, int n_ls) {
  const int i = blockIdx.x;
  __shared__ double red[(DMAXS * 2 + 1) * 8];
  double zi[DMAXS];
#pragma unroll
  for (int k = 0; k < DMAXS; ++k) zi[k] = k < d ? zs[(int64_t)i * d + k] : 0.0;
  double al[DMAXS], az[DMAXS], av = 0.0;
#pragma unroll
  for (int k = 0; k < DMAXS; ++k) al[k] = az[k] = 0.0;
  for (int j = threadIdx.x; j < m; j += blockDim.x) {
    const double g = GK[(int64_t)i * ldm + j];
    double dz[DMAXS], sq = 0.0;
#pragma unroll
    for (int k = 0; k < DMAXS; ++k) {
      dz[k] = k < d ? zi[k] - zs[(int64_t)j * d + k] : 0.0;
      sq += dz[k] * dz[k];
    }
    double k1, c1;
    kval_dcoef<double>(kind, sq, 1.0, k1, c1, kshape<double>(kind, theta, n_ls));
    av += g * k1;
#pragma unroll
    for (int k = 0; k < DMAXS; ++k) {
      al[k] += g * c1 * dz[k] * dz[k];
      az[k] += 2.0 * g * c1 * dz[k];
    }
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  for (int k = 0; k < 2 * d + 1; ++k) {
    // slot k: [0, d) lengthscale terms, [d, 2d) Z terms, 2d variance term
    double v = av;
    if (k < 2 * d) {
      const int idx = k < d ? k : k - d;
      v = 0.0;
#pragma unroll
      for (int q = 0; q < DMAXS; ++q)
        if (q == idx) v = (k < d) ? al[q] : az[q];
    }
    v = warp_sum(v);
    if (l == 0) red[k * 8 + w] = v;
  }
  __syncthreads();
  if (threadIdx.x < 2 * d + 1) {
    const int k = threadIdx.x;
    double t = 0.0;
    for (int q = 0; q < 8; ++q) t += red[k * 8 + q];
    if (k < d)
      thK[(int64_t)i * (d + 1) + k] = t;
    else if (k < 2 * d)
      dzK[(int64_t)i * d + (k - d)] = t;
    else
      thK[(int64_t)i * (d + 1) + d] = t;
  }
}

// Fused Phi adjoint: for row tile I (AB rows of Z) and column tiles j = s, s+S, ...
//   G = H Phi + gamma d^T / s^2   (tile by tile, never stored)
// reduced against dPhi/dtheta and dPhi/dZ regenerated from the scaled inputs.
template <typename T>
__global__ void __launch_bounds__(256)
    sg_phi_adjoint(int kind, int m, int n, int d, const T* __restrict__ Ht, int64_t ldm,
                   const T* __restrict__ Phi, int64_t ldn, const T* __restrict__ zs,
                   const T* __restrict__ xs, const double* __restrict__ gam,
                   const double* __restrict__ dv, const double* __restrict__ theta, int n_ls,
                   double* __restrict__ thP, double* __restrict__ dzP) {
  constexpr int BKc = 16;
  extern __shared__ __align__(16) unsigned char sg_smem[];
  typedef T Row64[AB + 1];
  typedef T RowD[DMAXS + 1];
  typedef double RowDd[DMAXS + 1];
  Row64* As = reinterpret_cast<Row64*>(sg_smem);     // [BKc]
  Row64* Bs = As + BKc;                              // [BKc]
  Row64* Gs = Bs + BKc;                              // [AB]
  RowD* szi = reinterpret_cast<RowD*>(Gs + AB);      // [AB]
  RowD* sxj = szi + AB;                              // [AB]
  RowDd* sdz = reinterpret_cast<RowDd*>(
      (reinterpret_cast<uintptr_t>(sxj + AB) + 15) & ~static_cast<uintptr_t>(15));  // [AB]
  RowDd* sred = sdz + AB;                            // [8]
  const int I = blockIdx.x, split = blockIdx.y;
  const int i0 = I * AB;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const double sd = theta[n_ls + 1], s = sd * sd;
  for (int e = threadIdx.x; e < AB * DMAXS; e += 256) {
    const int r = e / DMAXS, k = e % DMAXS;
    szi[r][k] = (i0 + r < m && k < d) ? zs[(int64_t)(i0 + r) * d + k] : T(0);
    sdz[r][k] = 0.0;
  }
  double al[DMAXS], av = 0.0;
#pragma unroll
  for (int k = 0; k < DMAXS; ++k) al[k] = 0.0;
  const int ntile = (n + AB - 1) / AB;
  // element ownership in the reduction: 4 threads per row, 16 columns each
  const int er = threadIdx.x >> 2, ec = (threadIdx.x & 3) * 16;
  for (int J = split; J < ntile; J += ASPLIT) {
    const int j0 = J * AB;
    T acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b] = T(0);
    for (int c0 = 0; c0 < m; c0 += BKc) {
      __syncthreads();
      for (int e = threadIdx.x; e < AB * BKc; e += 256) {
        const int r = e / BKc, kk = e % BKc;
        As[kk][r] = (i0 + r < m && c0 + kk < m) ? Ht[(int64_t)(i0 + r) * ldm + c0 + kk] : T(0);
      }
      for (int e = threadIdx.x; e < AB * BKc; e += 256) {
        const int kk = e / AB, cc = e % AB;
        Bs[kk][cc] = (c0 + kk < m && j0 + cc < n) ? Phi[(int64_t)(c0 + kk) * ldn + j0 + cc] : T(0);
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < BKc; ++kk) {
        T av4[4], bv4[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) av4[a] = As[kk][ty + 16 * a];
#pragma unroll
        for (int b = 0; b < 4; ++b) bv4[b] = Bs[kk][tx + 16 * b];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) acc[a][b] = fma(av4[a], bv4[b], acc[a][b]);
      }
    }
    __syncthreads();
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) Gs[ty + 16 * a][tx + 16 * b] = acc[a][b];
    for (int e = threadIdx.x; e < AB * DMAXS; e += 256) {
      const int r = e / DMAXS, k = e % DMAXS;
      sxj[r][k] = (j0 + r < n && k < d) ? xs[(int64_t)(j0 + r) * d + k] : T(0);
    }
    __syncthreads();
    const int gi = i0 + er;
    double zacc[DMAXS];
#pragma unroll
    for (int k = 0; k < DMAXS; ++k) zacc[k] = 0.0;
    {
      const double gami = gi < m ? gam[gi] / (s * s) : 0.0;
      for (int cc = ec; cc < ec + 16 && gi < m; ++cc) {
        const int gj = j0 + cc;
        if (gj >= n) break;
        const T g = (T)((double)Gs[er][cc] + gami * dv[gj]);
        T dz[DMAXS], sq = T(0);
#pragma unroll
        for (int k = 0; k < DMAXS; ++k) {
          dz[k] = szi[er][k] - sxj[cc][k];
          sq += dz[k] * dz[k];
        }
        T k1, c1;
        kval_dcoef<T>(kind, sq, T(1), k1, c1, kshape<T>(kind, theta, n_ls));
        av += (double)(g * k1);
        const T gc = g * c1;
#pragma unroll
        for (int k = 0; k < DMAXS; ++k) {
          al[k] += (double)(gc * dz[k] * dz[k]);
          zacc[k] += (double)(gc * dz[k]);
        }
      }
    }
    // 4 consecutive lanes share a row: combine (whole warp), one lane adds
#pragma unroll
    for (int k = 0; k < DMAXS; ++k) {
      double v = zacc[k];
      v += __shfl_xor_sync(0xffffffffu, v, 1);
      v += __shfl_xor_sync(0xffffffffu, v, 2);
      zacc[k] = v;
    }
    if ((threadIdx.x & 3) == 0 && gi < m) {
#pragma unroll
      for (int k = 0; k < DMAXS; ++k) sdz[er][k] += zacc[k];
    }
  }
  __syncthreads();
  // theta partials of this block
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  for (int k = 0; k <= d; ++k) {
    // slot k: [0, d) lengthscale terms, d variance term
    double v = av;
    if (k < d) {
      v = 0.0;
#pragma unroll
      for (int q = 0; q < DMAXS; ++q)
        if (q == k) v = al[q];
    }
    v = warp_sum(v);
    if (l == 0) sred[w][k] = v;
  }
  __syncthreads();
  const int mt = gridDim.x;
  if (threadIdx.x <= d) {
    double t = 0.0;
    for (int q = 0; q < 8; ++q) t += sred[q][threadIdx.x];
    thP[((int64_t)split * mt + I) * (d + 1) + threadIdx.x] = t;
  }
  for (int e = threadIdx.x; e < AB * d; e += 256) {
    const int r = e / d, k = e % d;
    if (i0 + r < m) dzP[((int64_t)split * m + i0 + r) * d + k] = sdz[r][k];
  }
}

// value, theta gradient and the Z gradient from the reduced sums:
// sth[0..d] theta sums (Kzz and Phi parts), gzs[m][d] the Phi part of the Z
// sums, ddds = (d^T d, 1^T d)
__global__ void __launch_bounds__(256)
    sg_finalize(int n, int m, int d, const double* __restrict__ theta, int n_ls,
                const double* __restrict__ ldK, const double* __restrict__ ldU,
                const double* __restrict__ cv, const double* __restrict__ gam,
                const double* __restrict__ pgam, const double* __restrict__ phi1,
                const double* __restrict__ red, const double* __restrict__ sth,
                const double* __restrict__ ddds, const double* __restrict__ dzK,
                const double* __restrict__ gzs, const int* __restrict__ err, int want_grad,
                int* __restrict__ info, double* __restrict__ out_elbo,
                double* __restrict__ out_grad, double* __restrict__ out_gz) {
  __shared__ double sh[8];
  __shared__ double part[5][256];
  const int tid = threadIdx.x;
  {
    double a = 0.0, b = 0.0, cg = 0.0, gpg = 0.0, pg1 = 0.0;
    for (int i = tid; i < m; i += blockDim.x) {
      a += ldK[i];
      b += ldU[i];
      cg += cv[i] * gam[i];
      gpg += gam[i] * pgam[i];
      pg1 += phi1[i] * gam[i];
    }
    part[0][tid] = a;
    part[1][tid] = b;
    part[2][tid] = cg;
    part[3][tid] = gpg;
    part[4][tid] = pg1;
  }
  __syncthreads();
  if (tid < 5) {
    double t = 0.0;
    for (int q = 0; q < (int)blockDim.x; ++q) t += part[tid][q];
    sh[tid] = (tid < 2) ? 2.0 * t : t;  // log|K|, log|Su| from log-diagonals
  }
  __syncthreads();
  int inf = *info;
  if (inf == INT_MAX) inf = 0;
  if (inf == 0 && *err) inf = -1;  // a tensor-core wait timed out
  const double nan = __longlong_as_double(0x7ff8000000000000ULL);
  const double s2 = theta[n_ls], sd = theta[n_ls + 1], s = sd * sd;
  if (want_grad) {
    for (int e = tid; e < m * d; e += blockDim.x) {
      const int k = e % d;
      const double l = theta[n_ls == 1 ? 0 : k];
      out_gz[e] = inf ? nan : -s2 * (dzK[e] + gzs[e]) / l;
    }
  }
  if (tid != 0) return;
  *info = inf;
  const double ldK_ = sh[0], ldU_ = sh[1], cg = sh[2], gpg = sh[3], pg1 = sh[4], dd = ddds[0],
               ds = ddds[1];
  const double trKP = red[0], trUP = red[1];
  const double two_log_prob =
      -(double)n * log(2.0 * 3.141592653589793 * s) - (ldU_ - ldK_) - (dd / s - cg / (s * s));
  const double two_trace = (double)n * s2 / s - trKP / s;
  *out_elbo = inf ? nan : 0.5 * (two_log_prob - two_trace);
  if (!want_grad) return;
  if (n_ls == 1) {
    double a = 0.0;
    for (int k = 0; k < d; ++k) a += sth[k];
    out_grad[0] = inf ? nan : s2 * a / theta[0];
  } else {
    for (int k = 0; k < d; ++k) out_grad[k] = inf ? nan : s2 * sth[k] / theta[k];
  }
  out_grad[n_ls] = inf ? nan : sth[d] - (double)n / (2.0 * s);
  const double dFds = 0.5 * (-(double)n / s + trUP / (s * s) + dd / (s * s) - 2.0 * cg / (s * s * s) +
                             gpg / (s * s * s * s) + (double)n * s2 / (s * s) - trKP / (s * s));
  out_grad[n_ls + 1] = inf ? nan : 2.0 * sd * dFds;
  out_grad[n_ls + 2] = inf ? nan : ds / s - pg1 / (s * s);
}

// Copies the lower triangle of a symmetric m x m matrix into its upper one.
__global__ void sg_mirror(int m, int64_t ld, double* __restrict__ a) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)m * m) return;
  const int i = (int)(e / m), j = (int)(e % m);
  if (j <= i) return;
  a[(int64_t)i * ld + j] = a[(int64_t)j * ld + i];
}

__global__ void sg_zero(double* p, int count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) p[i] = 0.0;
}

// Side stream for the Kzz chain (its Cholesky factor, inverse and K^-1 do not
// depend on Phi or P, so they run beside the Phi generation and the P
// product), forked from and joined back into the caller's stream.  The mutex
// is held from the fork to the join so that concurrent calls cannot
// interleave their uses of the shared fork/join events (and is released
// before a sharded call's exchanges, which may wait for other ranks).
struct SgSide {
  cudaStream_t s = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};
std::mutex g_sg_mu;
SgSide g_sg_side[64];

cudaError_t sg_side(SgSide** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  SgSide& c = g_sg_side[dev];
  if (!c.s) {
    e = cudaEventCreateWithFlags(&c.fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c.join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c.s, cudaStreamNonBlocking);
    if (e != cudaSuccess) return e;
  }
  *out = &c;
  return cudaSuccess;
}

// Sum of a float64 region of the workspace over the ranks of a sharded call
// (gpk_collapsed_elbo_sharded); a no-op for a single-rank call.
struct Exchange {
  gpk_allreduce_fn fn = nullptr;
  void* user = nullptr;
  const void* ws = nullptr;
  gpk_status sum(const double* p, int64_t count, cudaStream_t s) const {
    if (!fn) return GPK_OK;
    const size_t off = (size_t)(reinterpret_cast<const char*>(p) - static_cast<const char*>(ws));
    return fn(user, off, count, s) == 0 ? GPK_OK : GPK_ERR_CUDA;
  }
};

// Su = (Kzz + jitter I) + P / s from the summed P
__global__ void sg_su(int m, int64_t ldm, const double* __restrict__ Kf,
                      const double* __restrict__ P64, const double* __restrict__ theta, int n_ls,
                      double jitter, double* __restrict__ Su) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)m * m) return;
  const int i = (int)(e / m), j = (int)(e % m);
  const double sd = theta[n_ls + 1];
  const int64_t o = (int64_t)i * ldm + j;
  Su[o] = Kf[o] + (i == j ? jitter : 0.0) + P64[o] / (sd * sd);
}

template <typename T>
gpk_status sgpr_run(int kind, int n, int m, int d, const double* x, int64_t ldx, const double* y,
                    const double* z, int64_t ldz, const double* theta, int n_ls, double jitter,
                    int want_grad, double* out_elbo, double* out_grad, double* out_gz, int* info,
                    void* ws, cudaStream_t s, const Exchange& ex = Exchange(),
                    int64_t n_total = -1) {
  constexpr bool mixed = SgprBuf<T>::kMixed;
  SgprBuf<T> b;
  sgpr_layout<T>(n, m, d, ws, b);
  const int64_t ldm = b.ldm;
  if (n_total < 0) n_total = n;
  sg_init<<<b.nb, 256, 0, s>>>(info, b.err, y, theta, n_ls, n, b.dv, b.ddpart);
  GPK_LAUNCH_CHECK();
  sg_zero<<<1, 64, 0, s>>>(b.red, 64);
  GPK_LAUNCH_CHECK();
  GPK_CUDA_TRY(scale_inputs<T>(x, ldx, n, d, theta, n_ls, b.xs, s));
  GPK_CUDA_TRY(scale_inputs<T>(z, ldz, m, d, theta, n_ls, b.zs, s));
  GPK_CUDA_TRY(scale_inputs<double>(z, ldz, m, d, theta, n_ls, b.zs64, s));
  // Kzz chain on the side stream: K (float64, full), Lz = chol(K + jitter I),
  // Mz = Lz^-1, Vz = Mz^T, K^-1 = Vz Vz^T
  std::unique_lock<std::mutex> lock(g_sg_mu);
  SgSide* side = nullptr;
  GPK_CUDA_TRY(sg_side(&side));
  const cudaStream_t ss = side->s;
  const unsigned mgrid = (unsigned)cdiv((int64_t)m * m, 256);
  GPK_CUDA_TRY(cudaEventRecord(side->fork, s));
  GPK_CUDA_TRY(cudaStreamWaitEvent(ss, side->fork, 0));
  GPK_CUDA_TRY(cross_cov_scaled<double, double>(kind, m, m, d, b.zs64, b.zs64, theta, n_ls, 0, 0.0,
                                                b.Kf, ldm, ss));
  GPK_CUDA_TRY(cross_cov_scaled<double, double>(kind, m, m, d, b.zs64, b.zs64, theta, n_ls, 2,
                                                jitter, b.Lz, ldm, ss));
  GPK_CUDA_TRY(potrf_lower<double>(b.Lz, ldm, m, b.ldK, info, nullptr, false, ss));
  GPK_CUDA_TRY(trtri_lower<double>(b.Lz, ldm, m, b.Mz, ldm, b.Vz, ldm, b.scr, ss));
  {
    GemmProb<double> p{};
    p.A = b.Vz;
    p.B = b.Vz;
    p.lda = p.ldb = ldm;
    p.a_tri = p.b_tri = TRI_UPPER;
    p.C = b.Kinv;
    p.ldc = ldm;
    p.M = p.N = p.K = m;
    p.c_lower = 1;
    p.alpha = 1.0;
    p.beta = 0.0;
    GPK_CUDA_TRY(gemm_nt<double>(p, 1, ss));
    sg_mirror<<<mgrid, 256, 0, ss>>>(m, ldm, b.Kinv);
    GPK_LAUNCH_CHECK();
  }
  GPK_CUDA_TRY(cudaEventRecord(side->join, ss));
  TcMap mphi, mh, mpt;
  if constexpr (mixed) {
    // Phi (both layouts, TF32 hi/lo), c = Phi d and Phi 1
    const int64_t npad = (int64_t)b.nchunks * KCHUNK;
    const dim3 grid((unsigned)b.nxb, (unsigned)cdiv(m, PG_I));
    if (d <= 8)
      sg_phi_gen<8><<<grid, 256, 0, s>>>(kind, m, n, npad, d, b.zs, b.xs, theta, n_ls, b.dv,
                                         b.Phh, b.Phl, b.PTh, b.PTl, ldm, b.cpart);
    else
      sg_phi_gen<DMAXS><<<grid, 256, 0, s>>>(kind, m, n, npad, d, b.zs, b.xs, theta, n_ls, b.dv,
                                             b.Phh, b.Phl, b.PTh, b.PTl, ldm, b.cpart);
    GPK_LAUNCH_CHECK();
    GPK_CUDA_TRY(colsum(b.cpart, b.nxb, 2 * (int64_t)m, b.cv, false, b.colpart, s));
    // P: lower triangles of Phi_k Phi_k^T per n-chunk (tensor cores, one
    // batched launch over the chunk-blocked operand, rows c * m + i), summed
    // in float64.  A tile's rows past m (read from the next chunk) only reach
    // outputs past m, which the epilogue drops.
    if (!tc_make_map(&mphi, b.Phh, b.Phl, (int64_t)b.nchunks * m, KCHUNK, KCHUNK) ||
        !tc_make_map(&mh, b.Hh, b.Hl, m, m, ldm) || !tc_make_map(&mpt, b.PTh, b.PTl, n, m, ldm))
      return GPK_ERR_CUDA;
    GPK_CUDA_TRY(cudaMemsetAsync(b.Pparts, 0, sizeof(float) * (size_t)b.nchunks * m * m, s));
    tc::TcParams p{};
    p.M = p.N = m;
    p.K = KCHUNK;
    p.a_zrow = p.b_zrow = m;
    p.c_lower = 1;
    p.force_shape = m >= 256 ? 2 : 0;  // wide tiles: the batch supplies the parallelism
    p.c0 = b.Pparts;
    p.ldc = m;
    p.c_zrow = m;
    p.alpha = 1.f;
    p.err = b.err;
    GPK_CUDA_TRY(tc_gemm_run(tc::MODE_ADD_F32, mphi, mphi, p, b.nchunks, s));
  } else {
    // Phi = K(z, x) (m x n), c = Phi d, phi1 = Phi 1
    GPK_CUDA_TRY(cross_cov_scaled<T, T>(kind, m, n, d, b.zs, b.xs, theta, n_ls, 0, 0.0, b.Phi,
                                        b.ldn, s));
    sg_phi_gemv<T><<<(int)cdiv((int64_t)m * 32, 256), 256, 0, s>>>(b.Phi, b.ldn, m, n, b.dv,
                                                                     b.cv, b.phi1);
    GPK_LAUNCH_CHECK();
    // P: lower triangles of Phi_k Phi_k^T per n-chunk, summed in float64
    const int full = n / KCHUNK;
    GemmProb<T> p{};
    p.A = b.Phi;
    p.B = b.Phi;
    p.lda = p.ldb = b.ldn;
    p.sA = p.sB = KCHUNK;
    p.C = b.Pparts;
    p.ldc = m;
    p.sC = (int64_t)m * m;
    p.M = p.N = m;
    p.K = KCHUNK;
    p.c_lower = 1;
    p.alpha = T(1);
    p.beta = T(0);
    if (full > 0) GPK_CUDA_TRY(gemm_nt<T>(p, full, s));
    const int rest = n - full * KCHUNK;
    if (rest > 0) {
      p.A = b.Phi + (int64_t)full * KCHUNK;
      p.B = p.A;
      p.C = b.Pparts + (int64_t)full * m * m;
      p.K = rest;
      GPK_CUDA_TRY(gemm_nt<T>(p, 1, s));
    }
  }
  GPK_CUDA_TRY(cudaStreamWaitEvent(s, side->join, 0));
  lock.unlock();  // the side stream's events are not used past the join
  sg_reduce_P<T><<<(int)cdiv((int64_t)m * m, 256), 256, 0, s>>>(b.Pparts, b.nchunks, m, ldm, b.Kf,
                                                                  theta, n_ls, jitter, b.P64, b.Su);
  GPK_LAUNCH_CHECK();
  GPK_CUDA_TRY(colsum(b.ddpart, b.nb, 2, b.ddds, false, b.colpart, s));
  if (ex.fn) {
    // the data-dependent statistics summed over the ranks' rows: P = Phi Phi^T,
    // c = Phi d and Phi 1, (d^T d, 1^T d); then Su from the summed P
    gpk_status st = ex.sum(b.P64, (int64_t)m * ldm, s);
    if (st == GPK_OK) st = ex.sum(b.cv, 2 * (int64_t)m, s);
    if (st == GPK_OK) st = ex.sum(b.ddds, 2, s);
    if (st != GPK_OK) return st;
    sg_su<<<(int)cdiv((int64_t)m * m, 256), 256, 0, s>>>(m, ldm, b.Kf, b.P64, theta, n_ls, jitter,
                                                         b.Su);
    GPK_LAUNCH_CHECK();
  }
  GPK_CUDA_TRY(potrf_lower<double>(b.Su, ldm, m, b.ldU, info, nullptr, true, s));
  GPK_CUDA_TRY(trtri_lower<double>(b.Su, ldm, m, b.Mu, ldm, b.Vu, ldm, b.scr, s));
  {  // Su^-1 = Vu Vu^T (lower triangle, then mirrored)
    GemmProb<double> p{};
    p.A = b.Vu;
    p.B = b.Vu;
    p.lda = p.ldb = ldm;
    p.a_tri = p.b_tri = TRI_UPPER;
    p.C = b.Suinv;
    p.ldc = ldm;
    p.M = p.N = p.K = m;
    p.c_lower = 1;
    p.alpha = 1.0;
    p.beta = 0.0;
    GPK_CUDA_TRY(gemm_nt<double>(p, 1, s));
    sg_mirror<<<mgrid, 256, 0, s>>>(m, ldm, b.Suinv);
    GPK_LAUNCH_CHECK();
    // T1 = K^-1 P ; KPK = T1 K^-1 (symmetric operands: NT form; KPK is
    // symmetric, so its lower triangle is formed and mirrored)
    GemmProb<double> q{};
    q.A = b.Kinv;
    q.B = b.P64;
    q.lda = q.ldb = ldm;
    q.C = b.T1;
    q.ldc = ldm;
    q.M = q.N = q.K = m;
    q.alpha = 1.0;
    q.beta = 0.0;
    GPK_CUDA_TRY(gemm_nt<double>(q, 1, s));
    q.A = b.T1;
    q.B = b.Kinv;
    q.C = b.KPK;
    q.c_lower = 1;
    GPK_CUDA_TRY(gemm_nt<double>(q, 1, s));
    sg_mirror<<<mgrid, 256, 0, s>>>(m, ldm, b.KPK);
    GPK_LAUNCH_CHECK();
  }
  GPK_CUDA_TRY(gemv_dense<double>(b.Suinv, ldm, m, m, b.cv, b.gam, s));
  GPK_CUDA_TRY(gemv_dense<double>(b.P64, ldm, m, m, b.gam, b.pgam, s));
  sg_combine<T><<<256, 256, 0, s>>>(m, ldm, b.Kinv, b.Suinv, b.KPK, b.P64, b.gam, theta, n_ls,
                                    b.Ht, b.Hh, b.Hl, b.gams, b.GK, b.red);
  GPK_LAUNCH_CHECK();
  if (want_grad) {
    sg_grad_kzz<<<m, 256, 0, s>>>(kind, m, d, ldm, b.zs64, b.GK, b.thK, b.dzK, theta, n_ls);
    GPK_LAUNCH_CHECK();
    if constexpr (mixed) {
      // G = H Phi + gamma d^T / s^2 on the tensor cores, reduced in the epilogue
      tc::TcParams p = sg_adj_params(n, m, d);
      p.n_true = n;
      p.kind = kind;
      p.kaptr = kind == GPK_RATIONAL_QUADRATIC ? theta + n_ls + 3 : nullptr;
      p.xs = b.xs;
      p.zs = b.zs;
      p.avec = b.gams;
      p.bvec = b.dv;
      p.gpart = b.thP;
      p.zpart = b.dzP;
      p.err = b.err;
      GPK_CUDA_TRY(tc_gemm_run(tc::MODE_SGPR, mh, mpt, p, 1, s));
      GPK_CUDA_TRY(colsum(b.thP, b.gtiles, d + 1, b.sth, false, b.colpart, s));
      GPK_CUDA_TRY(colsum(b.dzP, b.gcols, (int64_t)m * d, b.gzs, false, b.colpart, s));
    } else {
      const int mt = (m + AB - 1) / AB;
      dim3 grid(mt, ASPLIT);
      const size_t smem = (size_t)(2 * 16 + AB) * (AB + 1) * sizeof(T) +
                          (size_t)2 * AB * (DMAXS + 1) * sizeof(T) + 16 +
                          (size_t)(AB + 8) * (DMAXS + 1) * sizeof(double);
      cudaFuncSetAttribute(sg_phi_adjoint<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem);
      sg_phi_adjoint<T><<<grid, 256, smem, s>>>(kind, m, n, d, b.Ht, ldm, b.Phi, b.ldn, b.zs,
                                                b.xs, b.gam, b.dv, theta, n_ls, b.thP, b.dzP);
      GPK_LAUNCH_CHECK();
      GPK_CUDA_TRY(colsum(b.thP, (int64_t)ASPLIT * mt, d + 1, b.sth, false, b.colpart, s));
      GPK_CUDA_TRY(colsum(b.dzP, ASPLIT, (int64_t)m * d, b.gzs, false, b.colpart, s));
    }
    // the Phi parts of the gradient sums over the ranks' rows; the Kzz part,
    // identical on every rank, is added once after
    gpk_status st = ex.sum(b.sth, d + 1, s);
    if (st == GPK_OK) st = ex.sum(b.gzs, (int64_t)m * d, s);
    if (st != GPK_OK) return st;
    GPK_CUDA_TRY(colsum(b.thK, m, d + 1, b.sth, true, b.colpart, s));
  }
  sg_finalize<<<1, 256, 0, s>>>((int)n_total, m, d, theta, n_ls, b.ldK, b.ldU, b.cv, b.gam, b.pgam, b.phi1,
                                b.red, b.sth, b.ddds, b.dzK, b.gzs, b.err, want_grad, info,
                                out_elbo, out_grad, out_gz);
  GPK_LAUNCH_CHECK();
  return GPK_OK;
}

}  // namespace
}  // namespace gpk

using namespace gpk;

extern "C" size_t gpk_collapsed_elbo_workspace_bytes(int64_t n, int64_t m, int d, int precision) {
  if (n <= 0 || m <= 0 || d <= 0) return 256;
  if (precision == GPK_PREC_FP64) {
    SgprBuf<double> b;
    return sgpr_layout<double>(n, m, d, nullptr, b);
  }
  SgprBuf<float> b;
  return sgpr_layout<float>(n, m, d, nullptr, b);
}

extern "C" gpk_status gpk_collapsed_elbo(int kind, int64_t n, int64_t m, int d, const double* x,
                                         int64_t ldx, const double* y, const double* z,
                                         int64_t ldz, const double* theta, int n_ls,
                                         double jitter, int precision, int want_grad,
                                         double* out_elbo, double* out_grad, double* out_grad_z,
                                         int* info, void* workspace, size_t workspace_bytes,
                                         cudaStream_t stream) {
  if (kind < GPK_RBF || kind > GPK_RATIONAL_QUADRATIC) return GPK_ERR_BAD_ARG;
  if (n <= 0 || m <= 0 || n > (int64_t)1 << 28 || m > 16384) return GPK_ERR_BAD_ARG;
  if (d <= 0 || d > DMAXS || ldx < d || ldz < d || !(n_ls == 1 || n_ls == d))
    return GPK_ERR_BAD_ARG;
  if (precision != GPK_PREC_FP64 && precision != GPK_PREC_MIXED) return GPK_ERR_BAD_ARG;
  if (!x || !y || !z || !theta || !out_elbo || !info || !workspace) return GPK_ERR_BAD_ARG;
  if (want_grad && (!out_grad || !out_grad_z)) return GPK_ERR_BAD_ARG;
  if (workspace_bytes < gpk_collapsed_elbo_workspace_bytes(n, m, d, precision))
    return GPK_ERR_WORKSPACE;
  if (precision == GPK_PREC_FP64)
    return sgpr_run<double>(kind, (int)n, (int)m, d, x, ldx, y, z, ldz, theta, n_ls, jitter,
                            want_grad, out_elbo, out_grad, out_grad_z, info, workspace, stream);
  return sgpr_run<float>(kind, (int)n, (int)m, d, x, ldx, y, z, ldz, theta, n_ls, jitter,
                         want_grad, out_elbo, out_grad, out_grad_z, info, workspace, stream);
}

extern "C" gpk_status gpk_collapsed_elbo_sharded(
    int kind, int64_t n_local, int64_t n_total, int64_t m, int d, const double* x, int64_t ldx,
    const double* y, const double* z, int64_t ldz, const double* theta, int n_ls, double jitter,
    int precision, int want_grad, double* out_elbo, double* out_grad, double* out_grad_z,
    int* info, void* workspace, size_t workspace_bytes, cudaStream_t stream,
    gpk_allreduce_fn allreduce, void* user) {
  if (kind < GPK_RBF || kind > GPK_RATIONAL_QUADRATIC) return GPK_ERR_BAD_ARG;
  if (n_local <= 0 || n_total < n_local || m <= 0 || n_total > (int64_t)1 << 31 || m > 16384)
    return GPK_ERR_BAD_ARG;
  if (d <= 0 || d > DMAXS || ldx < d || ldz < d || !(n_ls == 1 || n_ls == d))
    return GPK_ERR_BAD_ARG;
  if (precision != GPK_PREC_FP64 && precision != GPK_PREC_MIXED) return GPK_ERR_BAD_ARG;
  if (!x || !y || !z || !theta || !out_elbo || !info || !workspace || !allreduce)
    return GPK_ERR_BAD_ARG;
  if (want_grad && (!out_grad || !out_grad_z)) return GPK_ERR_BAD_ARG;
  if (n_local > (int64_t)1 << 28) return GPK_ERR_BAD_ARG;
  if (workspace_bytes < gpk_collapsed_elbo_workspace_bytes(n_local, m, d, precision))
    return GPK_ERR_WORKSPACE;
  Exchange ex;
  ex.fn = allreduce;
  ex.user = user;
  ex.ws = workspace;
  if (precision == GPK_PREC_FP64)
    return sgpr_run<double>(kind, (int)n_local, (int)m, d, x, ldx, y, z, ldz, theta, n_ls, jitter,
                            want_grad, out_elbo, out_grad, out_grad_z, info, workspace, stream, ex,
                            n_total);
  return sgpr_run<float>(kind, (int)n_local, (int)m, d, x, ldx, y, z, ldz, theta, n_ls, jitter,
                         want_grad, out_elbo, out_grad, out_grad_z, info, workspace, stream, ex,
                         n_total);
}
