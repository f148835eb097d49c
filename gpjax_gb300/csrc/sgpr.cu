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
// The m x n work (Phi, P, c, the fused H Phi adjoint) runs in T (float64 for
// the plain form, float32 for the mixed form); the m x m algebra always runs
// in float64.  Reductions go through per-block partials summed in a fixed
// order.
#include <climits>
#include "gpk_internal.cuh"

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

template <typename T>
struct SgprBuf {
  int64_t ldn, ldm;
  int nchunks;
  T *zs, *xs, *Phi, *Pparts, *Ht;
  double *zs64, *Kf, *Lz, *Mz, *Vz, *Kinv, *Su, *Mu, *Vu, *Suinv, *P64, *T1, *KPK, *GK, *scr;
  double *dv, *cv, *phi1, *gam, *pgam, *ldK, *ldU, *red, *thK, *dzK, *thP, *dzP;
};

template <typename T>
size_t sgpr_layout(int64_t n, int64_t m, int d, void* ws, SgprBuf<T>& b) {
  Arena a(ws);
  b.ldn = pad64(n);
  b.ldm = pad64(m);
  b.nchunks = (int)((n + KCHUNK - 1) / KCHUNK);
  const size_t mm = (size_t)m * b.ldm;
  b.zs = a.take<T>((size_t)m * d);
  b.xs = a.take<T>((size_t)n * d);
  b.Phi = a.take<T>((size_t)m * b.ldn);
  b.Pparts = a.take<T>((size_t)b.nchunks * m * m);
  b.Ht = a.take<T>(mm);
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
  b.cv = a.take<double>(m);
  b.phi1 = a.take<double>(m);
  b.gam = a.take<double>(m);
  b.pgam = a.take<double>(m);
  b.ldK = a.take<double>(m);
  b.ldU = a.take<double>(m);
  b.red = a.take<double>(64);
  b.thK = a.take<double>((size_t)m * (d + 1));
  b.dzK = a.take<double>((size_t)m * d);
  const int mt = (int)((m + AB - 1) / AB);
  b.thP = a.take<double>((size_t)ASPLIT * mt * (d + 1));
  b.dzP = a.take<double>((size_t)ASPLIT * m * d);
  return a.off + 256;
}

__global__ void sg_init(int* info, const double* __restrict__ y, const double* __restrict__ theta,
                        int n_ls, int n, double* __restrict__ dv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) *info = INT_MAX;
  if (i < n) dv[i] = y[i] - theta[n_ls + 2];
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

// H (in T), GK (float64) and the traces tr(K^-1 P), tr(Su^-1 P) (block partials)
template <typename T>
__global__ void sg_combine(int m, int64_t ldm, const double* __restrict__ Kinv,
                           const double* __restrict__ Suinv, const double* __restrict__ KPK,
                           const double* __restrict__ P64, const double* __restrict__ gam,
                           const double* __restrict__ theta, int n_ls, T* __restrict__ Ht,
                           double* __restrict__ GK, double* __restrict__ red) {
  const double sd = theta[n_ls + 1], s = sd * sd;
  double tK = 0.0, tU = 0.0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < (int64_t)m * m;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / m), j = (int)(e % m);
    const int64_t o = (int64_t)i * ldm + j;
    const double ki = Kinv[o], ui = Suinv[o], gg = gam[i] * gam[j], p = P64[o];
    Ht[o] = (T)((ki - ui) / s - gg / (s * s * s));
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
                double* __restrict__ dzK) {
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
    kval_dcoef<double>(kind, sq, 1.0, k1, c1);
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
        kval_dcoef<T>(kind, sq, T(1), k1, c1);
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

// value, theta gradient and the Z gradient from all partials
__global__ void __launch_bounds__(256)
    sg_finalize(int n, int m, int d, const double* __restrict__ theta, int n_ls,
                const double* __restrict__ ldK, const double* __restrict__ ldU,
                const double* __restrict__ dv, const double* __restrict__ cv,
                const double* __restrict__ gam, const double* __restrict__ pgam,
                const double* __restrict__ phi1, const double* __restrict__ red,
                const double* __restrict__ thK, const double* __restrict__ dzK,
                const double* __restrict__ thP, const double* __restrict__ dzP, int mt,
                int want_grad, int* __restrict__ info, double* __restrict__ out_elbo,
                double* __restrict__ out_grad, double* __restrict__ out_gz) {
  __shared__ double sh[8];
  __shared__ double sth[GPK_MAX_D + 2];
  __shared__ double part[7][256];
  const int tid = threadIdx.x;
  {
    double a = 0.0, b = 0.0, cg = 0.0, gpg = 0.0, pg1 = 0.0, dd = 0.0, ds = 0.0;
    for (int i = tid; i < m; i += blockDim.x) {
      a += ldK[i];
      b += ldU[i];
      cg += cv[i] * gam[i];
      gpg += gam[i] * pgam[i];
      pg1 += phi1[i] * gam[i];
    }
    for (int j = tid; j < n; j += blockDim.x) {
      dd += dv[j] * dv[j];
      ds += dv[j];
    }
    part[0][tid] = a;
    part[1][tid] = b;
    part[2][tid] = cg;
    part[3][tid] = gpg;
    part[4][tid] = pg1;
    part[5][tid] = dd;
    part[6][tid] = ds;
  }
  __syncthreads();
  if (tid < 7) {
    double t = 0.0;
    for (int q = 0; q < (int)blockDim.x; ++q) t += part[tid][q];
    sh[tid] = (tid < 2) ? 2.0 * t : t;  // log|K|, log|Su| from log-diagonals
  }
  __syncthreads();
  if (want_grad) {
    for (int k = tid; k <= d; k += blockDim.x) {
      double t = 0.0;
      for (int i = 0; i < m; ++i) t += thK[(int64_t)i * (d + 1) + k];
      for (int q = 0; q < ASPLIT * mt; ++q) t += thP[(int64_t)q * (d + 1) + k];
      sth[k] = t;
    }
  }
  __syncthreads();
  int inf = *info;
  if (inf == INT_MAX) inf = 0;
  const double nan = __longlong_as_double(0x7ff8000000000000ULL);
  const double s2 = theta[n_ls], sd = theta[n_ls + 1], s = sd * sd;
  if (want_grad) {
    for (int e = tid; e < m * d; e += blockDim.x) {
      const int i = e / d, k = e % d;
      double t = dzK[e];
      for (int q = 0; q < ASPLIT; ++q) t += dzP[((int64_t)q * m + i) * d + k];
      const double l = theta[n_ls == 1 ? 0 : k];
      out_gz[e] = inf ? nan : -s2 * t / l;
    }
  }
  if (tid != 0) return;
  *info = inf;
  const double ldK_ = sh[0], ldU_ = sh[1], cg = sh[2], gpg = sh[3], pg1 = sh[4], dd = sh[5],
               ds = sh[6];
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

__global__ void sg_zero(double* p, int count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) p[i] = 0.0;
}

template <typename T>
gpk_status sgpr_run(int kind, int n, int m, int d, const double* x, int64_t ldx, const double* y,
                    const double* z, int64_t ldz, const double* theta, int n_ls, double jitter,
                    int want_grad, double* out_elbo, double* out_grad, double* out_gz, int* info,
                    void* ws, cudaStream_t s) {
  SgprBuf<T> b;
  sgpr_layout<T>(n, m, d, ws, b);
  const int64_t ldm = b.ldm;
  sg_init<<<(int)cdiv(n, 256), 256, 0, s>>>(info, y, theta, n_ls, n, b.dv);
  GPK_LAUNCH_CHECK();
  sg_zero<<<1, 64, 0, s>>>(b.red, 64);
  GPK_LAUNCH_CHECK();
  GPK_CUDA_TRY(scale_inputs<T>(x, ldx, n, d, theta, n_ls, b.xs, s));
  GPK_CUDA_TRY(scale_inputs<T>(z, ldz, m, d, theta, n_ls, b.zs, s));
  GPK_CUDA_TRY(scale_inputs<double>(z, ldz, m, d, theta, n_ls, b.zs64, s));
  // Phi = K(z, x) (m x n, T), c = Phi d, phi1 = Phi 1
  GPK_CUDA_TRY(cross_cov_scaled<T, T>(kind, m, n, d, b.zs, b.xs, theta, n_ls, 0, 0.0, b.Phi, b.ldn,
                                      s));
  sg_phi_gemv<T><<<(int)cdiv((int64_t)m * 32, 256), 256, 0, s>>>(b.Phi, b.ldn, m, n, b.dv, b.cv,
                                                                   b.phi1);
  GPK_LAUNCH_CHECK();
  // P: lower triangles of Phi_k Phi_k^T per n-chunk, summed in float64
  {
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
  // K (float64, full) and Lz
  GPK_CUDA_TRY(cross_cov_scaled<double, double>(kind, m, m, d, b.zs64, b.zs64, theta, n_ls, 0, 0.0,
                                                b.Kf, ldm, s));
  GPK_CUDA_TRY(cross_cov_scaled<double, double>(kind, m, m, d, b.zs64, b.zs64, theta, n_ls, 2,
                                                jitter, b.Lz, ldm, s));
  sg_reduce_P<T><<<(int)cdiv((int64_t)m * m, 256), 256, 0, s>>>(b.Pparts, b.nchunks, m, ldm, b.Kf,
                                                                  theta, n_ls, jitter, b.P64, b.Su);
  GPK_LAUNCH_CHECK();
  GPK_CUDA_TRY(potrf_lower<double>(b.Lz, ldm, m, b.ldK, info, nullptr, false, s));
  GPK_CUDA_TRY(trtri_lower<double>(b.Lz, ldm, m, b.Mz, ldm, b.Vz, ldm, b.scr, s));
  GPK_CUDA_TRY(potrf_lower<double>(b.Su, ldm, m, b.ldU, info, nullptr, true, s));
  GPK_CUDA_TRY(trtri_lower<double>(b.Su, ldm, m, b.Mu, ldm, b.Vu, ldm, b.scr, s));
  {  // K^-1 = Vz Vz^T, Su^-1 = Vu Vu^T (full squares)
    GemmProb<double> p{};
    p.A = b.Vz;
    p.B = b.Vz;
    p.lda = p.ldb = ldm;
    p.a_tri = p.b_tri = TRI_UPPER;
    p.C = b.Kinv;
    p.ldc = ldm;
    p.M = p.N = p.K = m;
    p.alpha = 1.0;
    p.beta = 0.0;
    GPK_CUDA_TRY(gemm_nt<double>(p, 1, s));
    p.A = b.Vu;
    p.B = b.Vu;
    p.C = b.Suinv;
    GPK_CUDA_TRY(gemm_nt<double>(p, 1, s));
    // T1 = K^-1 P ; KPK = T1 K^-1   (symmetric operands: NT form)
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
    GPK_CUDA_TRY(gemm_nt<double>(q, 1, s));
  }
  GPK_CUDA_TRY(gemv_dense<double>(b.Suinv, ldm, m, m, b.cv, b.gam, s));
  GPK_CUDA_TRY(gemv_dense<double>(b.P64, ldm, m, m, b.gam, b.pgam, s));
  sg_combine<T><<<256, 256, 0, s>>>(m, ldm, b.Kinv, b.Suinv, b.KPK, b.P64, b.gam, theta, n_ls,
                                    b.Ht, b.GK, b.red);
  GPK_LAUNCH_CHECK();
  const int mt = (m + AB - 1) / AB;
  if (want_grad) {
    sg_grad_kzz<<<m, 256, 0, s>>>(kind, m, d, ldm, b.zs64, b.GK, b.thK, b.dzK);
    GPK_LAUNCH_CHECK();
    dim3 grid(mt, ASPLIT);
    const size_t smem = (size_t)(2 * 16 + AB) * (AB + 1) * sizeof(T) +
                        (size_t)2 * AB * (DMAXS + 1) * sizeof(T) + 16 +
                        (size_t)(AB + 8) * (DMAXS + 1) * sizeof(double);
    cudaFuncSetAttribute(sg_phi_adjoint<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    sg_phi_adjoint<T><<<grid, 256, smem, s>>>(kind, m, n, d, b.Ht, ldm, b.Phi, b.ldn, b.zs, b.xs,
                                           b.gam, b.dv, theta, n_ls, b.thP, b.dzP);
    GPK_LAUNCH_CHECK();
  }
  sg_finalize<<<1, 256, 0, s>>>(n, m, d, theta, n_ls, b.ldK, b.ldU, b.dv, b.cv, b.gam, b.pgam,
                                b.phi1, b.red, b.thK, b.dzK, b.thP, b.dzP, mt, want_grad, info,
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
  if (kind < GPK_RBF || kind > GPK_MATERN52) return GPK_ERR_BAD_ARG;
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
