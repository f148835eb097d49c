// Register-tiled CUDA-core main loop shared by the SIMT GEMM and the fused
// inverse-product/gradient kernel: acc += A[i0:i0+BM, k] * B[j0:j0+BN, k]^T.
#pragma once
#include "gpk_internal.cuh"

namespace gpk {

template <typename T> struct GemmCfg;
template <> struct GemmCfg<double> {
  static constexpr int BM = 64, BN = 64, BK = 16, TM = 4, TN = 4;
};
template <> struct GemmCfg<float> {
  static constexpr int BM = 128, BN = 128, BK = 16, TM = 8, TN = 8;
};
// Quarter-size tiles for products whose full-size grid would leave most SMs
// idle (float64 throughput per SM is low on this part, so a lone 64 x 64
// tile is slow): four times the CTAs, same 256 threads.
template <typename T> struct GemmCfgSmall;
template <> struct GemmCfgSmall<double> {
  static constexpr int BM = 32, BN = 32, BK = 16, TM = 2, TN = 2;
};
template <> struct GemmCfgSmall<float> {
  static constexpr int BM = 64, BN = 64, BK = 16, TM = 4, TN = 4;
};

// Linear lower-triangle tile index t -> (I, J), I >= J.  A float32 estimate
// corrected by the integer loops (every thread of a CTA calls this; float64
// square roots are slow on this part).
__device__ __forceinline__ void tri_index(int t, int& I, int& J) {
  int i = (int)((sqrtf(8.f * (float)t + 1.f) - 1.f) * 0.5f);
  while (i * (i + 1) / 2 > t) --i;
  while ((i + 1) * (i + 2) / 2 <= t) ++i;
  I = i;
  J = t - i * (i + 1) / 2;
}

template <typename T>
__device__ __forceinline__ T load_masked(const T* P, int64_t ld, int r, int c, int rows, int khi,
                                         int tri) {
  if (r >= rows || c >= khi) return T(0);
  if (tri == TRI_LOWER && c > r) return T(0);
  if (tri == TRI_UPPER && c < r) return T(0);
  return P[(int64_t)r * ld + c];
}

// K range of tile (i0, j0) given the operands' triangular structure.
template <int BM, int BN, int BK>
__device__ __forceinline__ void tile_krange(int K, int a_tri, int b_tri, int i0, int j0, int& klo,
                                            int& khi) {
  klo = 0;
  khi = K;
  if (a_tri == TRI_LOWER) khi = min(khi, i0 + BM);
  if (a_tri == TRI_UPPER) klo = max(klo, i0);
  if (b_tri == TRI_LOWER) khi = min(khi, j0 + BN);
  if (b_tri == TRI_UPPER) klo = max(klo, j0);
  klo = (klo / BK) * BK;
}

template <typename T, typename Cfg = GemmCfg<T>>
struct SimtSmem {
  T As[Cfg::BK][Cfg::BM + 4];
  T Bs[Cfg::BK][Cfg::BN + 4];
};

template <typename T, typename Cfg = GemmCfg<T>>
__device__ __forceinline__ void simt_tile_mma(const T* A, int64_t lda, int M, int a_tri, const T* B,
                                              int64_t ldb, int N, int b_tri, int i0, int j0,
                                              int klo, int khi, SimtSmem<T, Cfg>& sm,
                                              T (&acc)[Cfg::TM][Cfg::TN]) {
  constexpr int BM = Cfg::BM, BN = Cfg::BN, BK = Cfg::BK;
  constexpr int TM = Cfg::TM, TN = Cfg::TN;
  constexpr int NTX = BN / TN, NTY = BM / TM, NT = NTX * NTY;
  const int tx = threadIdx.x % NTX, ty = threadIdx.x / NTX;
  for (int k0 = klo; k0 < khi; k0 += BK) {
    for (int e = threadIdx.x; e < BM * BK; e += NT) {
      int r = e / BK, kk = e % BK;
      sm.As[kk][r] = load_masked(A, lda, i0 + r, k0 + kk, M, khi, a_tri);
    }
    for (int e = threadIdx.x; e < BN * BK; e += NT) {
      int r = e / BK, kk = e % BK;
      sm.Bs[kk][r] = load_masked(B, ldb, j0 + r, k0 + kk, N, khi, b_tri);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T av[TM], bv[TN];
#pragma unroll
      for (int a = 0; a < TM; ++a) av[a] = sm.As[kk][ty + a * NTY];
#pragma unroll
      for (int b = 0; b < TN; ++b) bv[b] = sm.Bs[kk][tx + b * NTX];
#pragma unroll
      for (int a = 0; a < TM; ++a)
#pragma unroll
        for (int b = 0; b < TN; ++b) acc[a][b] = fma(av[a], bv[b], acc[a][b]);
    }
    __syncthreads();
  }
}

}  // namespace gpk
