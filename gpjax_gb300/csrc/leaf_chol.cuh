// The 128 x 128 leaf of the recursive Cholesky + inverse: one CTA of 512
// threads factors a diagonal block of the (Schur-complemented) matrix with
// pivots from a float64 diagonal track and inverts it, in float32 with
// float-float pivots.  Shared by the tensor-core factorisation
// (mixed_tc.cu), which stores M as TF32 hi/lo pairs, and the persistent
// batched factorisation (batched.cu), which stores it as float32.
#pragma once
#include "gpk_common.cuh"

namespace gpk {

constexpr int LEAF = 128;
constexpr int LEAF_NT = 512;  // threads of the leaf kernel

constexpr int LEAF_PB = 32;             // panel width
constexpr int LEAF_LDT = LEAF + 4;      // k-major L and row-major M: 16-byte rows
constexpr int LEAF_TLD = 64 + 4;        // merge product rows
constexpr int LEAF_WNT = LEAF_NT - 32;  // panel-loop threads; the last warp inverts diagonal blocks

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

__device__ __forceinline__ void bar_sync_n(int id, int n) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}
__device__ __forceinline__ void bar_arrive_n(int id, int n) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory");
}

__device__ __forceinline__ void fma2x4(float (&acc)[2][4], const float2 a, const float4 b) {
  const float av[2] = {a.x, a.y}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(av[u], bv[v], acc[u][v]);
}

__device__ __forceinline__ void fma4x4(float (&acc)[4][4], const float4 a, const float4 b) {
  const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(av[u], bv[v], acc[u][v]);
}

// Columns [k0, k0+nk) of the block into k-major L (lane = row: conflict-free)
__device__ __forceinline__ void leaf_load_cols(const float* __restrict__ A, int64_t lda, int o,
                                               float* LT, int k0, int nk, int t, int nth) {
  constexpr int N = LEAF, CH = 8;  // float4 loads in flight per thread
  const int total = N * (nk / 4);
  for (int base = t; base < total; base += CH * nth) {
    float4 v[CH];
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int e = base + u * nth;
      if (e < total)
        v[u] = *reinterpret_cast<const float4*>(A + (int64_t)(o + e % N) * lda + o + k0 + 4 * (e / N));
    }
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int e = base + u * nth;
      if (e < total) {
        const int i = e % N, k = k0 + 4 * (e / N);
        LT[(k + 0) * LEAF_LDT + i] = v[u].x;
        LT[(k + 1) * LEAF_LDT + i] = v[u].y;
        LT[(k + 2) * LEAF_LDT + i] = v[u].z;
        LT[(k + 3) * LEAF_LDT + i] = v[u].w;
      }
    }
  }
}


inline size_t leaf_smem_bytes() {
  return (size_t)(2 * LEAF * LEAF_LDT + 64 * LEAF_TLD + 5 * LEAF) * sizeof(float);
}

// One CTA: Cholesky of the 128 x 128 diagonal block at (o, o) and its inverse.
// Pivots come from the float64 diagonal track, carried as float-float pairs.
//  * blocked right-looking factor over 32-wide panels (warps 0..14): one warp
//    factors the diagonal block in registers, one thread per row substitutes
//    the rows below it, then a rank-32 update of the lower trailing part from
//    the k-major L (4 x 4 tiles, float4 operands);
//  * the last warp inverts each 32 x 32 diagonal block as soon as it is
//    factored (handed over through a named barrier) and writes it out;
//  * two doubling merges M21 = -M22 (L21 M11), 2 x 4 register tiles, fill
//    the rest of M.
// Hands the lower blocks of M and the upper blocks of V = M^T (from the
// row-major M in shared memory) to out.put_m / out.put_v and writes half the
// log of each pivot; the caller supplies the 160 KB of shared memory
// (leaf_smem_bytes) and 512 threads.
template <class Out>
__device__ __forceinline__ void leaf_chol_inv_body(const float* __restrict__ A, int64_t lda, int o,
                                                   const double* __restrict__ dtrack,
                                                   double* __restrict__ logdiag,
                                                   int* __restrict__ info, const Out& out,
                                                   float* leaf_smem) {
  constexpr int N = LEAF, NT = LEAF_NT, PB = LEAF_PB, LDT = LEAF_LDT, TLD = LEAF_TLD,
                WNT = LEAF_WNT;
  static_assert(N == 128 && NT == 512, "tile maps below assume a 128-wide leaf and 512 threads");
  float* LT = leaf_smem;      // [N][LDT]  LT[k][i] = L[i][k]
  float* Ms = LT + N * LDT;   // [N][LDT]  M = L^-1, row-major
  float* Tt = Ms + N * LDT;   // [64][TLD] merge products; column buffer of the diagonal factor
  float* Dh = Tt + 64 * TLD;  // float-float diagonal track
  float* Dlo = Dh + N;
  float* Ph = Dlo + N;        // float-float pivots
  float* Pl = Ph + N;
  float* Rl = Pl + N;         // 1 / diag(L)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // ---- the block into k-major L, the diagonal track, M = 0 ----
  leaf_load_cols(A, lda, o, LT, 0, N, tid, NT);
  for (int e = tid; e < N * LDT / 4; e += NT)
    reinterpret_cast<float4*>(Ms)[e] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (tid < N) {
    const double dv = dtrack[o + tid];
    const float hi = (float)dv;
    Dh[tid] = hi;
    Dlo[tid] = (float)(dv - (double)hi);
  }
  __syncthreads();

  if (warp < WNT / 32) {
    // ---- blocked right-looking Cholesky over 32-wide panels (warps 0..14) ----
    for (int p = 0; p < N / PB; ++p) {
      const int c0 = p * PB;
      if (warp == 0) {
        // P1: the diagonal block in registers, lane = row; the next pivot
        // comes from a float32 candidate one FMA away while the float-float
        // track is updated off that dependency chain; the new column is
        // broadcast through a double-buffered shared row
        const int row = c0 + lane;
        float r[PB];
#pragma unroll
        for (int k = 0; k < PB; ++k) r[k] = LT[(c0 + k) * LDT + row];
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
          const bool below = lane > j;
          const float npf = fmaf(-lij, lij, dh) + dlo;
          float nh = dh, nl = dlo;
          ff_sub_sq(nh, nl, lij);
          r[j] = below ? lij : r[j];
          pf = below ? npf : pf;
          dh = below ? nh : dh;
          dlo = below ? nl : dlo;
          float* colb = Tt + (j & 1) * PB;  // double-buffered column
          colb[lane] = lij;
          __syncwarp();
#pragma unroll
          for (int g = (j + 1) / 4; g < PB / 4; ++g) {
            const float4 c4 = *reinterpret_cast<const float4*>(colb + 4 * g);
            if (4 * g + 0 > j) r[4 * g + 0] = fmaf(-lij, c4.x, r[4 * g + 0]);
            if (4 * g + 1 > j) r[4 * g + 1] = fmaf(-lij, c4.y, r[4 * g + 1]);
            if (4 * g + 2 > j) r[4 * g + 2] = fmaf(-lij, c4.z, r[4 * g + 2]);
            if (4 * g + 3 > j) r[4 * g + 3] = fmaf(-lij, c4.w, r[4 * g + 3]);
          }
        }
#pragma unroll
        for (int k = 0; k < PB; ++k) LT[(c0 + k) * LDT + row] = (k < lane) ? r[k] : 0.f;
        bar_arrive_n(2 + p, 64);  // diagonal block p is final: hand it to the inverting warp
      }
      bar_sync_n(1, WNT);
      // P2: rows below the panel by substitution, one thread per row
      const int r0 = c0 + PB, R = N - r0;
      if (tid < R) {
        const int row = r0 + tid;
        float a[PB], rl[PB];
#pragma unroll
        for (int k = 0; k < PB; ++k) a[k] = LT[(c0 + k) * LDT + row];
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
            if (4 * g + 3 > m) {  // column m of the diagonal block: zeros on and above it
              const float4 l = *reinterpret_cast<const float4*>(LT + (c0 + m) * LDT + c0 + 4 * g);
              if (4 * g + 0 > m) a[4 * g + 0] = fmaf(-x, l.x, a[4 * g + 0]);
              if (4 * g + 1 > m) a[4 * g + 1] = fmaf(-x, l.y, a[4 * g + 1]);
              if (4 * g + 2 > m) a[4 * g + 2] = fmaf(-x, l.z, a[4 * g + 2]);
              a[4 * g + 3] = fmaf(-x, l.w, a[4 * g + 3]);
            }
          }
        }
#pragma unroll
        for (int k = 0; k < PB; ++k) LT[(c0 + k) * LDT + row] = a[k];
      }
      bar_sync_n(1, WNT);
      // P3: rank-32 update of the lower trailing part, 4 x 4 tiles enumerated
      // by tile column (a warp's lanes share the column and walk the rows);
      // other threads take the squares off the float-float diagonal track
      if (R > 0) {
        const int T = R / 4, ntiles = T * (T + 1) / 2;
        for (int t = tid; t < ntiles; t += WNT) {
          int tc = 0, rem = t;
          while (rem >= T - tc) {
            rem -= T - tc;
            ++tc;
          }
          const int R0 = r0 + 4 * (tc + rem), C0 = r0 + 4 * tc;
          float acc[4][4];
#pragma unroll
          for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
#pragma unroll 8
          for (int k = 0; k < PB; ++k)
            fma4x4(acc, *reinterpret_cast<const float4*>(LT + (c0 + k) * LDT + R0),
                   *reinterpret_cast<const float4*>(LT + (c0 + k) * LDT + C0));
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            float4* d = reinterpret_cast<float4*>(LT + (C0 + v) * LDT + R0);
            float4 x = *d;
            x.x -= acc[0][v];
            x.y -= acc[1][v];
            x.z -= acc[2][v];
            x.w -= acc[3][v];
            *d = x;
          }
        }
        if (tid >= WNT - R) {
          const int row = r0 + tid - (WNT - R);
          float dh = Dh[row], dlo = Dlo[row];
#pragma unroll
          for (int k = 0; k < PB; ++k) ff_sub_sq(dh, dlo, LT[(c0 + k) * LDT + row]);
          Dh[row] = dh;
          Dlo[row] = dlo;
        }
        bar_sync_n(1, WNT);
      }
    }
  } else {
    // ---- last warp: invert each diagonal block as soon as it is factored
    //      (lane = column; right-looking, float4 reads down L's columns) and
    //      write it out, M and V = M^T ----
    for (int p = 0; p < N / PB; ++p) {
      const int c0 = p * PB, cc = lane;
      bar_sync_n(2 + p, 64);
      float acc[PB], mc[PB];
#pragma unroll
      for (int i = 0; i < PB; ++i) acc[i] = 0.f;
#pragma unroll
      for (int k = 0; k < PB; ++k) {
        const float rlk = Rl[c0 + k];
        mc[k] = rlk * ((k == cc) ? 1.f - acc[k] : -acc[k]);  // zero for k < cc
#pragma unroll
        for (int g = 0; g < PB / 4; ++g) {
          if (4 * g + 3 > k) {
            const float4 l = *reinterpret_cast<const float4*>(LT + (c0 + k) * LDT + c0 + 4 * g);
            if (4 * g + 0 > k) acc[4 * g + 0] = fmaf(l.x, mc[k], acc[4 * g + 0]);
            if (4 * g + 1 > k) acc[4 * g + 1] = fmaf(l.y, mc[k], acc[4 * g + 1]);
            if (4 * g + 2 > k) acc[4 * g + 2] = fmaf(l.z, mc[k], acc[4 * g + 2]);
            acc[4 * g + 3] = fmaf(l.w, mc[k], acc[4 * g + 3]);
          }
        }
      }
#pragma unroll
      for (int i = 0; i < PB; ++i) Ms[(c0 + i) * LDT + c0 + cc] = mc[i];
      __syncwarp();
      out.put_m(Ms, c0, PB, c0, PB, lane, 32);
      out.put_v(Ms, c0, PB, c0, PB, lane, 32);
    }
  }
  __syncthreads();
  if (tid >= 384) {  // idle during every merge phase below
    const int i = tid - 384;
    const double pv = (double)Ph[i] + (double)Pl[i];
    logdiag[o + i] = 0.5 * log(pv);
    if (!(pv > 0.0)) atomicMin(info, o + i + 1);
  }
  // ---- off-diagonal blocks of M by doubling merges, M21 = -M22 (L21 M11),
  //      2 x 4 tiles with float2 / float4 operands: both 32-wide pairs, then 64 ----
  if (tid < 256) {  // T = L21 M11 for the pairs at 0 and 64 (lanes walk row pairs)
    const int pr = tid >> 7, b = tid & 127, ob = pr * 64;
    const int i0 = (b & 15) * 2, j0 = (b >> 4) * 4;
    float acc[2][4] = {};
#pragma unroll 4
    for (int c = j0; c < PB; ++c) {  // M11[c][j] = 0 for c < j
      const float2 a2 = *reinterpret_cast<const float2*>(LT + (ob + c) * LDT + ob + PB + i0);
      const float4 b4 = *reinterpret_cast<const float4*>(Ms + (ob + c) * LDT + ob + j0);
      fma2x4(acc, a2, b4);
    }
    float* T = Tt + pr * PB * TLD;
#pragma unroll
    for (int u = 0; u < 2; ++u)
      *reinterpret_cast<float4*>(T + (i0 + u) * TLD + j0) =
          make_float4(acc[u][0], acc[u][1], acc[u][2], acc[u][3]);
  }
  __syncthreads();
  if (tid < 256) {  // M21 = -M22 T
    const int pr = tid >> 7, b = tid & 127, ob = pr * 64;
    const int i0 = (b & 15) * 2, j0 = (b >> 4) * 4;
    const float* T = Tt + pr * PB * TLD;
    float acc[2][4] = {};
#pragma unroll 2
    for (int c4 = 0; c4 <= (i0 + 1) / 4; ++c4) {  // M22[i][c] = 0 for c > i
      const float4 m0 = *reinterpret_cast<const float4*>(Ms + (ob + PB + i0) * LDT + ob + PB + 4 * c4);
      const float4 m1 = *reinterpret_cast<const float4*>(Ms + (ob + PB + i0 + 1) * LDT + ob + PB + 4 * c4);
      fma2x4(acc, make_float2(m0.x, m1.x), *reinterpret_cast<const float4*>(T + (4 * c4 + 0) * TLD + j0));
      fma2x4(acc, make_float2(m0.y, m1.y), *reinterpret_cast<const float4*>(T + (4 * c4 + 1) * TLD + j0));
      fma2x4(acc, make_float2(m0.z, m1.z), *reinterpret_cast<const float4*>(T + (4 * c4 + 2) * TLD + j0));
      fma2x4(acc, make_float2(m0.w, m1.w), *reinterpret_cast<const float4*>(T + (4 * c4 + 3) * TLD + j0));
    }
#pragma unroll
    for (int u = 0; u < 2; ++u)
      *reinterpret_cast<float4*>(Ms + (ob + PB + i0 + u) * LDT + ob + j0) =
          make_float4(-acc[u][0], -acc[u][1], -acc[u][2], -acc[u][3]);
  }
  __syncthreads();
  {  // T = L21 M11 for the 64-wide halves (lanes walk row pairs)
    const int i0 = (tid & 31) * 2, j0 = (tid >> 5) * 4;
    float acc[2][4] = {};
#pragma unroll 4
    for (int c = j0; c < 64; ++c) {
      const float2 a2 = *reinterpret_cast<const float2*>(LT + c * LDT + 64 + i0);
      const float4 b4 = *reinterpret_cast<const float4*>(Ms + c * LDT + j0);
      fma2x4(acc, a2, b4);
    }
#pragma unroll
    for (int u = 0; u < 2; ++u)
      *reinterpret_cast<float4*>(Tt + (i0 + u) * TLD + j0) =
          make_float4(acc[u][0], acc[u][1], acc[u][2], acc[u][3]);
  }
  __syncthreads();
  {  // M21 = -M22 T
    const int i0 = (tid & 31) * 2, j0 = (tid >> 5) * 4;
    float acc[2][4] = {};
#pragma unroll 2
    for (int c4 = 0; c4 <= (i0 + 1) / 4; ++c4) {
      const float4 m0 = *reinterpret_cast<const float4*>(Ms + (64 + i0) * LDT + 64 + 4 * c4);
      const float4 m1 = *reinterpret_cast<const float4*>(Ms + (64 + i0 + 1) * LDT + 64 + 4 * c4);
      fma2x4(acc, make_float2(m0.x, m1.x), *reinterpret_cast<const float4*>(Tt + (4 * c4 + 0) * TLD + j0));
      fma2x4(acc, make_float2(m0.y, m1.y), *reinterpret_cast<const float4*>(Tt + (4 * c4 + 1) * TLD + j0));
      fma2x4(acc, make_float2(m0.z, m1.z), *reinterpret_cast<const float4*>(Tt + (4 * c4 + 2) * TLD + j0));
      fma2x4(acc, make_float2(m0.w, m1.w), *reinterpret_cast<const float4*>(Tt + (4 * c4 + 3) * TLD + j0));
    }
#pragma unroll
    for (int u = 0; u < 2; ++u)
      *reinterpret_cast<float4*>(Ms + (64 + i0 + u) * LDT + j0) =
          make_float4(-acc[u][0], -acc[u][1], -acc[u][2], -acc[u][3]);
  }
  __syncthreads();
  // ---- the 64-wide merge result: M rows 64.., columns ..63 and its transpose ----
  out.put_m(Ms, 64, 64, 0, 64, tid, NT);
  out.put_v(Ms, 0, 64, 64, 64, tid, NT);
  out.put_m(Ms, PB, PB, 0, PB, tid, NT);
  out.put_m(Ms, 3 * PB, PB, 2 * PB, PB, tid, NT);
  out.put_v(Ms, 0, PB, PB, PB, tid, NT);
  out.put_v(Ms, 2 * PB, PB, 3 * PB, PB, tid, NT);
}

}  // namespace gpk
