// tcgen05 split-TF32 NT GEMM: kernel, tensor-map encoding and launch helpers.
// See tc_gemm.cuh for the arithmetic.
#include <mutex>
#include "tc_gemm.cuh"
#include "tc_ptx.cuh"

namespace gpk {
namespace tc {

// float-float accumulation (hi, lo) += a with the rounding error of the
// addition kept (Knuth's two-sum); the _rn forms keep it from being contracted
__device__ __forceinline__ void ff_add(float& hi, float& lo, float a) {
  const float s = __fadd_rn(hi, a);
  const float bb = __fsub_rn(s, hi);
  lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(a, bb)));
  hi = s;
}

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void split_tf32(float x, float& hi, float& lo) {
  hi = tf32_rna(x);
  lo = tf32_rna(x - hi);
}

// ---------------------------------------------------------------------------
// The kernel
// ---------------------------------------------------------------------------
// Four tile shapes (TS).  Narrow (0): 128 x 128 outputs, 32-wide K slices in
// 128B swizzle, 3 stages of 64 KB, 4 accumulator buffers of 128 TMEM
// columns.  Wide (1, large GEMMs): 128 x 256 outputs, 16-wide K slices in 64B
// swizzle, 4 stages of 48 KB, 2 buffers of 256 columns: a quarter fewer
// operand bytes, from L2 and from shared memory, per multiply-add.  Half (2,
// small GEMMs): 128 x 64 outputs, 32-wide slices, 4 stages of 48 KB, 4 buffers
// of 64 columns: twice the CTAs of the narrow tile where that leaves SMs idle.
// Wide float16 (3): the wide tile's byte geometry (64-byte K slice rows, 64B
// swizzle, 4 stages of 48 KB) holding 32 float16 K elements per slice, two
// kind::f16 MMAs of K = 16 per slice.
template <int TS>
struct Tile {
  static constexpr bool F16 = TS == 3;
  static constexpr bool WIDE = TS == 1 || TS == 3;
  static constexpr int ELEM = F16 ? 2 : 4;  // operand bytes
  static constexpr int BN = WIDE ? 256 : (TS == 2 ? 64 : 128);
  static constexpr int BK = TS == 1 ? 16 : 32;
  static constexpr int STAGES = TS == 0 ? 3 : 4;
  static constexpr int SWZ = BK * ELEM;  // bytes of one K slice row
  static constexpr int A_BYTES = BM * BK * ELEM;
  static constexpr int B_BYTES = BN * BK * ELEM;
  static constexpr int STAGE_BYTES = 2 * (A_BYTES + B_BYTES);  // A_hi, A_lo, B_hi, B_lo
  static constexpr int NBUF = BN >= 128 ? 512 / BN : 4;        // TMEM accumulator buffers
  static constexpr int TMEM_COLS = NBUF * BN;                  // a power of two >= 32
  static constexpr int HC = BN / 2;  // accumulator columns owned by one epilogue thread
  static constexpr int TLD = BN + 4; // staged output tile row stride (floats)
  static constexpr int KSTEP = F16 ? 16 : 8;  // K elements per MMA (32 bytes either way)
  static constexpr int KS = BK / KSTEP;       // MMA K steps per K slice
  // MMA K steps (3 products each) summed by one TMEM accumulator before the
  // epilogue drains it.  The accumulator truncates each MMA's sum toward zero,
  // so a segment of k steps biases the tile by about k units of 2^-24 toward
  // zero on one-signed data (measured: 4 steps -3.3, 1 step -0.8).  The
  // narrow and half tiles, which carry every product of the small and middle
  // recursion nodes, drain after every step (this takes the mixed MLL from
  // 1.4e-5 to 4e-7 relative error on an RBF problem with condition number
  // ~4e3); the wide tiles of the large products drain every 4 steps, which
  // their epilogue keeps up with.
  static constexpr int KPSEG = (TS == 0 || TS == 2) ? 1 : 4;
};

template <int STAGES_>
struct SmemCtl {
  uint64_t full[STAGES_];
  uint64_t empty[STAGES_];
  uint64_t tfull[4];   // accumulator segment ready (MMA -> epilogue)
  uint64_t tempty[4];  // accumulator segment drained (epilogue -> MMA)
  uint64_t mdone;      // MMAs issued before an abort have completed
  uint32_t tmem;
  int abort_flag;
};

// The tensor-core float32 accumulator truncates toward zero (measured on
// positive products: a 12-MMA accumulator loses 3.3 units of 2^-24 of its
// magnitude on average, whatever K; more on operands of wide dynamic range),
// so each accumulator only sums Tile::KPSEG K steps, the hi*hi MMAs come after
// the cross products, and the epilogue warps drain finished segments into
// round-to-nearest float32 registers while the MMA thread fills the next of
// NBUF TMEM buffers.
constexpr int EPI_WARPS = 8;   // epilogue warps: two per TMEM lane quarter
constexpr int EPI_THREADS = EPI_WARPS * 32;

// Launch index -> output tile (I, J), grouped so that the CTAs resident at
// one time share operand panels in L2: groups of TILE_GROUP tile rows, walked
// column by column (consecutive CTAs take consecutive rows of one column).
// Row tiles are BM high, column tiles bn wide; for c_lower only tiles holding
// elements on or below the diagonal exist: row tile I reaches column tiles
// J < ncols(I), and column tile J starts at row tile imin(J).
constexpr int TILE_GROUP = 8;
__host__ __device__ inline int lower_ncols(int I, int tiles_n, int bn) {
  return min(tiles_n, (I * BM + BM - 1) / bn + 1);
}
__host__ __device__ inline void tile_of(int t, int c_lower, int tiles_m, int tiles_n, int bn,
                                        int& I, int& J) {
  constexpr int G = TILE_GROUP;
  if (!c_lower) {
    const int g = t / (G * tiles_n), l = t % (G * tiles_n);
    const int rows = min(G, tiles_m - g * G);
    J = l / rows;
    I = g * G + l % rows;
    return;
  }
  int g = 0, base = 0, rows = 0;
  for (;; ++g) {
    rows = min(G, tiles_m - g * G);
    int cnt = 0;
    for (int r = 0; r < rows; ++r) cnt += lower_ncols(g * G + r, tiles_n, bn);
    if (t < base + cnt) break;
    base += cnt;
  }
  int l = t - base;
  const int full_cols = lower_ncols(g * G, tiles_n, bn);  // every row of the group reaches these
  if (l < full_cols * rows) {
    J = l / rows;
    I = g * G + l % rows;
    return;
  }
  l -= full_cols * rows;
  for (J = full_cols;; ++J) {
    const int num = J * bn - BM + 1;
    const int imin = num > 0 ? (num + BM - 1) / BM : 0;
    const int r0 = max(g * G, imin);
    const int cnt = g * G + rows - r0;
    if (l < cnt) {
      I = r0 + l;
      return;
    }
    l -= cnt;
  }
}

// Number of launch indices tile_of maps (the grid of one GEMM).
__host__ __device__ inline int tile_count(int c_lower, int tiles_m, int tiles_n, int bn) {
  if (!c_lower) return tiles_m * tiles_n;
  int cnt = 0;
  for (int I = 0; I < tiles_m; ++I) cnt += lower_ncols(I, tiles_n, bn);
  return cnt;
}

// MODE: epilogue.  TS: tile shape (Tile<TS>).  DM: bound on the input
// dimension of the MODE_GRAD epilogue (registers scale with it).
template <int MODE, int TS, int DM>
__global__ void __launch_bounds__(NUM_THREADS, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap ta_hi, const __grid_constant__ CUtensorMap ta_lo,
                   const __grid_constant__ CUtensorMap tb_hi, const __grid_constant__ CUtensorMap tb_lo,
                   const __grid_constant__ TcParams p) {
  using TL = Tile<TS>;
  constexpr int BN = TL::BN, BK = TL::BK, STAGES = TL::STAGES, NBUF = TL::NBUF, HC = TL::HC,
                TLD = TL::TLD, STAGE_BYTES = TL::STAGE_BYTES, A_BYTES = TL::A_BYTES,
                B_BYTES = TL::B_BYTES;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* tiles = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  SmemCtl<STAGES>* ctl = reinterpret_cast<SmemCtl<STAGES>*>(tiles + STAGES * STAGE_BYTES);
  float* gx = reinterpret_cast<float*>(ctl + 1);  // MODE_GRAD: column points and alphas
  float* ga = gx + BN * DM;
  float* gsc = ga + BN;  // MODE_GRAD: column scales of a scaled operand
  double* gred = reinterpret_cast<double*>(gsc + BN);
  float* otile = reinterpret_cast<float*>(tiles);  // output tile, reuses the operand ring

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int z = blockIdx.z;
  int I, J;
  tile_of(blockIdx.x, p.c_lower, p.tiles_m, p.tiles_n, BN, I, J);
  const int i0 = I * BM, j0 = J * BN;
  int klo = 0, khi = p.K;
  if (p.a_tri == TRI_LOWER) khi = min(khi, i0 + BM);
  if (p.a_tri == TRI_UPPER) klo = max(klo, i0);
  if (p.b_tri == TRI_LOWER) khi = min(khi, j0 + BN);
  if (p.b_tri == TRI_UPPER) klo = max(klo, j0);
  klo = (klo / BK) * BK;
  const int nk = khi > klo ? (khi - klo + BK - 1) / BK : 0;
  const int nseg = (nk * TL::KS + TL::KPSEG - 1) / TL::KPSEG;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&ctl->full[s], 1);
      mbar_init(&ctl->empty[s], 1);
    }
    for (int b = 0; b < NBUF; ++b) {
      mbar_init(&ctl->tfull[b], 1);
      mbar_init(&ctl->tempty[b], EPI_WARPS);  // one arrival per epilogue warp
    }
    mbar_init(&ctl->mdone, 1);
    ctl->abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&ctl->tmem)),
                 "r"(TL::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  pdl_wait();  // everything above touched no input of the previous kernel
  pdl_trigger();
  const uint32_t tmem = ctl->tmem;
  volatile int* abort_flag = &ctl->abort_flag;
  const long long wlim = p.wait_cycles > 0 ? p.wait_cycles : kWaitCycles;

  if (warp == 0) {
    if (lane == 0 && nk > 0) {
      const int ay = i0 + p.a_row0 + z * p.a_zrow, ax0 = p.a_col0 + z * p.a_zcol;
      const int by = j0 + p.b_row0 + z * p.b_zrow, bx0 = p.b_col0 + z * p.b_zcol;
      int issued = 0;
      for (int kc = 0; kc < nk; ++kc) {
        const int s = kc % STAGES;
        if (kc >= STAGES) {
          if (!mbar_wait(&ctl->empty[s], ((kc / STAGES) - 1) & 1, abort_flag, p.err, wlim)) break;
        }
        uint8_t* st = tiles + s * STAGE_BYTES;
        const int k = klo + kc * BK;
        mbar_expect_tx(&ctl->full[s], STAGE_BYTES);
        tma_load_2d(st, &ta_hi, ax0 + k, ay, &ctl->full[s]);
        tma_load_2d(st + A_BYTES, &ta_lo, ax0 + k, ay, &ctl->full[s]);
        tma_load_2d(st + 2 * A_BYTES, &tb_hi, bx0 + k, by, &ctl->full[s]);
        tma_load_2d(st + 2 * A_BYTES + B_BYTES, &tb_lo, bx0 + k, by, &ctl->full[s]);
        ++issued;
      }
      // the copies of the last STAGES slices land before the CTA can exit (on
      // the normal path the MMA thread has already waited for them; after an
      // abort they may still be in flight)
      for (int kc = max(0, issued - STAGES); kc < issued; ++kc)
        mbar_wait_own(&ctl->full[kc % STAGES], (kc / STAGES) & 1, wlim);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = TL::F16 ? idesc_f16(BM, BN) : idesc_tf32(BM, BN);
      constexpr int KS = TL::KS, KP = TL::KPSEG;
      const int nks = nk * KS;  // MMA K steps of this tile
      bool ok = true, issued_mma = false;
      if (p.test_stall)  // self-test: wait on a barrier nothing arrives at
        ok = mbar_wait(&ctl->mdone, 0, abort_flag, p.err, wlim);
      for (int kc = 0; kc < nk && ok; ++kc) {
        const int s = kc % STAGES;
        ok = mbar_wait(&ctl->full[s], (kc / STAGES) & 1, abort_flag, p.err, wlim);
        if (!ok) break;
        tc_fence_after();
        const uint32_t sb = smem_u32(tiles + s * STAGE_BYTES);
        const uint64_t ahi = sdesc<TL::SWZ>(sb), alo = sdesc<TL::SWZ>(sb + A_BYTES);
        const uint64_t bhi = sdesc<TL::SWZ>(sb + 2 * A_BYTES);
        const uint64_t blo = sdesc<TL::SWZ>(sb + 2 * A_BYTES + B_BYTES);
#pragma unroll
        for (int k4 = 0; k4 < KS; ++k4) {
          // segment of KP K steps per TMEM accumulator buffer
          const int ks = kc * KS + k4, seg = ks / KP, b = seg % NBUF;
          const uint32_t tacc = tmem + (uint32_t)(b * BN);
          const bool first = (ks % KP) == 0;
          if (first && seg >= NBUF) {
            ok = mbar_wait(&ctl->tempty[b], ((seg / NBUF) - 1) & 1, abort_flag, p.err, wlim);
            if (!ok) break;
            tc_fence_after();
          }
          issued_mma = true;
          // the two cross products (about 2^-11 of the result) before the
          // hi*hi product, so the running sum carrying them is small
          const uint64_t off = (uint64_t)((k4 * 32) >> 4);  // 32 bytes per MMA K step
          if (TL::F16) {
            mma_f16(tacc, alo + off, bhi + off, idesc, first ? 0u : 1u);
            mma_f16(tacc, ahi + off, blo + off, idesc, 1u);
            mma_f16(tacc, ahi + off, bhi + off, idesc, 1u);
          } else {
            mma_tf32(tacc, alo + off, bhi + off, idesc, first ? 0u : 1u);
            mma_tf32(tacc, ahi + off, blo + off, idesc, 1u);
            mma_tf32(tacc, ahi + off, bhi + off, idesc, 1u);
          }
          if ((ks % KP) == KP - 1 || ks == nks - 1) mma_commit(&ctl->tfull[b]);
        }
        if (!ok) break;
        mma_commit(&ctl->empty[s]);
      }
      if (!ok && issued_mma) {
        // after an abort, the MMAs already issued finish before TMEM is freed
        mma_commit(&ctl->mdone);
        mbar_wait_own(&ctl->mdone, 0, wlim);
      }
    }
    __syncwarp();
  } else {
    // ---------------- epilogue warps 2..9 ----------------
    // two warps per TMEM lane quarter; each owns one row and HC columns of it
    const int q = warp & 3;  // TMEM lane quarter this warp may access
    const int ew = warp - 2;
    const int hcol = (ew >> 2) * HC;  // first tile column this thread owns
    const int r = q * 32 + lane;
    const int gi = i0 + r;  // row within the problem
    const int et = threadIdx.x - 64;
    const float ka = p.kaptr ? (float)*p.kaptr : 1.f;  // kernel shape parameter
    if (MODE == MODE_GRAD || MODE == MODE_SGPR) {
      // column points and column coefficients of this tile
      const double* cvec = MODE == MODE_GRAD ? p.avec : p.bvec;
      for (int e = et; e < BN * DM; e += EPI_THREADS) {
        const int c = e / DM, k = e % DM;
        const int gj = j0 + c;
        gx[e] = (gj < p.n_true && k < p.d) ? p.xs[(int64_t)gj * p.d + k] : 0.f;
      }
      for (int c = et; c < BN; c += EPI_THREADS) {
        const int gj = j0 + c;
        ga[c] = (cvec && gj < p.n_true) ? (float)cvec[gj] : 0.f;
      }
    }
    if (p.ra)  // column scales of a float16 B operand (1 where rb is absent)
      for (int c = et; c < BN; c += EPI_THREADS)
        gsc[c] = (p.rb && j0 + c < p.N) ? p.rb[j0 + c] : 1.f;
    // drain the accumulator segments into float32 registers (round to nearest)
    float acc[HC];
#pragma unroll
    for (int c = 0; c < HC; ++c) acc[c] = 0.f;
    bool have = true;
    // single-step segments of the half tile are drained two per round trip
    constexpr int DR = (TL::KPSEG == 1 && HC == 32) ? 2 : 1;
    for (int seg = 0; seg < nseg; seg += DR) {
      const int b = seg % NBUF;
      const bool two = DR == 2 && seg + 1 < nseg;
      const int b1 = (seg + 1) % NBUF;
      bool ready = mbar_wait(&ctl->tfull[b], (seg / NBUF) & 1, abort_flag, p.err, wlim);
      if (two && ready)
        ready = mbar_wait(&ctl->tfull[b1], ((seg + 1) / NBUF) & 1, abort_flag, p.err, wlim);
      have = __all_sync(0xffffffffu, ready);
      if (!have) break;
      tc_fence_after();
      const uint32_t tb = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * BN + hcol);
      if (HC == 32) {
        uint32_t v0[32], v1[32];
        tmem_ld32_nowait(tb, v0);
        if (two) tmem_ld32_nowait(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b1 * BN + hcol), v1);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int k = 0; k < 32; ++k) acc[k] += __uint_as_float(v0[k]);
        if (two) {
#pragma unroll
          for (int k = 0; k < 32; ++k) acc[k] += __uint_as_float(v1[k]);
        }
      } else if (HC == 64) {
        uint32_t v0[32], v1[32];
        tmem_ld32_nowait(tb, v0);
        tmem_ld32_nowait(tb + 32, v1);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int k = 0; k < 32; ++k) {
          acc[k] += __uint_as_float(v0[k]);
          acc[32 + k] += __uint_as_float(v1[k]);
        }
      } else {
#pragma unroll
        for (int cc = 0; cc < HC; cc += 16) {
          uint32_t v0[16];
          tmem_ld16_nowait(tb + cc, v0);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int k = 0; k < 16; ++k) acc[cc + k] += __uint_as_float(v0[k]);
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) {
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&ctl->tempty[b]))
                     : "memory");
        if (two)
          asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&ctl->tempty[b1]))
                       : "memory");
      }
    }
    if (p.ra) {
      // undo the float16 operands' power-of-two row scales (exact)
      asm volatile("bar.sync 1, %0;" ::"r"(EPI_THREADS) : "memory");  // gsc staged
      const float rsi = gi < p.M ? p.ra[gi] : 1.f;
#pragma unroll
      for (int c = 0; c < HC; ++c) acc[c] *= rsi * gsc[hcol + c];
    }
    if (MODE == MODE_ADD_F32 || MODE == MODE_STORE_SPLIT) {
      // dtrack: sum of squares of this row's outputs (float64)
      // in float-float (exact squares by FMA, Knuth's two-sum), not float64:
      // per-element float64 arithmetic here ran at this part's float64 rate
      if (MODE == MODE_STORE_SPLIT && p.dtrack && have && gi < p.M) {
        float sh = 0.f, sl = 0.f;
#pragma unroll
        for (int c = 0; c < HC; ++c) {
          const float w = (j0 + hcol + c < p.N) ? p.alpha * acc[c] : 0.f;
          const float q = __fmul_rn(w, w);
          const float qe = fmaf(w, w, -q);  // q + qe = w^2 exactly
          const float t = __fadd_rn(sh, q);
          const float bb = __fsub_rn(t, sh);
          const float te = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bb)), __fsub_rn(q, bb));
          sh = t;
          sl = __fadd_rn(sl, __fadd_rn(te, qe));
        }
        atomicAdd(&p.dtrack[p.c_row0 + (int64_t)z * p.c_zrow + gi], -((double)sh + (double)sl));
      }
      // stage the tile, then write whole rows (coalesced, 4 floats per lane)
      asm volatile("bar.sync 1, %0;" ::"r"(EPI_THREADS) : "memory");  // ring is free
#pragma unroll
      for (int c = 0; c < HC; c += 4)
        *reinterpret_cast<float4*>(&otile[r * TLD + hcol + c]) =
            have ? make_float4(p.alpha * acc[c], p.alpha * acc[c + 1], p.alpha * acc[c + 2],
                               p.alpha * acc[c + 3])
                 : make_float4(0.f, 0.f, 0.f, 0.f);
      asm volatile("bar.sync 1, %0;" ::"r"(EPI_THREADS) : "memory");
      if (have) {
        const int64_t crow0 = p.c_row0 + (int64_t)z * p.c_zrow + i0;
        const int64_t ccol = p.c_col0 + (int64_t)z * p.c_zcol + j0;
        if (MODE == MODE_ADD_F32 && p.c0) {
          // C += tile: each warp issues RB rows of C loads before it adds and
          // stores, so the read-modify-write does not serialise on load latency
          constexpr int RB = 8;
          constexpr int NRC = BM * BN / 128;  // warp passes of 32 float4 groups (rows of BN / 4)
          for (int rc0 = ew; rc0 < NRC; rc0 += EPI_WARPS * RB) {
            float4 cv[RB];
            bool f4[RB];
#pragma unroll
            for (int u = 0; u < RB; ++u) {
              const int rc = rc0 + u * EPI_WARPS;
              const int g = rc * 32 + lane, rr = g / (BN / 4), c4 = (g % (BN / 4)) * 4;
              const int grow = i0 + rr;
              const int64_t base = (crow0 + rr) * p.ldc + ccol + c4;
              f4[u] = rc < NRC && grow < p.M && (j0 + c4 + 3 < p.N) &&
                      !(p.c_lower && j0 + c4 + 3 > grow) && ((base & 3) == 0);
              if (f4[u]) cv[u] = *reinterpret_cast<const float4*>(p.c0 + base);
            }
#pragma unroll
            for (int u = 0; u < RB; ++u) {
              const int rc = rc0 + u * EPI_WARPS;
              const int g = rc * 32 + lane, rr = g / (BN / 4), c4 = (g % (BN / 4)) * 4;
              const int grow = i0 + rr;
              if (rc >= NRC || grow >= p.M) continue;
              const float4 w4 = *reinterpret_cast<const float4*>(&otile[rr * TLD + c4]);
              const int64_t base = (crow0 + rr) * p.ldc + ccol + c4;
              if (f4[u]) {
                const float4 nv =
                    make_float4(cv[u].x + w4.x, cv[u].y + w4.y, cv[u].z + w4.z, cv[u].w + w4.w);
                *reinterpret_cast<float4*>(p.c0 + base) = nv;
                if (p.s0) {
                  float hv[4], lv[4];
                  const float nvv[4] = {nv.x, nv.y, nv.z, nv.w};
#pragma unroll
                  for (int k = 0; k < 4; ++k) split_tf32(nvv[k], hv[k], lv[k]);
                  *reinterpret_cast<float4*>(p.s0 + base) = make_float4(hv[0], hv[1], hv[2], hv[3]);
                  *reinterpret_cast<float4*>(p.s1 + base) = make_float4(lv[0], lv[1], lv[2], lv[3]);
                }
              } else {
                const float wv[4] = {w4.x, w4.y, w4.z, w4.w};
                for (int k = 0; k < 4; ++k) {
                  const int gj = j0 + c4 + k;
                  if (gj < p.N && !(p.c_lower && gj > grow)) {
                    const float nv = p.c0[base + k] + wv[k];
                    p.c0[base + k] = nv;
                    if (p.s0) split_tf32(nv, p.s0[base + k], p.s1[base + k]);
                  }
                }
              }
            }
          }
        }
        if (MODE == MODE_STORE_SPLIT && p.c0) {
          for (int rc = ew; rc < BM * BN / 128; rc += EPI_WARPS) {
            const int g = rc * 32 + lane, rr = g / (BN / 4), c4 = (g % (BN / 4)) * 4;
            const int grow = i0 + rr;
            if (grow >= p.M) continue;
            const float4 w4 = *reinterpret_cast<const float4*>(&otile[rr * TLD + c4]);
            const float wv[4] = {w4.x, w4.y, w4.z, w4.w};
            const int64_t base = (crow0 + rr) * p.ldc + ccol + c4;
            const bool full4 = (j0 + c4 + 3 < p.N) && !(p.c_lower && j0 + c4 + 3 > grow) &&
                               ((base & 3) == 0);
            {
              float hv[4], lv[4];
#pragma unroll
              for (int k = 0; k < 4; ++k) split_tf32(wv[k], hv[k], lv[k]);
              if (full4) {
                *reinterpret_cast<float4*>(p.c0 + base) = make_float4(hv[0], hv[1], hv[2], hv[3]);
                *reinterpret_cast<float4*>(p.c1 + base) = make_float4(lv[0], lv[1], lv[2], lv[3]);
              } else {
                for (int k = 0; k < 4; ++k) {
                  const int gj = j0 + c4 + k;
                  if (gj < p.N && !(p.c_lower && gj > grow)) {
                    p.c0[base + k] = hv[k];
                    p.c1[base + k] = lv[k];
                  }
                }
              }
            }
          }
        }
        if (MODE == MODE_STORE_SPLIT && p.t0) {
          // transposed: output row = tile column j, lanes over tile rows i
          const int64_t trow0 = p.t_row0 + (int64_t)z * p.t_zrow + j0;
          const int64_t tcol = p.t_col0 + (int64_t)z * p.t_zcol + i0;
          for (int cc = ew; cc < BN; cc += EPI_WARPS) {
            if (j0 + cc >= p.N) break;
            const int64_t base = (trow0 + cc) * p.ldt + tcol;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const int ii = lane + 32 * k;  // 32 consecutive rows -> one coalesced line
              if (i0 + ii < p.M) {
                float hv, lv;
                split_tf32(otile[ii * TLD + cc], hv, lv);
                p.t0[base + ii] = hv;
                p.t1[base + ii] = lv;
              }
            }
          }
        }
      }
    }
    if (MODE == MODE_GRAD) {
      // the finished W tile goes through the (now idle) operand ring, row
      // stride BN + 1 so that lanes on consecutive rows hit distinct banks:
      // the reduction below then holds no accumulator registers
      constexpr int GLD = BN + 1;
      asm volatile("bar.sync 1, %0;" ::"r"(EPI_THREADS) : "memory");  // gx / ga staged, ring free
#pragma unroll
      for (int c = 0; c < HC; ++c) otile[r * GLD + hcol + c] = have ? acc[c] : 0.f;
      // W tile -> reduction against dK/dtheta (unit variance); an aborted wait
      // contributes zeros but still joins the reduction barrier
      float xi[DM];
#pragma unroll
      for (int k = 0; k < DM; ++k)
        xi[k] = (gi < p.n_true && k < p.d) ? p.xs[(int64_t)gi * p.d + k] : 0.f;
      const float ai = (p.avec && gi < p.n_true) ? (float)p.avec[gi] : 0.f;  // null: -W terms only
      // per-thread sums in float-float (float64 here ran at this part's float64 rate)
      float glh[DM], gll[DM];
#pragma unroll
      for (int k = 0; k < DM; ++k) glh[k] = gll[k] = 0.f;
      double gnoise = 0.0;
      float gvh = 0.f, gvl = 0.f;
      with_kind(p.kind, [&](auto kind_c) {  // one loop per kernel kind
        constexpr int KIND = decltype(kind_c)::value;
        // coordinates in pairs: packed float32x2 arithmetic halves the
        // per-element instruction count of the distance and of the
        // lengthscale sums, which bound this epilogue
        constexpr int DP = DM / 2;
        f32x2 xi2[DP];
#pragma unroll
        for (int kp = 0; kp < DP; ++kp) xi2[kp] = f2_pack(xi[2 * kp], xi[2 * kp + 1]);
        // warps whose elements all lie strictly below the diagonal and inside
        // n take a loop without per-element checks (f = 2 throughout)
        const bool inner = __all_sync(0xffffffffu, have && gi < p.n_true &&
                                                       j0 + hcol + HC <= p.n_true &&
                                                       j0 + hcol + HC - 1 < gi);
        auto cols = [&](auto inner_c) {
          constexpr bool INNER = decltype(inner_c)::value;
#pragma unroll
      for (int cb = 0; cb < HC / 32; ++cb) {
        f32x2 pl2[DP];
#pragma unroll
        for (int kp = 0; kp < DP; ++kp) pl2[kp] = f2_pack(0.f, 0.f);
        float pvar = 0.f;
#pragma unroll 8
        for (int k = 0; k < 32; ++k) {
          const int c = hcol + cb * 32 + k;
          const int gj = j0 + c;
          if (!INNER && (!have || gi >= p.n_true || gj >= p.n_true || gj > gi)) continue;
          const float w = otile[r * GLD + c];
          const float f = (INNER || gi != gj) ? 2.f : 1.f;
          const float coef = f * (ai * ga[c] - w);
          const f32x2* gx2 = reinterpret_cast<const f32x2*>(gx + c * DM);
          f32x2 dsq2[DP];
          f32x2 s2 = f2_pack(0.f, 0.f);
#pragma unroll
          for (int kp = 0; kp < DP; ++kp) {
            const f32x2 df = f2_sub(xi2[kp], gx2[kp]);
            dsq2[kp] = f2_mul(df, df);
            s2 = f2_add(s2, dsq2[kp]);
          }
          const float sq = f2_lo(s2) + f2_hi(s2);
          float k1, c1;
          kval_dcoef_k<KIND, float>(sq, 1.f, k1, c1, ka);
          pvar = fmaf(coef, k1, pvar);
          const float cc = coef * c1;
          const f32x2 cc2 = f2_pack(cc, cc);
#pragma unroll
          for (int kp = 0; kp < DP; ++kp) pl2[kp] = f2_fma(cc2, dsq2[kp], pl2[kp]);
        }
#pragma unroll
        for (int kp = 0; kp < DP; ++kp) {
          ff_add(glh[2 * kp], gll[2 * kp], f2_lo(pl2[kp]));
          ff_add(glh[2 * kp + 1], gll[2 * kp + 1], f2_hi(pl2[kp]));
        }
        ff_add(gvh, gvl, pvar);
      }
        };
        if (inner)
          cols(std::integral_constant<bool, true>{});
        else
          cols(std::integral_constant<bool, false>{});
      });
      // the diagonal's noise term, outside the column loop (float64 there
      // would run for every element of an if-converted branch)
      {
        const int cd = gi - j0;  // this row's diagonal column within the tile
        if (have && gi < p.n_true && cd >= hcol && cd < hcol + HC) {
          const float w = otile[r * GLD + cd];
          gnoise = (double)ai * (double)ai - (double)w;
        }
      }
      // reduce over the 4 epilogue warps into gpart[tile]
      const int slots = p.d + 2;
      for (int sidx = 0; sidx < slots; ++sidx) {
        double val;
        if (sidx < p.d) {
          val = 0.0;
#pragma unroll
          for (int kk = 0; kk < DM; ++kk)
            if (kk == sidx) val = (double)glh[kk] + (double)gll[kk];
        } else if (sidx == p.d) {
          val = (double)gvh + (double)gvl;
        } else {
          val = gnoise;
        }
        val = warp_sum(val);
        if (lane == 0) gred[sidx * EPI_WARPS + ew] = val;
      }
      asm volatile("bar.sync 1, %0;" ::"r"(EPI_THREADS) : "memory");
      const int tile_id = blockIdx.x + (int)gridDim.x * z;
      for (int sidx = et; sidx < slots; sidx += EPI_THREADS) {
        double tot = 0.0;
        for (int w8 = 0; w8 < EPI_WARPS; ++w8) tot += gred[sidx * EPI_WARPS + w8];
        p.gpart[(int64_t)tile_id * slots + sidx] = tot;
      }
    }
    if (MODE == MODE_SGPR) {
      // G = acc + avec_i bvec_j (rows: inducing points z_i, columns: data
      // points x_j), contracted against the unit-variance kernel and its
      // derivatives: per tile  sum_ij G k1, sum_ij G c1 (z_ik - x_jk)^2  and
      // per row  sum_j G c1 (z_ik - x_jk)
      constexpr int GLD = BN + 1;
      static_assert(BM * GLD * 4 + BM * DM * 8 <= STAGES * STAGE_BYTES, "staging exceeds the ring");
      double* zrow = reinterpret_cast<double*>(otile + BM * GLD);  // [BM][DM], second half-row
      asm volatile("bar.sync 1, %0;" ::"r"(EPI_THREADS) : "memory");  // gx / ga staged, ring free
#pragma unroll
      for (int c = 0; c < HC; ++c) otile[r * GLD + hcol + c] = have ? acc[c] : 0.f;
      const bool row_ok = have && gi < p.M;
      float zi[DM];
#pragma unroll
      for (int k = 0; k < DM; ++k) zi[k] = (row_ok && k < p.d) ? p.zs[(int64_t)gi * p.d + k] : 0.f;
      const float ai = row_ok ? (float)p.avec[gi] : 0.f;
      float glh[DM], gll[DM], gzh[DM], gzl[DM];  // float-float sums
#pragma unroll
      for (int k = 0; k < DM; ++k) glh[k] = gll[k] = gzh[k] = gzl[k] = 0.f;
      float gvh = 0.f, gvl = 0.f;
      with_kind(p.kind, [&](auto kind_c) {  // one loop per kernel kind
        constexpr int KIND = decltype(kind_c)::value;
        // coordinates in pairs (packed float32x2 arithmetic, as in MODE_GRAD)
        constexpr int DP = DM / 2;
        f32x2 zi2[DP];
#pragma unroll
        for (int kp = 0; kp < DP; ++kp) zi2[kp] = f2_pack(zi[2 * kp], zi[2 * kp + 1]);
#pragma unroll 1
      for (int cb = 0; cb < HC / 32; ++cb) {
        f32x2 pl2[DP], pz2[DP];
#pragma unroll
        for (int kp = 0; kp < DP; ++kp) pl2[kp] = pz2[kp] = f2_pack(0.f, 0.f);
        float pvar = 0.f;
#pragma unroll 4
        for (int k = 0; k < 32; ++k) {
          const int c = hcol + cb * 32 + k;
          if (!row_ok || j0 + c >= p.n_true) continue;
          const float g = fmaf(ai, ga[c], otile[r * GLD + c]);
          const f32x2* gx2 = reinterpret_cast<const f32x2*>(gx + c * DM);
          f32x2 df2[DP];
          f32x2 s2 = f2_pack(0.f, 0.f);
#pragma unroll
          for (int kp = 0; kp < DP; ++kp) {
            df2[kp] = f2_sub(zi2[kp], gx2[kp]);
            s2 = f2_fma(df2[kp], df2[kp], s2);
          }
          const float sq = f2_lo(s2) + f2_hi(s2);
          float k1, c1;
          kval_dcoef_k<KIND, float>(sq, 1.f, k1, c1, ka);
          pvar = fmaf(g, k1, pvar);
          const float gc = g * c1;
          const f32x2 gc2 = f2_pack(gc, gc);
#pragma unroll
          for (int kp = 0; kp < DP; ++kp) {
            const f32x2 t = f2_mul(gc2, df2[kp]);
            pz2[kp] = f2_add(pz2[kp], t);
            pl2[kp] = f2_fma(t, df2[kp], pl2[kp]);
          }
        }
#pragma unroll
        for (int kp = 0; kp < DP; ++kp) {
          ff_add(glh[2 * kp], gll[2 * kp], f2_lo(pl2[kp]));
          ff_add(glh[2 * kp + 1], gll[2 * kp + 1], f2_hi(pl2[kp]));
          ff_add(gzh[2 * kp], gzl[2 * kp], f2_lo(pz2[kp]));
          ff_add(gzh[2 * kp + 1], gzl[2 * kp + 1], f2_hi(pz2[kp]));
        }
        ff_add(gvh, gvl, pvar);
      }
      });
      // per-row z partials: the two threads of a row combine in a fixed order
      if (hcol != 0) {
#pragma unroll
        for (int kk = 0; kk < DM; ++kk) zrow[r * DM + kk] = (double)gzh[kk] + (double)gzl[kk];
      }
      // theta partials: reduce over the epilogue warps into gpart[tile]
      const int slots = p.d + 1;
      for (int sidx = 0; sidx < slots; ++sidx) {
        double val = (double)gvh + (double)gvl;
        if (sidx < p.d) {
          val = 0.0;
#pragma unroll
          for (int kk = 0; kk < DM; ++kk)
            if (kk == sidx) val = (double)glh[kk] + (double)gll[kk];
        }
        val = warp_sum(val);
        if (lane == 0) gred[sidx * EPI_WARPS + ew] = val;
      }
      asm volatile("bar.sync 1, %0;" ::"r"(EPI_THREADS) : "memory");
      if (hcol == 0 && gi < p.M) {
        double* zp = p.zpart + ((int64_t)z * p.tiles_n + J) * (int64_t)p.M * p.d + (int64_t)gi * p.d;
#pragma unroll
        for (int kk = 0; kk < DM; ++kk)
          if (kk < p.d) zp[kk] = row_ok ? ((double)gzh[kk] + (double)gzl[kk]) + zrow[r * DM + kk] : 0.0;
      }
      const int tile_id = blockIdx.x + (int)gridDim.x * z;
      for (int sidx = et; sidx < slots; sidx += EPI_THREADS) {
        double tot = 0.0;
        for (int w8 = 0; w8 < EPI_WARPS; ++w8) tot += gred[sidx * EPI_WARPS + w8];
        p.gpart[(int64_t)tile_id * slots + sidx] = tot;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TL::TMEM_COLS)
                 : "memory");
  }
}

// ---------------------------------------------------------------------------
// TF32 split of a float32 matrix
// ---------------------------------------------------------------------------
__global__ void tf32_split_kernel(const float* __restrict__ src, int64_t lds, int rows, int cols,
                                  float* __restrict__ hi, float* __restrict__ lo, int64_t ldo) {
  pdl_wait();
  pdl_trigger();
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)rows * cols) return;
  const int r = (int)(e / cols), c = (int)(e % cols);
  float h, l;
  split_tf32(src[(int64_t)r * lds + c], h, l);
  hi[(int64_t)r * ldo + c] = h;
  lo[(int64_t)r * ldo + c] = l;
}

}  // namespace tc

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(f);
  });
  return fn;
}

// float32 row-major [rows, cols] with leading dimension ld; box bk x box_rows
// (bk = 32: 128B swizzle, bk = 16: 64B swizzle; one K slice row per box row)
static bool make_map(CUtensorMap* m, const void* base, int64_t rows, int64_t cols, int64_t ld,
                     int bk, int box_rows, int elem = 4) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  if ((reinterpret_cast<uintptr_t>(base) & 15u) != 0 || ((ld * elem) & 15) != 0) return false;
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(ld * elem)};
  cuuint32_t box[2] = {(cuuint32_t)bk, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  const int row_bytes = bk * elem;  // 128 -> 128B swizzle, 64 -> 64B swizzle
  CUresult r = fn(m, elem == 2 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                  2, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE,
                  row_bytes == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

template <int TS>
static size_t tc_smem_bytes() {
  using TL = tc::Tile<TS>;
  return 1024 + (size_t)TL::STAGES * TL::STAGE_BYTES + sizeof(tc::SmemCtl<TL::STAGES>) +
         (size_t)TL::BN * tc::GRAD_DMAX * 4 + 2 * TL::BN * 4 +
         (size_t)(tc::GRAD_DMAX + 2) * 8 * sizeof(double) + 64;
}

bool tc_make_map(TcMap* m, const float* hi, const float* lo, int64_t rows, int64_t cols,
                 int64_t ld) {
  using N = tc::Tile<0>;
  using W = tc::Tile<1>;
  using H = tc::Tile<2>;
  return make_map(&m->hi, hi, rows, cols, ld, N::BK, tc::BM) &&
         make_map(&m->lo, lo, rows, cols, ld, N::BK, tc::BM) &&
         make_map(&m->wa_hi, hi, rows, cols, ld, W::BK, tc::BM) &&
         make_map(&m->wa_lo, lo, rows, cols, ld, W::BK, tc::BM) &&
         make_map(&m->wb_hi, hi, rows, cols, ld, W::BK, W::BN) &&
         make_map(&m->wb_lo, lo, rows, cols, ld, W::BK, W::BN) &&
         make_map(&m->hb_hi, hi, rows, cols, ld, H::BK, H::BN) &&
         make_map(&m->hb_lo, lo, rows, cols, ld, H::BK, H::BN);
}

bool tc_make_map_f16(TcMap* m, const void* hi, const void* lo, int64_t rows, int64_t cols,
                     int64_t ld) {
  using F = tc::Tile<3>;
  return make_map(&m->fa_hi, hi, rows, cols, ld, F::BK, tc::BM, 2) &&
         make_map(&m->fa_lo, lo, rows, cols, ld, F::BK, tc::BM, 2) &&
         make_map(&m->fb_hi, hi, rows, cols, ld, F::BK, F::BN, 2) &&
         make_map(&m->fb_lo, lo, rows, cols, ld, F::BK, F::BN, 2);
}

// Tile shape per problem: wide once a GEMM has several waves of tiles (the
// adjoint epilogue keeps 128 accumulator columns per thread only with DM =
// 8), half where narrow tiles would leave most SMs idle, narrow otherwise.
static int tile_shape(int mode, const tc::TcParams& p) {
  if (p.force_shape > 0) return p.force_shape - 1;
  if (mode == tc::MODE_SGPR) return (p.N >= 2048 && p.d <= 8) ? 1 : 0;
  if (p.M >= 2048 && p.N >= 2048 && (mode != tc::MODE_GRAD || p.d <= 8)) return 1;
  const int tm = (p.M + tc::BM - 1) / tc::BM, tn = (p.N + 127) / 128;
  if (mode != tc::MODE_GRAD && tc::tile_count(p.c_lower, tm, tn, 128) <= 76) return 2;
  return 0;
}

static int tile_bn(int ts) {
  return ts == 1 || ts == 3 ? tc::Tile<1>::BN : (ts == 2 ? tc::Tile<2>::BN : tc::Tile<0>::BN);
}

int tc_gemm_col_tiles(int mode, const tc::TcParams& p) {
  const int bn = tile_bn(tile_shape(mode, p));
  return (p.N + bn - 1) / bn;
}

int tc_gemm_tiles(int mode, const tc::TcParams& p) {
  const int bn = tile_bn(tile_shape(mode, p));
  const int tm = (p.M + tc::BM - 1) / tc::BM, tn = (p.N + bn - 1) / bn;
  return tc::tile_count(p.c_lower, tm, tn, bn);
}

template <int MODE, int TS, int DM>
static void launch_one(const TcMap& A, const TcMap& B, const tc::TcParams& p0, int batch,
                       cudaStream_t s, bool pdl) {
  using TL = tc::Tile<TS>;
  tc::TcParams p = p0;
  p.tiles_m = (p.M + tc::BM - 1) / tc::BM;
  p.tiles_n = (p.N + TL::BN - 1) / TL::BN;
  dim3 grid(tc::tile_count(p.c_lower, p.tiles_m, p.tiles_n, TL::BN), 1, batch);
  const size_t smem = tc_smem_bytes<TS>();
  cudaFuncSetAttribute(tc::tc_gemm_kernel<MODE, TS, DM>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  PdlAttr attr(pdl);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(tc::NUM_THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = attr.a;
  cfg.numAttrs = 1;
  if (TS == 3)
    cudaLaunchKernelEx(&cfg, tc::tc_gemm_kernel<MODE, TS, DM>, A.fa_hi, A.fa_lo, B.fb_hi,
                       B.fb_lo, p);
  else if (TS == 1)
    cudaLaunchKernelEx(&cfg, tc::tc_gemm_kernel<MODE, TS, DM>, A.wa_hi, A.wa_lo, B.wb_hi,
                       B.wb_lo, p);
  else if (TS == 2)
    cudaLaunchKernelEx(&cfg, tc::tc_gemm_kernel<MODE, TS, DM>, A.hi, A.lo, B.hb_hi, B.hb_lo, p);
  else
    cudaLaunchKernelEx(&cfg, tc::tc_gemm_kernel<MODE, TS, DM>, A.hi, A.lo, B.hi, B.lo, p);
}

cudaError_t tc_gemm_run(int mode, const TcMap& A, const TcMap& B, const tc::TcParams& p,
                        int batch, cudaStream_t s, bool pdl) {
  if (p.M <= 0 || p.N <= 0 || batch <= 0) return cudaSuccess;
  const int ts = tile_shape(mode, p);
  switch (mode) {
    case tc::MODE_ADD_F32:
      if (ts == 3)
        launch_one<tc::MODE_ADD_F32, 3, tc::GRAD_DMAX>(A, B, p, batch, s, pdl);
      else if (ts == 1)
        launch_one<tc::MODE_ADD_F32, 1, tc::GRAD_DMAX>(A, B, p, batch, s, pdl);
      else if (ts == 2)
        launch_one<tc::MODE_ADD_F32, 2, tc::GRAD_DMAX>(A, B, p, batch, s, pdl);
      else
        launch_one<tc::MODE_ADD_F32, 0, tc::GRAD_DMAX>(A, B, p, batch, s, pdl);
      break;
    case tc::MODE_STORE_SPLIT:
      if (ts == 3)
        launch_one<tc::MODE_STORE_SPLIT, 3, tc::GRAD_DMAX>(A, B, p, batch, s, pdl);
      else if (ts == 1)
        launch_one<tc::MODE_STORE_SPLIT, 1, tc::GRAD_DMAX>(A, B, p, batch, s, pdl);
      else if (ts == 2)
        launch_one<tc::MODE_STORE_SPLIT, 2, tc::GRAD_DMAX>(A, B, p, batch, s, pdl);
      else
        launch_one<tc::MODE_STORE_SPLIT, 0, tc::GRAD_DMAX>(A, B, p, batch, s, pdl);
      break;
    case tc::MODE_GRAD:
      if (ts == 3)
        launch_one<tc::MODE_GRAD, 3, 8>(A, B, p, batch, s, pdl);
      else if (ts == 1)
        launch_one<tc::MODE_GRAD, 1, 8>(A, B, p, batch, s, pdl);
      else
        launch_one<tc::MODE_GRAD, 0, tc::GRAD_DMAX>(A, B, p, batch, s, pdl);
      break;
    case tc::MODE_SGPR:
      if (ts == 1)
        launch_one<tc::MODE_SGPR, 1, 8>(A, B, p, batch, s, pdl);
      else if (p.d <= 8)
        launch_one<tc::MODE_SGPR, 0, 8>(A, B, p, batch, s, pdl);
      else
        launch_one<tc::MODE_SGPR, 0, tc::GRAD_DMAX>(A, B, p, batch, s, pdl);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return launch_status();
}

cudaError_t tc_gemm_launch(int mode, const TcMat& A, const TcMat& B, const tc::TcParams& p,
                           int batch, cudaStream_t s) {
  TcMap ma, mb;
  if (!tc_make_map(&ma, A.hi, A.lo, A.rows, A.cols, A.ld) ||
      !tc_make_map(&mb, B.hi, B.lo, B.rows, B.cols, B.ld))
    return cudaErrorInvalidValue;
  return tc_gemm_run(mode, ma, mb, p, batch, s);
}

cudaError_t tf32_split(const float* src, int64_t lds, int rows, int cols, float* hi, float* lo,
                       int64_t ldo, cudaStream_t s, bool pdl) {
  const int64_t total = (int64_t)rows * cols;
  if (total <= 0) return cudaSuccess;
  PdlAttr attr(pdl);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)cdiv(total, 256));
  cfg.blockDim = dim3(256);
  cfg.stream = s;
  cfg.attrs = attr.a;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, tc::tf32_split_kernel, src, lds, rows, cols, hi, lo, ldo);
  return launch_status();
}

}  // namespace gpk

// ---------------------------------------------------------------------------
// C ABI: standalone split-TF32 GEMM, C = beta*C + alpha * A B^T
// ---------------------------------------------------------------------------
using namespace gpk;

static size_t gemm_ws_layout(int64_t M, int64_t N, int64_t K, void* ws, float** ahi, float** alo,
                             float** bhi, float** blo, int64_t* ldk) {
  const int64_t ld = ((K + 31) / 32) * 32;
  *ldk = ld;
  char* b = static_cast<char*>(ws);
  size_t off = 0;
  auto take = [&](int64_t rows) {
    off = (off + 255) & ~size_t(255);
    float* p = b ? reinterpret_cast<float*>(b + off) : nullptr;
    off += (size_t)rows * ld * 4;
    return p;
  };
  *ahi = take(M);
  *alo = take(M);
  *bhi = take(N);
  *blo = take(N);
  return off + 256;
}

extern "C" size_t gpk_gemm_tf32x3_workspace_bytes(int64_t M, int64_t N, int64_t K) {
  float *a, *b, *c, *d;
  int64_t ld;
  return gemm_ws_layout(M, N, K, nullptr, &a, &b, &c, &d, &ld);
}

__global__ void scale_matrix_kernel(float* C, int64_t ldc, int M, int N, float beta) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)M * N) return;
  float* p = C + (e / N) * ldc + (e % N);
  *p = beta == 0.f ? 0.f : beta * *p;
}

extern "C" gpk_status gpk_gemm_tf32x3(int64_t M, int64_t N, int64_t K, float alpha,
                                      const float* A, int64_t lda, const float* B, int64_t ldb,
                                      float beta, float* C, int64_t ldc, int lower_only,
                                      int* err_flag, void* workspace, size_t workspace_bytes,
                                      cudaStream_t stream) {
  if (M < 0 || N < 0 || K < 0 || lda < K || ldb < K || ldc < N) return GPK_ERR_BAD_ARG;
  if (M > (1 << 24) || N > (1 << 24) || K > (1 << 24)) return GPK_ERR_BAD_ARG;
  if (lower_only && M != N) return GPK_ERR_BAD_ARG;
  if (M == 0 || N == 0) return GPK_OK;
  if (!A || !B || !C || !workspace) return GPK_ERR_BAD_ARG;
  if (workspace_bytes < gpk_gemm_tf32x3_workspace_bytes(M, N, K)) return GPK_ERR_WORKSPACE;
  float *ahi, *alo, *bhi, *blo;
  int64_t ld;
  gemm_ws_layout(M, N, K, workspace, &ahi, &alo, &bhi, &blo, &ld);
  if (beta != 1.f) {
    scale_matrix_kernel<<<(int)cdiv(M * N, 256), 256, 0, stream>>>(C, ldc, (int)M, (int)N, beta);
    GPK_LAUNCH_CHECK();
  }
  if (K == 0) return GPK_OK;
  GPK_CUDA_TRY(tf32_split(A, lda, (int)M, (int)K, ahi, alo, ld, stream));
  GPK_CUDA_TRY(tf32_split(B, ldb, (int)N, (int)K, bhi, blo, ld, stream));
  tc::TcParams p{};
  p.M = (int)M;
  p.N = (int)N;
  p.K = (int)K;
  p.c_lower = lower_only ? 1 : 0;
  p.c0 = C;
  p.ldc = ldc;
  p.alpha = alpha;
  p.err = err_flag;
  TcMat a{ahi, alo, M, K, ld}, b{bhi, blo, N, K, ld};
  GPK_CUDA_TRY(tc_gemm_launch(tc::MODE_ADD_F32, a, b, p, 1, stream));
  return GPK_OK;
}

// ---------------------------------------------------------------------------
// C ABI: self-test of the bounded waits.  One 256 x 256 x 256 GEMM whose MMA
// thread waits on a barrier that nothing arrives at, with a 20M-cycle limit
// (about 10 ms): the wait runs out, the CTA sets *err_flag, lets its own TMA
// copies land, frees its tensor memory and returns -- the path a device-side
// stall takes in any product call.
// ---------------------------------------------------------------------------
static constexpr int64_t kSelfTestN = 256;

extern "C" size_t gpk_selftest_wait_timeout_workspace_bytes(void) {
  return gpk_gemm_tf32x3_workspace_bytes(kSelfTestN, kSelfTestN, kSelfTestN) +
         (size_t)kSelfTestN * kSelfTestN * 4 + 256;
}

extern "C" gpk_status gpk_selftest_wait_timeout(int* err_flag, void* workspace,
                                                size_t workspace_bytes, cudaStream_t stream) {
  if (!err_flag || !workspace || workspace_bytes < gpk_selftest_wait_timeout_workspace_bytes())
    return GPK_ERR_BAD_ARG;
  const int64_t n = kSelfTestN;
  GPK_CUDA_TRY(cudaMemsetAsync(workspace, 0, workspace_bytes, stream));
  float *ahi, *alo, *bhi, *blo;
  int64_t ld;
  const size_t g = gemm_ws_layout(n, n, n, workspace, &ahi, &alo, &bhi, &blo, &ld);
  float* C = reinterpret_cast<float*>(static_cast<char*>(workspace) + ((g + 255) & ~size_t(255)));
  tc::TcParams p{};
  p.M = p.N = p.K = (int)n;
  p.c0 = C;
  p.ldc = n;
  p.alpha = 1.f;
  p.err = err_flag;
  p.wait_cycles = 20000000LL;
  p.test_stall = 1;
  TcMat a{ahi, alo, n, n, ld}, b{bhi, blo, n, n, ld};
  GPK_CUDA_TRY(tc_gemm_launch(tc::MODE_ADD_F32, a, b, p, 1, stream));
  return GPK_OK;
}
