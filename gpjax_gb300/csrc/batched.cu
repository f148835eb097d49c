// Persistent batched exact-GP marginal log-likelihood and gradient: many
// independent GPs of uneven n (Bayesian-optimisation candidates, multi-start
// hyperparameter fits) in ONE launch.  Per instance the quantity is the one of
// mll.cu -- conjugate_mll (gpjax/objectives.py:36-107) and its gradient
// 1/2 tr((alpha alpha^T - Sigma^-1) dSigma/dtheta) -- in float32 with float64
// pivots (a float-float diagonal track), float-float residuals for the
// refinement of alpha and float64 sums.
//
// Schedule.  A plan (built once, outside any stream capture) holds the
// instance descriptors on the device, a queue of instance indices sorted by n
// (largest first) and a tile configuration per instance chosen by the
// autotuner.  Each execution zeroes the queue head and launches one grid of
// one CTA per SM; a CTA takes the next queue entry with an atomic add and runs
// the whole instance in its workspace slot, then takes the next.  The largest
// instances start first and the small ones fill in behind them, so the SMs
// finish together.  CTAs never wait on one another.
//
// Per instance (padded to n_pad, a multiple of 128, with an identity block):
//   Gram: lower 128-blocks of Sigma (float32) and its float64 diagonal;
//   factor: left-looking over 128-wide block columns: the column updated by
//     one product over all earlier panels, its diagonal block factored and
//     inverted by leaf_chol_inv_body, the panel below solved by substitution;
//   inverse: M = L^-1 by the recursive merge M21 = -M22 (L21 M11);
//   alpha = M^T M diff, refined against float-float residuals (twice, or
//     once when the first correction is below 1e-5 of alpha);
//   W = M^T M tile by tile, reduced at once against dK/dtheta (adjoint).
// Every product runs as 128 x 128 output tiles, one at a time on the whole
// CTA, in the configuration the autotuner picks per n range: on the CUDA
// cores (512 threads, 8 x 4 outputs per thread, K slices of 16 or 32
// double-buffered through shared memory) or on the tcgen05 tensor cores
// (split TF32, TMEM accumulators; tile_mma_tc).
#include <algorithm>
#include <climits>
#include <map>
#include <mutex>
#include <vector>
#include "gpk_internal.cuh"
#include "simt_tile.cuh"
#include "leaf_chol.cuh"
#include "mll_finalize.cuh"
#include "tc_ptx.cuh"

namespace gpk {
namespace {

constexpr int BNT = LEAF_NT;  // threads per CTA (the leaf's 512)
constexpr int TT = 128;       // output tile edge = leaf size
constexpr int SLD = TT + 4;   // staged K-slice rows (16-byte aligned)
constexpr int WLD = TT + 4;   // W tile rows in shared memory (float4 rows)
constexpr int BDM = 16;       // input dimension bound of the batched kernel
constexpr int XLD = BDM + 2;  // staged input rows (pairs stay 8-byte aligned)
constexpr int NP_MAX = 4096;  // largest padded instance
constexpr int NCFG = 3;       // tile configurations: K slices of 16 or 32 (CUDA cores),
                              // K slices of 32 on the tensor cores

// floats of the product staging area: the K-slice double buffer (or the W
// tile), then the staged inputs and alphas of a tile's rows and columns
__host__ __device__ constexpr int stage_floats() {
  return 4 * 32 * SLD > TT * WLD ? 4 * 32 * SLD : TT * WLD;
}
__host__ __device__ constexpr int prod_floats() { return stage_floats() + 2 * TT * XLD + 2 * TT; }

struct BatchInst {
  const double* x;
  const double* y;
  const double* theta;
  double* out_mll;
  double* out_grad;
  int* info;
  int64_t ldx;
  int64_t slot_off;   // byte offset of the instance's slot in the workspace
  int64_t tpart_off;  // first of its ntiles * (d + 2) per-tile gradient partials
  int n, d, kind, n_ls, cfg, ntiles;
};

// Per-execution counters (zeroed before each launch): the queue head, then
// per instance "published" (its M and alpha are final), the next unclaimed
// adjoint tile and the number of finished tiles.
struct BatchArgs {
  const BatchInst* inst;
  const int* queue;  // instance indices, largest n first
  int* head;         // next queue position
  int* published;    // [count]
  int* next_tile;    // [count]
  int* tiles_done;   // [count]
  double* tpart;     // per-tile gradient partials
  int count;
  char* ws;          // one slot per instance
  int want_grad;
  double jitter;
  int force_cfg;     // >= 0: every instance with this configuration (autotuner trials,
                     // gpk_batch_plan_force_config)
  long long wait_cycles;  // bound on an idle CTA's wait for published tiles
  long long tc_stall;     // self-test (0: off), see tc_wait
};

struct Slot {
  float *A, *L, *M, *xs;
  double *dtrack, *logdiag, *diff, *alpha;
  float *rf, *zf, *ahf;  // ahf: alpha in float32 (the adjoint tiles' operand)
};

__host__ __device__ inline size_t al256(size_t b) { return (b + 255) & ~size_t(255); }

// Slot of one instance of padded size np (matrices with leading dimension np).
__host__ __device__ inline size_t slot_layout(int np, char* base, Slot* s) {
  const size_t mat = al256((size_t)np * np * sizeof(float));
  const size_t vd = al256((size_t)np * sizeof(double)), vf = al256((size_t)np * sizeof(float));
  const size_t xsb = al256((size_t)np * BDM * sizeof(float));
  if (s) {
    char* p = base;
    s->A = reinterpret_cast<float*>(p);
    s->L = reinterpret_cast<float*>(p += mat);
    s->M = reinterpret_cast<float*>(p += mat);
    s->xs = reinterpret_cast<float*>(p += mat);
    s->dtrack = reinterpret_cast<double*>(p += xsb);
    s->logdiag = reinterpret_cast<double*>(p += vd);
    s->diff = reinterpret_cast<double*>(p += vd);
    s->alpha = reinterpret_cast<double*>(p += vd);
    s->rf = reinterpret_cast<float*>(p += vd);
    s->zf = reinterpret_cast<float*>(p += vf);
    s->ahf = reinterpret_cast<float*>(p += vf);
  }
  return 3 * mat + xsb + 4 * vd + 3 * vf;
}

// ---------------------------------------------------------------------------
// One 128 x 128 output tile on the whole CTA (512 threads, 8 x 4 outputs each):
//   acc[u][v] = sum_{k in [klo, khi)} A(i, k) B(j, k)
// for rows i = i0 + tile_row(u) (ty*4 + (u & 3) + 64 (u >> 2)) and columns
// j = j0 + tx*4 + v, with ty = tid / 32 and tx = tid % 32 (a warp shares its
// rows: the A fragment loads are broadcasts).  Operand element (m, k) sits at
// P[m * ld + k] (KM = false: rows hold K) or P[k * ld + m] (KM = true).  K
// slices of BK are loaded into registers one slice ahead and stored into the
// other half of a double buffer.
// ---------------------------------------------------------------------------
template <int BK, bool KM>
__device__ __forceinline__ void slice_load(const float* __restrict__ P, int ld, int r0, int k0,
                                           float4 (&r)[BK / 16]) {
#pragma unroll
  for (int v = 0; v < BK / 16; ++v) {
    const int e = threadIdx.x + v * BNT;
    if constexpr (KM) {
      const int k = e / (TT / 4), m = 4 * (e % (TT / 4));
      r[v] = *reinterpret_cast<const float4*>(P + (int64_t)(k0 + k) * ld + r0 + m);
    } else {
      const int m = e / (BK / 4), k = 4 * (e % (BK / 4));
      r[v] = *reinterpret_cast<const float4*>(P + (int64_t)(r0 + m) * ld + k0 + k);
    }
  }
}

template <int BK, bool KM>
__device__ __forceinline__ void slice_store(float* S, const float4 (&r)[BK / 16]) {
#pragma unroll
  for (int v = 0; v < BK / 16; ++v) {
    const int e = threadIdx.x + v * BNT;
    if constexpr (KM) {
      const int k = e / (TT / 4), m = 4 * (e % (TT / 4));
      *reinterpret_cast<float4*>(S + k * SLD + m) = r[v];
    } else {
      const int m = e / (BK / 4), k = 4 * (e % (BK / 4));
      S[(k + 0) * SLD + m] = r[v].x;
      S[(k + 1) * SLD + m] = r[v].y;
      S[(k + 2) * SLD + m] = r[v].z;
      S[(k + 3) * SLD + m] = r[v].w;
    }
  }
}

template <int BK, bool AKM, bool BKM>
__device__ __forceinline__ void tile_mma_simt(const float* __restrict__ A, int lda,
                                              const float* __restrict__ B, int ldb, int i0,
                                              int j0, int klo, int khi, float* S,
                                              float (&acc)[8][4]) {
  float* As = S;                 // [2][BK][SLD]
  float* Bs = S + 2 * BK * SLD;  // [2][BK][SLD]
  const int ty = threadIdx.x >> 5, tx = threadIdx.x & 31;
  if (klo >= khi) return;
  float4 ra[BK / 16], rb[BK / 16];
  slice_load<BK, AKM>(A, lda, i0, klo, ra);
  slice_load<BK, BKM>(B, ldb, j0, klo, rb);
  slice_store<BK, AKM>(As, ra);
  slice_store<BK, BKM>(Bs, rb);
  __syncthreads();
  int st = 0;
  for (int k0 = klo; k0 < khi; k0 += BK) {
    const bool more = k0 + BK < khi;
    if (more) {
      slice_load<BK, AKM>(A, lda, i0, k0 + BK, ra);
      slice_load<BK, BKM>(B, ldb, j0, k0 + BK, rb);
    }
    const float* as = As + st * BK * SLD;
    const float* bs = Bs + st * BK * SLD;
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      const float4 a0 = *reinterpret_cast<const float4*>(as + kk * SLD + ty * 4);
      const float4 a1 = *reinterpret_cast<const float4*>(as + kk * SLD + 64 + ty * 4);
      const float4 b0 = *reinterpret_cast<const float4*>(bs + kk * SLD + tx * 4);
      const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float bv[4] = {b0.x, b0.y, b0.z, b0.w};
#pragma unroll
      for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(av[u], bv[v], acc[u][v]);
    }
    if (more) {
      slice_store<BK, AKM>(As + (st ^ 1) * BK * SLD, ra);
      slice_store<BK, BKM>(Bs + (st ^ 1) * BK * SLD, rb);
    }
    __syncthreads();
    st ^= 1;
  }
}

__device__ __forceinline__ int tile_row(int u) {
  return (threadIdx.x >> 5) * 4 + (u & 3) + ((u >> 2) << 6);
}
__device__ __forceinline__ int tile_col(int v) { return (threadIdx.x & 31) * 4 + v; }

// ---------------------------------------------------------------------------
// The same 128 x 128 tile on the tensor cores (configuration TC_BK).  K
// slices of 32 float32 elements are copied from memory by cp.async into one
// of two raw stages (32 KB each, two slices in flight), then split into TF32
// hi / lo by all 512 threads and stored into the 128B-swizzled K-major layout
// the MMA reads (one split stage of A_hi, A_lo, B_hi, B_lo, 64 KB, 1024-byte
// aligned).  Thread 0 issues the slice's 3 products (A_lo B_hi, A_hi B_lo,
// then A_hi B_hi) x 4 K steps of tcgen05.mma kind::tf32 into one of two TMEM
// accumulators and commits to that accumulator's mbarrier; while they run,
// every thread adds the previous slice's accumulator (its 32 columns) to
// float32 registers (round to nearest: 12 MMAs per TMEM accumulation) and
// the next raw slice lands.  The finished tile goes through shared memory
// into the CUDA-core fragment layout of tile_mma_simt, so every epilogue is
// shared.  Waits on the MMA barriers are bounded (kTcWait cycles); a timeout
// sets the CTA's error flag, after which no wait is attempted and the
// instance reports info = -1.
// ---------------------------------------------------------------------------
constexpr int TC_BK = 0;        // template value of the tensor-core configuration
constexpr int TC_STAGE = 65536; // bytes of the split stage
constexpr int TC_RAW = 32768;   // bytes of one raw stage (A, then B)
constexpr long long kTcWait = 4000000000LL;

struct TcState {
  uint64_t bar[2];  // MMA completion, one per accumulator
  uint64_t never;   // self-test: a barrier nothing arrives on
  uint64_t fin;     // kernel end after a timeout: every MMA issued has completed
  long long stall;  // self-test: > 0 makes the CTA's first MMA wait also wait on `never`
  uint32_t n[2];    // completions consumed so far (parity = n & 1)
  uint32_t issued[2];  // commits made
  uint32_t tmem;    // base of 256 TMEM columns (two 128-column accumulators)
  int err;          // a wait timed out
  int stalled;      // the self-test wait ran out
};
__device__ __forceinline__ TcState& tc_state() {
  __shared__ TcState st;
  return st;
}

// element (r, k) of a 128-row, 32-column float32 K slice in the 128B swizzle
__device__ __forceinline__ uint32_t sw128(int r, int k) {
  return (uint32_t)(r * 128 + ((((k >> 2) ^ (r & 7))) << 4) + ((k & 3) << 2));
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(tc::smem_u32(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Raw copy of one operand's K slice (1024 16-byte chunks, two per thread):
// rows of 32 floats (KM = false: raw[m * 32 + k]) or rows of 128 (KM = true:
// raw[k * 128 + m]), both as they lie in memory (a warp copies 512
// contiguous bytes per row group).
template <bool KM>
__device__ __forceinline__ void tc_copy(const float* __restrict__ P, int ld, int r0, int k0,
                                        float* raw) {
#pragma unroll
  for (int v = 0; v < 2; ++v) {
    const int e = threadIdx.x + v * BNT;
    if constexpr (KM) {
      const int k = e >> 5, m = 4 * (e & 31);
      cp_async16(raw + k * TT + m, P + (int64_t)(k0 + k) * ld + r0 + m);
    } else {
      const int m = e >> 3, k = 4 * (e & 7);
      cp_async16(raw + m * 32 + k, P + (int64_t)(r0 + m) * ld + k0 + k);
    }
  }
}

__device__ __forceinline__ float4 tf32_hi4(float4 x) {
  return make_float4(tf32_rna_f(x.x), tf32_rna_f(x.y), tf32_rna_f(x.z), tf32_rna_f(x.w));
}

// Split of a raw slice into the swizzled hi / lo buffers: each thread forms
// four consecutive k of one row m and stores them as one 16-byte chunk
// (KM: lanes run over m, so the four column reads and the swizzled stores
// are free of bank conflicts).
template <bool KM>
__device__ __forceinline__ void tc_split(const float* raw, char* hi, char* lo) {
#pragma unroll
  for (int v = 0; v < 2; ++v) {
    const int e = threadIdx.x + v * BNT;
    int m, k;
    float4 x;
    if constexpr (KM) {
      m = e & (TT - 1);
      k = 4 * (e >> 7);
      x = make_float4(raw[k * TT + m], raw[(k + 1) * TT + m], raw[(k + 2) * TT + m],
                      raw[(k + 3) * TT + m]);
    } else {
      m = e >> 3;
      k = 4 * (e & 7);
      x = *reinterpret_cast<const float4*>(raw + m * 32 + k);
    }
    const float4 h = tf32_hi4(x);
    const float4 l = tf32_hi4(make_float4(x.x - h.x, x.y - h.y, x.z - h.z, x.w - h.w));
    const uint32_t o = sw128(m, k);
    *reinterpret_cast<float4*>(hi + o) = h;
    *reinterpret_cast<float4*>(lo + o) = l;
  }
}

// Wait for the n-th completion (from 0) of accumulator b's barrier.  With
// the self-test on, the CTA's first wait first waits (st.stall cycles) on a
// barrier that nothing arrives on and records that it ran out; the MMAs are
// still waited for, so none is in flight when the CTA moves on.
__device__ __forceinline__ void tc_wait(int b, uint32_t n) {
  TcState& st = tc_state();
  if (*(volatile int*)&st.err) return;
  if (st.stall > 0 && !*(volatile int*)&st.stalled) {
    if (!tc::mbar_wait_own(&st.never, 0u, st.stall)) st.stalled = 1;
  }
  if (!tc::mbar_wait_own(&st.bar[b], n & 1u, kTcWait)) st.err = 1;
}

__device__ __forceinline__ bool tc_failed() {
  TcState& st = tc_state();
  return *(volatile int*)&st.err || *(volatile int*)&st.stalled;
}

// The tensor-core staging region: the start of the dynamic shared memory,
// 1024-byte aligned for the swizzle.  It overlaps the CUDA-core staging area
// and the leaf's storage, neither of which is live during a tile product (the
// epilogue runs after the tile has been moved to registers).  Kept within the
// leaf's footprint so that the L1 share of the SM does not shrink.
__host__ __device__ constexpr size_t tc_region_bytes() {
  return 1024 + (size_t)TC_STAGE + 2 * (size_t)TC_RAW;
}

// Kernel start (every thread): barriers, counters, 256 TMEM columns.
__device__ void tc_setup(long long stall) {
  TcState& st = tc_state();
  if (threadIdx.x == 0) {
    tc::mbar_init(&st.bar[0], 1);
    tc::mbar_init(&st.bar[1], 1);
    tc::mbar_init(&st.never, 1);
    tc::mbar_init(&st.fin, 1);
    st.stall = stall;
    st.n[0] = st.n[1] = 0;
    st.issued[0] = st.issued[1] = 0;
    st.err = 0;
    st.stalled = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if ((threadIdx.x >> 5) == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     tc::smem_u32(&st.tmem)),
                 "r"(256)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
}

// Kernel end (every thread): after a timeout (when later waits were skipped
// and the counters no longer tell which MMAs were seen to complete), thread
// 0, which issued every MMA, commits once more to `fin` -- it arrives when
// all of them have completed -- and waits for that (bounded) before the TMEM
// columns are released.
__device__ void tc_teardown() {
  TcState& st = tc_state();
  __syncthreads();
  if (threadIdx.x == 0 && st.err && (st.issued[0] | st.issued[1])) {
    tc::mma_commit(&st.fin);
    tc::mbar_wait_own(&st.fin, 0u, kTcWait);
  }
  tc::tc_fence_before();
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) {
    tc::tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(st.tmem), "r"(256)
                 : "memory");
  }
}

template <bool AKM, bool BKM, bool ACC_IN>
__device__ void tile_mma_tc(const float* __restrict__ A, int lda, const float* __restrict__ B,
                            int ldb, int i0, int j0, int klo, int khi, float* S,
                            float (&acc)[8][4]) {
  TcState& st = tc_state();
  char* base =
      reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(S) + 1023) & ~uintptr_t(1023));
  char* sp = base;  // split stage: A_hi, A_lo, B_hi, B_lo
  auto raw = [&](int sl) {  // raw stage of slice sl
    return reinterpret_cast<float*>(base + TC_STAGE + (sl & 1) * TC_RAW);
  };
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nsl = (khi - klo) / 32;
  // completions consumed per accumulator (the same in every thread; two
  // scalars, not an array indexed at run time, which would live in memory)
  uint32_t nb0 = st.n[0], nb1 = st.n[1];
  float c32[32];
  if constexpr (ACC_IN) {  // the incoming accumulator (fragment layout) to the row layout
    float* Cs = reinterpret_cast<float*>(base);
#pragma unroll
    for (int u = 0; u < 8; ++u)
      *reinterpret_cast<float4*>(Cs + tile_row(u) * SLD + tile_col(0)) =
          make_float4(acc[u][0], acc[u][1], acc[u][2], acc[u][3]);
    __syncthreads();
    const float* row = Cs + (32 * (warp & 3) + lane) * SLD + 32 * (warp >> 2);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const float4 t = *reinterpret_cast<const float4*>(row + 4 * q);
      c32[4 * q] = t.x;
      c32[4 * q + 1] = t.y;
      c32[4 * q + 2] = t.z;
      c32[4 * q + 3] = t.w;
    }
    __syncthreads();
  } else {
#pragma unroll
    for (int k = 0; k < 32; ++k) c32[k] = 0.f;
  }
  auto copy = [&](int sl) {  // raw stage sl & 1; one commit group per call
    if (sl < nsl) {
      float* r = raw(sl);
      tc_copy<AKM>(A, lda, i0, klo + 32 * sl, r);
      tc_copy<BKM>(B, ldb, j0, klo + 32 * sl, r + TT * 32);
    }
    cp_async_commit();
  };
  auto drain = [&](int b) {  // accumulator b, complete, into c32
    const uint32_t ta =
        st.tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(b * 128 + 32 * (warp >> 2));
#pragma unroll
    for (int h = 0; h < 2; ++h) {  // two 16-column loads: fewer live registers
      uint32_t v[16];
      tc::tmem_ld16_nowait(ta + 16 * h, v);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int k = 0; k < 16; ++k) c32[16 * h + k] += __uint_as_float(v[k]);
    }
  };
  if (nsl > 0) {
    copy(0);
    copy(1);
  }
  for (int sl = 0; sl < nsl; ++sl) {
    cp_async_wait<1>();  // this thread's copies of slice sl have landed
    __syncthreads();     // everyone's; the accumulator drained last iteration is free
    if (sl > 0) {        // the MMAs of slice sl - 1 read the split stage: wait for them
      tc_wait((sl - 1) & 1, ((sl - 1) & 1) ? nb1 : nb0);
      tc::tc_fence_after();
    }
    const float* r = raw(sl);
    tc_split<AKM>(r, sp, sp + 16384);
    tc_split<BKM>(r + TT * 32, sp + 32768, sp + 49152);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc::tc_fence_before();
    __syncthreads();  // the split stage is written; raw stage sl & 1 is free
    copy(sl + 2);
    if (threadIdx.x == 0) {
      tc::tc_fence_after();
      const uint32_t a = tc::smem_u32(sp);
      const uint64_t ahi = tc::sdesc<128>(a), alo = tc::sdesc<128>(a + 16384);
      const uint64_t bhi = tc::sdesc<128>(a + 32768), blo = tc::sdesc<128>(a + 49152);
      const uint32_t tacc = st.tmem + (uint32_t)((sl & 1) * 128);
      constexpr uint32_t idesc = tc::idesc_tf32(128, 128);
      // the small cross products first, the hi x hi products last: the
      // accumulator's roundings at the size of the result happen 4 times
      // per slice instead of 12
#pragma unroll
      for (int ks = 0; ks < 4; ++ks)
        tc::mma_tf32(tacc, alo + 2 * ks, bhi + 2 * ks, idesc, ks ? 1u : 0u);
#pragma unroll
      for (int ks = 0; ks < 4; ++ks) tc::mma_tf32(tacc, ahi + 2 * ks, blo + 2 * ks, idesc, 1u);
#pragma unroll
      for (int ks = 0; ks < 4; ++ks) tc::mma_tf32(tacc, ahi + 2 * ks, bhi + 2 * ks, idesc, 1u);
      tc::mma_commit(&st.bar[sl & 1]);
      st.issued[sl & 1] += 1;
    }
    if (sl > 0) {  // slice sl - 1's accumulator, complete since the wait above
      drain((sl - 1) & 1);
      if ((sl - 1) & 1) ++nb1; else ++nb0;
      tc::tc_fence_before();  // ordered before the next barrier, after which it is rewritten
    }
  }
  cp_async_wait<0>();
  if (nsl > 0) {
    const int b = (nsl - 1) & 1;
    tc_wait(b, b ? nb1 : nb0);
    tc::tc_fence_after();
    drain(b);
    if (b) ++nb1; else ++nb0;
    tc::tc_fence_before();
  }
  __syncthreads();  // every thread past its waits and loads: the counters, and the stages
  if (threadIdx.x == 0) {
    st.n[0] = nb0;
    st.n[1] = nb1;
  }
  // the tile through shared memory into the CUDA-core fragment layout
  float* Cs = reinterpret_cast<float*>(base);
  const int r = 32 * (warp & 3) + lane, c0 = 32 * (warp >> 2);
#pragma unroll
  for (int q = 0; q < 8; ++q)
    *reinterpret_cast<float4*>(Cs + r * SLD + c0 + 4 * q) =
        make_float4(c32[4 * q], c32[4 * q + 1], c32[4 * q + 2], c32[4 * q + 3]);
  __syncthreads();
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const float4 t = *reinterpret_cast<const float4*>(Cs + tile_row(u) * SLD + tile_col(0));
    acc[u][0] = t.x;
    acc[u][1] = t.y;
    acc[u][2] = t.z;
    acc[u][3] = t.w;
  }
  __syncthreads();
}

// acc += the tile's product (ACC_IN: acc holds a starting value; else zeros)
template <int BK, bool AKM, bool BKM, bool ACC_IN = false>
__device__ __forceinline__ void tile_mma(const float* __restrict__ A, int lda,
                                         const float* __restrict__ B, int ldb, int i0, int j0,
                                         int klo, int khi, float* S, float (&acc)[8][4]) {
  if constexpr (BK == TC_BK)
    tile_mma_tc<AKM, BKM, ACC_IN>(A, lda, B, ldb, i0, j0, klo, khi, S, acc);
  else
    tile_mma_simt<BK, AKM, BKM>(A, lda, B, ldb, i0, j0, klo, khi, S, acc);
}

// A product over tm x tn output tiles (the lower ones when lower), one tile
// at a time on the whole CTA.  kr(i0, j0, klo, khi) gives a tile's K range
// (the triangles of the operands), init(i0, j0, acc) the accumulator's
// starting value when ACC_IN (else zeros), ep(i0, j0, acc, S) consumes it (S:
// the staging area, free until the next barrier).
template <int BK, bool AKM, bool BKM, bool ACC_IN, class KR, class IN, class EP>
__device__ void product_from(int tm, int tn, bool lower, const float* A, int lda,
                             const float* B, int ldb, KR kr, IN init, EP ep, float* smem) {
  const int nt = lower ? tm * (tm + 1) / 2 : tm * tn;
  for (int t = 0; t < nt; ++t) {
    int I, J;
    if (lower) {
      tri_index(t, I, J);
    } else {
      I = t / tn;
      J = t % tn;
    }
    int klo, khi;
    kr(I * TT, J * TT, klo, khi);
    float acc[8][4];
    if constexpr (ACC_IN) {
      init(I * TT, J * TT, acc);
    } else {
#pragma unroll
      for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
    }
    tile_mma<BK, AKM, BKM, ACC_IN>(A, lda, B, ldb, I * TT, J * TT, klo, khi, smem, acc);
    ep(I * TT, J * TT, acc, smem);
  }
  __syncthreads();
}

template <int BK, bool AKM, bool BKM, class KR, class EP>
__device__ void product(int tm, int tn, bool lower, const float* A, int lda, const float* B,
                        int ldb, KR kr, EP ep, float* smem) {
  product_from<BK, AKM, BKM, false>(
      tm, tn, lower, A, lda, B, ldb, kr, [](int, int, float(&)[8][4]) {}, ep, smem);
}

// C tile (rows i0.., columns j0..) = alpha acc (+ C when add), float4 rows
__device__ __forceinline__ void put_tile(float* C, int ldc, int i0, int j0,
                                         const float (&acc)[8][4], float alpha, bool add) {
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    float* c = C + (int64_t)(i0 + tile_row(u)) * ldc + j0 + tile_col(0);
    float4 v = make_float4(alpha * acc[u][0], alpha * acc[u][1], alpha * acc[u][2],
                           alpha * acc[u][3]);
    if (add) {
      const float4 o = *reinterpret_cast<const float4*>(c);
      v.x += o.x;
      v.y += o.y;
      v.z += o.z;
      v.w += o.w;
    }
    *reinterpret_cast<float4*>(c) = v;
  }
}

// The leaf's M blocks as plain float32 (its V = M^T blocks are not kept).
struct LeafOutPlain {
  float* M;
  int64_t ldm;
  int o;
  __device__ void put_m(const float* Ms, int r0, int nr, int c0, int nc, int t, int nth) const {
    const int q4 = nc / 4;
    for (int e = t; e < nr * q4; e += nth) {
      const int i = r0 + e / q4, c = c0 + 4 * (e % q4);
      *reinterpret_cast<float4*>(M + (int64_t)(o + i) * ldm + o + c) =
          *reinterpret_cast<const float4*>(Ms + i * LEAF_LDT + c);
    }
  }
  __device__ void put_v(const float*, int, int, int, int, int, int) const {}
};

// dtrack[o + r] -= sum_k L[o + r][c0 + k]^2 (k < w) for rows r < rows: one
// warp per row, float-float squares, float64 total.
__device__ __noinline__ void track_rows(const float* L, int ld, int o, int rows, int c0, int w,
                           double* dtrack) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int r = warp; r < rows; r += BNT / 32) {
    const float* row = L + (int64_t)(o + r) * ld + c0;
    float hi = 0.f, lo = 0.f;
    for (int k = lane * 4; k < w; k += 128) {
      const float4 v = *reinterpret_cast<const float4*>(row + k);
      ff_sub_sq(hi, lo, v.x);
      ff_sub_sq(hi, lo, v.y);
      ff_sub_sq(hi, lo, v.z);
      ff_sub_sq(hi, lo, v.w);
    }
    const double s = warp_sum((double)hi + (double)lo);
    if (lane == 0) dtrack[o + r] += s;
  }
}

// The merge of an inner node of the inverse (block at (o, o), size sz,
// left child h): T = L21 M11, stored transposed in L's unused upper part, and
// M21 = -M22 T into M.
template <int BK>
__device__ void node_up(const Slot& S, int ld, int o, int h, int h2, float* smem) {
  const float* L21 = S.L + (int64_t)(o + h) * ld + o;
  const float* M11 = S.M + (int64_t)o * ld + o;
  // T = L21 M11 (h2 x h; M11[k][j] = 0 for k < j), stored transposed:
  // Tt[j][i] at L[(o + j) * ld + o + h + i]
  float* Tt = S.L + (int64_t)o * ld + o + h;
  product<BK, false, true>(
      h2 / TT, h / TT, false, L21, ld, M11, ld,
      [&](int, int j0, int& klo, int& khi) { klo = j0; khi = h; },
      [&](int i0, int j0, const float (&acc)[8][4], float*) {
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          float* c = Tt + (int64_t)(j0 + tile_col(v)) * ld + i0;
#pragma unroll
          for (int ub = 0; ub < 2; ++ub)
            *reinterpret_cast<float4*>(c + tile_row(4 * ub)) =
                make_float4(acc[4 * ub][v], acc[4 * ub + 1][v], acc[4 * ub + 2][v],
                            acc[4 * ub + 3][v]);
        }
      },
      smem);
  // M21 = -M22 T: M22[i][k] = 0 for k > i; T(k, j) = Tt[j][k]
  const float* M22 = S.M + (int64_t)(o + h) * ld + o + h;
  float* M21 = S.M + (int64_t)(o + h) * ld + o;
  product<BK, false, false>(
      h2 / TT, h / TT, false, M22, ld, Tt, ld,
      [&](int i0, int, int& klo, int& khi) { klo = 0; khi = min(h2, i0 + TT); },
      [&](int i0, int j0, const float (&acc)[8][4], float*) {
        put_tile(M21, ld, i0, j0, acc, -1.f, false);
      },
      smem);
}

// X L_kk^T = A_panel for the R rows below a diagonal block: forward
// substitution, one thread per row, 32 columns at a time in registers (the
// solved columns of the row are read back from X).  L_kk comes from the
// leaf's shared memory, still in place: LT[k][i] = L[i][k] below the
// diagonal (zeros on and above it) and Rl[i] = 1 / L[i][i].  Substitution is
// backward stable; X = A_panel M_kk^T with the leaf's inverse is not, and on
// a smooth RBF instance (n = 1068, d = 2, condition number 8.8e6) the
// product form drove a later pivot negative.
__device__ __noinline__ void panel_solve(const float* __restrict__ Ap, float* __restrict__ Xp, int ld, int R,
                            const float* leaf_smem) {
  constexpr int LDT = LEAF_LDT, PB = 32;
  const float* LT = leaf_smem;
  const float* Rl = leaf_smem + 2 * LEAF * LEAF_LDT + 64 * LEAF_TLD + 4 * LEAF;
  for (int row = threadIdx.x; row < R; row += BNT) {
    const float* ar = Ap + (int64_t)row * ld;
    float* xr = Xp + (int64_t)row * ld;
    for (int cb = 0; cb < LEAF / PB; ++cb) {
      const int c0 = cb * PB;
      float a[PB];
#pragma unroll
      for (int g = 0; g < PB / 4; ++g) {
        const float4 v = *reinterpret_cast<const float4*>(ar + c0 + 4 * g);
        a[4 * g] = v.x;
        a[4 * g + 1] = v.y;
        a[4 * g + 2] = v.z;
        a[4 * g + 3] = v.w;
      }
      for (int m = 0; m < c0; ++m) {  // the solved columns
        const float xm = xr[m];
#pragma unroll
        for (int g = 0; g < PB / 4; ++g) {
          const float4 l = *reinterpret_cast<const float4*>(LT + m * LDT + c0 + 4 * g);
          a[4 * g] = fmaf(-xm, l.x, a[4 * g]);
          a[4 * g + 1] = fmaf(-xm, l.y, a[4 * g + 1]);
          a[4 * g + 2] = fmaf(-xm, l.z, a[4 * g + 2]);
          a[4 * g + 3] = fmaf(-xm, l.w, a[4 * g + 3]);
        }
      }
#pragma unroll
      for (int j = 0; j < PB; ++j) {  // within the block
        const float xj = a[j] * Rl[c0 + j];
        a[j] = xj;
#pragma unroll
        for (int g = 0; g < PB / 4; ++g) {
          if (4 * g + 3 > j) {
            const float4 l = *reinterpret_cast<const float4*>(LT + (c0 + j) * LDT + c0 + 4 * g);
            if (4 * g + 0 > j) a[4 * g] = fmaf(-xj, l.x, a[4 * g]);
            if (4 * g + 1 > j) a[4 * g + 1] = fmaf(-xj, l.y, a[4 * g + 1]);
            if (4 * g + 2 > j) a[4 * g + 2] = fmaf(-xj, l.z, a[4 * g + 2]);
            a[4 * g + 3] = fmaf(-xj, l.w, a[4 * g + 3]);
          }
        }
      }
#pragma unroll
      for (int g = 0; g < PB / 4; ++g)
        *reinterpret_cast<float4*>(xr + c0 + 4 * g) =
            make_float4(a[4 * g], a[4 * g + 1], a[4 * g + 2], a[4 * g + 3]);
    }
  }
}

// The leaf, the substitution, the GEMVs, the residual and the finalisation
// are kept out of line (__noinline__): with everything inlined,
// one register allocation serves the whole kernel and the tile loops paid for
// the other phases' live ranges (the tensor-core configuration ran 2.8%
// faster with them out of line, results unchanged bit for bit).
__device__ __noinline__ void leaf_call(const Slot& S, int ld, int o, int* info, float* smem) {
  leaf_chol_inv_body(S.A, ld, o, S.dtrack, S.logdiag, info, LeafOutPlain{S.M, ld, o}, smem);
}

// Cholesky + inverse of the padded matrix.
//  * Factor: left-looking over 128-wide block columns.  Block column o is
//    brought up to date by ONE product, A[o:, o:o+128] -= L[o:, :o]
//    L[o:o+128, :o]^T (K = o: every earlier panel at once, each output tile
//    read and written once); the leaf then factors and inverts the diagonal
//    block (pivots from the float64 diagonal track), the panel below is
//    solved by substitution against L_kk (panel_solve) and the diagonal
//    track loses its row sums of squares.  (The right-looking order,
//    A22 -= X X^T after every panel, rewrote the trailing matrix once per
//    panel: its read-modify-write traffic bound the factor with one CTA per
//    SM.  The recursive form L21 = A21 M11^T with a recursively formed M11
//    amplified rounding by the condition number of L11: on ill-conditioned
//    RBF instances its log-determinant erred ~10x more than this panel
//    form.)
//  * Inverse: M = L^-1 by the recursion's merge step, post-order over the
//    tree with 128 leaves and left child h = 128 * ceil(sz / 256):
//    T = L21 M11, M21 = -M22 T (node_up), every thread on the same path.
template <int BK>
__device__ void chol_inv(const Slot& S, int ld, int np, int* info, float* smem) {
  for (int o = 0; o < np; o += TT) {
    if (o > 0) {  // block column o minus the products of the panels to its left
      const float* Lr = S.L + (int64_t)o * ld;  // rows o.. of L, columns < o
      float* Ac = S.A + (int64_t)o * ld + o;
      // the accumulator starts at -A and takes the panels in order, so
      // every rounding is relative to the partly reduced entry as in the
      // right-looking order (summing the panels first and subtracting once
      // lost a factor ~6 of log-determinant accuracy on an n = 1500 RBF
      // instance)
      product_from<BK, false, false, true>(
          (np - o) / TT, 1, false, Lr, ld, Lr, ld,
          [&](int, int, int& klo, int& khi) { klo = 0; khi = o; },
          [&](int i0, int j0, float(&acc)[8][4]) {
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const float4 c = *reinterpret_cast<const float4*>(
                  Ac + (int64_t)(i0 + tile_row(u)) * ld + j0 + tile_col(0));
              acc[u][0] = -c.x;
              acc[u][1] = -c.y;
              acc[u][2] = -c.z;
              acc[u][3] = -c.w;
            }
          },
          [&](int i0, int j0, const float (&acc)[8][4], float*) {
            put_tile(Ac, ld, i0, j0, acc, -1.f, false);
          },
          smem);
    }
    __syncthreads();  // the column and track_rows' dtrack writes before the leaf reads them
    leaf_call(S, ld, o, info, smem);
    __syncthreads();
    const int R = np - o - TT;
    if (R <= 0) break;
    float* Lp = S.L + (int64_t)(o + TT) * ld + o;
    panel_solve(S.A + (int64_t)(o + TT) * ld + o, Lp, ld, R, smem);
    __syncthreads();
    track_rows(S.L, ld, o + TT, R, o, TT, S.dtrack);
  }
  constexpr int DEPTH = 8;  // np <= 4096: at most 6 levels
  int so[DEPTH], ss[DEPTH], sst[DEPTH];
  int top = 0;
  so[0] = 0;
  ss[0] = np;
  sst[0] = 0;
  while (top >= 0) {
    const int o = so[top], sz = ss[top];
    if (sz == TT) {
      --top;
      continue;
    }
    const int h = ((sz / 2 + TT - 1) / TT) * TT, h2 = sz - h;
    if (sst[top] < 2) {  // left child, then right child
      const int first = sst[top] == 0;
      sst[top] += 1;
      ++top;
      so[top] = first ? o : o + h;
      ss[top] = first ? h : h2;
      sst[top] = 0;
    } else {
      node_up<BK>(S, ld, o, h, h2, smem);
      --top;
    }
  }
}

__device__ __forceinline__ float dot4(float4 m, float4 v, float s) {
  return fmaf(m.w, v.w, fmaf(m.z, v.z, fmaf(m.y, v.y, fmaf(m.x, v.x, s))));
}

// z = M r (lower), one warp per row, float accumulation.  The two GEMVs of a
// solve read M from memory (np^2 / 2 floats each) with one CTA per SM, so
// they are written for bytes in flight: eight (then four) independent
// 16-byte loads per lane before the first FMA.
__device__ __noinline__ void gemv_lower(const float* M, int ld, int np, const float* r, float* z) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = warp; i < np; i += BNT / 32) {
    const float* row = M + (int64_t)i * ld;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    int k = lane * 4;
    // entries past i inside the float4 that holds i are zeros of M's
    // diagonal block; every load starts at k <= i
    for (; k + 896 <= i; k += 1024) {
      float4 m[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) m[q] = *reinterpret_cast<const float4*>(row + k + 128 * q);
#pragma unroll
      for (int q = 0; q < 8; q += 4) {
        s0 = dot4(m[q], *reinterpret_cast<const float4*>(r + k + 128 * q), s0);
        s1 = dot4(m[q + 1], *reinterpret_cast<const float4*>(r + k + 128 * (q + 1)), s1);
        s2 = dot4(m[q + 2], *reinterpret_cast<const float4*>(r + k + 128 * (q + 2)), s2);
        s3 = dot4(m[q + 3], *reinterpret_cast<const float4*>(r + k + 128 * (q + 3)), s3);
      }
    }
    for (; k + 384 <= i; k += 512) {
      const float4 m0 = *reinterpret_cast<const float4*>(row + k);
      const float4 m1 = *reinterpret_cast<const float4*>(row + k + 128);
      const float4 m2 = *reinterpret_cast<const float4*>(row + k + 256);
      const float4 m3 = *reinterpret_cast<const float4*>(row + k + 384);
      s0 = dot4(m0, *reinterpret_cast<const float4*>(r + k), s0);
      s1 = dot4(m1, *reinterpret_cast<const float4*>(r + k + 128), s1);
      s2 = dot4(m2, *reinterpret_cast<const float4*>(r + k + 256), s2);
      s3 = dot4(m3, *reinterpret_cast<const float4*>(r + k + 384), s3);
    }
    for (; k <= i; k += 128)
      s0 = dot4(*reinterpret_cast<const float4*>(row + k), *reinterpret_cast<const float4*>(r + k),
                s0);
    const float s = warp_sum((s0 + s1) + (s2 + s3));
    if (lane == 0) z[i] = s;
  }
}

// alpha (+)= M^T z by 128-column chunks: warp w takes rows c0 + w, c0 + w +
// 16, ... (a float4 of 4 columns per lane, four rows in flight), the 16
// warps' partial sums meet in shared memory (red: 16 x 128 floats).  Rows of
// the diagonal block reach past the diagonal into its zeros.
__device__ __noinline__ void gemv_upper_t(const float* M, int ld, int np, const float* z, double* alpha,
                             bool accumulate, float* red) {
  constexpr int NW = BNT / 32;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int c0 = 0; c0 < np; c0 += TT) {
    const float* col = M + c0 + 4 * lane;
    float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f), a1 = a0;
    int i = c0 + warp;
    for (; i + 7 * NW < np; i += 8 * NW) {
      float4 m[8];
      float zz[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        m[q] = *reinterpret_cast<const float4*>(col + (int64_t)(i + q * NW) * ld);
        zz[q] = z[i + q * NW];
      }
#pragma unroll
      for (int q = 0; q < 8; q += 2) {
        a0.x = fmaf(m[q].x, zz[q], a0.x); a0.y = fmaf(m[q].y, zz[q], a0.y);
        a0.z = fmaf(m[q].z, zz[q], a0.z); a0.w = fmaf(m[q].w, zz[q], a0.w);
        a1.x = fmaf(m[q + 1].x, zz[q + 1], a1.x); a1.y = fmaf(m[q + 1].y, zz[q + 1], a1.y);
        a1.z = fmaf(m[q + 1].z, zz[q + 1], a1.z); a1.w = fmaf(m[q + 1].w, zz[q + 1], a1.w);
      }
    }
    for (; i + 3 * NW < np; i += 4 * NW) {
      const float4 m0 = *reinterpret_cast<const float4*>(col + (int64_t)i * ld);
      const float4 m1 = *reinterpret_cast<const float4*>(col + (int64_t)(i + NW) * ld);
      const float4 m2 = *reinterpret_cast<const float4*>(col + (int64_t)(i + 2 * NW) * ld);
      const float4 m3 = *reinterpret_cast<const float4*>(col + (int64_t)(i + 3 * NW) * ld);
      const float z0 = z[i], z1 = z[i + NW], z2 = z[i + 2 * NW], z3 = z[i + 3 * NW];
      a0.x = fmaf(m0.x, z0, a0.x); a0.y = fmaf(m0.y, z0, a0.y);
      a0.z = fmaf(m0.z, z0, a0.z); a0.w = fmaf(m0.w, z0, a0.w);
      a1.x = fmaf(m1.x, z1, a1.x); a1.y = fmaf(m1.y, z1, a1.y);
      a1.z = fmaf(m1.z, z1, a1.z); a1.w = fmaf(m1.w, z1, a1.w);
      a0.x = fmaf(m2.x, z2, a0.x); a0.y = fmaf(m2.y, z2, a0.y);
      a0.z = fmaf(m2.z, z2, a0.z); a0.w = fmaf(m2.w, z2, a0.w);
      a1.x = fmaf(m3.x, z3, a1.x); a1.y = fmaf(m3.y, z3, a1.y);
      a1.z = fmaf(m3.z, z3, a1.z); a1.w = fmaf(m3.w, z3, a1.w);
    }
    for (; i < np; i += NW) {
      const float4 m0 = *reinterpret_cast<const float4*>(col + (int64_t)i * ld);
      const float z0 = z[i];
      a0.x = fmaf(m0.x, z0, a0.x); a0.y = fmaf(m0.y, z0, a0.y);
      a0.z = fmaf(m0.z, z0, a0.z); a0.w = fmaf(m0.w, z0, a0.w);
    }
    *reinterpret_cast<float4*>(red + warp * TT + 4 * lane) =
        make_float4(a0.x + a1.x, a0.y + a1.y, a0.z + a1.z, a0.w + a1.w);
    __syncthreads();
    if (threadIdx.x < TT) {
      float s = 0.f;
#pragma unroll
      for (int w = 0; w < NW; ++w) s += red[w * TT + threadIdx.x];
      const int j = c0 + threadIdx.x;
      alpha[j] = accumulate ? alpha[j] + (double)s : (double)s;
    }
    __syncthreads();
  }
}

// rf = rhs as float32 (rhs: float64, zeros past n)
__device__ void to_float(const double* rhs, int np, float* rf) {
  for (int i = threadIdx.x; i < np; i += BNT) rf[i] = (float)rhs[i];
}

// alpha (+)= M^T M rhs (red: 16 x 128 floats of shared memory)
__device__ void solve_apply(const Slot& S, int ld, int np, const double* rhs, bool accumulate,
                            float* red) {
  to_float(rhs, np, S.rf);
  __syncthreads();
  gemv_lower(S.M, ld, np, S.rf, S.zf);
  __syncthreads();
  gemv_upper_t(S.M, ld, np, S.zf, S.alpha, accumulate, red);
  __syncthreads();
}

// float-float accumulation (hi, lo) += a (two-sum, not contracted)
__device__ __forceinline__ void ff_add_b(float& hi, float& lo, float a) {
  const float s = __fadd_rn(hi, a);
  const float bb = __fsub_rn(s, hi);
  lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(a, bb)));
  hi = s;
}

// r = diff - Sigma alpha for rows < n (zeros past n) into rres (float64),
// Sigma regenerated from the scaled inputs, products summed in float-float.
// ah / al: alpha split into float hi / lo parts (shared memory).  The
// columns go by chunks of RCH inputs staged in shared memory (gx, odd row
// stride); a warp takes a row, its lanes the chunk's columns, and each
// row's chunk sums add up in float64 in rres.
constexpr int RCH = 512;
__device__ __noinline__ void residual(const BatchInst& I, const Slot& S, int np, float s2, float ka,
                         double noise_diag, const float* ah, const float* al, double* rres,
                         float* gx) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n = I.n, d = I.d, sd = d | 1;
  for (int i = threadIdx.x; i < np; i += BNT) rres[i] = 0.0;
  with_kind(I.kind, [&](auto kind_c) {
    constexpr int KIND = decltype(kind_c)::value;
    for (int c0 = 0; c0 < n; c0 += RCH) {
      const int cn = min(RCH, n - c0);
      __syncthreads();  // the previous chunk is done with gx (and rres is zeroed)
      for (int e = threadIdx.x; e < cn * d; e += BNT)
        gx[(e / d) * sd + e % d] = S.xs[c0 * d + e];
      __syncthreads();
      for (int i = warp; i < n; i += BNT / 32) {
        float xi[BDM];
#pragma unroll
        for (int k = 0; k < BDM; ++k) xi[k] = k < d ? S.xs[i * d + k] : 0.f;
        float sh = 0.f, sl = 0.f;
        for (int jl = lane; jl < cn; jl += 32) {
          const float* xj = gx + jl * sd;
          float sq = 0.f;
#pragma unroll
          for (int k = 0; k < BDM; ++k) {
            if (k < d) {
              const float df = xi[k] - xj[k];
              sq = fmaf(df, df, sq);
            }
          }
          const float kv = kval<float>(KIND, sq, s2, ka);
          const int j = c0 + jl;
          const float p = kv * ah[j];
          const float pe = fmaf(kv, ah[j], -p);
          ff_add_b(sh, sl, p);
          sl = fmaf(kv, al[j], sl + pe);
        }
        const double t = warp_sum((double)sh + (double)sl);
        if (lane == 0) rres[i] += t;
      }
    }
  });
  __syncthreads();
  for (int i = threadIdx.x; i < np; i += BNT)
    rres[i] = i < n ? S.diff[i] - (rres[i] + noise_diag * S.alpha[i]) : 0.0;
}

// One W tile (shared memory, row stride WLD) contracted against dK/dtheta:
// coordinates in DP pairs (packed float32x2 arithmetic), per-thread float32
// sums over its 64 elements, then per warp in float64 into wred[slot][warp].
template <int KIND, int DP>
__device__ __forceinline__ void adj_tile(int i0, int j0, int n, int d, float ka,
                                         const float* Ws, const float* sxi, const float* sxj,
                                         const float* sai, const float* saj, double* wred,
                                         int warp, int lane) {
  constexpr int NW = BNT / 32;
  f32x2 pl2[DP];
#pragma unroll
  for (int kp = 0; kp < DP; ++kp) pl2[kp] = f2_pack(0.f, 0.f);
  float pvar = 0.f, pnoise = 0.f;
#pragma unroll 2
  for (int m = 0; m < TT * TT / BNT; ++m) {
    const int e = threadIdx.x + m * BNT, r = e >> 7, c = e & 127;
    const int gi = i0 + r, gj = j0 + c;
    if (gi >= n || gj >= n || gj > gi) continue;
    const float w = Ws[r * WLD + c];
    const float coef = (gi == gj ? 1.f : 2.f) * (sai[r] * saj[c] - w);
    const f32x2* xi2 = reinterpret_cast<const f32x2*>(sxi + r * XLD);
    const f32x2* xj2 = reinterpret_cast<const f32x2*>(sxj + c * XLD);
    f32x2 dsq2[DP];
    f32x2 s2 = f2_pack(0.f, 0.f);
#pragma unroll
    for (int kp = 0; kp < DP; ++kp) {
      const f32x2 df = f2_sub(xi2[kp], xj2[kp]);
      dsq2[kp] = f2_mul(df, df);
      s2 = f2_add(s2, dsq2[kp]);
    }
    float k1, c1;
    kval_dcoef_k<KIND, float>(f2_lo(s2) + f2_hi(s2), 1.f, k1, c1, ka);
    pvar = fmaf(coef, k1, pvar);
    const float cc = coef * c1;
    const f32x2 cc2 = f2_pack(cc, cc);
#pragma unroll
    for (int kp = 0; kp < DP; ++kp) pl2[kp] = f2_fma(cc2, dsq2[kp], pl2[kp]);
    if (gi == gj) pnoise += fmaf(sai[r], sai[r], -w);
  }
  for (int s = 0; s < d + 2; ++s) {
    float v = s == d ? pvar : pnoise;
#pragma unroll
    for (int kp = 0; kp < DP; ++kp) {  // (pairs past d hold the zero padding)
      if (s < d && 2 * kp == s) v = f2_lo(pl2[kp]);
      if (s < d && 2 * kp + 1 == s) v = f2_hi(pl2[kp]);
    }
    const double t = warp_sum((double)v);
    if (lane == 0) wred[s * NW + warp] += t;
  }
}

// The adjoint: W = M^T M (lower tiles, M[k][i] = 0 for k < i), contracted at
// once with (alpha alpha^T - W) o dK/dtheta (unit variance).  Each thread sums
// its elements of a tile in float32 (64 terms); the tile's sums go, per warp
// and in float64, into the warp's own slots of wred (fixed order: the result
// is reproducible).  sg[d + 2] (shared memory) receives the lengthscale sums,
// the variance sum and the noise sum.
// One adjoint tile t (lower tiles of W = M^T M, M[k][i] = 0 for k < i) of an
// instance whose M and alpha are final, on any CTA: the W tile contracted
// with (alpha alpha^T - W) o dK/dtheta in the epilogue, its d + 2 partial
// sums written to tpart[t] (per-warp float64 sums added in a fixed order, so
// the result does not depend on which CTA ran the tile).  Returns true on
// the CTA that finished the instance's last tile.
template <int BK>
__device__ bool adjoint_tile(const BatchArgs& a, int id, const BatchInst& I, const Slot& S,
                             int t, float* smem, double* wred) {
  const int d = I.d, n = I.n, np = ((n + TT - 1) / TT) * TT, ld = np;
  constexpr int NW = BNT / 32;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float ka = kshape<float>(I.kind, I.theta, I.n_ls);
  int bi, bj;
  tri_index(t, bi, bj);
  const int i0 = bi * TT, j0 = bj * TT;
  for (int e = threadIdx.x; e < (d + 2) * NW; e += BNT) wred[e] = 0.0;
  float acc[8][4];
#pragma unroll
  for (int u = 0; u < 8; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
  tile_mma<BK, true, true>(S.M, ld, S.M, ld, i0, j0, i0, np, smem, acc);
  float* Ws = smem;                          // [TT][WLD]
  float* sxi = smem + stage_floats();        // [TT][XLD]
  float* sxj = sxi + TT * XLD;
  float* sai = sxj + TT * XLD;               // alpha of the tile's rows
  float* saj = sai + TT;                     // and columns
#pragma unroll
  for (int u = 0; u < 8; ++u)
    *reinterpret_cast<float4*>(Ws + tile_row(u) * WLD + tile_col(0)) =
        make_float4(acc[u][0], acc[u][1], acc[u][2], acc[u][3]);
  for (int e = threadIdx.x; e < TT * BDM; e += BNT) {
    const int r = e / BDM, k = e % BDM;
    sxi[r * XLD + k] = (i0 + r < n && k < d) ? S.xs[(i0 + r) * d + k] : 0.f;
    sxj[r * XLD + k] = (j0 + r < n && k < d) ? S.xs[(j0 + r) * d + k] : 0.f;
  }
  for (int e = threadIdx.x; e < TT; e += BNT) {
    sai[e] = S.ahf[i0 + e];
    saj[e] = S.ahf[j0 + e];
  }
  __syncthreads();
  with_kind(I.kind, [&](auto kind_c) {
    constexpr int KIND = decltype(kind_c)::value;
    const int dp = (d + 1) / 2;
    if (dp <= 2)
      adj_tile<KIND, 2>(i0, j0, n, d, ka, Ws, sxi, sxj, sai, saj, wred, warp, lane);
    else if (dp <= 4)
      adj_tile<KIND, 4>(i0, j0, n, d, ka, Ws, sxi, sxj, sai, saj, wred, warp, lane);
    else
      adj_tile<KIND, 8>(i0, j0, n, d, ka, Ws, sxi, sxj, sai, saj, wred, warp, lane);
  });
  __syncthreads();
  double* tp = a.tpart + I.tpart_off + (int64_t)t * (d + 2);
  for (int s = threadIdx.x; s < d + 2; s += BNT) {
    double v = 0.0;
    for (int w = 0; w < NW; ++w) v += wred[s * NW + w];
    tp[s] = v;
  }
  __shared__ int s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();  // the partials before the count
    s_last = atomicAdd(&a.tiles_done[id], 1) == I.ntiles - 1;
  }
  __syncthreads();
  return s_last;
}

// The outputs of an instance from its slot (any CTA): log-determinant,
// quadratic form and alpha sum in compensated float64, the gradient slots
// summed over the tiles' partials in tile order.
__device__ __noinline__ void finish_instance(const BatchArgs& a, const BatchInst& I, const Slot& S,
                                bool failed, double* sg) {
  const int n = I.n, d = I.d;
  const bool grad = a.want_grad && !failed;
  __threadfence();  // every tile's partials (written on other SMs) before reading them
  for (int s = threadIdx.x; s < d + 2; s += BNT) {
    double v = 0.0;
    if (grad)
      for (int t = 0; t < I.ntiles; ++t) v += a.tpart[I.tpart_off + (int64_t)t * (d + 2) + s];
    sg[s] = v;
  }
  __syncthreads();
  const double logdet =
      2.0 * block_ksum(n, [&](int i) { return failed ? 0.0 : S.logdiag[i]; });
  const double quad = block_ksum(n, [&](int i) { return failed ? 0.0 : S.diff[i] * S.alpha[i]; });
  const double asum = block_ksum(n, [&](int i) { return failed ? 0.0 : S.alpha[i]; });
  if (threadIdx.x == 0)
    finalize_outputs(n, d, I.theta, I.n_ls, a.jitter, logdet, quad, asum, sg, a.want_grad,
                     I.info, I.out_mll, a.want_grad ? I.out_grad : nullptr);
  __syncthreads();
}

// Everything of an instance before its adjoint, on the CTA that took it from
// the queue: Gram, factor and inverse, alpha refined.  Returns true if
// the factorisation failed.
template <int BK>
__device__ bool instance_front(const BatchArgs& a, const BatchInst& I, const Slot& S,
                               float* smem) {
  const int n = I.n, d = I.d;
  const int np = ((n + TT - 1) / TT) * TT;
  const int ld = np;
  const double* th = I.theta;
  const double s2d = th[I.n_ls], sd = th[I.n_ls + 1], cst = th[I.n_ls + 2];
  const float s2 = (float)s2d;
  const float ka = kshape<float>(I.kind, th, I.n_ls);
  const double noise_diag = a.jitter + sd * sd;
  if (threadIdx.x == 0) *I.info = INT_MAX;
  // scaled inputs, diff, diagonal track, zeroed diagonal blocks of M
  for (int e = threadIdx.x; e < n * d; e += BNT) {
    const int i = e / d, k = e % d;
    const double l = I.n_ls == 1 ? th[0] : th[k];
    S.xs[e] = (float)(I.x[(int64_t)i * I.ldx + k] / l);
  }
  for (int i = threadIdx.x; i < np; i += BNT) {
    S.diff[i] = i < n ? I.y[i] - cst : 0.0;
    S.dtrack[i] = i < n ? s2d + noise_diag : 1.0;
  }
  for (int e = threadIdx.x; e < np * TT; e += BNT) {
    const int i = e / TT, c = e % TT;
    S.M[(int64_t)i * ld + (i / TT) * TT + c] = 0.f;
  }
  __syncthreads();
  // Gram: lower 128-blocks (diagonal blocks in full), identity past n.  The
  // block's row and column inputs are staged in shared memory with an odd
  // row stride (a warp reads 32 consecutive columns' coordinates without
  // bank conflicts); the kernel kind is resolved outside the loops.
  {
    const int nb = np / TT, nt = nb * (nb + 1) / 2;
    const int sd = d | 1;
    float* gxi = smem;              // [TT][sd]
    float* gxj = smem + TT * (BDM + 1);
    with_kind(I.kind, [&](auto kind_c) {
      constexpr int KIND = decltype(kind_c)::value;
      for (int t = 0; t < nt; ++t) {
        int bi, bj;
        tri_index(t, bi, bj);
        for (int e = threadIdx.x; e < TT * d; e += BNT) {
          const int r = e / d, k = e % d;
          gxi[r * sd + k] = bi * TT + r < n ? S.xs[(bi * TT + r) * d + k] : 0.f;
          gxj[r * sd + k] = bj * TT + r < n ? S.xs[(bj * TT + r) * d + k] : 0.f;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < TT * TT; e += BNT) {
          const int il = e / TT, jl = e % TT;
          const int i = bi * TT + il, j = bj * TT + jl;
          float v;
          if (i >= n || j >= n) {
            v = i == j ? 1.f : 0.f;
          } else {
            float sq = 0.f;
            for (int k = 0; k < d; ++k) {
              const float df = gxi[il * sd + k] - gxj[jl * sd + k];
              sq = fmaf(df, df, sq);
            }
            v = kval<float>(KIND, sq, s2, ka);
            if (i == j) v = (float)((double)v + noise_diag);
          }
          S.A[(int64_t)i * ld + j] = v;
        }
        __syncthreads();
      }
    });
  }
  __syncthreads();
  chol_inv<BK>(S, ld, np, I.info, smem);
  __syncthreads();
  const bool failed = *(volatile int*)I.info != INT_MAX;
  __syncthreads();
  if (failed) return true;
  // alpha = Sigma^-1 diff, refined (twice, or once: see below)
  float* ah = smem;          // [np] alpha hi
  float* al = smem + np;     // [np] alpha lo
  double* rres = reinterpret_cast<double*>(smem + 2 * np);  // [np]
  float* red = smem + 4 * np;  // [16][128] GEMV partial sums, then the residual's
                               // staged inputs [RCH][BDM + 1]
  solve_apply(S, ld, np, S.diff, false, red);
  __shared__ double s_cmax[BNT / 32], s_amax[BNT / 32];
  for (int it = 0; it < 2; ++it) {
    for (int i = threadIdx.x; i < np; i += BNT) {
      const double v = S.alpha[i];
      const float hi = (float)v;
      ah[i] = hi;
      al[i] = (float)(v - (double)hi);
    }
    __syncthreads();
    residual(I, S, np, s2, ka, noise_diag, ah, al, rres, red + 16 * TT);
    __syncthreads();
    solve_apply(S, ld, np, rres, true, red);
    if (it == 0) {
      // Refinement contracts the error by about the size of its first
      // correction relative to alpha; below 1e-5 the second correction would
      // be below ~1e-10 of alpha, under the float32 factor's own effect on
      // the MLL, and is skipped (most instances of a batch).
      double cm = 0.0, am = 0.0;
      for (int i = threadIdx.x; i < np; i += BNT) {
        const double v = S.alpha[i];
        cm = fmax(cm, fabs(v - ((double)ah[i] + (double)al[i])));
        am = fmax(am, fabs(v));
      }
      for (int off = 16; off > 0; off >>= 1) {
        cm = fmax(cm, __shfl_xor_sync(0xffffffffu, cm, off));
        am = fmax(am, __shfl_xor_sync(0xffffffffu, am, off));
      }
      if ((threadIdx.x & 31) == 0) {
        s_cmax[threadIdx.x >> 5] = cm;
        s_amax[threadIdx.x >> 5] = am;
      }
      __syncthreads();
      cm = 0.0;
      am = 0.0;
      for (int w = 0; w < BNT / 32; ++w) {
        cm = fmax(cm, s_cmax[w]);
        am = fmax(am, s_amax[w]);
      }
      __syncthreads();
      if (cm <= 1e-5 * am) break;
    }
  }
  for (int i = threadIdx.x; i < np; i += BNT) S.ahf[i] = (float)S.alpha[i];
  __syncthreads();
  return false;
}

// One CTA per SM.  A CTA first works through the adjoint tiles of the last
// instance it prepared; then takes the next instance from the size-sorted
// queue (Gram, factor, inverse, alpha) and publishes it; when the queue is
// empty it takes unclaimed adjoint tiles of any published instance, waiting
// (at most wait_cycles in total) while some instance is still being prepared.
// Whoever finishes an instance's last tile writes its outputs.  An idle CTA
// that stops waiting changes nothing but speed: the owner of an instance
// claims all of its tiles that nobody else has.
__global__ void __launch_bounds__(BNT, 1) batch_mll_kernel(const __grid_constant__ BatchArgs a) {
  extern __shared__ __align__(16) float smem[];
  __shared__ double s_red[(GPK_MAX_D + 2) * 17];
  // the slot's pointers and the instance's descriptor live in shared memory
  // (read where used) rather than in ~40 registers for the whole instance
  __shared__ Slot s_slot;
  __shared__ BatchInst s_inst;
  __shared__ int s_mode, s_id, s_tile, s_own;
  __shared__ long long s_wait0;
  if (threadIdx.x == 0) {
    s_own = -1;
    s_wait0 = -1;
  }
  tc_setup(a.tc_stall);
  for (;;) {
    if (threadIdx.x == 0) {
      int mode = 0, id = -1, tile = -1;
      // 1) the tiles of the instance this CTA prepared
      if (s_own >= 0) {
        const int t = atomicAdd(&a.next_tile[s_own], 1);
        if (t < a.inst[s_own].ntiles) {
          mode = 2;
          id = s_own;
          tile = t;
        } else {
          s_own = -1;
        }
      }
      // 2) the next instance of the queue
      if (mode == 0) {
        const int q = atomicAdd(a.head, 1);
        if (q < a.count) {
          mode = 1;
          id = a.queue[q];
        }
      }
      // 3) unclaimed tiles of published instances
      if (mode == 0) {
        bool all_published = true;
        for (int i = 0; i < a.count && mode == 0; ++i) {
          if (!*(volatile int*)&a.published[i]) {
            all_published = false;
            continue;
          }
          if (*(volatile int*)&a.next_tile[i] >= a.inst[i].ntiles) continue;
          const int t = atomicAdd(&a.next_tile[i], 1);
          if (t < a.inst[i].ntiles) {
            mode = 2;
            id = i;
            tile = t;
          }
        }
        if (mode == 0) {
          if (all_published) {
            mode = 3;  // nothing left anywhere
          } else {
            const long long now = clock64();
            if (s_wait0 < 0) s_wait0 = now;
            mode = now - s_wait0 > a.wait_cycles ? 3 : 4;
          }
        }
      }
      if (mode == 2) __threadfence();  // the instance's slot after its "published" flag
      if (id >= 0) {
        s_inst = a.inst[id];
        const int np = ((s_inst.n + TT - 1) / TT) * TT;
        slot_layout(np, a.ws + s_inst.slot_off, &s_slot);
      }
      s_mode = mode;
      s_id = id;
      s_tile = tile;
    }
    __syncthreads();
    const int mode = s_mode;
    if (mode == 3) break;
    if (mode == 4) {
      if (threadIdx.x == 0) __nanosleep(2000);
      __syncthreads();
      continue;
    }
    const int id = s_id;
    const int cfg = a.force_cfg >= 0 ? a.force_cfg : s_inst.cfg;
    if (mode == 1) {
      bool failed = cfg == 0   ? instance_front<16>(a, s_inst, s_slot, smem)
                    : cfg == 1 ? instance_front<32>(a, s_inst, s_slot, smem)
                               : instance_front<TC_BK>(a, s_inst, s_slot, smem);
      if (tc_failed()) {  // a tensor-core wait timed out: the instance fails
        __syncthreads();
        if (threadIdx.x == 0) *s_inst.info = -1;
        failed = true;
      }
      const bool tiles = !failed && a.want_grad && s_inst.ntiles > 0;
      if (!tiles) finish_instance(a, s_inst, s_slot, failed, s_red);
      if (threadIdx.x == 0) {
        if (!tiles) atomicExch(&a.next_tile[id], 1 << 30);  // no tiles to claim
        __threadfence();  // the slot's M and alpha before the flag
        atomicExch(&a.published[id], 1);
        s_own = tiles ? id : -1;
      }
    } else {
      const bool last =
          cfg == 0   ? adjoint_tile<16>(a, id, s_inst, s_slot, s_tile, smem, s_red)
          : cfg == 1 ? adjoint_tile<32>(a, id, s_inst, s_slot, s_tile, smem, s_red)
                     : adjoint_tile<TC_BK>(a, id, s_inst, s_slot, s_tile, smem, s_red);
      if (tc_failed() && threadIdx.x == 0) atomicExch(s_inst.info, -1);
      if (last) finish_instance(a, s_inst, s_slot, false, s_red + GPK_MAX_D + 2 + 16 * 18);
    }
    __syncthreads();  // everyone is done with the shared descriptors before thread 0 rewrites them
  }
  tc_teardown();
}

// The queued instances of a partial launch (autotuner trial): not yet
// published, tiles claimed from 0.
__global__ void batch_reset_kernel(const int* queue, int count, int* published, int* next_tile) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < count) {
    published[queue[q]] = 0;
    next_tile[queue[q]] = 0;
  }
}

size_t batch_smem_bytes(int np_max) {
  // the largest of: the product staging area, the tensor-core region, the
  // leaf, the refinement vectors
  const size_t prod = std::max((size_t)prod_floats() * sizeof(float), tc_region_bytes());
  const size_t leaf = leaf_smem_bytes();
  const size_t refine = (size_t)np_max * (2 * sizeof(float) + sizeof(double)) +
                        (size_t)(16 * TT + RCH * (BDM + 1)) * sizeof(float);
  return std::max(std::max(prod, leaf), refine);
}

}  // namespace
}  // namespace gpk

using namespace gpk;

// ---------------------------------------------------------------------------
// Plans
// ---------------------------------------------------------------------------
struct gpk_batch_plan_s {
  int device = 0;
  int count = 0;
  int np_max = 0;
  int want_grad = 1;
  double jitter = 0.0;
  int grid = 0;
  size_t ws_bytes = 0;          // one slot per instance
  size_t smem = 0;
  BatchInst* d_inst = nullptr;  // device copies of the descriptors
  int* d_queue = nullptr;       // size-sorted instance indices
  int* d_state = nullptr;       // head, published[count], next_tile[count], tiles_done[count]
  double* d_tpart = nullptr;    // per-tile gradient partials
  int force_cfg = -1;           // >= 0: every instance runs this configuration
  long long tc_stall = 0;       // self-test of the bounded tensor-core waits (0: off)
};

namespace {
// Autotuner results, kept for the process: (device, n_pad) -> configuration.
std::mutex g_tune_mu;
std::map<std::pair<int, int>, int> g_tune;

// Wait bound of an idle CTA for instances still being prepared (~2 s of SM
// clock; an execution takes tens of milliseconds).
constexpr long long kIdleWaitCycles = 4000000000LL;

cudaError_t launch_batch(const gpk_batch_plan_s& P, void* ws, int force_cfg, int count,
                         const int* queue, cudaStream_t s) {
  BatchArgs a{};
  a.inst = P.d_inst;
  a.queue = queue;
  a.head = P.d_state;
  a.published = P.d_state + 1;
  a.next_tile = a.published + P.count;
  a.tiles_done = a.next_tile + P.count;
  a.tpart = P.d_tpart;
  a.count = count;
  a.ws = static_cast<char*>(ws);
  a.want_grad = P.want_grad;
  a.jitter = P.jitter;
  a.force_cfg = force_cfg;
  a.wait_cycles = kIdleWaitCycles;
  a.tc_stall = P.tc_stall;
  // instances outside the queue (autotuner trials) count as published with
  // no tiles: 1 in published[], a huge next_tile
  cudaError_t e = cudaMemsetAsync(P.d_state, 0, sizeof(int) * (1 + 3 * (size_t)P.count), s);
  if (e == cudaSuccess && count < P.count) {
    e = cudaMemsetAsync(a.published, 0x01, sizeof(int) * P.count, s);  // any non-zero word
    if (e == cudaSuccess) e = cudaMemsetAsync(a.next_tile, 0x7f, sizeof(int) * P.count, s);
  }
  if (e != cudaSuccess) return e;
  if (count < P.count) {  // the trial's instances: not published, tiles from 0
    batch_reset_kernel<<<(count + 255) / 256, 256, 0, s>>>(queue, count, a.published, a.next_tile);
    e = launch_status();
    if (e != cudaSuccess) return e;
  }
  const int grid = std::min(P.grid, std::max(count, 1));
  batch_mll_kernel<<<grid, BNT, P.smem, s>>>(a);
  return launch_status();
}

// Times every configuration on up to one grid of the plan's instances of
// each n_pad (their outputs are overwritten by the next execution) and
// keeps, per (device, n_pad), the fastest of those that fail the fewest of
// the trial's instances.
gpk_status autotune(gpk_batch_plan_s& P, const std::vector<int>& np_of, const std::vector<int>& order,
                    const int* d_info) {
  std::map<int, std::vector<int>> by_np;
  for (int i : order) by_np[np_of[i]].push_back(i);
  std::vector<int> todo;
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    for (auto& kv : by_np)
      if (!g_tune.count({P.device, kv.first})) todo.push_back(kv.first);
  }
  if (todo.empty()) return GPK_OK;
  std::vector<int> hinfo(P.count);
  const size_t ws_bytes = P.ws_bytes;
  void* ws = nullptr;
  int* dq = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  gpk_status st = GPK_OK;
  if (cudaMalloc(&ws, ws_bytes) != cudaSuccess || cudaMalloc(&dq, sizeof(int) * P.count) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    st = GPK_ERR_CUDA;
  for (size_t b = 0; st == GPK_OK && b < todo.size(); ++b) {
    std::vector<int>& ids = by_np[todo[b]];
    const int m = std::min((int)ids.size(), P.grid);
    if (cudaMemcpy(dq, ids.data(), sizeof(int) * m, cudaMemcpyHostToDevice) != cudaSuccess) {
      st = GPK_ERR_CUDA;
      break;
    }
    float best = 0.f;
    int best_cfg = 0, best_fail = INT_MAX;
    for (int cfg = 0; cfg < NCFG && st == GPK_OK; ++cfg) {
      float ms = 0.f;
      for (int rep = 0; rep < 2; ++rep) {  // the first run warms up
        if (cudaEventRecord(e0, s) != cudaSuccess || launch_batch(P, ws, cfg, m, dq, s) != cudaSuccess ||
            cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
            cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
          st = GPK_ERR_CUDA;
          break;
        }
      }
      // failed instances of the trial (a configuration must not lose an
      // instance that another one factors)
      int fails = 0;
      if (st == GPK_OK) {
        if (cudaMemcpy(hinfo.data(), d_info, sizeof(int) * P.count, cudaMemcpyDeviceToHost) !=
            cudaSuccess) {
          st = GPK_ERR_CUDA;
          break;
        }
        for (int q = 0; q < m; ++q) fails += hinfo[ids[q]] != 0;
      }
      if (st == GPK_OK && (fails < best_fail || (fails == best_fail && ms < best))) {
        best = ms;
        best_cfg = cfg;
        best_fail = fails;
      }
    }
    if (st == GPK_OK) {
      std::lock_guard<std::mutex> lock(g_tune_mu);
      g_tune[{P.device, todo[b]}] = best_cfg;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (s) cudaStreamDestroy(s);
  if (dq) cudaFree(dq);
  if (ws) cudaFree(ws);
  return st;
}
}  // namespace

extern "C" gpk_status gpk_batch_plan_create(int count, const int* kind, const int64_t* n,
                                            const int* d, const double* const* x,
                                            const int64_t* ldx, const double* const* y,
                                            const double* const* theta, const int* n_ls,
                                            double jitter, int want_grad,
                                            double* const* out_mll, double* const* out_grad,
                                            int* info, int autotune_flag, gpk_batch_plan* plan) {
  if (!plan) return GPK_ERR_BAD_ARG;
  *plan = nullptr;
  if (count <= 0 || !kind || !n || !d || !x || !ldx || !y || !theta || !n_ls || !out_mll ||
      !info || (want_grad && !out_grad) || !(jitter >= 0.0))
    return GPK_ERR_BAD_ARG;
  int np_max = 0;
  std::vector<int> np_of(count);
  std::vector<BatchInst> hv(count);
  for (int i = 0; i < count; ++i) {
    if (kind[i] < GPK_RBF || kind[i] > GPK_RATIONAL_QUADRATIC || n[i] <= 0 || d[i] <= 0 ||
        ldx[i] < d[i] || (n_ls[i] != 1 && n_ls[i] != d[i]) || !x[i] || !y[i] || !theta[i] ||
        !out_mll[i] || (want_grad && !out_grad[i]))
      return GPK_ERR_BAD_ARG;
    if (n[i] > NP_MAX || d[i] > BDM) return GPK_ERR_UNSUPPORTED;
    np_of[i] = (int)((n[i] + TT - 1) / TT) * TT;
    np_max = std::max(np_max, np_of[i]);
    hv[i] = BatchInst{};
    hv[i].x = x[i];
    hv[i].y = y[i];
    hv[i].theta = theta[i];
    hv[i].out_mll = out_mll[i];
    hv[i].out_grad = want_grad ? out_grad[i] : nullptr;
    hv[i].info = info + i;
    hv[i].ldx = ldx[i];
    hv[i].n = (int)n[i];
    hv[i].d = d[i];
    hv[i].kind = kind[i];
    hv[i].n_ls = n_ls[i];
  }
  // one workspace slot per instance; the adjoint's lower 128-tiles and their
  // partial sums
  size_t ws_bytes = 0;
  int64_t tpart = 0;
  for (int i = 0; i < count; ++i) {
    const int nb = np_of[i] / TT;
    hv[i].slot_off = (int64_t)ws_bytes;
    ws_bytes += al256(slot_layout(np_of[i], nullptr, nullptr));
    hv[i].ntiles = want_grad ? nb * (nb + 1) / 2 : 0;
    hv[i].tpart_off = tpart;
    tpart += (int64_t)hv[i].ntiles * (d[i] + 2);
  }
  std::vector<int> order(count);
  for (int i = 0; i < count; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return n[a] > n[b]; });
  auto* P = new gpk_batch_plan_s;
  auto fail = [&](gpk_status st) {
    gpk_batch_plan_destroy(P);
    return st;
  };
  if (cudaGetDevice(&P->device) != cudaSuccess) return fail(GPK_ERR_CUDA);
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, P->device) != cudaSuccess)
    return fail(GPK_ERR_CUDA);
  P->count = count;
  P->np_max = np_max;
  P->want_grad = want_grad ? 1 : 0;
  P->jitter = jitter;
  P->smem = batch_smem_bytes(np_max);
  P->ws_bytes = ws_bytes;
  if (cudaFuncSetAttribute(batch_mll_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)P->smem) != cudaSuccess)
    return fail(GPK_ERR_CUDA);
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_mll_kernel, BNT, P->smem) !=
          cudaSuccess ||
      per_sm < 1)
    return fail(GPK_ERR_UNSUPPORTED);
  P->grid = sms * per_sm;
  if (cudaMalloc(&P->d_inst, sizeof(BatchInst) * count) != cudaSuccess ||
      cudaMalloc(&P->d_queue, sizeof(int) * count) != cudaSuccess ||
      cudaMalloc(&P->d_state, sizeof(int) * (1 + 3 * (size_t)count)) != cudaSuccess ||
      cudaMalloc(&P->d_tpart, sizeof(double) * (size_t)std::max<int64_t>(tpart, 1)) != cudaSuccess)
    return fail(GPK_ERR_CUDA);
  if (cudaMemcpy(P->d_inst, hv.data(), sizeof(BatchInst) * count, cudaMemcpyHostToDevice) !=
          cudaSuccess ||
      cudaMemcpy(P->d_queue, order.data(), sizeof(int) * count, cudaMemcpyHostToDevice) !=
          cudaSuccess)
    return fail(GPK_ERR_CUDA);
  if (autotune_flag) {
    const gpk_status st = autotune(*P, np_of, order, info);
    if (st != GPK_OK) return fail(st);
  }
  // configurations per instance from the tuned table (K slices of 32 where untuned)
  bool changed = false;
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    for (int i = 0; i < count; ++i) {
      auto it = g_tune.find({P->device, np_of[i]});
      const int cfg = it != g_tune.end() ? it->second : 1;
      if (hv[i].cfg != cfg) {
        hv[i].cfg = cfg;
        changed = true;
      }
    }
  }
  if (changed && cudaMemcpy(P->d_inst, hv.data(), sizeof(BatchInst) * count,
                            cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(GPK_ERR_CUDA);
  *plan = P;
  return GPK_OK;
}

extern "C" size_t gpk_batch_plan_workspace_bytes(gpk_batch_plan plan) {
  return plan ? plan->ws_bytes : 0;
}

extern "C" int gpk_batch_plan_config(gpk_batch_plan plan, int64_t n) {
  if (!plan || n <= 0 || n > NP_MAX) return -1;
  const int np = (int)((n + TT - 1) / TT) * TT;
  std::lock_guard<std::mutex> lock(g_tune_mu);
  auto it = g_tune.find({plan->device, np});
  return it != g_tune.end() ? it->second : 1;
}

extern "C" int gpk_batch_plan_config_count(void) { return NCFG; }

extern "C" gpk_status gpk_batch_plan_force_config(gpk_batch_plan plan, int cfg) {
  if (!plan || cfg < -1 || cfg >= NCFG) return GPK_ERR_BAD_ARG;
  plan->force_cfg = cfg;
  return GPK_OK;
}

extern "C" gpk_status gpk_batch_plan_selftest_stall(gpk_batch_plan plan, long long cycles) {
  if (!plan || cycles < 0 || cycles > kIdleWaitCycles) return GPK_ERR_BAD_ARG;
  plan->tc_stall = cycles;
  return GPK_OK;
}

extern "C" gpk_status gpk_batch_plan_execute(gpk_batch_plan plan, void* workspace,
                                             size_t workspace_bytes, cudaStream_t stream) {
  if (!plan || !workspace) return GPK_ERR_BAD_ARG;
  if (workspace_bytes < gpk_batch_plan_workspace_bytes(plan)) return GPK_ERR_WORKSPACE;
  GPK_CUDA_TRY(launch_batch(*plan, workspace, plan->force_cfg, plan->count, plan->d_queue, stream));
  return GPK_OK;
}

extern "C" gpk_status gpk_batch_plan_destroy(gpk_batch_plan plan) {
  if (!plan) return GPK_OK;
  if (plan->d_inst) cudaFree(plan->d_inst);
  if (plan->d_queue) cudaFree(plan->d_queue);
  if (plan->d_state) cudaFree(plan->d_state);
  if (plan->d_tpart) cudaFree(plan->d_tpart);
  delete plan;
  return GPK_OK;
}
