// Split-TF32 NT GEMM on the 5th-generation tensor cores (tcgen05, sm_103a).
//
//   acc[i, j] = sum_k A[i, k] B[j, k],  A = A_hi + A_lo, B = B_hi + B_lo
//   computed as A_lo B_hi + A_hi B_lo + A_hi B_hi
// where *_hi is the operand rounded to TF32 and *_lo the TF32 rounding of the
// remainder (both stored as float32 bit patterns with zero low 13 bits), which
// recovers float32-class products on the TF32 pipe.  One tile shape takes the
// same split in float16 instead (same 11-bit significand, twice the MMA rate,
// half the operand bytes), on operands whose rows were scaled by powers of
// two into float16's range; the epilogue undoes the scales exactly.  Operands
// are staged by TMA (swizzled) into a shared-memory ring, one elected thread
// issues tcgen05.mma into float32 accumulators in tensor memory, and eight
// epilogue warps read them back with tcgen05.ld and apply a fused epilogue
// (trailing update, split store with optional transpose, the MLL adjoint
// reduction or the SGPR adjoint reduction).  Four tile shapes (128 x 128;
// 128 x 256 for large problems; 128 x 64 where few tiles would leave SMs idle;
// 128 x 256 on float16 operands) share the code.  Every mbarrier wait is
// bounded: on timeout the CTA sets an error flag, drains its own copies and
// returns.
#pragma once
#include <cuda.h>
#include "gpk_internal.cuh"

namespace gpk {
namespace tc {

constexpr int BM = 128;                        // output tile rows (TMEM lanes)
constexpr int NUM_THREADS = 320;               // w0 TMA, w1 MMA + TMEM, w2..w9 epilogue
constexpr int GRAD_DMAX = 16;                  // largest input dimension of the adjoint epilogue

enum Mode { MODE_ADD_F32 = 0, MODE_STORE_SPLIT = 1, MODE_GRAD = 2, MODE_SGPR = 3 };

struct TcParams {
  int M, N, K;
  int a_row0, a_col0, b_row0, b_col0;   // origin of A and B inside their tensor maps
  int a_zrow, a_zcol, b_zrow, b_zcol;   // per-batch (blockIdx.z) origin increments
  int a_tri, b_tri, c_lower;
  int tiles_m, tiles_n;
  int force_shape;  // 0: chosen per problem; 1 + Tile shape index to force one
  // outputs (MODE_ADD_F32: c0 += alpha*acc; MODE_STORE_SPLIT: hi/lo of alpha*acc
  // into c0/c1 at (i, j) and t0/t1 at (j, i))
  float *c0, *c1, *t0, *t1;
  float *s0, *s1;  // MODE_ADD_F32, optional: TF32 hi/lo of the updated C, same layout as c0
  int64_t ldc, ldt;
  int64_t c_row0, c_col0, c_zrow, c_zcol;
  int64_t t_row0, t_col0, t_zrow, t_zcol;
  float alpha;
  double* dtrack;  // optional: dtrack[c_row0 + i] -= sum_j (alpha*acc)^2
  // adjoint epilogues.  MODE_GRAD (exact GP, square symmetric): rows and
  // columns both index xs, avec = alpha.  MODE_SGPR (rows = inducing points
  // zs, columns = data points xs): G = acc + avec_i * bvec_j, reduced against
  // dK/dtheta into gpart[tile] and against dK/dz into zpart[column tile][row].
  // optional, every mode: acc[i, j] *= ra[i] * rb[j] before the epilogue uses
  // it (the inverse power-of-two row scales of float16 operands A and B;
  // indices are rows of the product, 0 <= i < M, 0 <= j < N)
  const float* ra;
  const float* rb;
  int n_true, d, kind;
  const double* kaptr;  // device pointer to the rational-quadratic alpha (kshape); null: 1
  const float* xs;
  const float* zs;
  const double* avec;
  const double* bvec;
  double* gpart;
  double* zpart;
  int* err;
  long long wait_cycles;  // bound of every mbarrier wait in SM clocks; 0: about two seconds
  int test_stall;         // self-test only: the MMA thread waits on a barrier nothing arrives at
};

}  // namespace tc

// Host helpers (tc_gemm.cu).
struct TcMat {
  const float* hi;
  const float* lo;
  int64_t rows, cols, ld;  // extent of the whole array the tensor map covers
};

// Launches one (batched) split-TF32 NT GEMM; maps are encoded from A and B.
cudaError_t tc_gemm_launch(int mode, const TcMat& A, const TcMat& B, const tc::TcParams& p,
                           int batch, cudaStream_t s);

// Pre-encoded hi/lo tensor maps of one split operand array (encode once per
// call, reuse for every GEMM that reads the array at some origin).
struct TcMap {
  CUtensorMap hi, lo;        // narrow tile: box 32 x 128
  CUtensorMap wa_hi, wa_lo;  // wide tile, A side: box 16 x 128
  CUtensorMap wb_hi, wb_lo;  // wide tile, B side: box 16 x 256
  CUtensorMap hb_hi, hb_lo;  // half tile, B side: box 32 x 64
  CUtensorMap fa_hi, fa_lo;  // float16 wide tile, A side: box 32 x 128
  CUtensorMap fb_hi, fb_lo;  // float16 wide tile, B side: box 32 x 256
};
bool tc_make_map(TcMap* m, const float* hi, const float* lo, int64_t rows, int64_t cols,
                 int64_t ld);
// float16 hi/lo operand pair (2-byte elements, ld in elements): fills the fa/fb
// maps, used by the float16 wide tile shape (index 3; force_shape = 4).
bool tc_make_map_f16(TcMap* m, const void* hi, const void* lo, int64_t rows, int64_t cols,
                     int64_t ld);
// pdl: launch as a programmatic dependent of the previous kernel in the stream
// (only where that previous stream operation is a kernel launch).
cudaError_t tc_gemm_run(int mode, const TcMap& A, const TcMap& B, const tc::TcParams& p,
                        int batch, cudaStream_t s, bool pdl = false);
// Grid size (output tiles) tc_gemm_run launches for this mode and problem; the
// MODE_GRAD epilogue writes one gpart row per tile.
int tc_gemm_tiles(int mode, const tc::TcParams& p);
// Column tiles of that grid (MODE_SGPR writes zpart[column tile][row]).
int tc_gemm_col_tiles(int mode, const tc::TcParams& p);

// hi/lo TF32 split of a float32 matrix (rows x cols, ld) into hi/lo (ldo).
cudaError_t tf32_split(const float* src, int64_t lds, int rows, int cols, float* hi, float* lo,
                       int64_t ldo, cudaStream_t s, bool pdl = false);

}  // namespace gpk
