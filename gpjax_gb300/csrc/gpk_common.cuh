// Shared device helpers for the gpk library: pointwise stationary kernels and
// their derivatives, status handling and small reductions.
#pragma once
#include <type_traits>
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>
#include "gpk.h"

#define GPK_MAX_D 32  // largest input dimension handled by the register paths

namespace gpk {

// ---------------------------------------------------------------------------
// Pointwise stationary kernels on the scaled squared distance
//   sq = sum_d ((x_d - y_d) / l_d)^2
// RBF       k = s2 exp(-sq/2)                          (kernels/stationary/rbf.py:40-44)
// Matern32  k = s2 (1 + sqrt3 t) exp(-sqrt3 t)         (matern32.py:41-54)
// Matern52  k = s2 (1 + sqrt5 t + 5/3 t^2) exp(-sqrt5 t) (matern52.py:42-53)
// Matern12  k = s2 exp(-t)                             (matern12.py:44-48)
// RationalQuadratic  k = s2 (1 + sq / (2 alpha))^-alpha (rational_quadratic.py:76-83)
// with t = sqrt(max(sq, 1e-36)) (stationary/utils.py:56-67).
//
// dcoef(sq) returns c with dk/dl_d = c * (x_d - y_d)^2 / l_d^3 and
// dk/dx_d = -c * (x_d - y_d) / l_d^2; the 1e-36 floor has zero derivative,
// which matches differentiating max(sq, 1e-36) below the floor.
// ---------------------------------------------------------------------------
template <typename T> struct Consts;
template <> struct Consts<double> {
  static __device__ __forceinline__ double floor_() { return 1e-36; }
};
template <> struct Consts<float> {
  // 1e-36 is a normal float (FLT_MIN ~ 1.18e-38), so the same floor applies.
  static __device__ __forceinline__ float floor_() { return 1e-36f; }
};

__device__ __forceinline__ double d_exp(double x) { return exp(x); }
__device__ __forceinline__ float d_exp(float x) { return expf(x); }
__device__ __forceinline__ double d_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float d_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double d_log(double x) { return log(x); }
__device__ __forceinline__ float d_log(float x) { return logf(x); }

__device__ __forceinline__ double d_log1p(double x) { return log1p(x); }
__device__ __forceinline__ float d_log1p(float x) { return log1pf(x); }

// Shape parameter of the kernel: alpha of the rational quadratic, read from
// theta[n_ls + 3] (after the mean constant); 1 (unused) for the others.
template <typename T>
__device__ __forceinline__ T kshape(int kind, const double* theta, int n_ls) {
  return kind == GPK_RATIONAL_QUADRATIC ? (T)theta[n_ls + 3] : T(1);
}

// The Matern-1/2 and rational-quadratic evaluations are out of line: kval and
// kval_dcoef run once per matrix element inside the Gram, adjoint and GEMM
// epilogue loops, and inlined (if-converted) extra branches there would cost
// every kernel kind their exp, log1p and divisions.
template <typename T>
struct KvDc {
  T k, c;
};

template <typename T>
__device__ __noinline__ KvDc<T> kval_dcoef_m12(T sq, T s2) {
  const bool above = sq > Consts<T>::floor_();
  const T t = d_sqrt(above ? sq : Consts<T>::floor_());
  KvDc<T> r;
  r.k = s2 * d_exp(-t);
  r.c = above ? r.k / t : T(0);  // -2 dk/dsq = s2 exp(-t) / t; zero below the floor
  return r;
}

template <typename T>
__device__ __noinline__ KvDc<T> kval_dcoef_rq(T sq, T s2, T ka) {
  const T u = sq / (T(2) * ka);
  KvDc<T> r;
  r.k = s2 * d_exp(-ka * d_log1p(u));
  r.c = r.k / (T(1) + u);  // -2 dk/dsq = s2 (1 + sq / (2 alpha))^-(alpha + 1)
  return r;
}

template <typename T>
__device__ __forceinline__ T kval(int kind, T sq, T s2, T ka = T(1)) {
  if (kind == GPK_RBF) return s2 * d_exp(T(-0.5) * sq);
  if (kind >= GPK_MATERN12)
    return kind == GPK_MATERN12 ? kval_dcoef_m12<T>(sq, s2).k : kval_dcoef_rq<T>(sq, s2, ka).k;
  T t = d_sqrt(sq > Consts<T>::floor_() ? sq : Consts<T>::floor_());
  if (kind == GPK_MATERN32) {
    const T r3 = T(1.7320508075688772);
    return s2 * (T(1) + r3 * t) * d_exp(-r3 * t);
  }
  const T r5 = T(2.23606797749979);
  return s2 * (T(1) + r5 * t + T(5.0 / 3.0) * (t * t)) * d_exp(-r5 * t);
}

// value and derivative coefficient together (one exp)
template <typename T>
__device__ __forceinline__ void kval_dcoef(int kind, T sq, T s2, T& k, T& c, T ka = T(1)) {
  if (kind == GPK_RBF) {
    k = s2 * d_exp(T(-0.5) * sq);
    c = k;
    return;
  }
  if (kind >= GPK_MATERN12) {
    const KvDc<T> r = kind == GPK_MATERN12 ? kval_dcoef_m12<T>(sq, s2) : kval_dcoef_rq<T>(sq, s2, ka);
    k = r.k;
    c = r.c;
    return;
  }
  T t = d_sqrt(sq > Consts<T>::floor_() ? sq : Consts<T>::floor_());
  if (kind == GPK_MATERN32) {
    const T r3 = T(1.7320508075688772);
    T e = s2 * d_exp(-r3 * t);
    k = (T(1) + r3 * t) * e;
    c = T(3) * e;
    return;
  }
  const T r5 = T(2.23606797749979);
  T e = s2 * d_exp(-r5 * t);
  k = (T(1) + r5 * t + T(5.0 / 3.0) * (t * t)) * e;
  c = T(5.0 / 3.0) * (T(1) + r5 * t) * e;
}

// kval_dcoef with the kernel kind fixed at compile time, for loops that
// dispatch on the kind once outside (GEMM epilogues): each kind's loop holds
// only its own arithmetic.
template <int KIND, typename T>
__device__ __forceinline__ void kval_dcoef_k(T sq, T s2, T& k, T& c, T ka = T(1)) {
  if constexpr (KIND == GPK_RBF) {
    k = s2 * d_exp(T(-0.5) * sq);
    c = k;
  } else if constexpr (KIND == GPK_MATERN12) {
    const bool above = sq > Consts<T>::floor_();
    const T t = d_sqrt(above ? sq : Consts<T>::floor_());
    k = s2 * d_exp(-t);
    c = above ? k / t : T(0);
  } else if constexpr (KIND == GPK_RATIONAL_QUADRATIC) {
    const T u = sq / (T(2) * ka);
    k = s2 * d_exp(-ka * d_log1p(u));
    c = k / (T(1) + u);
  } else {
    kval_dcoef<T>(KIND, sq, s2, k, c, ka);  // Matern-3/2, Matern-5/2
  }
}

// Calls f(std::integral_constant<int, KIND>{}) for the runtime kind.
template <typename F>
__device__ __forceinline__ void with_kind(int kind, F&& f) {
  switch (kind) {
    case GPK_RBF: f(std::integral_constant<int, GPK_RBF>{}); break;
    case GPK_MATERN32: f(std::integral_constant<int, GPK_MATERN32>{}); break;
    case GPK_MATERN52: f(std::integral_constant<int, GPK_MATERN52>{}); break;
    case GPK_MATERN12: f(std::integral_constant<int, GPK_MATERN12>{}); break;
    default: f(std::integral_constant<int, GPK_RATIONAL_QUADRATIC>{}); break;
  }
}

// Packed float32 pairs (sm_100 and later): one instruction for two lanes'
// worth of add / sub / mul / fma, each element rounded as its scalar form.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 f2_pack(float a, float b) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float f2_lo(f32x2 v) { return __uint_as_float((unsigned)v); }
__device__ __forceinline__ float f2_hi(f32x2 v) { return __uint_as_float((unsigned)(v >> 32)); }
__device__ __forceinline__ f32x2 f2_add(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 f2_sub(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 f2_mul(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 f2_fma(f32x2 a, f32x2 b, f32x2 c) {
  f32x2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}

// float32 -> TF32 (10 explicit mantissa bits), round to nearest, ties away
// from zero; the result is a float32 bit pattern with the low 13 bits clear.
__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// warp / block reductions
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sums v over the block into *out with one atomicAdd per warp.
__device__ __forceinline__ void block_atomic_add(double* out, double v) {
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, v);
}

__host__ __device__ inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Counts kernel launches made by the library (reported by gpk_launch_count);
// every launch site reads its status through launch_status().
void count_launch();
inline cudaError_t launch_status() {
  count_launch();
  return cudaGetLastError();
}

}  // namespace gpk

#define GPK_CUDA_TRY(...)                                    \
  do {                                                       \
    cudaError_t _e = (__VA_ARGS__);                          \
    if (_e != cudaSuccess) return GPK_ERR_CUDA;              \
  } while (0)

// Programmatic dependent launch.  A kernel launched with the attribute may
// start while its predecessor in the stream is finishing: it does its
// input-independent set-up, then pdl_wait() blocks until the predecessor has
// completed and its writes are visible; pdl_trigger() lets this kernel's own
// successor launch.  Both are no-ops for a kernel launched without it.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
struct PdlAttr {
  cudaLaunchAttribute a[1];
  explicit PdlAttr(bool on) {
    a[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    a[0].val.programmaticStreamSerializationAllowed = on ? 1 : 0;
  }
};

#define GPK_LAUNCH_CHECK()                                   \
  do {                                                       \
    cudaError_t _e = gpk::launch_status();                   \
    if (_e != cudaSuccess) return GPK_ERR_CUDA;              \
  } while (0)
