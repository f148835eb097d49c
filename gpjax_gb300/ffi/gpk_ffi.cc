// XLA FFI custom-call handlers over the gpk C ABI, for JAX callers.
//
// Each handler unpacks the XLA buffers and attributes, takes its workspace
// from XLA's scratch allocator (the library itself never allocates), calls
// the C entry point on XLA's CUDA stream and turns a non-zero gpk_status into
// an FFI error.  gpjax_gb300/jax_ffi.py registers them with
// jax.ffi.register_ffi_target and wraps the objectives in jax.custom_vjp.
// Built only where jaxlib's headers exist (jax.ffi.include_dir()).
//
// Handlers, with the reference functions they stand in for:
//   GpkConjugateMll   gpjax/objectives.py:36-107 (value and theta gradient)
//   GpkCollapsedElbo  gpjax/objectives.py:321-416 (value, theta and Z gradients)
//   GpkPredict        gpjax/gps.py:443-526 (predictive mean and variance)
#include <cstdint>
#include <optional>

#include <cuda_runtime.h>

#include "gpk.h"
#include "xla/ffi/api/ffi.h"

namespace ffi = xla::ffi;

namespace {

ffi::Error status_error(const char* fn, int st) {
  if (st == GPK_OK) return ffi::Error::Success();
  return ffi::Error(ffi::ErrorCode::kInternal,
                    std::string(fn) + " failed: " + gpk_status_string(st));
}

// x [n, d] row-major; y [n] or [n, 1]; theta [n_ls + 3] (+ alpha for the
// rational quadratic).  Outputs: mll [], grad [theta size], info [].
ffi::Error ConjugateMllImpl(cudaStream_t stream, ffi::ScratchAllocator scratch,
                            ffi::Buffer<ffi::F64> x, ffi::Buffer<ffi::F64> y,
                            ffi::Buffer<ffi::F64> theta, int32_t kind, int32_t n_ls,
                            double jitter, int32_t precision, int32_t want_grad,
                            ffi::ResultBuffer<ffi::F64> mll, ffi::ResultBuffer<ffi::F64> grad,
                            ffi::ResultBuffer<ffi::S32> info) {
  const auto dx = x.dimensions();
  if (dx.size() != 2) return ffi::Error::InvalidArgument("x must be [n, d]");
  const int64_t n = dx[0];
  const int d = static_cast<int>(dx[1]);
  if (static_cast<int64_t>(y.element_count()) != n)
    return ffi::Error::InvalidArgument("y must hold n values");
  if (static_cast<int64_t>(grad->element_count()) < n_ls + 3)
    return ffi::Error::InvalidArgument("grad must hold n_ls + 3 values");
  const size_t bytes = gpk_conjugate_mll_workspace_bytes(n, d, precision);
  std::optional<void*> ws = scratch.Allocate(bytes, 256);
  if (!ws.has_value()) return ffi::Error(ffi::ErrorCode::kResourceExhausted, "gpk workspace");
  return status_error("gpk_conjugate_mll",
                      gpk_conjugate_mll(kind, n, d, x.typed_data(), d, y.typed_data(),
                                        theta.typed_data(), n_ls, jitter, precision, want_grad,
                                        mll->typed_data(), grad->typed_data(),
                                        info->typed_data(), *ws, bytes, stream));
}

// x [n, d], y [n], z [m, d], theta; outputs elbo [], grad [theta size],
// grad_z [m, d], info [].
ffi::Error CollapsedElboImpl(cudaStream_t stream, ffi::ScratchAllocator scratch,
                             ffi::Buffer<ffi::F64> x, ffi::Buffer<ffi::F64> y,
                             ffi::Buffer<ffi::F64> z, ffi::Buffer<ffi::F64> theta, int32_t kind,
                             int32_t n_ls, double jitter, int32_t precision, int32_t want_grad,
                             ffi::ResultBuffer<ffi::F64> elbo, ffi::ResultBuffer<ffi::F64> grad,
                             ffi::ResultBuffer<ffi::F64> grad_z,
                             ffi::ResultBuffer<ffi::S32> info) {
  const auto dx = x.dimensions(), dz = z.dimensions();
  if (dx.size() != 2 || dz.size() != 2 || dz[1] != dx[1])
    return ffi::Error::InvalidArgument("x must be [n, d] and z [m, d]");
  const int64_t n = dx[0], m = dz[0];
  const int d = static_cast<int>(dx[1]);
  const size_t bytes = gpk_collapsed_elbo_workspace_bytes(n, m, d, precision);
  std::optional<void*> ws = scratch.Allocate(bytes, 256);
  if (!ws.has_value()) return ffi::Error(ffi::ErrorCode::kResourceExhausted, "gpk workspace");
  return status_error(
      "gpk_collapsed_elbo",
      gpk_collapsed_elbo(kind, n, m, d, x.typed_data(), d, y.typed_data(), z.typed_data(), d,
                         theta.typed_data(), n_ls, jitter, precision, want_grad,
                         elbo->typed_data(), grad->typed_data(), grad_z->typed_data(),
                         info->typed_data(), *ws, bytes, stream));
}

// x [n, d], y [n], xt [t, d], theta; outputs mean [t], var [t], info [].
ffi::Error PredictImpl(cudaStream_t stream, ffi::ScratchAllocator scratch,
                       ffi::Buffer<ffi::F64> x, ffi::Buffer<ffi::F64> y,
                       ffi::Buffer<ffi::F64> xt, ffi::Buffer<ffi::F64> theta, int32_t kind,
                       int32_t n_ls, double jitter, double prior_jitter, int32_t precision,
                       ffi::ResultBuffer<ffi::F64> mean, ffi::ResultBuffer<ffi::F64> var,
                       ffi::ResultBuffer<ffi::S32> info) {
  const auto dx = x.dimensions(), dt = xt.dimensions();
  if (dx.size() != 2 || dt.size() != 2 || dt[1] != dx[1])
    return ffi::Error::InvalidArgument("x must be [n, d] and xt [t, d]");
  const int64_t n = dx[0], t = dt[0];
  const int d = static_cast<int>(dx[1]);
  const size_t bytes = gpk_predict_workspace_bytes(n, t, d, precision);
  std::optional<void*> ws = scratch.Allocate(bytes, 256);
  if (!ws.has_value()) return ffi::Error(ffi::ErrorCode::kResourceExhausted, "gpk workspace");
  return status_error("gpk_predict",
                      gpk_predict(kind, n, t, d, x.typed_data(), d, y.typed_data(),
                                  xt.typed_data(), d, theta.typed_data(), n_ls, jitter,
                                  prior_jitter, precision, mean->typed_data(),
                                  var->typed_data(), nullptr, 0, info->typed_data(), *ws, bytes,
                                  stream));
}

}  // namespace

XLA_FFI_DEFINE_HANDLER_SYMBOL(GpkConjugateMll, ConjugateMllImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Ctx<ffi::ScratchAllocator>()
                                  .Arg<ffi::Buffer<ffi::F64>>()  // x
                                  .Arg<ffi::Buffer<ffi::F64>>()  // y
                                  .Arg<ffi::Buffer<ffi::F64>>()  // theta
                                  .Attr<int32_t>("kind")
                                  .Attr<int32_t>("n_ls")
                                  .Attr<double>("jitter")
                                  .Attr<int32_t>("precision")
                                  .Attr<int32_t>("want_grad")
                                  .Ret<ffi::Buffer<ffi::F64>>()   // mll
                                  .Ret<ffi::Buffer<ffi::F64>>()   // grad
                                  .Ret<ffi::Buffer<ffi::S32>>());  // info

XLA_FFI_DEFINE_HANDLER_SYMBOL(GpkCollapsedElbo, CollapsedElboImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Ctx<ffi::ScratchAllocator>()
                                  .Arg<ffi::Buffer<ffi::F64>>()  // x
                                  .Arg<ffi::Buffer<ffi::F64>>()  // y
                                  .Arg<ffi::Buffer<ffi::F64>>()  // z
                                  .Arg<ffi::Buffer<ffi::F64>>()  // theta
                                  .Attr<int32_t>("kind")
                                  .Attr<int32_t>("n_ls")
                                  .Attr<double>("jitter")
                                  .Attr<int32_t>("precision")
                                  .Attr<int32_t>("want_grad")
                                  .Ret<ffi::Buffer<ffi::F64>>()   // elbo
                                  .Ret<ffi::Buffer<ffi::F64>>()   // grad
                                  .Ret<ffi::Buffer<ffi::F64>>()   // grad_z
                                  .Ret<ffi::Buffer<ffi::S32>>());  // info

XLA_FFI_DEFINE_HANDLER_SYMBOL(GpkPredict, PredictImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Ctx<ffi::ScratchAllocator>()
                                  .Arg<ffi::Buffer<ffi::F64>>()  // x
                                  .Arg<ffi::Buffer<ffi::F64>>()  // y
                                  .Arg<ffi::Buffer<ffi::F64>>()  // xt
                                  .Arg<ffi::Buffer<ffi::F64>>()  // theta
                                  .Attr<int32_t>("kind")
                                  .Attr<int32_t>("n_ls")
                                  .Attr<double>("jitter")
                                  .Attr<double>("prior_jitter")
                                  .Attr<int32_t>("precision")
                                  .Ret<ffi::Buffer<ffi::F64>>()   // mean
                                  .Ret<ffi::Buffer<ffi::F64>>()   // var
                                  .Ret<ffi::Buffer<ffi::S32>>());  // info
