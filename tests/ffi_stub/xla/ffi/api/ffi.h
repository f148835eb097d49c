// Compile-only stand-in for the XLA FFI header (jaxlib's xla/ffi/api/ffi.h),
// covering the part of its API that gpjax_gb300/ffi/gpk_ffi.cc uses, so that a
// CPU test can type-check the handlers against include/gpk.h where jaxlib is
// not installed.  Nothing here runs.
#pragma once
#include <cstddef>
#include <cstdint>
#include <optional>
#include <string>

namespace xla {
namespace ffi {

enum class ErrorCode { kInvalidArgument, kInternal, kResourceExhausted };

class Error {
 public:
  Error() = default;
  Error(ErrorCode, std::string) {}
  static Error Success() { return Error(); }
  static Error InvalidArgument(std::string) { return Error(); }
  static Error Internal(std::string) { return Error(); }
};

enum DataType { F64, S32 };
template <DataType T> struct Native;
template <> struct Native<F64> { using type = double; };
template <> struct Native<S32> { using type = int32_t; };

struct Dims {
  size_t size() const { return 0; }
  int64_t operator[](size_t) const { return 0; }
};

template <DataType T>
struct Buffer {
  typename Native<T>::type* typed_data() const { return nullptr; }
  Dims dimensions() const { return Dims(); }
  size_t element_count() const { return 0; }
};

template <typename B>
struct Result {
  B* operator->() { return &b; }
  B b;
};
template <DataType T>
using ResultBuffer = Result<Buffer<T>>;

struct ScratchAllocator {
  std::optional<void*> Allocate(size_t, size_t) { return std::nullopt; }
};

template <typename T>
struct PlatformStream {};

struct Binding {
  template <typename T> Binding Ctx() { return *this; }
  template <typename T> Binding Arg() { return *this; }
  template <typename T> Binding Attr(const char*) { return *this; }
  template <typename T> Binding Ret() { return *this; }
};

struct Ffi {
  static Binding Bind() { return Binding(); }
};

}  // namespace ffi
}  // namespace xla

#define XLA_FFI_DEFINE_HANDLER_SYMBOL(name, impl, binding) \
  extern "C" const void* name() {                          \
    (void)(binding);                                       \
    return reinterpret_cast<const void*>(&impl);           \
  }
