// Compile-time stand-in for the XLA FFI header, for checking vivsim_gb300/xla/vs_xla_ffi.cc
// where jaxlib (which ships the real header) is not installed.  Test infrastructure only.
//
// It declares just the names the handlers use (buffers, results, errors, the CUDA stream and
// scratch-allocator contexts, span attributes and the binding builder) and adds one check of
// its own: XLA_FFI_DEFINE_HANDLER_SYMBOL static_asserts that the handler's parameter list is
// exactly the list the binding describes (context, then arguments, results and attributes in
// binding order; a Ret<T> is a Result<T> parameter).  Nothing here runs.
#pragma once

#include <cstddef>
#include <cstdint>
#include <optional>
#include <string>
#include <type_traits>

namespace xla::ffi {

enum class ErrorCode { kOk, kInternal, kInvalidArgument, kResourceExhausted };

class Error {
 public:
  Error() = default;
  Error(ErrorCode code, std::string message) : code_(code), message_(std::move(message)) {}
  static Error Success() { return Error(); }
  ErrorCode code() const { return code_; }

 private:
  ErrorCode code_ = ErrorCode::kOk;
  std::string message_;
};

enum class DataType : uint8_t { INVALID, PRED, S8, S16, S32, S64, U8, U16, U32, U64, F16, F32, F64 };
inline constexpr DataType PRED = DataType::PRED;
inline constexpr DataType S8 = DataType::S8;
inline constexpr DataType S32 = DataType::S32;
inline constexpr DataType U8 = DataType::U8;
inline constexpr DataType F32 = DataType::F32;
inline constexpr DataType F64 = DataType::F64;

template <typename T>
class Span {
 public:
  Span(T* data, size_t size) : data_(data), size_(size) {}
  size_t size() const { return size_; }
  T* begin() const { return data_; }
  T* end() const { return data_ + size_; }
  T& operator[](size_t i) const { return data_[i]; }

 private:
  T* data_;
  size_t size_;
};

class AnyBuffer {
 public:
  DataType element_type() const { return type_; }
  Span<const int64_t> dimensions() const { return Span<const int64_t>(dims_, rank_); }
  void* untyped_data() const { return data_; }
  size_t element_count() const { return count_; }
  size_t size_bytes() const { return bytes_; }

 private:
  DataType type_ = DataType::INVALID;
  const int64_t* dims_ = nullptr;
  size_t rank_ = 0, count_ = 0, bytes_ = 0;
  void* data_ = nullptr;
};

template <typename T>
class Result {
 public:
  T* operator->() const { return value_; }
  T& operator*() const { return *value_; }

 private:
  T* value_ = nullptr;
};

template <typename T>
struct PlatformStream {};

class ScratchAllocator {
 public:
  std::optional<void*> Allocate(size_t, size_t = 1) { return std::nullopt; }
};

// ---- binding builder: each step appends the handler parameter type it stands for
template <typename T>
struct CtxParam;
template <typename S>
struct CtxParam<PlatformStream<S>> {
  using type = S;
};
template <>
struct CtxParam<ScratchAllocator> {
  using type = ScratchAllocator;
};

template <typename... Params>
struct Binding {
  template <typename C>
  constexpr Binding<Params..., typename CtxParam<C>::type> Ctx() const {
    return {};
  }
  template <typename A>
  constexpr Binding<Params..., A> Arg() const {
    return {};
  }
  template <typename R>
  constexpr Binding<Params..., Result<R>> Ret() const {
    return {};
  }
  template <typename A>
  constexpr Binding<Params..., A> Attr(const char*) const {
    return {};
  }
};

struct Ffi {
  static constexpr Binding<> Bind() { return {}; }
};

template <typename Fn, typename... Params>
constexpr bool handler_matches(Fn*, Binding<Params...>) {
  return std::is_same_v<Fn, Error(Params...)>;
}

}  // namespace xla::ffi

#define XLA_FFI_DEFINE_HANDLER_SYMBOL(name, fn, binding)                                             \
  static_assert(::xla::ffi::handler_matches(&fn, binding),                                          \
                "handler " #fn ": parameters differ from the binding of " #name);                    \
  extern "C" int name(void*) { return 0; }
