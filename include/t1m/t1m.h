// t1m.h — drop-in C++ API of the GB300 contraction engine.
//
// Same names, template parameters and call signatures as the reference's
// header (MatthiasReumann/t1m include/t1m/t1m.h):
//   TensorScalar concepts            t1m.h:15-27
//   memory_layout {row_major, col_major}   t1m.h:29
//   tensor<T, ndim>(dims, data, layout)    t1m.h:31-66
//   contract(alpha, a, la, b, lb, beta, c, lc[, ctx])  real    t1m.h:560-568
//   contract(a, la, b, lb, c, lc[, ctx])               complex t1m.h:570-577
// with the reference's semantics C <- C + alpha*A*B (beta ignored; alpha = 1
// for the complex overload).  Differences a user sees:
//   * the trailing BLIS `const cntx_t*` becomes `t1m::context*` (device,
//     stream, method); the default is a per-thread context on device 0;
//   * row_major is implemented (the reference leaves its strides
//     uninitialised, t1m.h:51-52);
//   * the data pointer may be host memory (staged to the GPU and back) or
//     device memory (used in place, asynchronous on the context's stream);
//   * errors throw: std::bad_alloc (allocation, as in the reference),
//     std::invalid_argument (labels/extents), std::runtime_error (CUDA).
// Extensions without a reference counterpart: contract_scaled (complex
// alpha/beta, BLAS semantics), contract_vjp (adjoint), and the method switch.
//
// Everything forwards to the C-ABI in t1m_capi.h (libt1m_cuda.so).
#pragma once

#include <array>
#include <complex>
#include <cstddef>
#include <cstdint>
#include <new>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "../t1m_capi.h"

namespace t1m {

template <typename T>
concept TensorScalarArithmetic = std::is_same_v<T, float> || std::is_same_v<T, double>;

template <typename T>
concept TensorScalarCompound =
    std::is_same_v<T, std::complex<float>> || std::is_same_v<T, std::complex<double>>;

template <typename T>
concept TensorScalar = TensorScalarArithmetic<T> || TensorScalarCompound<T>;

namespace detail {
template <class T> struct real_of { using type = T; };
template <class R> struct real_of<std::complex<R>> { using type = R; };
template <class T> constexpr int dtype_of() {
  if constexpr (std::is_same_v<T, float>) return T1M_FLOAT32;
  else if constexpr (std::is_same_v<T, double>) return T1M_FLOAT64;
  else if constexpr (std::is_same_v<T, std::complex<float>>) return T1M_COMPLEX64;
  else return T1M_COMPLEX128;
}
}  // namespace detail

template <typename T>
using underlying_scalar_t = typename detail::real_of<T>::type;

enum memory_layout : std::uint8_t { row_major, col_major };

/// Non-owning view of a dense tensor (t1m.h:31-66).
template <TensorScalar T, std::size_t ndim> class tensor {
 public:
  using dim_array = std::array<std::size_t, ndim>;
  using stride_array = std::array<std::size_t, ndim>;

  explicit tensor(const dim_array& dims, T* data, memory_layout layout = col_major)
      : data_(data), layout_{layout}, dims_(dims) {}

  [[nodiscard]] constexpr std::size_t rank() const noexcept { return ndim; }
  [[nodiscard]] constexpr dim_array dims() const noexcept { return dims_; }
  /// Element strides; col_major: s0 = 1, si = s(i-1)*d(i-1); row_major:
  /// the last mode is unit stride.
  [[nodiscard]] constexpr stride_array strides() const {
    stride_array s{};
    std::size_t acc = 1;
    if (layout_ == col_major) {
      for (std::size_t i = 0; i < ndim; ++i) { s[i] = acc; acc *= dims_[i]; }
    } else {
      for (std::size_t i = ndim; i-- > 0;) { s[i] = acc; acc *= dims_[i]; }
    }
    return s;
  }
  [[nodiscard]] T* data() noexcept { return data_; }
  [[nodiscard]] const T* data() const noexcept { return data_; }
  [[nodiscard]] constexpr memory_layout layout() const noexcept { return layout_; }

 private:
  T* data_;
  memory_layout layout_;
  std::array<std::size_t, ndim> dims_;
};

/// Replaces the reference's BLIS `cntx_t*`: device, stream and method.
class context {
 public:
  explicit context(int device = 0) {
    const int st = t1m_create(&h_, device);
    if (st != T1M_OK) throw std::runtime_error(std::string("t1m_create: ") + t1m_status_string(st));
  }
  ~context() { if (h_) t1m_destroy(h_); }
  context(const context&) = delete;
  context& operator=(const context&) = delete;

  void set_method(t1m_method m) { check(t1m_set_method(h_, m)); }
  /// Number of K partitions (0 = automatic).
  void set_split_k(int splits) { check(t1m_set_split_k(h_, splits)); }
  /// Cap on each optional tensor-core workspace in bytes (-1 = none, 0 = off).
  void set_workspace_limit(int64_t bytes) { check(t1m_set_workspace_limit(h_, bytes)); }
  /// Tile form of tensor-core products (T1M_TILE_AUTO / _ONE / _PAIR).
  void set_tile_form(int form) { check(t1m_set_tile_form(h_, form)); }
  /// Bound on grouped launches' dependency waits in microseconds (0 = default).
  void set_wait_limit(int64_t us) { check(t1m_set_wait_limit(h_, us)); }
  /// Tune single tensor-core contractions per shape class (cached).
  void set_autotune(bool on) { check(t1m_set_autotune(h_, on ? 1 : 0)); }
  /// Run on a caller-owned cudaStream_t (nullptr = the context's own stream).
  void set_stream(void* stream) { check(t1m_set_stream(h_, stream)); }
  void synchronize() { check(t1m_synchronize(h_)); }
  [[nodiscard]] t1m_context* handle() const noexcept { return h_; }

  void check(int st) const {
    if (st == T1M_OK) return;
    const std::string msg = std::string(t1m_status_string(st)) + ": " + t1m_last_error(h_);
    if (st == T1M_ERR_ALLOC) throw std::bad_alloc();
    if (st == T1M_ERR_LABELS || st == T1M_ERR_INVALID_ARGUMENT) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
  }

 private:
  t1m_context* h_ = nullptr;
};

/// The calling thread's context on device 0.
inline context* default_context() {
  thread_local context ctx(0);
  return &ctx;
}

namespace detail {
template <class T, std::size_t N>
struct view {
  std::array<int64_t, (N > 0 ? N : 1)> ext{};
  t1m_tensor t{};
  explicit view(const tensor<T, N>& x) {
    const auto d = x.dims();
    for (std::size_t i = 0; i < N; ++i) ext[i] = static_cast<int64_t>(d[i]);
    t.ndim = static_cast<int32_t>(N);
    t.layout = x.layout() == col_major ? T1M_COL_MAJOR : T1M_ROW_MAJOR;
    t.extents = ext.data();
    t.strides = nullptr;
    t.data = const_cast<T*>(x.data());
  }
};

template <class T, std::size_t NA, std::size_t NB, std::size_t NC>
void run(context* ctx, T alpha, const tensor<T, NA>& a, const std::string& la,
         const tensor<T, NB>& b, const std::string& lb, T beta, tensor<T, NC>& c,
         const std::string& lc, uint32_t flags) {
  view<T, NA> va(a);
  view<T, NB> vb(b);
  view<T, NC> vc(c);
  ctx->check(t1m_contract(ctx->handle(), dtype_of<T>(), &alpha, &va.t, la.c_str(), &vb.t,
                          lb.c_str(), &beta, &vc.t, lc.c_str(), flags, nullptr));
}
}  // namespace detail

/// Real contraction, reference semantics C <- C + alpha*A*B (t1m.h:560-568).
template <TensorScalarArithmetic T, std::size_t ndim_a, std::size_t ndim_b, std::size_t ndim_c>
void contract(const T alpha, const tensor<T, ndim_a>& a, const std::string& labels_a,
              const tensor<T, ndim_b>& b, const std::string& labels_b, const T beta,
              tensor<T, ndim_c>& c, const std::string& labels_c,
              context* ctx = default_context()) {
  detail::run(ctx, alpha, a, labels_a, b, labels_b, beta, c, labels_c, T1M_FLAG_ACCUMULATE);
}

/// Complex contraction, reference semantics C <- C + A*B (t1m.h:570-577).
template <TensorScalarCompound T, std::size_t ndim_a, std::size_t ndim_b, std::size_t ndim_c>
void contract(const tensor<T, ndim_a>& a, const std::string& labels_a,
              const tensor<T, ndim_b>& b, const std::string& labels_b, tensor<T, ndim_c>& c,
              const std::string& labels_c, context* ctx = default_context()) {
  detail::run(ctx, T(1), a, labels_a, b, labels_b, T(0), c, labels_c, T1M_FLAG_ACCUMULATE);
}

/// C <- alpha*A*B + beta*C for any TensorScalar, complex alpha/beta allowed
/// (no reference counterpart).  beta == 0 does not read C.
template <TensorScalar T, std::size_t ndim_a, std::size_t ndim_b, std::size_t ndim_c>
void contract_scaled(const T alpha, const tensor<T, ndim_a>& a, const std::string& labels_a,
                     const tensor<T, ndim_b>& b, const std::string& labels_b, const T beta,
                     tensor<T, ndim_c>& c, const std::string& labels_c,
                     context* ctx = default_context()) {
  detail::run(ctx, alpha, a, labels_a, b, labels_b, beta, c, labels_c, 0u);
}

/// Adjoint of C = A*B (no reference counterpart): dA = dC * conj(B) and
/// dB = conj(A) * dC in the conjugate-Wirtinger convention (for real T, plain
/// transposed products).  dA / dB are overwritten; either may be null.
/// Forwards to t1m_contract_vjp.
template <TensorScalar T, std::size_t ndim_a, std::size_t ndim_b, std::size_t ndim_c>
void contract_vjp(const tensor<T, ndim_c>& dc, const std::string& labels_c,
                  const tensor<T, ndim_a>& a, const std::string& labels_a,
                  const tensor<T, ndim_b>& b, const std::string& labels_b,
                  tensor<T, ndim_a>* da, tensor<T, ndim_b>* db,
                  context* ctx = default_context()) {
  detail::view<T, ndim_c> vdc(dc);
  detail::view<T, ndim_a> va(a);
  detail::view<T, ndim_b> vb(b);
  if (da) {
    detail::view<T, ndim_a> vda(*da);
    ctx->check(t1m_contract_vjp(ctx->handle(), detail::dtype_of<T>(), &vdc.t, labels_c.c_str(),
                                &va.t, labels_a.c_str(), &vb.t, labels_b.c_str(), &vda.t, nullptr,
                                0u, nullptr));
  }
  if (db) {
    detail::view<T, ndim_b> vdb(*db);
    ctx->check(t1m_contract_vjp(ctx->handle(), detail::dtype_of<T>(), &vdc.t, labels_c.c_str(),
                                &va.t, labels_a.c_str(), &vb.t, labels_b.c_str(), nullptr, &vdb.t,
                                0u, nullptr));
  }
}

}  // namespace t1m
