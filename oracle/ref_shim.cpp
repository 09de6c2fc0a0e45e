// C-ABI shim over the UNMODIFIED reference headers (test infrastructure only).
//
// Built by oracle/build.py only where the reference tree is present, against
// the project-written BLIS stand-in in oracle/standin/blis.h, into
// oracle/_ref/libt1m_ref.so.  It exposes the reference's internal hot-path
// functions and its public contract() so the oracle restatements (numpy in
// oracle/numpy_oracle.py, C++ in oracle/port/t1m_port.cpp) can be pinned
// against the reference itself.  Nothing of the reference is copied here: this
// file only instantiates its templates.
//
// Reference entry points wrapped:
//   get_index_bundles   include/t1m/t1m.h:90-136
//   get_scatter         include/t1m/t1m.h:141-174
//   get_block_scatter   include/t1m/t1m.h:179-205
//   pack_block          include/t1m/t1m.h:341-404
//   unpack              include/t1m/t1m.h:406-430
//   contract            include/t1m/t1m.h:560-577
#include <array>
#include <complex>
#include <cstring>
#include <span>
#include <string>
#include <vector>

#include "t1m/t1m.h"

namespace {

using t1m::col_major;
using t1m::tensor;
using t1m::internal::index_bundle;

template <class T, std::size_t N>
tensor<T, N> make_tensor(const long* dims, void* data) {
  std::array<std::size_t, N> d{};
  for (std::size_t i = 0; i < N; ++i) d[i] = static_cast<std::size_t>(dims[i]);
  return tensor<T, N>(d, static_cast<T*>(data), col_major);
}

template <std::size_t N>
long scatter_n(const long* dims, const long* strides, int nidx, const long* idx,
               long* out) {
  std::array<std::size_t, N> d{}, s{};
  for (std::size_t i = 0; i < N; ++i) {
    d[i] = static_cast<std::size_t>(dims[i]);
    s[i] = static_cast<std::size_t>(strides[i]);
  }
  std::vector<std::size_t> ind(idx, idx + nidx);
  std::vector<std::size_t> r = t1m::internal::get_scatter<N>(
      ind, std::span<const std::size_t, N>(d), std::span<const std::size_t, N>(s));
  for (std::size_t i = 0; i < r.size(); ++i) out[i] = static_cast<long>(r[i]);
  return static_cast<long>(r.size());
}

index_bundle make_bundle(int nx, const long* X, int ny, const long* Y) {
  index_bundle b;
  for (int i = 0; i < nx; ++i) b.X.push_back(static_cast<std::size_t>(X[i]));
  for (int i = 0; i < ny; ++i) b.Y.push_back(static_cast<std::size_t>(Y[i]));
  return b;
}

// Real scalar of T (the reference's underlying_scalar_t cannot be named for
// real T; its templates deduce U from the destination pointer instead).
template <class T> struct real_of { using type = T; };
template <class R> struct real_of<std::complex<R>> { using type = R; };

template <class T, std::size_t N>
int pack_n(int label, const long* dims, const index_bundle& bundle, long br,
           long bc, long length, const void* src, void* dest) {
  using U = typename real_of<T>::type;
  auto t = make_tensor<T, N>(dims, const_cast<void*>(src));
  t1m::internal::matrix_layout layout(t, bundle, static_cast<std::size_t>(br),
                                      static_cast<std::size_t>(bc));
  auto view = layout.to_view();
  if (label == 0)
    t1m::internal::pack_block<T, t1m::internal::A>(view, length, t.data(),
                                                   static_cast<U*>(dest));
  else
    t1m::internal::pack_block<T, t1m::internal::B>(view, length, t.data(),
                                                   static_cast<U*>(dest));
  return 0;
}

template <class T, std::size_t N>
int unpack_n(const long* dims, const index_bundle& bundle, long br, long bc,
             const void* src, void* dest) {
  using U = typename real_of<T>::type;
  auto t = make_tensor<T, N>(dims, dest);
  t1m::internal::matrix_layout layout(t, bundle, static_cast<std::size_t>(br),
                                      static_cast<std::size_t>(bc));
  t1m::internal::unpack<T>(layout.to_view(), static_cast<const U*>(src),
                           static_cast<T*>(dest));
  return 0;
}

struct ContractArgs {
  const long *da, *db, *dc;
  void *a, *b, *c;
  const char *la, *lb, *lc;
  double alpha, beta;
};

template <class T, std::size_t NA, std::size_t NB, std::size_t NC>
int run_contract(const ContractArgs& x) {
  auto a = make_tensor<T, NA>(x.da, x.a);
  auto b = make_tensor<T, NB>(x.db, x.b);
  auto c = make_tensor<T, NC>(x.dc, x.c);
  if constexpr (t1m::TensorScalarCompound<T>) {
    t1m::contract(a, x.la, b, x.lb, c, x.lc);
  } else {
    t1m::contract(static_cast<T>(x.alpha), a, x.la, b, x.lb,
                  static_cast<T>(x.beta), c, x.lc);
  }
  return 0;
}

template <class T, std::size_t NA, std::size_t NB>
int dispatch_c(int nc, const ContractArgs& x) {
  switch (nc) {
    case 1: return run_contract<T, NA, NB, 1>(x);
    case 2: return run_contract<T, NA, NB, 2>(x);
    case 3: return run_contract<T, NA, NB, 3>(x);
    case 4: return run_contract<T, NA, NB, 4>(x);
  }
  return -1;
}

template <class T, std::size_t NA>
int dispatch_b(int nb, int nc, const ContractArgs& x) {
  switch (nb) {
    case 1: return dispatch_c<T, NA, 1>(nc, x);
    case 2: return dispatch_c<T, NA, 2>(nc, x);
    case 3: return dispatch_c<T, NA, 3>(nc, x);
    case 4: return dispatch_c<T, NA, 4>(nc, x);
  }
  return -1;
}

template <class T>
int dispatch_a(int na, int nb, int nc, const ContractArgs& x) {
  switch (na) {
    case 1: return dispatch_b<T, 1>(nb, nc, x);
    case 2: return dispatch_b<T, 2>(nb, nc, x);
    case 3: return dispatch_b<T, 3>(nb, nc, x);
    case 4: return dispatch_b<T, 4>(nb, nc, x);
  }
  return -1;
}

}  // namespace

extern "C" {

// Bundles as six position lists (A.X, A.Y, B.X, B.Y, C.X, C.Y), each written
// to out + 16*i with its length in counts[i].
int t1mref_index_bundles(const char* la, const char* lb, const char* lc,
                         long* out, int* counts) {
  auto [A, B, C] = t1m::internal::get_index_bundles(la, lb, lc);
  const std::vector<std::size_t>* v[6] = {&A.X, &A.Y, &B.X, &B.Y, &C.X, &C.Y};
  for (int i = 0; i < 6; ++i) {
    counts[i] = static_cast<int>(v[i]->size());
    for (std::size_t j = 0; j < v[i]->size(); ++j)
      out[16 * i + j] = static_cast<long>((*v[i])[j]);
  }
  return 0;
}

long t1mref_scatter(int ndim, const long* dims, const long* strides, int nidx,
                    const long* idx, long* out) {
  switch (ndim) {
    case 1: return scatter_n<1>(dims, strides, nidx, idx, out);
    case 2: return scatter_n<2>(dims, strides, nidx, idx, out);
    case 3: return scatter_n<3>(dims, strides, nidx, idx, out);
    case 4: return scatter_n<4>(dims, strides, nidx, idx, out);
    case 5: return scatter_n<5>(dims, strides, nidx, idx, out);
    case 6: return scatter_n<6>(dims, strides, nidx, idx, out);
  }
  return -1;
}

long t1mref_block_scatter(const long* scat, long n, long b, long* out) {
  std::vector<std::size_t> s(scat, scat + n);
  std::vector<std::size_t> r =
      t1m::internal::get_block_scatter(s, static_cast<std::size_t>(b));
  for (std::size_t i = 0; i < r.size(); ++i) out[i] = static_cast<long>(r[i]);
  return static_cast<long>(r.size());
}

// dtype: 0 float, 2 complex<float>.  label: 0 = A (column slivers), 1 = B.
int t1mref_pack_block(int dtype, int label, int ndim, const long* dims, int nx,
                      const long* X, int ny, const long* Y, long br, long bc,
                      long length, const void* src, void* dest) {
  const index_bundle bundle = make_bundle(nx, X, ny, Y);
#define T1MREF_PACK(T)                                                         \
  switch (ndim) {                                                              \
    case 2: return pack_n<T, 2>(label, dims, bundle, br, bc, length, src, dest); \
    case 3: return pack_n<T, 3>(label, dims, bundle, br, bc, length, src, dest); \
    case 4: return pack_n<T, 4>(label, dims, bundle, br, bc, length, src, dest); \
  }
  if (dtype == 0) { T1MREF_PACK(float) }
  if (dtype == 2) { T1MREF_PACK(std::complex<float>) }
#undef T1MREF_PACK
  return -1;
}

int t1mref_unpack(int dtype, int ndim, const long* dims, int nx, const long* X,
                  int ny, const long* Y, long br, long bc, const void* src,
                  void* dest) {
  const index_bundle bundle = make_bundle(nx, X, ny, Y);
#define T1MREF_UNPACK(T)                                               \
  switch (ndim) {                                                      \
    case 2: return unpack_n<T, 2>(dims, bundle, br, bc, src, dest);    \
    case 3: return unpack_n<T, 3>(dims, bundle, br, bc, src, dest);    \
    case 4: return unpack_n<T, 4>(dims, bundle, br, bc, src, dest);    \
  }
  if (dtype == 0) { T1MREF_UNPACK(float) }
  if (dtype == 2) { T1MREF_UNPACK(std::complex<float>) }
#undef T1MREF_UNPACK
  return -1;
}

// dtype: 0 float, 1 double, 2 complex<float>, 3 complex<double>.  All tensors
// are column-major (the only layout the reference implements, t1m.h:44-53).
// Real types take alpha/beta; the complex overload has neither (t1m.h:570-577).
int t1mref_contract(int dtype, int na, const long* da, void* a, const char* la,
                    int nb, const long* db, void* b, const char* lb, int nc,
                    const long* dc, void* c, const char* lc, double alpha,
                    double beta) {
  ContractArgs x{da, db, dc, a, b, c, la, lb, lc, alpha, beta};
  switch (dtype) {
    case 0: return dispatch_a<float>(na, nb, nc, x);
    case 1: return dispatch_a<double>(na, nb, nc, x);
    case 2: return dispatch_a<std::complex<float>>(na, nb, nc, x);
    case 3: return dispatch_a<std::complex<double>>(na, nb, nc, x);
  }
  return -1;
}

}  // extern "C"
