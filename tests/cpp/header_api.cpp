// Exercises the drop-in C++ API (include/t1m/t1m.h) the way the reference's
// example and tests use theirs (example/example.cpp, test/test_contraction.cpp):
// tensor views over caller-owned memory and t1m::contract by label strings.
// Exit status 0 = all checks passed.
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "t1m/t1m.h"

namespace {

template <class T> T rnd(unsigned& s) {
  s = s * 1664525u + 1013904223u;
  return static_cast<T>((s >> 8) * (1.0 / 16777216.0) * 2.0 - 1.0);
}

int fails = 0;
void expect(bool ok, const char* what) {
  if (!ok) {
    std::printf("FAIL: %s\n", what);
    ++fails;
  }
}

}  // namespace

int main() {
  unsigned seed = 7;
  // The reference's example: abc,bd->acd, extents 10, complex<float>, col-major.
  constexpr std::size_t d = 10;
  std::vector<std::complex<float>> A(d * d * d), B(d * d), C(d * d * d, {1.0f, -1.0f});
  for (auto& x : A) x = {rnd<float>(seed), rnd<float>(seed)};
  for (auto& x : B) x = {rnd<float>(seed), rnd<float>(seed)};
  const std::vector<std::complex<float>> C0 = C;
  t1m::tensor<std::complex<float>, 3> a({d, d, d}, A.data());
  t1m::tensor<std::complex<float>, 2> b({d, d}, B.data());
  t1m::tensor<std::complex<float>, 3> c({d, d, d}, C.data());
  t1m::contract(a, "abc", b, "bd", c, "acd");
  double err = 0, ref_max = 0;
  for (std::size_t ia = 0; ia < d; ++ia)
    for (std::size_t ic = 0; ic < d; ++ic)
      for (std::size_t id = 0; id < d; ++id) {
        std::complex<double> s = C0[ia + d * ic + d * d * id];
        for (std::size_t ib = 0; ib < d; ++ib)
          s += std::complex<double>(A[ia + d * ib + d * d * ic]) *
               std::complex<double>(B[ib + d * id]);
        const std::complex<double> got = C[ia + d * ic + d * d * id];
        err = std::max(err, std::abs(got - s));
        ref_max = std::max(ref_max, std::abs(s));
      }
  expect(err / ref_max < 1e-5, "complex<float> abc,bd->acd (C += A*B)");

  // Real overload: C += alpha*A*B, beta ignored (reference semantics), row-major.
  std::vector<double> RA(4 * 5), RB(5 * 3), RC(4 * 3, 2.0);
  for (auto& x : RA) x = rnd<double>(seed);
  for (auto& x : RB) x = rnd<double>(seed);
  t1m::tensor<double, 2> ra({4, 5}, RA.data(), t1m::row_major);
  t1m::tensor<double, 2> rb({5, 3}, RB.data(), t1m::row_major);
  t1m::tensor<double, 2> rc({4, 3}, RC.data(), t1m::row_major);
  t1m::contract(0.5, ra, "ik", rb, "kj", 123.0, rc, "ij");
  double rerr = 0;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 2.0;
      for (int k = 0; k < 5; ++k) s += 0.5 * RA[i * 5 + k] * RB[k * 3 + j];
      rerr = std::max(rerr, std::abs(s - RC[i * 3 + j]));
    }
  expect(rerr < 1e-12, "double row-major ik,kj->ij (beta ignored)");

  // Label errors throw std::invalid_argument.
  bool threw = false;
  try {
    t1m::contract(a, "abb", b, "bd", c, "acd");
  } catch (const std::invalid_argument&) {
    threw = true;
  }
  expect(threw, "repeated label throws invalid_argument");

  // BLAS-semantics extension with complex alpha/beta.
  std::vector<std::complex<double>> ZA(6 * 7), ZB(7 * 8), ZC(6 * 8, {0.5, 0.25});
  for (auto& x : ZA) x = {rnd<double>(seed), rnd<double>(seed)};
  for (auto& x : ZB) x = {rnd<double>(seed), rnd<double>(seed)};
  const auto ZC0 = ZC;
  t1m::tensor<std::complex<double>, 2> za({6, 7}, ZA.data());
  t1m::tensor<std::complex<double>, 2> zb({7, 8}, ZB.data());
  t1m::tensor<std::complex<double>, 2> zc({6, 8}, ZC.data());
  const std::complex<double> alpha(1.0, 0.5), beta(0.25, 0.0);
  t1m::contract_scaled(alpha, za, "ik", zb, "kj", beta, zc, "ij");
  double zerr = 0;
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 8; ++j) {
      std::complex<double> s = 0;
      for (int k = 0; k < 7; ++k) s += ZA[i + 6 * k] * ZB[k + 7 * j];
      zerr = std::max(zerr, std::abs(alpha * s + beta * ZC0[i + 6 * j] - ZC[i + 6 * j]));
    }
  expect(zerr < 1e-12, "complex<double> contract_scaled");

  // Adjoint of C = A*B: dA[i,k] = sum_j dC[i,j] conj(B[k,j]),
  // dB[k,j] = sum_i conj(A[i,k]) dC[i,j].
  std::vector<std::complex<double>> DC(6 * 8), DA(6 * 7), DB(7 * 8);
  for (auto& x : DC) x = {rnd<double>(seed), rnd<double>(seed)};
  t1m::tensor<std::complex<double>, 2> dc({6, 8}, DC.data());
  t1m::tensor<std::complex<double>, 2> da({6, 7}, DA.data());
  t1m::tensor<std::complex<double>, 2> db({7, 8}, DB.data());
  t1m::contract_vjp(dc, "ij", za, "ik", zb, "kj", &da, &db);
  double verr = 0;
  for (int i = 0; i < 6; ++i)
    for (int k = 0; k < 7; ++k) {
      std::complex<double> s = 0;
      for (int j = 0; j < 8; ++j) s += DC[i + 6 * j] * std::conj(ZB[k + 7 * j]);
      verr = std::max(verr, std::abs(s - DA[i + 6 * k]));
    }
  for (int k = 0; k < 7; ++k)
    for (int j = 0; j < 8; ++j) {
      std::complex<double> s = 0;
      for (int i = 0; i < 6; ++i) s += std::conj(ZA[i + 6 * k]) * DC[i + 6 * j];
      verr = std::max(verr, std::abs(s - DB[k + 7 * j]));
    }
  expect(verr < 1e-12, "complex<double> contract_vjp (dA, dB)");

  std::printf("%s\n", fails ? "header api FAILED" : "header api ok");
  return fails ? 1 : 0;
}
