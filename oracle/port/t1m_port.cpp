// t1m_port: CPU restatement of the reference's contraction algorithm.
//
// TEST INFRASTRUCTURE ONLY.  This is the oracle: the tests, the smoke check
// and the CPU-baseline leg of bench.py call it to check and to time against.
// The product path (libt1m_cuda.so) never links or calls it.
//
// It restates, with dynamic rank and arbitrary element strides, the
// block-scatter + five-loop + 1M algorithm of include/t1m/t1m.h:
//   index bundles            t1m.h:90-136   (sorted labels; contracted = A n B)
//   scatter vectors          t1m.h:141-174  (first bundle mode varies fastest)
//   five loops jc/pc/ic/jr/ir t1m.h:466-507 (real) and t1m.h:508-554 (1M)
//   1M A packing [re -im; im re], 1M B packing re/im rows   t1m.h:309-337
//   micro-tile into a zeroed buffer, then C += tile         t1m.h:543-548
// with the block sizes and micro-kernel of the BLIS stand-in
// (oracle/standin/blis.h).  Packing is a pure gather, so the packed panels are
// the same values the reference packs; the micro-kernel and the per-KC-chunk
// "C += tile" order are the same, so results agree bit for bit with the
// reference built against the same stand-in (pinned by tests/test_oracle.py).
//
// Semantics follow the reference exactly: C <- C + alpha*A*B for real types
// (beta only multiplies the zeroed scratch tile, t1m.h:497-502), and
// C <- C + A*B for complex types (t1m.h:570-577).
//
// Extra over the reference: nthreads > 1 splits N into disjoint column slabs,
// one per thread (each C element is still produced by exactly the same
// arithmetic, so the bits do not depend on the thread count).
#include <algorithm>
#include <complex>
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "blis.h"

namespace {

struct Operand {
  int ndim;
  const int64_t* dims;
  const int64_t* strides;
  std::string labels;
};

struct Bundles {
  std::vector<int> AX, AY, BX, BY, CX, CY;
};

// Restatement of get_index_bundles (t1m.h:90-136).
bool index_bundles(const std::string& la, const std::string& lb,
                   const std::string& lc, Bundles* out) {
  std::string a = la, b = lb;
  std::sort(a.begin(), a.end());
  std::sort(b.begin(), b.end());
  std::string contracted, free_a, free_b;
  std::set_intersection(a.begin(), a.end(), b.begin(), b.end(),
                        std::back_inserter(contracted));
  std::set_difference(a.begin(), a.end(), b.begin(), b.end(),
                      std::back_inserter(free_a));
  std::set_difference(b.begin(), b.end(), a.begin(), a.end(),
                      std::back_inserter(free_b));
  for (char ch : contracted) {
    out->AY.push_back(static_cast<int>(la.find(ch)));
    out->BX.push_back(static_cast<int>(lb.find(ch)));
  }
  for (char ch : free_a) {
    out->AX.push_back(static_cast<int>(la.find(ch)));
    size_t p = lc.find(ch);
    if (p == std::string::npos) return false;
    out->CX.push_back(static_cast<int>(p));
  }
  for (char ch : free_b) {
    out->BY.push_back(static_cast<int>(lb.find(ch)));
    size_t p = lc.find(ch);
    if (p == std::string::npos) return false;
    out->CY.push_back(static_cast<int>(p));
  }
  return true;
}

// Restatement of get_scatter (t1m.h:141-174): offsets of every element of a
// bundle, the bundle's first mode varying fastest.
std::vector<int64_t> scatter(const std::vector<int>& modes, const Operand& t) {
  std::vector<int64_t> out{0};
  // Fold from the last mode down so the first mode ends up fastest.
  for (int i = static_cast<int>(modes.size()) - 1; i >= 0; --i) {
    const int64_t d = t.dims[modes[i]], s = t.strides[modes[i]];
    std::vector<int64_t> next;
    next.reserve(out.size() * d);
    for (int64_t hi : out)
      for (int64_t j = 0; j < d; ++j) next.push_back(hi + j * s);
    out.swap(next);
  }
  return out;
}

struct Problem {
  std::vector<int64_t> rsA, csA, rsB, csB, rsC, csC;  // M,K / K,N / M,N
};

template <class U>
void ukernel(long m, long n, long k, const U* alpha, const U* a, const U* b,
             const U* beta, U* c, long mr) {
  auxinfo_t aux{};
  if constexpr (std::is_same_v<U, float>)
    bli_sgemm_ukernel(m, n, k, alpha, a, b, beta, c, 1, mr, &aux,
                      bli_gks_query_cntx());
  else
    bli_dgemm_ukernel(m, n, k, alpha, a, b, beta, c, 1, mr, &aux,
                      bli_gks_query_cntx());
}

// One column slab [n_begin, n_end) of the five-loop algorithm.
template <class T, class U, bool kComplex>
void run_slab(const Problem& p, const T* A, const T* B, T* C, U alpha, U beta,
              int64_t n_begin, int64_t n_end) {
  const cntx_t* cntx = bli_gks_query_cntx();
  const num_t dt = std::is_same_v<U, float> ? BLIS_FLOAT : BLIS_DOUBLE;
  cntx_t* cx = const_cast<cntx_t*>(cntx);
  const int64_t MR = bli_cntx_get_blksz_def_dt(dt, BLIS_MR, cx);
  const int64_t NR = bli_cntx_get_blksz_def_dt(dt, BLIS_NR, cx);
  const int64_t MC = bli_cntx_get_blksz_def_dt(dt, BLIS_MC, cx);
  const int64_t KC = bli_cntx_get_blksz_def_dt(dt, BLIS_KC, cx);
  const int64_t NC = bli_cntx_get_blksz_def_dt(dt, BLIS_NC, cx);

  const int64_t M = static_cast<int64_t>(p.rsA.size());
  const int64_t K = static_cast<int64_t>(p.csA.size());
  // Complex: the loops step KC/2 and MC/2 complex entries (t1m.h:512, 521).
  const int64_t kstep = kComplex ? KC / 2 : KC;
  const int64_t mstep = kComplex ? MC / 2 : MC;

  std::vector<U> panel_a(static_cast<size_t>(MC * KC));
  std::vector<U> panel_b(static_cast<size_t>(KC * NC));
  std::vector<U> tile(static_cast<size_t>(MR * NR));

  for (int64_t jc = n_begin; jc < n_end; jc += NC) {
    const int64_t nc = std::min(NC, n_end - jc);
    for (int64_t pc = 0; pc < K; pc += kstep) {
      const int64_t kc = std::min(kstep, K - pc);
      const int64_t kreal = kComplex ? 2 * kc : kc;
      // B panel: NR-wide row-major slivers, sliver j at offset j*KC.
      std::fill(panel_b.begin(), panel_b.end(), U(0));
      for (int64_t j = 0; j < nc; ++j) {
        U* sl = panel_b.data() + (j / NR) * NR * KC;
        const int64_t jj = j % NR;
        const int64_t cn = p.csB[jc + j];
        for (int64_t k = 0; k < kc; ++k) {
          const T v = B[p.rsB[pc + k] + cn];
          if constexpr (kComplex) {
            sl[(2 * k) * NR + jj] = v.real();
            sl[(2 * k + 1) * NR + jj] = v.imag();
          } else {
            sl[k * NR + jj] = v;
          }
        }
      }
      for (int64_t ic = 0; ic < M; ic += mstep) {
        const int64_t mc = std::min(mstep, M - ic);
        const int64_t mreal = kComplex ? 2 * mc : mc;
        // A panel: MR-tall column-major slivers, real row r at r*KC.
        std::fill(panel_a.begin(), panel_a.end(), U(0));
        for (int64_t i = 0; i < mc; ++i) {
          const int64_t ri = kComplex ? 2 * i : i;
          U* sl = panel_a.data() + (ri / MR) * MR * KC;
          const int64_t ii = ri % MR;
          const int64_t rm = p.rsA[ic + i];
          for (int64_t k = 0; k < kc; ++k) {
            const T v = A[rm + p.csA[pc + k]];
            if constexpr (kComplex) {
              // 2x2 real block [re -im; im re] (t1m.h:319-323).
              sl[(2 * k) * MR + ii] = v.real();
              sl[(2 * k) * MR + ii + 1] = v.imag();
              sl[(2 * k + 1) * MR + ii] = -v.imag();
              sl[(2 * k + 1) * MR + ii + 1] = v.real();
            } else {
              sl[k * MR + ii] = v;
            }
          }
        }
        for (int64_t jr = 0; jr < nc; jr += NR) {
          const U* sb = panel_b.data() + KC * jr;
          const int64_t n = std::min(NR, nc - jr);
          for (int64_t ir = 0; ir < mreal; ir += MR) {
            const U* sa = panel_a.data() + ir * KC;
            const int64_t m = std::min(MR, mreal - ir);
            std::fill(tile.begin(), tile.end(), U(0));
            ukernel<U>(m, n, kreal, &alpha, sa, sb, &beta, tile.data(), MR);
            // C += tile (t1m.h:406-430); 1M rows 2k/2k+1 are re/im.
            if constexpr (kComplex) {
              const int64_t crow = ic + ir / 2;
              for (int64_t l = 0; l < n; ++l) {
                const int64_t cn = p.csC[jc + jr + l];
                for (int64_t k = 0; k < m / 2; ++k) {
                  const U re = tile[2 * k + l * MR];
                  const U im = tile[2 * k + 1 + l * MR];
                  C[p.rsC[crow + k] + cn] += T(re, im);
                }
              }
            } else {
              for (int64_t l = 0; l < n; ++l) {
                const int64_t cn = p.csC[jc + jr + l];
                for (int64_t k = 0; k < m; ++k)
                  C[p.rsC[ic + ir + k] + cn] += tile[k + l * MR];
              }
            }
          }
        }
      }
    }
  }
}

template <class T, class U, bool kComplex>
int run(const Problem& p, const void* A, const void* B, void* C, U alpha,
        U beta, int nthreads) {
  const int64_t N = static_cast<int64_t>(p.csB.size());
  const cntx_t* cntx = bli_gks_query_cntx();
  const num_t dt = std::is_same_v<U, float> ? BLIS_FLOAT : BLIS_DOUBLE;
  const int64_t NR =
      bli_cntx_get_blksz_def_dt(dt, BLIS_NR, const_cast<cntx_t*>(cntx));
  const T* a = static_cast<const T*>(A);
  const T* b = static_cast<const T*>(B);
  T* c = static_cast<T*>(C);
  if (nthreads <= 1 || N <= NR) {
    run_slab<T, U, kComplex>(p, a, b, c, alpha, beta, 0, N);
    return 0;
  }
  // Slabs are whole NR groups so each thread's slivers line up like the
  // single-threaded run's.
  const int64_t groups = (N + NR - 1) / NR;
  const int64_t nt = std::min<int64_t>(nthreads, groups);
  std::vector<std::thread> pool;
  for (int64_t t = 0; t < nt; ++t) {
    const int64_t g0 = groups * t / nt, g1 = groups * (t + 1) / nt;
    const int64_t n0 = g0 * NR, n1 = std::min(N, g1 * NR);
    pool.emplace_back([=, &p] { run_slab<T, U, kComplex>(p, a, b, c, alpha, beta, n0, n1); });
  }
  for (auto& th : pool) th.join();
  return 0;
}

}  // namespace

extern "C" {

// dtype: 0 float, 1 double, 2 complex<float>, 3 complex<double>.
// Strides are in elements (any layout).  alpha/beta point to a real scalar of
// the underlying type and are read for real dtypes only (the reference's
// complex overload has neither).  Returns 0, or -1 on a label error.
int t1m_port_contract(int dtype, int na, const int64_t* da, const int64_t* sa,
                      const void* a, const char* la, int nb, const int64_t* db,
                      const int64_t* sb, const void* b, const char* lb, int nc,
                      const int64_t* dc, const int64_t* sc, void* c,
                      const char* lc, const void* alpha, const void* beta,
                      int nthreads) {
  Operand A{na, da, sa, la}, B{nb, db, sb, lb}, C{nc, dc, sc, lc};
  Bundles bd;
  if (!index_bundles(A.labels, B.labels, C.labels, &bd)) return -1;
  Problem p;
  p.rsA = scatter(bd.AX, A);
  p.csA = scatter(bd.AY, A);
  p.rsB = scatter(bd.BX, B);
  p.csB = scatter(bd.BY, B);
  p.rsC = scatter(bd.CX, C);
  p.csC = scatter(bd.CY, C);
  switch (dtype) {
    case 0:
      return run<float, float, false>(p, a, b, c, *static_cast<const float*>(alpha),
                                      *static_cast<const float*>(beta), nthreads);
    case 1:
      return run<double, double, false>(p, a, b, c, *static_cast<const double*>(alpha),
                                        *static_cast<const double*>(beta), nthreads);
    case 2:
      return run<std::complex<float>, float, true>(p, a, b, c, 1.0f, 0.0f, nthreads);
    case 3:
      return run<std::complex<double>, double, true>(p, a, b, c, 1.0, 0.0, nthreads);
  }
  return -1;
}

}  // extern "C"
