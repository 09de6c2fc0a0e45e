// Minimal BLIS stand-in for the oracle (test infrastructure only).
//
// The reference library (include/t1m/t1m.h, include/t1m/bli/mappings.h) needs
// BLIS for two things: the block-size query (mappings.h:118-127) and the real
// GEMM micro-kernel (mappings.h:91-99, called at t1m.h:500 and t1m.h:546).
// BLIS itself is a third-party, un-vendored dependency with no pinned version
// (reference CMakeLists.txt:23-24 only does find_library), and it is not
// installed here.  This header supplies exactly the declarations the
// reference's hot path uses, written from the calling contract t1m relies on:
//
//   * A sliver: MR x k, column-major, leading dimension MR (t1m.h:381, 491).
//   * B sliver: k x NR, row-major, leading dimension NR (t1m.h:393, 485).
//   * C tile:   m x n (m <= MR, n <= NR) at c[i*rs_c + j*cs_c]; t1m always
//               passes rs_c = 1, cs_c = MR (t1m.h:501, 547).
//   * c <- beta*c + alpha*(a*b); with beta == 0 the old c is not read
//     (BLIS convention).
//
// The arithmetic is a plain fused-multiply-add chain over p = 0..k-1 per
// output element (std::fma, so x86-64 and aarch64 builds agree bit for bit).
// It is NOT BLIS's assembly kernel: the exact bits of BLIS are unpinned.
#pragma once

#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdint>

typedef long dim_t;
typedef long inc_t;

typedef enum { BLIS_FLOAT = 0, BLIS_DOUBLE = 1 } num_t;
typedef enum { BLIS_MR = 0, BLIS_NR, BLIS_MC, BLIS_KC, BLIS_NC } bszid_t;
typedef enum { BLIS_NO_CONJUGATE = 0 } conj_t;

struct scomplex { float real, imag; };
struct dcomplex { double real, imag; };

// Block sizes of the stand-in context.  MC is a multiple of MR and NC of NR so
// that 1M cells of MR/2 rows never straddle two MR-blocks (the hazard of the
// reference's slice_rows, t1m.h:226-231, stays dormant).
struct cntx_t {
  dim_t blksz[2][5];
};

namespace t1m_standin {
constexpr dim_t S_MR = 8, S_NR = 12, S_MC = 128, S_KC = 256, S_NC = 4080;
constexpr dim_t D_MR = 6, D_NR = 8, D_MC = 72, D_KC = 256, D_NC = 4080;

inline const cntx_t* default_cntx() {
  static const cntx_t c = {{{S_MR, S_NR, S_MC, S_KC, S_NC},
                            {D_MR, D_NR, D_MC, D_KC, D_NC}}};
  return &c;
}

template <typename U, int MR, int NR>
inline void ukernel(dim_t m, dim_t n, dim_t k, const U* alpha, const U* a,
                    const U* b, const U* beta, U* c, inc_t rs_c, inc_t cs_c) {
  U acc[MR][NR];
  for (int i = 0; i < MR; ++i)
    for (int j = 0; j < NR; ++j) acc[i][j] = U(0);
  for (dim_t p = 0; p < k; ++p) {
    const U* ap = a + p * MR;
    const U* bp = b + p * NR;
    for (int i = 0; i < MR; ++i)
      for (int j = 0; j < NR; ++j) acc[i][j] = std::fma(ap[i], bp[j], acc[i][j]);
  }
  for (dim_t i = 0; i < m; ++i) {
    for (dim_t j = 0; j < n; ++j) {
      U& cij = c[i * rs_c + j * cs_c];
      cij = (*beta == U(0)) ? (*alpha) * acc[i][j]
                            : (*beta) * cij + (*alpha) * acc[i][j];
    }
  }
}
}  // namespace t1m_standin

struct auxinfo_t {
  int unused;
};

inline const cntx_t* bli_gks_query_cntx() { return t1m_standin::default_cntx(); }

inline dim_t bli_cntx_get_blksz_def_dt(num_t dt, bszid_t bs, cntx_t* cntx) {
  return cntx->blksz[dt == BLIS_DOUBLE ? 1 : 0][bs];
}

inline void bli_sgemm_ukernel(dim_t m, dim_t n, dim_t k, const float* alpha,
                              const float* a, const float* b, const float* beta,
                              float* c, inc_t rs_c, inc_t cs_c,
                              const auxinfo_t*, const cntx_t*) {
  t1m_standin::ukernel<float, t1m_standin::S_MR, t1m_standin::S_NR>(
      m, n, k, alpha, a, b, beta, c, rs_c, cs_c);
}

inline void bli_dgemm_ukernel(dim_t m, dim_t n, dim_t k, const double* alpha,
                              const double* a, const double* b,
                              const double* beta, double* c, inc_t rs_c,
                              inc_t cs_c, const auxinfo_t*, const cntx_t*) {
  t1m_standin::ukernel<double, t1m_standin::D_MR, t1m_standin::D_NR>(
      m, n, k, alpha, a, b, beta, c, rs_c, cs_c);
}
