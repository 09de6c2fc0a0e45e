// Host-side label analysis and block-scatter descriptor builder.
//
// Follows the reference's index bundling (include/t1m/t1m.h:90-136) and
// scatter vectors (t1m.h:141-174), with three deliberate differences:
//  * inputs are validated (the reference has no validation; a repeated label,
//    an extent mismatch or a label in A, B and C is undefined behaviour there);
//  * the order of modes inside a bundle is chosen for memory access (unit-
//    stride mode first), consistently across the two tensors sharing the
//    bundle.  M and N order do not change any result; K order only changes
//    the summation order;
//  * empty bundles (outer products, a 0-mode C) are allowed: their scatter
//    vector is {0} (the reference dereferences parts.back() of an empty vector,
//    t1m.h:173).
#include <algorithm>
#include <cstring>
#include <string>

#include "internal.h"
#include "t1m_capi.h"

namespace t1m {
namespace gb300 {
namespace {

bool valid_label(char ch) {
  return (ch >= 'a' && ch <= 'z') || (ch >= 'A' && ch <= 'Z') ||
         (ch >= '0' && ch <= '9');
}

// Offsets of every element of the bundle, first mode fastest (t1m.h:162-173).
std::vector<int64_t> scatter(const std::vector<Mode>& modes, bool second) {
  int64_t n = 1;
  for (const Mode& m : modes) n *= m.extent;
  std::vector<int64_t> out(static_cast<size_t>(n));
  for (int64_t i = 0; i < n; ++i) {
    int64_t rem = i, off = 0;
    for (const Mode& m : modes) {
      const int64_t j = rem % m.extent;
      rem /= m.extent;
      off += j * (second ? m.s1 : m.s0);
    }
    out[static_cast<size_t>(i)] = off;
  }
  return out;
}

int64_t uniform_stride(const std::vector<int64_t>& v) {
  if (v.size() < 2) return 0;
  const int64_t s = v[1] - v[0];
  for (size_t i = 2; i < v.size(); ++i)
    if (v[i] - v[i - 1] != s) return -1;
  return s;
}

// Put a unit-stride mode of the primary tensor first, the rest by ascending
// stride (this keeps consecutive indices adjacent in memory wherever the
// layout allows it).  Ties keep the reference's alphabetical order.
void order_modes(std::vector<Mode>* modes, bool primary_second) {
  std::stable_sort(modes->begin(), modes->end(), [&](const Mode& x, const Mode& y) {
    const int64_t sx = primary_second ? x.s1 : x.s0;
    const int64_t sy = primary_second ? y.s1 : y.s0;
    return sx < sy;
  });
}

int64_t span(int n, const int64_t* e, const int64_t* s) {
  int64_t sp = 1;
  for (int i = 0; i < n; ++i) {
    if (e[i] == 0) return 0;
    sp += (e[i] - 1) * s[i];
  }
  return sp;
}

}  // namespace

int build_plan(int dtype, int na, const int64_t* ea, const int64_t* sa,
               const char* la, int nb, const int64_t* eb, const int64_t* sb,
               const char* lb, int nc, const int64_t* ec, const int64_t* sc,
               const char* lc, HostPlan* plan, std::string* err) {
  const std::string A(la), B(lb), Cs(lc);
  if (static_cast<int>(A.size()) != na || static_cast<int>(B.size()) != nb ||
      static_cast<int>(Cs.size()) != nc) {
    *err = "label string length differs from tensor rank";
    return T1M_ERR_LABELS;
  }
  struct Info {
    int pa = -1, pb = -1, pc = -1;
  };
  Info info[128];
  auto note = [&](const std::string& s, int which) -> bool {
    for (size_t i = 0; i < s.size(); ++i) {
      const unsigned char ch = static_cast<unsigned char>(s[i]);
      if (!valid_label(static_cast<char>(ch))) {
        *err = std::string("invalid label character '") + s[i] + "'";
        return false;
      }
      int& slot = which == 0 ? info[ch].pa : which == 1 ? info[ch].pb : info[ch].pc;
      if (slot >= 0) {
        *err = std::string("label '") + s[i] + "' repeated within one tensor";
        return false;
      }
      slot = static_cast<int>(i);
    }
    return true;
  };
  if (!note(A, 0) || !note(B, 1) || !note(Cs, 2)) return T1M_ERR_LABELS;

  for (int i = 0; i < na; ++i)
    if (ea[i] < 0 || sa[i] < 0) { *err = "negative extent or stride in A"; return T1M_ERR_INVALID_ARGUMENT; }
  for (int i = 0; i < nb; ++i)
    if (eb[i] < 0 || sb[i] < 0) { *err = "negative extent or stride in B"; return T1M_ERR_INVALID_ARGUMENT; }
  for (int i = 0; i < nc; ++i)
    if (ec[i] < 0 || sc[i] < 0) { *err = "negative extent or stride in C"; return T1M_ERR_INVALID_ARGUMENT; }

  plan->dtype = dtype;
  plan->modes_m.clear();
  plan->modes_n.clear();
  plan->modes_k.clear();
  plan->modes_b.clear();
  plan->batch = 1;
  // Walk labels in sorted order, as the reference's set operations do.
  for (int ch = 0; ch < 128; ++ch) {
    const Info& x = info[ch];
    const bool inA = x.pa >= 0, inB = x.pb >= 0, inC = x.pc >= 0;
    if (!inA && !inB && !inC) continue;
    if (inA && inB) {
      if (inC) {
        // Batch (Hadamard) label: one independent product per index.
        if (ea[x.pa] != eb[x.pb] || ea[x.pa] != ec[x.pc]) {
          *err = std::string("extent mismatch for batch label '") + static_cast<char>(ch) + "'";
          return T1M_ERR_LABELS;
        }
        plan->modes_b.push_back({ea[x.pa], sa[x.pa], sb[x.pb], sc[x.pc], static_cast<char>(ch)});
        plan->batch *= ea[x.pa];
        continue;
      }
      if (ea[x.pa] != eb[x.pb]) {
        *err = std::string("extent mismatch for contracted label '") + static_cast<char>(ch) + "'";
        return T1M_ERR_LABELS;
      }
      plan->modes_k.push_back({ea[x.pa], sa[x.pa], sb[x.pb], static_cast<char>(ch)});
    } else if (inA) {
      if (!inC) {
        *err = std::string("free label '") + static_cast<char>(ch) + "' of A missing from C";
        return T1M_ERR_LABELS;
      }
      if (ea[x.pa] != ec[x.pc]) {
        *err = std::string("extent mismatch for label '") + static_cast<char>(ch) + "'";
        return T1M_ERR_LABELS;
      }
      plan->modes_m.push_back({ea[x.pa], sa[x.pa], sc[x.pc], static_cast<char>(ch)});
    } else if (inB) {
      if (!inC) {
        *err = std::string("free label '") + static_cast<char>(ch) + "' of B missing from C";
        return T1M_ERR_LABELS;
      }
      if (eb[x.pb] != ec[x.pc]) {
        *err = std::string("extent mismatch for label '") + static_cast<char>(ch) + "'";
        return T1M_ERR_LABELS;
      }
      plan->modes_n.push_back({eb[x.pb], sb[x.pb], sc[x.pc], static_cast<char>(ch)});
    } else {
      *err = std::string("label '") + static_cast<char>(ch) + "' of C appears in neither A nor B";
      return T1M_ERR_LABELS;
    }
  }

  // Mode order: M follows A, N follows B; K follows B whenever B has a
  // unit-stride contracted mode, else A.  When both have one (but different
  // ones) the operand in the other order is gathered element by element, and
  // the B tile (128 columns) is twice the A tile (64 rows) in the complex64
  // kernels, so B keeps its contiguous K runs.
  order_modes(&plan->modes_m, false);
  order_modes(&plan->modes_n, false);
  bool k_by_b = false;
  for (const Mode& m : plan->modes_k) k_by_b |= (m.s1 == 1 && m.extent > 1);
  order_modes(&plan->modes_k, k_by_b);

  plan->rsA = scatter(plan->modes_m, false);
  plan->rsC = scatter(plan->modes_m, true);
  plan->csB = scatter(plan->modes_n, false);
  plan->csC = scatter(plan->modes_n, true);
  plan->csA = scatter(plan->modes_k, false);
  plan->rsB = scatter(plan->modes_k, true);
  plan->M = static_cast<int64_t>(plan->rsA.size());
  plan->N = static_cast<int64_t>(plan->csB.size());
  plan->K = static_cast<int64_t>(plan->csA.size());
  plan->uA_m = uniform_stride(plan->rsA);
  plan->uC_m = uniform_stride(plan->rsC);
  plan->uB_n = uniform_stride(plan->csB);
  plan->uC_n = uniform_stride(plan->csC);
  plan->uA_k = uniform_stride(plan->csA);
  plan->uB_k = uniform_stride(plan->rsB);
  plan->spanA = span(na, ea, sa);
  plan->spanB = span(nb, eb, sb);
  plan->spanC = span(nc, ec, sc);
  return T1M_OK;
}

}  // namespace gb300
}  // namespace t1m
