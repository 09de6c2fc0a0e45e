// C-ABI of libt1m_cuda.so (declared in include/t1m_capi.h).
//
// t1m_contract replaces the reference's t1m::contract (include/t1m/t1m.h:
// 560-577).  Per call it (1) validates and analyses the labels into a plan of
// scatter vectors (cached per shape on the device), (2) stages host operands
// to the device when the caller passed host pointers, (3) launches the kernel
// of the chosen method on the context's stream, and (4) copies C back for
// host operands.  Nothing runs on the CPU except label analysis and staging:
// a missing or failed kernel is an error, never a CPU fallback.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <list>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <unordered_map>

#include "internal.h"
#include "t1m_capi.h"

using namespace t1m::gb300;

namespace t1m {
namespace gb300 {
cudaError_t launch_dmma(int dtype, const GemmArgs& args, int splits, cudaStream_t stream,
                        int* kernels);
void dmma_tile(int* bm, int* bn, int* bk);
}  // namespace gb300
}  // namespace t1m

struct t1m_context {
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  int method = T1M_METHOD_AUTO;
  std::string last_error;
  cudaEvent_t ev[6] = {};
  // Around the main kernel of a tensor-core product (after its split, pack
  // or panel passes), when a timed single-product call arms them.
  cudaEvent_t mev[2] = {};
  bool mev_armed = false;
  bool mev_recorded = false;
  // Device-side error word written by kernels whose bounded waits ran out.
  int* d_err = nullptr;
  // Plan cache: key -> (host plan, device scatter vectors), LRU bounded.
  struct Entry {
    std::string key;
    HostPlan host;
    DevicePlan dev;
  };
  std::list<Entry> plans;
  std::unordered_map<std::string, std::list<Entry>::iterator> index;
  // Staging buffers for host operands (grow only).
  void* stage[3] = {nullptr, nullptr, nullptr};
  size_t stage_bytes[3] = {0, 0, 0};
  // Split-K workspace (grow only) and the forced split count (0 = automatic).
  void* work = nullptr;
  size_t work_bytes = 0;
  // B-panel and operand-pack workspaces of the tensor-core kernels (grow
  // only), one set per compute stream of the slab pipeline.
  void* panel[2] = {nullptr, nullptr};
  size_t panel_bytes[2] = {0, 0};
  void* pack[2] = {nullptr, nullptr};
  size_t pack_bytes[2] = {0, 0};
  // Host-buffer pipeline: pieces of its resident operand, split once for
  // every slab (grow only; an optional workspace like the panels).
  void* res_pieces = nullptr;
  size_t res_pieces_bytes = 0;
  // ... and of its streamed operand, each slab split once for both halves.
  void* slab_pieces = nullptr;
  size_t slab_pieces_bytes = 0;
  int split_k = 0;
  // Arrival counters of the persistent kernel's in-kernel split-K reduction
  // (zeroed when allocated; the kernel leaves them at zero; zeroed again
  // after a kernel reported an error).
  int* fix_ctr = nullptr;
  int64_t fix_cap = 0;
  bool fix_dirty = false;
  // Cap on each optional workspace (panels, packs); -1 = none.
  int64_t opt_work_limit = -1;
  // T1M_TILE_* form of tensor-core products.
  int tile_form = T1M_TILE_AUTO;
  // Bound on grouped launches' dependency waits (us, 0 = kernel default) and
  // the SM clock (kHz) that converts it to clock64 cycles.
  int64_t wait_limit_us = 0;
  int clock_khz = 2070000;
  // Tune single tensor-core contractions (tile form, split count) per shape
  // class, cached with the grouped launches' choices.
  bool autotune = false;
  // T1M_PATH_* code of the last tensor-core product of the current call.
  int last_path = 0;
  int num_sms = 152;
  // Host-operand pipeline: copy-in and copy-out streams beside the compute
  // stream, ordering events (see run_pipelined).
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  // Second compute stream of the slab pipeline: consecutive slabs alternate
  // between the context stream and this one, so the last wave of one slab's
  // kernel shares the SMs with the first of the next.
  cudaStream_t compute2 = nullptr;
  static constexpr int kPipeEvents = 3 + 8 + 2 * 8 + 2 + 2 + 8;
  cudaEvent_t pev[kPipeEvents] = {};
};

namespace t1m {
namespace gb300 {

int auto_method(int dtype, const HostPlan& plan) {
  if ((dtype == T1M_COMPLEX64 || dtype == T1M_FLOAT32) && tc_supported(kMethodTcAuto, dtype, plan) &&
      plan.M * plan.N * plan.K >= int64_t(1) << (dtype == T1M_FLOAT32 ? 20 : 18))
    return kMethodTcAuto;
  return T1M_METHOD_PLAIN;
}

int64_t accuracy_k_limit(int method, int dtype) {
  const bool cplx = dtype == T1M_COMPLEX64;
  if (dtype != T1M_COMPLEX64 && dtype != T1M_FLOAT32) return 0;
  if (method == T1M_METHOD_PLAIN) return cplx ? 128 : 256;
  if (method == kMethodTcAuto || method == T1M_METHOD_TC_3XTF32 || method == T1M_METHOD_TC_BF16X6)
    return cplx ? 4096 : 8192;
  return 0;
}

}  // namespace gb300
}  // namespace t1m

namespace {

constexpr size_t kMaxPlans = 4096;

size_t elem_size(int dtype) {
  switch (dtype) {
    case T1M_FLOAT32: return 4;
    case T1M_FLOAT64: return 8;
    case T1M_COMPLEX64: return 8;
    case T1M_COMPLEX128: return 16;
  }
  return 0;
}

int fail(t1m_context* ctx, int status, const std::string& msg) {
  if (ctx) ctx->last_error = msg;
  return status;
}

int cuda_fail(t1m_context* ctx, cudaError_t e, const char* what) {
  return fail(ctx, T1M_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

bool resolve_strides(const t1m_tensor* t, int64_t* out) {
  const int n = t->ndim;
  if (t->layout == T1M_STRIDED) {
    if (n > 0 && !t->strides) return false;
    for (int i = 0; i < n; ++i) out[i] = t->strides[i];
    return true;
  }
  int64_t acc = 1;
  if (t->layout == T1M_COL_MAJOR) {
    for (int i = 0; i < n; ++i) { out[i] = acc; acc *= t->extents[i]; }
    return true;
  }
  if (t->layout == T1M_ROW_MAJOR) {
    for (int i = n - 1; i >= 0; --i) { out[i] = acc; acc *= t->extents[i]; }
    return true;
  }
  return false;
}

std::string plan_key(int dtype, const t1m_tensor* a, const int64_t* sa, const char* la,
                     const t1m_tensor* b, const int64_t* sb, const char* lb,
                     const t1m_tensor* c, const int64_t* sc, const char* lc) {
  std::string k = std::to_string(dtype);
  auto add = [&](const t1m_tensor* t, const int64_t* s, const char* l) {
    k += '|';
    k += l;
    for (int i = 0; i < t->ndim; ++i) {
      k += ',' + std::to_string(t->extents[i]) + ':' + std::to_string(s[i]);
    }
  };
  add(a, sa, la);
  add(b, sb, lb);
  add(c, sc, lc);
  return k;
}

int upload_plan(t1m_context* ctx, const HostPlan& hp, DevicePlan* dp) {
  const std::vector<int64_t>* vs[6] = {&hp.rsA, &hp.csA, &hp.rsB, &hp.csB, &hp.rsC, &hp.csC};
  size_t total = 0;
  for (auto* v : vs) total += (v->size() + 1) * sizeof(int64_t);
  void* block = nullptr;
  cudaError_t e = cudaMalloc(&block, total);
  if (e != cudaSuccess) return fail(ctx, T1M_ERR_ALLOC, std::string("plan allocation: ") + cudaGetErrorString(e));
  std::vector<int64_t> host;
  host.reserve(total / sizeof(int64_t));
  const int64_t* ptrs[6];
  size_t off = 0;
  for (int i = 0; i < 6; ++i) {
    ptrs[i] = static_cast<const int64_t*>(block) + off;
    host.insert(host.end(), vs[i]->begin(), vs[i]->end());
    host.push_back(0);
    off += vs[i]->size() + 1;
  }
  e = cudaMemcpy(block, host.data(), total, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(block);
    return cuda_fail(ctx, e, "plan upload");
  }
  dp->block = block;
  dp->bytes = total;
  dp->rsA = ptrs[0]; dp->csA = ptrs[1]; dp->rsB = ptrs[2];
  dp->csB = ptrs[3]; dp->rsC = ptrs[4]; dp->csC = ptrs[5];
  return T1M_OK;
}

bool is_device_pointer(const void* p) {
  if (!p) return false;
  cudaPointerAttributes attr{};
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

int ensure_stage(t1m_context* ctx, int i, size_t bytes) {
  if (ctx->stage_bytes[i] >= bytes) return T1M_OK;
  if (ctx->stage[i]) cudaFree(ctx->stage[i]);
  ctx->stage[i] = nullptr;
  ctx->stage_bytes[i] = 0;
  cudaError_t e = cudaMalloc(&ctx->stage[i], bytes);
  if (e != cudaSuccess) return fail(ctx, T1M_ERR_ALLOC, std::string("staging allocation: ") + cudaGetErrorString(e));
  ctx->stage_bytes[i] = bytes;
  return T1M_OK;
}

// Read (and clear) the kernels' error word; only called after a stream sync.
int check_device_error(t1m_context* ctx) {
  int code = 0;
  cudaError_t e = cudaMemcpy(&code, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "read kernel status");
  if (code == 0) return T1M_OK;
  cudaMemset(ctx->d_err, 0, sizeof(int));
  ctx->fix_dirty = true;  // a kernel cut short may leave arrival counters set
  return fail(ctx, T1M_ERR_KERNEL_TIMEOUT,
              "a bounded device-side wait timed out (kernel code " + std::to_string(code) + ")");
}

int choose_method(const t1m_context* ctx, int dtype, const HostPlan& plan) {
  return ctx->method != T1M_METHOD_AUTO ? ctx->method : auto_method(dtype, plan);
}

// Workspace cap of split-K (bytes of partial products).
constexpr size_t kMaxWorkBytes = size_t(2) << 30;

// Number of K splits: enough CTAs for about one full wave when the output
// has too few tiles, each split keeping at least four K-steps; forced by
// t1m_set_split_k.  Returns the split count and its K length (a multiple of
// the kernel's K-step).
// Under T1M_METHOD_AUTO (`promote`) the split count is also at least
// ceil(K / accuracy_k_limit), so every FP32 partial stays within the 1e-6
// error bound and the partials are summed in FP64.
int choose_splits(const t1m_context* ctx, int method, int dtype, int64_t M, int64_t N,
                  int64_t K, size_t elem, int64_t* k_per_split, bool promote = false) {
  int bm, bn, bk, per_sm;
  if (method == T1M_METHOD_PLAIN) {
    simt_tile(dtype, &bm, &bn, &bk);
    per_sm = 2;
  } else if (method == T1M_METHOD_DMMA) {
    dmma_tile(&bm, &bn, &bk);
    per_sm = 8;
  } else {
    tc_tile(dtype, &bm, &bn, &bk);
    per_sm = 1;
  }
  const int64_t tiles = ((M + bm - 1) / bm) * ((N + bn - 1) / bn);
  const int64_t ksteps = (K + bk - 1) / bk;
  int64_t s = 1;
  if (ctx->split_k > 0) {
    s = ctx->split_k;
  } else {
    const int64_t target = int64_t(ctx->num_sms) * per_sm;
    if (tiles < target / 2 && ksteps >= 8)
      s = std::min<int64_t>((target + tiles - 1) / tiles, ksteps / 4);
    const int64_t lim = promote ? accuracy_k_limit(method, dtype) : 0;
    if (lim > 0) s = std::max<int64_t>(s, (K + lim - 1) / lim);
  }
  s = std::max<int64_t>(1, std::min<int64_t>({s, ksteps, 4096}));
  while (s > 1 && size_t(s) * size_t(M) * size_t(N) * elem > kMaxWorkBytes) --s;
  const int64_t steps_per = (ksteps + s - 1) / s;
  *k_per_split = steps_per * bk;
  return static_cast<int>((ksteps + steps_per - 1) / steps_per);
}

int ensure_work(t1m_context* ctx, size_t bytes) {
  if (ctx->work_bytes >= bytes) return T1M_OK;
  if (ctx->work) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->work);
  }
  ctx->work = nullptr;
  ctx->work_bytes = 0;
  cudaError_t e = cudaMalloc(&ctx->work, bytes);
  if (e != cudaSuccess)
    return fail(ctx, T1M_ERR_ALLOC, std::string("split-K workspace: ") + cudaGetErrorString(e));
  ctx->work_bytes = bytes;
  return T1M_OK;
}

// B-panel and operand-pack workspaces: both are optimisations, so a failed
// allocation leaves the product on the in-kernel path instead of failing it.
bool ensure_opt_work(cudaStream_t user, void** buf, size_t* have, size_t bytes) {
  if (*have >= bytes) return true;
  if (*buf) {
    cudaStreamSynchronize(user);  // the only stream that uses this buffer
    cudaFree(*buf);
  }
  *buf = nullptr;
  *have = 0;
  if (cudaMalloc(buf, bytes) != cudaSuccess) {
    cudaGetLastError();
    *buf = nullptr;
    return false;
  }
  *have = bytes;
  return true;
}

// Tuned tile form and split count of a single tensor-core product (defined
// with the tuning cache below); false when none applies.
bool tuned_product(t1m_context* ctx, int method, int dtype, size_t es, const HostPlan& hp,
                   const GemmArgs& g, cudaStream_t s, int slot, int* form, int* splits,
                   int64_t* k_per_split);

// One product C = alpha*A*B (+ beta*C) on stream s, its operands already in
// g (shifted for a batch index or a slab): method checks, split-K (raw
// partials in the workspace, FP64 reduction with the epilogue) and the
// kernel launch.  Adds the kernels it launched to *kernels.
int launch_product(t1m_context* ctx, int method, int dtype, size_t es, const HostPlan& hp,
                   const GemmArgs& g, cudaStream_t s, int* kernels, int* used_method,
                   int* splits_out, int slot, bool allow_split,
                   const PiecesReady* ready = nullptr) {
  int nk = 0;
  int splits = 1;
  bool reduced = false;  // the split product was reduced inside its kernel
  cudaError_t e = cudaSuccess;
  if (g.K == 0) {
    // C <- beta*C (or unchanged): nothing to multiply; handled by the plain
    // kernel with an empty K loop.
    e = launch_simt(dtype, g, 1, s, &nk);
    *used_method = T1M_METHOD_PLAIN;
  } else {
    const bool dmma_ok =
        method == T1M_METHOD_DMMA && (dtype == T1M_FLOAT64 || dtype == T1M_COMPLEX128);
    if (method != T1M_METHOD_PLAIN && !dmma_ok && !tc_supported(method, dtype, hp))
      return fail(ctx, T1M_ERR_UNSUPPORTED,
                  std::string("method ") + std::to_string(method) +
                      " is not available for this dtype/contraction");
    int64_t kps = g.K;
    // Blocks of the host-buffer pipeline never split: the whole product runs
    // unsplit on the device-buffer path, and concurrent blocks must not share
    // the split-K workspace.
    splits = allow_split ? choose_splits(ctx, method, dtype, g.M, g.N, g.K, es, &kps,
                                         ctx->method == T1M_METHOD_AUTO)
                         : 1;
    int form = ctx->tile_form;
    if (allow_split && ctx->autotune && ctx->split_k == 0 && ctx->tile_form == T1M_TILE_AUTO &&
        method != T1M_METHOD_PLAIN && method != T1M_METHOD_DMMA) {
      int tf = 0, ts = 0;
      int64_t tk = 0;
      if (tuned_product(ctx, method, dtype, es, hp, g, s, slot, &tf, &ts, &tk)) {
        form = tf;
        splits = ts;
        kps = tk;
      }
    }
    // Split-K: the main kernel writes raw partial products (alpha = 1,
    // beta = 0) into dense workspace slices, m fastest; the reduction sums
    // them in FP64 and applies the epilogue.
    GemmArgs gm = g;
    if (splits > 1) {
      if (int st = ensure_work(ctx, size_t(splits) * size_t(g.M) * size_t(g.N) * es)) return st;
      gm.C = ctx->work;
      gm.rsC = nullptr;
      gm.csC = nullptr;
      gm.uC_m = 1;
      gm.uC_n = g.M;
      gm.alpha[0] = 1.0;
      gm.alpha[1] = 0.0;
      gm.beta[0] = gm.beta[1] = 0.0;
      gm.flags = (g.flags & (kFlagConjA | kFlagConjB)) | kFlagBetaZero;
      gm.k_per_split = kps;
      gm.c_split_stride = g.M * g.N;
    }
    if (method == T1M_METHOD_PLAIN) {
      e = launch_simt(dtype, gm, splits, s, &nk);
    } else if (method == T1M_METHOD_DMMA) {
      e = launch_dmma(dtype, gm, splits, s, &nk);
    } else {
      std::string err;
      int ran = method;
      // Workspaces of this compute stream (slot 1: the pipeline's second).
      const auto within = [&](size_t bytes) {
        return ctx->opt_work_limit < 0 || bytes <= static_cast<size_t>(ctx->opt_work_limit);
      };
      // The panel workspace also holds operand pieces where they run.
      const size_t pcb = tc_pieces_count(method, dtype, gm, hp, form) > 0
                             ? tc_pieces_bytes(dtype, method, gm.M, gm.N, gm.K, ready)
                             : 0;
      const size_t pb = std::max(tc_panel_bytes(dtype, gm.M, gm.N, gm.K), pcb);
      const bool pan = pb > 0 && within(pb) &&
                       ensure_opt_work(s, &ctx->panel[slot], &ctx->panel_bytes[slot], pb);
      const size_t kb = tc_pack_bytes(dtype, hp);
      const bool pk = kb > 0 && within(kb) &&
                      ensure_opt_work(s, &ctx->pack[slot], &ctx->pack_bytes[slot], kb);
      // Arrival counters for the persistent kernel's in-kernel reduction of
      // a split product (the one-tile forms use the reduction kernel).
      constexpr int64_t kFixCap = int64_t(1) << 16;
      if (splits > 1 && !ctx->fix_ctr) {
        if (cudaMalloc(&ctx->fix_ctr, sizeof(int) * kFixCap) == cudaSuccess &&
            cudaMemset(ctx->fix_ctr, 0, sizeof(int) * kFixCap) == cudaSuccess) {
          ctx->fix_cap = kFixCap;
        } else {
          cudaGetLastError();
          if (ctx->fix_ctr) cudaFree(ctx->fix_ctr);
          ctx->fix_ctr = nullptr;
        }
      }
      if (ctx->fix_dirty && ctx->fix_ctr) {
        cudaMemsetAsync(ctx->fix_ctr, 0, sizeof(int) * size_t(ctx->fix_cap), s);
        ctx->fix_dirty = false;
      }
      TcFix fix{splits > 1 ? ctx->fix_ctr : nullptr, ctx->fix_cap, &g, false};
      e = launch_tc(method, dtype, gm, hp, splits, s, ctx->d_err, &nk, &err, &ran,
                    pan ? ctx->panel[slot] : nullptr, pan ? ctx->panel_bytes[slot] : 0,
                    pk ? ctx->pack[slot] : nullptr, pk ? ctx->pack_bytes[slot] : 0,
                    &ctx->last_path, form, ready, ctx->mev_armed ? ctx->mev : nullptr, &fix);
      reduced = fix.reduced;
      if (e == cudaSuccess && ctx->mev_armed) ctx->mev_recorded = true;
      *used_method = ran;
      if (e != cudaSuccess && !err.empty()) return fail(ctx, T1M_ERR_CUDA, err);
    }
    if (e == cudaSuccess && splits > 1 && !reduced) {
      e = launch_splitk_reduce(dtype, ctx->work, splits, g, s);
      ++nk;
    }
  }
  *kernels += nk;
  *splits_out = splits;
  if (e != cudaSuccess) return cuda_fail(ctx, e, "kernel launch");
  return T1M_OK;
}

// Host operands: the contraction is cut into slabs along N (B and C
// streamed, A resident) or along M (A and C streamed, B resident), so the
// host->device copy of slab i+1 and the device->host copy of slab i-1 run
// while slab i computes.  The slab dimension must be a uniform stride of both
// streamed tensors, larger than the spread of their other offsets: then every
// slab of them is one address range, disjoint from the others.
constexpr int kMaxSlabs = 8;
constexpr size_t kPipelineMinBytes = size_t(64) << 20;
constexpr size_t kSlabBytes = size_t(32) << 20;

struct Slabs {
  bool along_n = true;
  int count = 0;
  int64_t width = 0;       // columns (N) or rows (M) per slab, a multiple of 128
  int64_t x_lo = 0, x_hi = 0, ux = 0;  // streamed operand: offset spread, slab stride
  int64_t c_lo = 0, c_hi = 0, uc = 0;  // C: offset spread, slab stride
};

void spread(const std::vector<int64_t>& v, int64_t* lo, int64_t* hi) {
  *lo = v.empty() ? 0 : *std::min_element(v.begin(), v.end());
  *hi = v.empty() ? 0 : *std::max_element(v.begin(), v.end());
}

bool plan_slabs(const HostPlan& hp, size_t es, Slabs* sl) {
  if (hp.batch != 1 || hp.M <= 0 || hp.N <= 0 || hp.K <= 0) return false;
  int64_t bl, bh, al, ah, cnl, cnh, cml, cmh;
  spread(hp.rsB, &bl, &bh);   // B offsets of one column (over K)
  spread(hp.csA, &al, &ah);   // A offsets of one row (over K)
  spread(hp.rsC, &cml, &cmh); // C offsets of one column (over M)
  spread(hp.csC, &cnl, &cnh); // C offsets of one row (over N)
  const bool n_ok = hp.N >= 256 && hp.uB_n >= 1 && hp.uC_n >= 1 && bh - bl < hp.uB_n &&
                    cmh - cml < hp.uC_n;
  const bool m_ok = hp.M >= 256 && hp.uA_m >= 1 && hp.uC_m >= 1 && ah - al < hp.uA_m &&
                    cnh - cnl < hp.uC_m;
  if (!n_ok && !m_ok) return false;
  sl->along_n = n_ok;
  const int64_t len = n_ok ? hp.N : hp.M;
  const size_t streamed = size_t(n_ok ? hp.spanB : hp.spanA) * es + size_t(hp.spanC) * es;
  int64_t count = std::max<int64_t>(2, std::min<int64_t>(kMaxSlabs, streamed / kSlabBytes));
  sl->width = ((len + count - 1) / count + 127) / 128 * 128;
  sl->count = static_cast<int>((len + sl->width - 1) / sl->width);
  if (sl->count < 2) return false;
  if (n_ok) {
    sl->x_lo = bl; sl->x_hi = bh; sl->ux = hp.uB_n;
    sl->c_lo = cml; sl->c_hi = cmh; sl->uc = hp.uC_n;
  } else {
    sl->x_lo = al; sl->x_hi = ah; sl->ux = hp.uA_m;
    sl->c_lo = cnl; sl->c_hi = cnh; sl->uc = hp.uC_m;
  }
  return true;
}

}  // namespace

namespace {

// The slab pipeline (see plan_slabs).  Streams: copy_in (host->device), two
// compute streams (the context stream and compute2, alternating) and
// copy_out (device->host).  The resident operand (A for slabs along N, B for
// slabs along M) goes first, in two halves along its other dimension when
// each half is one 2-D region (unit stride there, uniform K stride): half 0,
// the first two streamed slabs, half 1, the remaining slabs.  A block (slab
// i, half h) is launched once its inputs are queued, on the next compute
// stream (each with its own workspaces), and waits for them by events; C
// slab i goes back once its blocks are done.  Blocks are disjoint outputs
// and multiples of the output tile, so the two compute streams may overlap
// and every output element is computed as on the device-buffer path.  The
// call returns once copy_out and compute2 have finished (the result is in
// host memory).
enum : int {
  kEvStart = 0,                      // earlier work on the context stream done
  kEvRes = 1,                        // + h: resident operand half h on the device
  kEvSlab = 3,                       // + i: streamed slab i (and its C range) on the device
  kEvDone = kEvSlab + kMaxSlabs,     // + 2 i + h: block (i, h) computed
  kEvOut = kEvDone + 2 * kMaxSlabs,  // copy_out finished
  kEvC2 = kEvOut + 1,                // compute2 finished
  kEvResPieces = kEvC2 + 1,          // + h: pieces of resident half h split
  kEvSlabPieces = kEvResPieces + 2,  // + i: pieces of streamed slab i split
  kEvCount = kEvSlabPieces + kMaxSlabs
};
static_assert(kEvCount <= t1m_context::kPipeEvents, "pipeline events");

int run_pipelined(t1m_context* ctx, int method, int dtype, size_t es, const HostPlan& hp,
                  const GemmArgs& g0, const t1m_tensor* a, const t1m_tensor* b,
                  const t1m_tensor* c, const Slabs& sl, bool readC, bool timing,
                  t1m_report* report) {
  cudaStream_t s = ctx->stream;
  const size_t bytesA = size_t(hp.spanA) * es, bytesB = size_t(hp.spanB) * es;
  const size_t bytesC = size_t(hp.spanC) * es;
  for (int i = 0; i < 3; ++i)
    if (int st = ensure_stage(ctx, i, i == 0 ? bytesA : i == 1 ? bytesB : bytesC)) return st;
  cudaError_t e = cudaSuccess;
  int64_t h2d = 0, d2h = 0;
  if (timing) cudaEventRecord(ctx->ev[0], s);
  // Earlier work on the context stream may still use the staging buffers.
  cudaEventRecord(ctx->pev[kEvStart], s);
  cudaStreamWaitEvent(ctx->copy_in, ctx->pev[kEvStart], 0);
  cudaStreamWaitEvent(ctx->copy_out, ctx->pev[kEvStart], 0);
  cudaStreamWaitEvent(ctx->compute2, ctx->pev[kEvStart], 0);

  // Resident operand and its halves: along N, A split along M (uA_m = 1,
  // rows of K at stride uA_k); along M, B split along N likewise.
  const int res = sl.along_n ? 0 : 1;
  const t1m_tensor* rt = sl.along_n ? a : b;
  const size_t rbytes = sl.along_n ? bytesA : bytesB;
  const int64_t rlen = sl.along_n ? hp.M : hp.N;                 // the halved dimension
  const int64_t ru = sl.along_n ? hp.uA_m : hp.uB_n;             // its stride in the operand
  const int64_t rk = sl.along_n ? hp.uA_k : hp.uB_k;             // the operand's K stride
  const int64_t cu = sl.along_n ? hp.uC_m : hp.uC_n;             // C's stride along it
  const int64_t half = (rlen / 2 + 127) / 128 * 128;
  const bool split = ru == 1 && rk >= rlen && cu >= 1 && rlen >= 256 && half < rlen;
  const int halves = split ? 2 : 1;
  auto copy_resident = [&](int h) -> cudaError_t {
    if (!split) {
      h2d += static_cast<int64_t>(rbytes);
      return cudaMemcpyAsync(ctx->stage[res], rt->data, rbytes, cudaMemcpyHostToDevice,
                             ctx->copy_in);
    }
    const int64_t lo = h * half, hi = h ? rlen : half;
    const size_t off = size_t(lo) * es, width = size_t(hi - lo) * es, pitch = size_t(rk) * es;
    h2d += static_cast<int64_t>(width) * hp.K;
    return cudaMemcpy2DAsync(static_cast<char*>(ctx->stage[res]) + off, pitch,
                             static_cast<const char*>(rt->data) + off, pitch, width,
                             static_cast<size_t>(hp.K), cudaMemcpyHostToDevice, ctx->copy_in);
  };

  const int xs = sl.along_n ? 1 : 0;
  const t1m_tensor* xt = sl.along_n ? b : a;
  // A C slab range that holds elements outside C (a strided view) goes to
  // the device first, so copying the range back leaves them as they were.
  const bool c_in = readC || hp.spanC != hp.M * hp.N;
  const int64_t len = sl.along_n ? hp.N : hp.M;
  auto copy_slab = [&](int i) -> cudaError_t {
    const int64_t lo = i * sl.width, hi = std::min(len, lo + sl.width);
    const int64_t x0 = lo * sl.ux + sl.x_lo, x1 = (hi - 1) * sl.ux + sl.x_hi + 1;
    const int64_t c0 = lo * sl.uc + sl.c_lo, c1 = (hi - 1) * sl.uc + sl.c_hi + 1;
    const size_t xo = size_t(x0) * es, xn = size_t(x1 - x0) * es;
    const size_t co = size_t(c0) * es, cn = size_t(c1 - c0) * es;
    cudaError_t r = cudaMemcpyAsync(static_cast<char*>(ctx->stage[xs]) + xo,
                                    static_cast<const char*>(xt->data) + xo, xn,
                                    cudaMemcpyHostToDevice, ctx->copy_in);
    h2d += static_cast<int64_t>(xn);
    if (r == cudaSuccess && c_in) {
      r = cudaMemcpyAsync(static_cast<char*>(ctx->stage[2]) + co,
                          static_cast<const char*>(c->data) + co, cn, cudaMemcpyHostToDevice,
                          ctx->copy_in);
      h2d += static_cast<int64_t>(cn);
    }
    if (r == cudaSuccess) r = cudaEventRecord(ctx->pev[kEvSlab + i], ctx->copy_in);
    return r;
  };

  int kernels = 0, used_method = method, splits = 1, nblock = 0;
  // Block (slab i, half h): the slab dimension shortened to the slab, the
  // halved dimension to the half, operands and C shifted accordingly
  // (uniform strides, so no scatter vector changes).
  auto block_args = [&](int i, int h) -> GemmArgs {
    const int64_t lo = i * sl.width, hi = std::min(len, lo + sl.width);
    const int64_t hlo = split ? h * half : 0, hhi = split ? (h ? rlen : half) : rlen;
    GemmArgs gs = g0;
    gs.A = ctx->stage[0];
    gs.B = ctx->stage[1];
    gs.C = ctx->stage[2];
    if (sl.along_n) {
      gs.N = hi - lo;
      gs.B = static_cast<const char*>(gs.B) + size_t(lo * hp.uB_n) * es;
      gs.C = static_cast<char*>(gs.C) + size_t(lo * hp.uC_n) * es;
      if (split) {
        gs.M = hhi - hlo;
        gs.A = static_cast<const char*>(gs.A) + size_t(hlo * hp.uA_m) * es;
        gs.C = static_cast<char*>(gs.C) + size_t(hlo * hp.uC_m) * es;
      }
    } else {
      gs.M = hi - lo;
      gs.A = static_cast<const char*>(gs.A) + size_t(lo * hp.uA_m) * es;
      gs.C = static_cast<char*>(gs.C) + size_t(lo * hp.uC_m) * es;
      if (split) {
        gs.N = hhi - hlo;
        gs.B = static_cast<const char*>(gs.B) + size_t(hlo * hp.uB_n) * es;
        gs.C = static_cast<char*>(gs.C) + size_t(hlo * hp.uC_n) * es;
      }
    }
    gs.k_per_split = hp.K;
    gs.c_split_stride = 0;
    return gs;
  };
  // Operand pieces: where the blocks run as pieces, the resident operand is
  // split once, half by half after its copy (on the context stream), into
  // its own workspace; every block then splits only its streamed slab.
  const int npieces = tc_pieces_count(method, dtype, block_args(0, 0), hp, ctx->tile_form);
  const int64_t ppitch = tc_pieces_pitch(hp.K);
  const int64_t prows = sl.along_n ? 2 * hp.M : hp.N;   // rows of the resident pieces
  const size_t pbytes = size_t(npieces) * size_t(prows) * size_t(ppitch) * 2u;
  const bool res_pieces =
      npieces > 0 && (ctx->opt_work_limit < 0 || pbytes <= size_t(ctx->opt_work_limit)) &&
      ensure_opt_work(s, &ctx->res_pieces, &ctx->res_pieces_bytes, pbytes);
  // Element offset of half h's first row in the resident pieces.
  auto pieces_row0 = [&](int h) -> int64_t {
    const int64_t hlo = split ? h * half : 0;
    return (sl.along_n ? 2 * hlo : hlo) * ppitch;
  };
  auto split_resident = [&](int h) -> cudaError_t {
    cudaStreamWaitEvent(s, ctx->pev[kEvRes + h], 0);
    void* out = static_cast<uint16_t*>(ctx->res_pieces) + pieces_row0(h);
    const cudaError_t r =
        tc_split_operand(npieces, sl.along_n, block_args(0, h), out, prows * ppitch, s);
    if (r == cudaSuccess) ++kernels;
    cudaEventRecord(ctx->pev[kEvResPieces + h], s);
    return r;
  };
  // The streamed operand's pieces: with the resident operand in halves, a
  // slab is used by two blocks; its first block splits it once into its own
  // rows of this workspace and the other block reuses them (the per-block
  // split did it twice: 16 splits of 42 MB moved at 4096^3 instead of 8).
  const int64_t srows = sl.along_n ? hp.N : 2 * hp.M;  // rows of the streamed pieces
  const size_t sbytes = size_t(npieces) * size_t(srows) * size_t(ppitch) * 2u;
  const bool slab_pieces =
      res_pieces && split &&
      (ctx->opt_work_limit < 0 || pbytes + sbytes <= size_t(ctx->opt_work_limit)) &&
      ensure_opt_work(s, &ctx->slab_pieces, &ctx->slab_pieces_bytes, sbytes);
  auto slab_row0 = [&](int i) -> int64_t {
    const int64_t lo = i * sl.width;
    return (sl.along_n ? lo : 2 * lo) * ppitch;
  };
  std::vector<char> slab_split(sl.count, 0);
  auto launch_block = [&](int i, int h) -> int {
    const int slot = nblock++ & 1;
    cudaStream_t cs = slot ? ctx->compute2 : s;
    cudaStreamWaitEvent(cs, ctx->pev[res_pieces ? kEvResPieces + h : kEvRes + h], 0);
    cudaStreamWaitEvent(cs, ctx->pev[kEvSlab + i], 0);
    const GemmArgs gs = block_args(i, h);
    PiecesReady ready;
    if (res_pieces) {
      const void* p = static_cast<const uint16_t*>(ctx->res_pieces) + pieces_row0(h);
      if (sl.along_n) {
        ready.a = p;
        ready.a_plane = prows * ppitch;
      } else {
        ready.b = p;
        ready.b_plane = prows * ppitch;
      }
    }
    if (slab_pieces) {
      void* sp = static_cast<uint16_t*>(ctx->slab_pieces) + slab_row0(i);
      if (!slab_split[i]) {
        const cudaError_t r = tc_split_operand(npieces, !sl.along_n, gs, sp, srows * ppitch, cs);
        if (r != cudaSuccess) return cuda_fail(ctx, r, "split streamed slab");
        ++kernels;
        cudaEventRecord(ctx->pev[kEvSlabPieces + i], cs);
        slab_split[i] = 1;
      } else {
        cudaStreamWaitEvent(cs, ctx->pev[kEvSlabPieces + i], 0);
      }
      if (sl.along_n) {
        ready.b = sp;
        ready.b_plane = srows * ppitch;
      } else {
        ready.a = sp;
        ready.a_plane = srows * ppitch;
      }
    }
    if (int st = launch_product(ctx, method, dtype, es, hp, gs, cs, &kernels, &used_method,
                                &splits, slot, false, res_pieces ? &ready : nullptr))
      return st;
    cudaEventRecord(ctx->pev[kEvDone + 2 * i + h], cs);
    return T1M_OK;
  };
  auto copy_back = [&](int i) -> cudaError_t {
    for (int h = 0; h < halves; ++h) cudaStreamWaitEvent(ctx->copy_out, ctx->pev[kEvDone + 2 * i + h], 0);
    const int64_t lo = i * sl.width, hi = std::min(len, lo + sl.width);
    const int64_t c0 = lo * sl.uc + sl.c_lo, c1 = (hi - 1) * sl.uc + sl.c_hi + 1;
    const size_t co = size_t(c0) * es, cn = size_t(c1 - c0) * es;
    d2h += static_cast<int64_t>(cn);
    return cudaMemcpyAsync(static_cast<char*>(c->data) + co,
                           static_cast<const char*>(ctx->stage[2]) + co, cn,
                           cudaMemcpyDeviceToHost, ctx->copy_out);
  };

  // Copies in order, each followed by the blocks it completes.
  if ((e = copy_resident(0)) != cudaSuccess) return cuda_fail(ctx, e, "copy resident operand");
  cudaEventRecord(ctx->pev[kEvRes], ctx->copy_in);
  if (res_pieces && (e = split_resident(0)) != cudaSuccess)
    return cuda_fail(ctx, e, "split resident operand");
  // Slabs before the second half: blocks of the first half keep the GPU busy
  // while the second half of the resident operand is copied.  When the
  // product's compute (estimated at 200 TFLOP/s on the tensor cores, 40 on
  // the plain kernel) outlasts the copies of all its operands, every slab's
  // first-half block goes first (the second half then arrives long before
  // the first-half blocks end); otherwise two, so that C slabs start going
  // back early.  Complex64 4096^3 (2.0 ms of compute, 1.3 ms of copies in):
  // two slabs left the GPU idle for about 0.2 ms while the second half of A
  // was in flight.
  const bool cplx = dtype == T1M_COMPLEX64 || dtype == T1M_COMPLEX128;
  const double est_flops = (cplx ? 8.0 : 2.0) * double(hp.M) * double(hp.N) * double(hp.K);
  const double est_compute_s = est_flops / (method == T1M_METHOD_PLAIN ? 40e12 : 200e12);
  const double est_copy_s = double(bytesA + bytesB + (readC ? bytesC : 0)) / 200e9;
  const int early = !split ? 0 : est_compute_s > est_copy_s ? sl.count : std::min(2, sl.count);
  for (int i = 0; i < early; ++i) {
    if ((e = copy_slab(i)) != cudaSuccess) return cuda_fail(ctx, e, "copy slab to device");
    if (int st = launch_block(i, 0)) return st;
  }
  if (split) {
    if ((e = copy_resident(1)) != cudaSuccess) return cuda_fail(ctx, e, "copy resident operand");
    cudaEventRecord(ctx->pev[kEvRes + 1], ctx->copy_in);
    if (res_pieces && (e = split_resident(1)) != cudaSuccess)
      return cuda_fail(ctx, e, "split resident operand");
    for (int i = 0; i < early; ++i) {
      if (int st = launch_block(i, 1)) return st;
      if ((e = copy_back(i)) != cudaSuccess) return cuda_fail(ctx, e, "copy C slab to host");
    }
  }
  for (int i = early; i < sl.count; ++i) {
    if ((e = copy_slab(i)) != cudaSuccess) return cuda_fail(ctx, e, "copy slab to device");
    for (int h = 0; h < halves; ++h)
      if (int st = launch_block(i, h)) return st;
    if ((e = copy_back(i)) != cudaSuccess) return cuda_fail(ctx, e, "copy C slab to host");
  }
  cudaEventRecord(ctx->pev[kEvOut], ctx->copy_out);
  cudaStreamWaitEvent(s, ctx->pev[kEvOut], 0);
  cudaEventRecord(ctx->pev[kEvC2], ctx->compute2);
  cudaStreamWaitEvent(s, ctx->pev[kEvC2], 0);
  if (timing) cudaEventRecord(ctx->ev[3], s);
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "contraction");
  if (int st = check_device_error(ctx)) return st;
  if (report) {
    std::memset(report, 0, sizeof(*report));
    report->method = used_method;
    report->split_k = splits;
    report->m = hp.M;
    report->n = hp.N;
    report->k = hp.K;
    const bool cplx = dtype == T1M_COMPLEX64 || dtype == T1M_COMPLEX128;
    report->flops = (cplx ? 8.0 : 2.0) * double(hp.M) * double(hp.N) * double(hp.K);
    report->h2d_bytes = h2d;
    report->d2h_bytes = d2h;
    report->kernels = kernels;
    report->path = ctx->last_path;
    if (timing) {
      // Copies and kernels overlap: the whole call is reported as kernel time.
      float t = 0;
      cudaEventElapsedTime(&t, ctx->ev[0], ctx->ev[3]);
      report->kernel_ms = t;
    }
  }
  return T1M_OK;
}

}  // namespace

extern "C" {

int t1m_version(int* major, int* minor, int* sm) {
  if (major) *major = 0;
  if (minor) *minor = 1;
  if (sm) *sm = 103;
  return T1M_OK;
}

const char* t1m_status_string(int status) {
  switch (status) {
    case T1M_OK: return "success";
    case T1M_ERR_INVALID_ARGUMENT: return "invalid argument";
    case T1M_ERR_LABELS: return "invalid labels or extents";
    case T1M_ERR_ALLOC: return "allocation failed";
    case T1M_ERR_CUDA: return "CUDA error";
    case T1M_ERR_UNSUPPORTED: return "unsupported method for this contraction";
    case T1M_ERR_KERNEL_TIMEOUT: return "device-side wait timed out";
    case T1M_ERR_NO_DEVICE: return "no usable CUDA device";
  }
  return "unknown status";
}

const char* t1m_last_error(const t1m_context* ctx) {
  return ctx ? ctx->last_error.c_str() : "null context";
}

int t1m_create(t1m_context** out, int device) {
  if (!out) return T1M_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= device || device < 0) {
    cudaGetLastError();
    return T1M_ERR_NO_DEVICE;
  }
  cudaDeviceProp prop{};
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return T1M_ERR_NO_DEVICE;
  if (prop.major != 10 || prop.minor != 3) return T1M_ERR_NO_DEVICE;  // sm_103 only
  auto* ctx = new (std::nothrow) t1m_context();
  if (!ctx) return T1M_ERR_ALLOC;
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
  for (int i = 0; i < 6 && e == cudaSuccess; ++i) e = cudaEventCreate(&ctx->ev[i]);
  for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaEventCreate(&ctx->mev[i]);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->copy_in, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->copy_out, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->compute2, cudaStreamNonBlocking);
  for (int i = 0; i < t1m_context::kPipeEvents && e == cudaSuccess; ++i)
    e = cudaEventCreateWithFlags(&ctx->pev[i], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_err, 64);
  if (e == cudaSuccess) e = cudaMemset(ctx->d_err, 0, 64);
  if (e != cudaSuccess) {
    t1m_destroy(ctx);
    return T1M_ERR_CUDA;
  }
  ctx->stream = ctx->own_stream;
  ctx->num_sms = prop.multiProcessorCount;
  int khz = 0;
  if (cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, device) == cudaSuccess && khz > 0)
    ctx->clock_khz = khz;
  *out = ctx;
  return T1M_OK;
}

int t1m_set_autotune(t1m_context* ctx, int on) {
  if (!ctx) return T1M_ERR_INVALID_ARGUMENT;
  ctx->autotune = on != 0;
  return T1M_OK;
}

int t1m_set_wait_limit(t1m_context* ctx, int64_t microseconds) {
  if (!ctx || microseconds < 0) return T1M_ERR_INVALID_ARGUMENT;
  ctx->wait_limit_us = microseconds;
  return T1M_OK;
}

int t1m_set_tile_form(t1m_context* ctx, int form) {
  if (!ctx || form < T1M_TILE_AUTO || form > T1M_TILE_PIECES) return T1M_ERR_INVALID_ARGUMENT;
  ctx->tile_form = form;
  return T1M_OK;
}

int t1m_set_workspace_limit(t1m_context* ctx, int64_t bytes) {
  if (!ctx || bytes < -1) return T1M_ERR_INVALID_ARGUMENT;
  ctx->opt_work_limit = bytes;
  return T1M_OK;
}

int t1m_set_split_k(t1m_context* ctx, int splits) {
  if (!ctx || splits < 0 || splits > 4096) return T1M_ERR_INVALID_ARGUMENT;
  ctx->split_k = splits;
  return T1M_OK;
}

int t1m_destroy(t1m_context* ctx) {
  if (!ctx) return T1M_ERR_INVALID_ARGUMENT;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (auto& e : ctx->plans) cudaFree(e.dev.block);
  for (int i = 0; i < 3; ++i)
    if (ctx->stage[i]) cudaFree(ctx->stage[i]);
  for (int i = 0; i < 6; ++i)
    if (ctx->ev[i]) cudaEventDestroy(ctx->ev[i]);
  for (int i = 0; i < 2; ++i)
    if (ctx->mev[i]) cudaEventDestroy(ctx->mev[i]);
  if (ctx->d_err) cudaFree(ctx->d_err);
  if (ctx->work) cudaFree(ctx->work);
  if (ctx->fix_ctr) cudaFree(ctx->fix_ctr);
  for (int i = 0; i < 2; ++i) {
    if (ctx->panel[i]) cudaFree(ctx->panel[i]);
    if (ctx->pack[i]) cudaFree(ctx->pack[i]);
  }
  if (ctx->res_pieces) cudaFree(ctx->res_pieces);
  if (ctx->slab_pieces) cudaFree(ctx->slab_pieces);
  if (ctx->compute2) {
    cudaStreamSynchronize(ctx->compute2);
    cudaStreamDestroy(ctx->compute2);
  }
  for (int i = 0; i < t1m_context::kPipeEvents; ++i)
    if (ctx->pev[i]) cudaEventDestroy(ctx->pev[i]);
  if (ctx->copy_in) {
    cudaStreamSynchronize(ctx->copy_in);
    cudaStreamDestroy(ctx->copy_in);
  }
  if (ctx->copy_out) {
    cudaStreamSynchronize(ctx->copy_out);
    cudaStreamDestroy(ctx->copy_out);
  }
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
  return T1M_OK;
}

int t1m_set_stream(t1m_context* ctx, void* stream) {
  if (!ctx) return T1M_ERR_INVALID_ARGUMENT;
  const cudaStream_t next = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
  // The context's workspaces (split-K partials, B panels) are reused by every
  // call: work queued on the previous stream finishes before the switch.
  if (next != ctx->stream && ctx->stream) {
    cudaSetDevice(ctx->device);
    const cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "drain the previous stream");
  }
  ctx->stream = next;
  return T1M_OK;
}

int t1m_set_method(t1m_context* ctx, int method) {
  if (!ctx || method < T1M_METHOD_AUTO || method > T1M_METHOD_DMMA)
    return T1M_ERR_INVALID_ARGUMENT;
  ctx->method = method;
  return T1M_OK;
}

int t1m_synchronize(t1m_context* ctx) {
  if (!ctx) return T1M_ERR_INVALID_ARGUMENT;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "synchronize");
  return check_device_error(ctx);
}

int t1m_analyze(int dtype, const t1m_tensor* a, const char* la, const t1m_tensor* b,
                const char* lb, const t1m_tensor* c, const char* lc, t1m_plan_info* info,
                char* err, int32_t err_len) {
  auto report = [&](int st, const std::string& msg) {
    if (err && err_len > 0) {
      std::strncpy(err, msg.c_str(), static_cast<size_t>(err_len) - 1);
      err[err_len - 1] = 0;
    }
    return st;
  };
  if (!a || !b || !c || !la || !lb || !lc) return report(T1M_ERR_INVALID_ARGUMENT, "null argument");
  if (elem_size(dtype) == 0) return report(T1M_ERR_INVALID_ARGUMENT, "unknown dtype");
  for (const t1m_tensor* t : {a, b, c}) {
    if (t->ndim < 0 || t->ndim > 64 || (t->ndim > 0 && !t->extents))
      return report(T1M_ERR_INVALID_ARGUMENT, "bad tensor rank or extents");
    if (t->layout < T1M_ROW_MAJOR || t->layout > T1M_STRIDED)
      return report(T1M_ERR_INVALID_ARGUMENT, "bad layout");
  }
  int64_t sa[64], sb[64], sc[64];
  if (!resolve_strides(a, sa) || !resolve_strides(b, sb) || !resolve_strides(c, sc))
    return report(T1M_ERR_INVALID_ARGUMENT, "strided tensor without strides");
  HostPlan hp;
  std::string msg;
  const int st = build_plan(dtype, a->ndim, a->extents, sa, la, b->ndim, b->extents, sb, lb,
                            c->ndim, c->extents, sc, lc, &hp, &msg);
  if (st != T1M_OK) return report(st, msg);
  if (info) {
    info->m = hp.M;
    info->n = hp.N;
    info->k = hp.K;
    info->modes_m = static_cast<int32_t>(hp.modes_m.size());
    info->modes_n = static_cast<int32_t>(hp.modes_n.size());
    info->modes_k = static_cast<int32_t>(hp.modes_k.size());
    info->reserved = 0;
  }
  return report(T1M_OK, "");
}

int t1m_contract(t1m_context* ctx, int dtype, const void* alpha, const t1m_tensor* a,
                 const char* la, const t1m_tensor* b, const char* lb, const void* beta,
                 const t1m_tensor* c, const char* lc, uint32_t flags, t1m_report* report) {
  if (!ctx) return T1M_ERR_INVALID_ARGUMENT;
  if (!a || !b || !c || !la || !lb || !lc || !alpha || !beta)
    return fail(ctx, T1M_ERR_INVALID_ARGUMENT, "null argument");
  const size_t es = elem_size(dtype);
  if (es == 0) return fail(ctx, T1M_ERR_INVALID_ARGUMENT, "unknown dtype");
  for (const t1m_tensor* t : {a, b, c}) {
    if (t->ndim < 0 || t->ndim > 64 || (t->ndim > 0 && !t->extents))
      return fail(ctx, T1M_ERR_INVALID_ARGUMENT, "bad tensor rank or extents");
    if (t->layout < T1M_ROW_MAJOR || t->layout > T1M_STRIDED)
      return fail(ctx, T1M_ERR_INVALID_ARGUMENT, "bad layout");
  }
  int64_t sa[64], sb[64], sc[64];
  if (!resolve_strides(a, sa) || !resolve_strides(b, sb) || !resolve_strides(c, sc))
    return fail(ctx, T1M_ERR_INVALID_ARGUMENT, "strided tensor without strides");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "set device");
  ctx->last_path = 0;

  // Plan (cached).
  const std::string key = plan_key(dtype, a, sa, la, b, sb, lb, c, sc, lc);
  t1m_context::Entry* entry = nullptr;
  auto it = ctx->index.find(key);
  if (it != ctx->index.end()) {
    ctx->plans.splice(ctx->plans.begin(), ctx->plans, it->second);
    entry = &*ctx->plans.begin();
  } else {
    t1m_context::Entry fresh;
    fresh.key = key;
    std::string err;
    int st = build_plan(dtype, a->ndim, a->extents, sa, la, b->ndim, b->extents, sb, lb,
                        c->ndim, c->extents, sc, lc, &fresh.host, &err);
    if (st != T1M_OK) return fail(ctx, st, err);
    st = upload_plan(ctx, fresh.host, &fresh.dev);
    if (st != T1M_OK) return st;
    ctx->plans.push_front(std::move(fresh));
    ctx->index[key] = ctx->plans.begin();
    entry = &*ctx->plans.begin();
    while (ctx->plans.size() > kMaxPlans) {
      auto& last = ctx->plans.back();
      cudaStreamSynchronize(ctx->stream);
      cudaFree(last.dev.block);
      ctx->index.erase(last.key);
      ctx->plans.pop_back();
    }
  }
  const HostPlan& hp = entry->host;
  const DevicePlan& dp = entry->dev;

  if (hp.spanC > 0 && !c->data) return fail(ctx, T1M_ERR_INVALID_ARGUMENT, "null C data");
  if (hp.M > 0 && hp.N > 0 && hp.K > 0 && (!a->data || !b->data))
    return fail(ctx, T1M_ERR_INVALID_ARGUMENT, "null A or B data");

  const int method = choose_method(ctx, dtype, hp);
  const bool timing = report && !(flags & T1M_FLAG_NO_TIMING);
  const bool cplx = dtype == T1M_COMPLEX64 || dtype == T1M_COMPLEX128;

  // Scalars (the reference's complex overload has alpha = 1, t1m.h:576).
  GemmArgs g{};
  g.M = hp.M; g.N = hp.N; g.K = hp.K;
  g.rsA = dp.rsA; g.csA = dp.csA; g.rsB = dp.rsB; g.csB = dp.csB;
  g.rsC = dp.rsC; g.csC = dp.csC;
  g.uA_m = hp.uA_m; g.uA_k = hp.uA_k; g.uB_k = hp.uB_k; g.uB_n = hp.uB_n;
  g.uC_m = hp.uC_m; g.uC_n = hp.uC_n;
  auto read_scalar = [&](const void* p, double* out) {
    switch (dtype) {
      case T1M_FLOAT32: out[0] = *static_cast<const float*>(p); out[1] = 0; break;
      case T1M_FLOAT64: out[0] = *static_cast<const double*>(p); out[1] = 0; break;
      case T1M_COMPLEX64: out[0] = static_cast<const float*>(p)[0]; out[1] = static_cast<const float*>(p)[1]; break;
      case T1M_COMPLEX128: out[0] = static_cast<const double*>(p)[0]; out[1] = static_cast<const double*>(p)[1]; break;
    }
  };
  read_scalar(alpha, g.alpha);
  read_scalar(beta, g.beta);
  g.flags = 0;
  if (flags & T1M_FLAG_ACCUMULATE) g.flags |= kFlagAccumulate;
  if ((flags & T1M_FLAG_CONJ_A) && cplx) g.flags |= kFlagConjA;
  if ((flags & T1M_FLAG_CONJ_B) && cplx) g.flags |= kFlagConjB;
  if (!(flags & T1M_FLAG_ACCUMULATE) && g.beta[0] == 0.0 && g.beta[1] == 0.0)
    g.flags |= kFlagBetaZero;

  // Host operands are staged.
  const bool devA = is_device_pointer(a->data), devB = is_device_pointer(b->data),
             devC = is_device_pointer(c->data);
  const size_t bytesA = static_cast<size_t>(hp.spanA) * es;
  const size_t bytesB = static_cast<size_t>(hp.spanB) * es;
  const size_t bytesC = static_cast<size_t>(hp.spanC) * es;
  const bool readC = (g.flags & kFlagAccumulate) || !(g.flags & kFlagBetaZero) || hp.K == 0;
  int64_t h2d = 0, d2h = 0;
  cudaStream_t s = ctx->stream;

  // All operands in host memory and large: slab pipeline (copies overlap the
  // kernels).  Not with forced split-K, and only where every slab runs
  // without split-K.
  Slabs sl;
  if (!devA && !devB && !devC && ctx->split_k == 0 && bytesA + bytesB + bytesC >= kPipelineMinBytes &&
      plan_slabs(hp, es, &sl)) {
    int64_t kps = 0;
    const int64_t sm = sl.along_n ? hp.M : sl.width, sn = sl.along_n ? sl.width : hp.N;
    if (method == T1M_METHOD_PLAIN || method == T1M_METHOD_DMMA || tc_supported(method, dtype, hp))
      if (choose_splits(ctx, method, dtype, sm, sn, hp.K, es, &kps,
                        ctx->method == T1M_METHOD_AUTO) == 1)
        return run_pipelined(ctx, method, dtype, es, hp, g, a, b, c, sl, readC, timing, report);
  }

  if (timing) cudaEventRecord(ctx->ev[0], s);
  g.A = a->data;
  g.B = b->data;
  g.C = c->data;
  if (!devA && bytesA) {
    if (int st = ensure_stage(ctx, 0, bytesA)) return st;
    if ((e = cudaMemcpyAsync(ctx->stage[0], a->data, bytesA, cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return cuda_fail(ctx, e, "copy A to device");
    g.A = ctx->stage[0];
    h2d += bytesA;
  }
  if (!devB && bytesB) {
    if (int st = ensure_stage(ctx, 1, bytesB)) return st;
    if ((e = cudaMemcpyAsync(ctx->stage[1], b->data, bytesB, cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return cuda_fail(ctx, e, "copy B to device");
    g.B = ctx->stage[1];
    h2d += bytesB;
  }
  if (!devC && bytesC) {
    if (int st = ensure_stage(ctx, 2, bytesC)) return st;
    if (readC || hp.spanC != hp.M * hp.N * hp.batch) {
      // C's gaps (strided C) must survive the copy back, so it is read too.
      if ((e = cudaMemcpyAsync(ctx->stage[2], c->data, bytesC, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_fail(ctx, e, "copy C to device");
      h2d += bytesC;
    }
    g.C = ctx->stage[2];
  }
  if (timing) cudaEventRecord(ctx->ev[1], s);
  ctx->mev_armed = timing;
  ctx->mev_recorded = false;

  int kernels = 0;
  int used_method = method;
  int splits = 1;
  // Batch labels: one product per batch index, operands shifted by the
  // index's offsets (the loop runs once without batch labels).
  const GemmArgs g_all = g;
  for (int64_t bi = 0; bi < hp.batch && hp.M > 0 && hp.N > 0; ++bi) {
    int64_t oa, ob, oc;
    batch_offsets(hp, bi, &oa, &ob, &oc);
    g = g_all;
    g.A = static_cast<const char*>(g_all.A) + oa * static_cast<int64_t>(es);
    g.B = static_cast<const char*>(g_all.B) + ob * static_cast<int64_t>(es);
    g.C = static_cast<char*>(g_all.C) + oc * static_cast<int64_t>(es);
    g.k_per_split = std::max<int64_t>(hp.K, 1);
    g.c_split_stride = 0;
    const int st = launch_product(ctx, method, dtype, es, hp, g, s, &kernels, &used_method,
                                  &splits, 0, true);
    if (st) {
      ctx->mev_armed = false;
      return st;
    }
  }
  ctx->mev_armed = false;
  if (timing) cudaEventRecord(ctx->ev[2], s);
  if (!devC && bytesC) {
    if ((e = cudaMemcpyAsync(c->data, ctx->stage[2], bytesC, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
      return cuda_fail(ctx, e, "copy C to host");
    d2h += bytesC;
  }
  if (timing) cudaEventRecord(ctx->ev[3], s);
  const bool host_result = (!devC && bytesC);
  if (host_result || timing) {
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "contraction");
    if (int st = check_device_error(ctx)) return st;
  }
  if (report) {
    std::memset(report, 0, sizeof(*report));
    report->method = used_method;
    report->split_k = splits;
    report->m = hp.M;
    report->n = hp.N;
    report->k = hp.K;
    report->flops =
        (cplx ? 8.0 : 2.0) * double(hp.M) * double(hp.N) * double(hp.K) * double(hp.batch);
    report->h2d_bytes = h2d;
    report->d2h_bytes = d2h;
    report->kernels = kernels;
    report->path = ctx->last_path;
    if (timing) {
      float t01 = 0, t12 = 0, t23 = 0;
      cudaEventElapsedTime(&t01, ctx->ev[0], ctx->ev[1]);
      cudaEventElapsedTime(&t12, ctx->ev[1], ctx->ev[2]);
      cudaEventElapsedTime(&t23, ctx->ev[2], ctx->ev[3]);
      report->h2d_ms = t01;
      report->kernel_ms = t12;
      report->d2h_ms = t23;
      float tm = 0;
      if (ctx->mev_recorded && cudaEventElapsedTime(&tm, ctx->mev[0], ctx->mev[1]) == cudaSuccess)
        report->main_ms = tm;
    }
  }
  return T1M_OK;
}

}  // extern "C"

extern "C" int t1m_contract_vjp(t1m_context* ctx, int dtype, const t1m_tensor* dc,
                                const char* lc, const t1m_tensor* a, const char* la,
                                const t1m_tensor* b, const char* lb, const t1m_tensor* da,
                                const t1m_tensor* db, uint32_t flags, t1m_report* report) {
  if (!ctx) return T1M_ERR_INVALID_ARGUMENT;
  if (!dc || !a || !b || !lc || !la || !lb) return fail(ctx, T1M_ERR_INVALID_ARGUMENT, "null argument");
  if (elem_size(dtype) == 0) return fail(ctx, T1M_ERR_INVALID_ARGUMENT, "unknown dtype");
  // One and zero of the dtype (complex: re, im).
  const double one_d[2] = {1.0, 0.0}, zero_d[2] = {0.0, 0.0};
  const float one_f[2] = {1.0f, 0.0f}, zero_f[2] = {0.0f, 0.0f};
  const bool single = dtype == T1M_FLOAT32 || dtype == T1M_COMPLEX64;
  const void* one = single ? static_cast<const void*>(one_f) : static_cast<const void*>(one_d);
  const void* zero = single ? static_cast<const void*>(zero_f) : static_cast<const void*>(zero_d);
  const uint32_t base = flags & (T1M_FLAG_ACCUMULATE | T1M_FLAG_NO_TIMING);
  t1m_report r1{}, r2{};
  if (da) {
    // dA[la] = sum over the free-B labels of dC[lc] * conj(B[lb]).
    const int st = t1m_contract(ctx, dtype, one, dc, lc, b, lb, zero, da, la,
                                base | T1M_FLAG_CONJ_B, report ? &r1 : nullptr);
    if (st != T1M_OK) return st;
  }
  if (db) {
    // dB[lb] = sum over the free-A labels of conj(A[la]) * dC[lc].
    const int st = t1m_contract(ctx, dtype, one, a, la, dc, lc, zero, db, lb,
                                base | T1M_FLAG_CONJ_A, report ? &r2 : nullptr);
    if (st != T1M_OK) return st;
  }
  if (report) {
    *report = da ? r1 : r2;
    if (da && db) {
      report->flops = r1.flops + r2.flops;
      report->kernel_ms = r1.kernel_ms + r2.kernel_ms;
      report->h2d_ms = r1.h2d_ms + r2.h2d_ms;
      report->d2h_ms = r1.d2h_ms + r2.d2h_ms;
      report->h2d_bytes = r1.h2d_bytes + r2.h2d_bytes;
      report->d2h_bytes = r1.d2h_bytes + r2.d2h_bytes;
      report->kernels = r1.kernels + r2.kernels;
      report->path = r2.path;
    }
  }
  return T1M_OK;
}

// ------------------------------------------------------------ grouped ---
// A batch of contractions (e.g. the updates of a tensor-network sweep) run
// as grouped launches: every complex64 contraction with enough rows and
// columns is a list of tiles of ONE persistent tensor-core launch; the rest
// (other dtypes, skinny outputs) are tiles of one grouped plain launch per
// tile shape.  Items may read the C of an earlier item (depends_on); when all
// items are tensor-core items the dependencies are resolved inside the one
// persistent launch, otherwise items run in dependency levels.  Optionally
// the whole batch is captured once in a CUDA graph.  The reference has no
// batching; its counterpart is a loop of t1m::contract calls.
#include "tc.h"

namespace {

enum Family : int { kFamTC = 0, kFamSimt = 1, kFamSimtSkinny = 2, kFamReduce = 3 };

// Split-K inside a grouped launch: every tile covers at most kGroupKCap
// complex (or real) K, so one long-K item (a skinny output over a big
// contracted bundle) spreads over many CTAs instead of leaving a tail of
// serial tiles; partials go to the group's workspace and one reduction per
// dependency level applies the epilogues.
constexpr int64_t kGroupKCap = 1024;
constexpr size_t kGroupWorkBytes = size_t(2) << 30;
constexpr size_t kGroupItemWorkBytes = size_t(256) << 20;

int group_splits(int dtype, int fam, const HostPlan& hp, size_t es, int64_t* k_per_split) {
  int bm = 0, bn = 0, bk = 0;
  if (fam == kFamTC) {
    tc_tile(dtype, &bm, &bn, &bk);
  } else {
    simt_tile(dtype, &bm, &bn, &bk);
    if (fam == kFamSimtSkinny) bk = 16;
  }
  const int64_t ksteps = std::max<int64_t>(1, (hp.K + bk - 1) / bk);
  // Families are chosen by the library, so the AUTO precision rule applies:
  // plain tiles accumulate sequentially and cover at most its K limit (the
  // skinny kernel's lanes each sum a 1/32 share, the tensor-core limit is
  // above the cap).
  int64_t cap = kGroupKCap;
  if (fam == kFamSimt) {
    const int64_t lim = accuracy_k_limit(T1M_METHOD_PLAIN, dtype);
    if (lim > 0) cap = std::min(cap, lim);
  }
  const int64_t cap_steps = std::max<int64_t>(1, cap / bk);
  int64_t s = (ksteps + cap_steps - 1) / cap_steps;
  s = std::max<int64_t>(1, std::min<int64_t>(s, 4096));
  while (s > 1 && size_t(s) * size_t(hp.M) * size_t(hp.N) * es > kGroupItemWorkBytes) --s;
  const int64_t steps_per = (ksteps + s - 1) / s;
  *k_per_split = steps_per * bk;
  return static_cast<int>((ksteps + steps_per - 1) / steps_per);
}

// Arguments of the main kernel of a split item: raw partial products (alpha 1,
// beta 0) into `splits` dense M x N slices of `work`, m fastest.
GemmArgs split_args(const GemmArgs& a, void* work, int64_t k_per_split) {
  GemmArgs w = a;
  w.C = work;
  w.rsC = nullptr;
  w.csC = nullptr;
  w.uC_m = 1;
  w.uC_n = a.M;
  w.alpha[0] = 1.0;
  w.alpha[1] = 0.0;
  w.beta[0] = w.beta[1] = 0.0;
  w.flags = (a.flags & (kFlagConjA | kFlagConjB)) | kFlagBetaZero;
  w.k_per_split = k_per_split;
  w.c_split_stride = a.M * a.N;
  return w;
}

// Autotuner cache: shape class -> family, measured once per process and
// persisted to a small versioned text file (T1M_TUNE_CACHE, default
// $HOME/.cache/t1m_gb300_tune.txt) keyed by GPU name, SM count and driver.
struct TuneCache {
  std::mutex mu;
  bool loaded = false;
  std::string path, header;
  std::unordered_map<std::string, int> choice;

  void load(int device) {
    const char* env_now = std::getenv("T1M_TUNE_CACHE");
    const char* home_now = std::getenv("HOME");
    const std::string want =
        env_now ? env_now : (home_now ? std::string(home_now) + "/.cache/t1m_gb300_tune.txt" : "");
    if (loaded && want == path) return;  // same file: the in-memory table is current
    loaded = true;
    choice.clear();
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, device);
    int drv = 0;
    cudaDriverGetVersion(&drv);
    header = std::string("t1m_gb300-tune v2 ") + prop.name + " sms=" +
             std::to_string(prop.multiProcessorCount) + " driver=" + std::to_string(drv);
    for (char& ch : header)
      if (ch == '\n') ch = ' ';
    const char* env = std::getenv("T1M_TUNE_CACHE");
    const char* home = std::getenv("HOME");
    path = env ? env : (home ? std::string(home) + "/.cache/t1m_gb300_tune.txt" : "");
    if (path.empty()) return;
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) return;
    char line[512];
    bool ok = std::fgets(line, sizeof(line), f) && header == std::string(line).substr(0, header.size());
    while (ok && std::fgets(line, sizeof(line), f)) {
      char key[400];
      int fam = 0;
      if (std::sscanf(line, "%399s %d", key, &fam) == 2) choice[key] = fam;
    }
    std::fclose(f);
  }
  void save() {
    if (path.empty()) return;
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) return;
    std::fprintf(f, "%s\n", header.c_str());
    for (auto& kv : choice) std::fprintf(f, "%s %d\n", kv.first.c_str(), kv.second);
    std::fclose(f);
  }
};
TuneCache g_tune;

int log2_bucket(int64_t v) {
  int b = 0;
  while ((int64_t(1) << (b + 1)) <= v) ++b;
  return b;
}

std::string shape_class(int dtype, const HostPlan& hp) {
  return std::to_string(dtype) + ":" + std::to_string(log2_bucket(hp.M)) + "," +
         std::to_string(log2_bucket(hp.N)) + "," + std::to_string(log2_bucket(hp.K));
}

// Single tensor-core products: per shape class (dtype, method, log2 of M, N,
// K, which operand directions have unit stride), the tile form (one CTA or
// CTA pairs) and the split count (the heuristic one, half or twice it, never
// below the precision rule's minimum) that ran fastest, measured once on
// the call's own operands into scratch outputs (the split workspace: the
// partials and a dense M x N result), three runs each after a warm-up.
// Choice code: form * 100 + split variant.
bool tuned_product(t1m_context* ctx, int method, int dtype, size_t es, const HostPlan& hp,
                   const GemmArgs& g, cudaStream_t s, int slot, int* form, int* splits,
                   int64_t* k_per_split) {
  int bm, bn, bk;
  tc_tile(dtype, &bm, &bn, &bk);
  const int64_t ksteps = (g.K + bk - 1) / bk;
  int64_t kps0 = 0;
  const int s0 = choose_splits(ctx, method, dtype, g.M, g.N, g.K, es, &kps0,
                               ctx->method == T1M_METHOD_AUTO);
  const int64_t lim = ctx->method == T1M_METHOD_AUTO ? accuracy_k_limit(method, dtype) : 0;
  const int64_t smin = lim > 0 ? (g.K + lim - 1) / lim : 1;
  auto variant = [&](int v) {
    int64_t sp = v == 0 ? s0 : v == 1 ? (s0 + 1) / 2 : 2 * int64_t(s0);
    sp = std::max<int64_t>({sp, smin, 1});
    sp = std::min<int64_t>({sp, ksteps, 4096});
    while (sp > 1 && size_t(sp + 1) * size_t(g.M) * size_t(g.N) * es > kMaxWorkBytes) --sp;
    const int64_t steps_per = (ksteps + sp - 1) / sp;
    *k_per_split = steps_per * bk;
    return static_cast<int>((ksteps + steps_per - 1) / steps_per);
  };
  const std::string key = "s:" + std::to_string(dtype) + ":" + std::to_string(method) + ":" +
                          std::to_string(log2_bucket(g.M)) + "," + std::to_string(log2_bucket(g.N)) +
                          "," + std::to_string(log2_bucket(g.K)) + ":" +
                          std::to_string(int(hp.uA_m == 1)) + std::to_string(int(hp.uA_k == 1)) +
                          std::to_string(int(hp.uB_k == 1)) + std::to_string(int(hp.uB_n == 1));
  std::lock_guard<std::mutex> lock(g_tune.mu);
  g_tune.load(ctx->device);
  auto it = g_tune.choice.find(key);
  int code = -1;
  if (it != g_tune.choice.end()) {
    code = it->second;
  } else {
    float best = 1e30f;
    for (int f : {T1M_TILE_ONE, T1M_TILE_PAIR, T1M_TILE_PIECES}) {
      // Pieces only where they run (else the same as pairs).
      if (f == T1M_TILE_PIECES && tc_pieces_count(method, dtype, g, hp, f) == 0) continue;
      int last_sp = -1;
      for (int v = 0; v < 3; ++v) {
        const int sp = variant(v);
        const int64_t kps = *k_per_split;
        if (sp == last_sp) continue;
        last_sp = sp;
        const size_t need = size_t(sp + 1) * size_t(g.M) * size_t(g.N) * es;
        if (ensure_work(ctx, need) != T1M_OK) return false;
        char* work = static_cast<char*>(ctx->work);
        // Raw partials (or the one dense result) into the workspace; the
        // reduction writes a dense M x N scratch after them.
        GemmArgs gm = g;
        gm.C = work;
        gm.rsC = gm.csC = nullptr;
        gm.uC_m = 1;
        gm.uC_n = g.M;
        gm.alpha[0] = 1.0;
        gm.alpha[1] = 0.0;
        gm.beta[0] = gm.beta[1] = 0.0;
        gm.flags = (g.flags & (kFlagConjA | kFlagConjB)) | kFlagBetaZero;
        gm.k_per_split = sp > 1 ? kps : g.K;
        gm.c_split_stride = sp > 1 ? g.M * g.N : 0;
        GemmArgs red = gm;
        red.C = work + size_t(sp) * size_t(g.M) * size_t(g.N) * es;
        const size_t pb = std::max(tc_panel_bytes(dtype, gm.M, gm.N, gm.K),
                                   tc_pieces_count(method, dtype, gm, hp, f) > 0
                                       ? tc_pieces_bytes(dtype, method, gm.M, gm.N, gm.K)
                                       : size_t(0));
        const bool pan = pb > 0 && (ctx->opt_work_limit < 0 || pb <= size_t(ctx->opt_work_limit)) &&
                         ensure_opt_work(s, &ctx->panel[slot], &ctx->panel_bytes[slot], pb);
        const size_t kb = tc_pack_bytes(dtype, hp);
        const bool pk = kb > 0 && (ctx->opt_work_limit < 0 || kb <= size_t(ctx->opt_work_limit)) &&
                        ensure_opt_work(s, &ctx->pack[slot], &ctx->pack_bytes[slot], kb);
        float total = 0;
        bool ok = true;
        for (int rep = 0; rep < 4 && ok; ++rep) {
          cudaEventRecord(ctx->ev[4], s);
          int nk = 0, ran = method;
          std::string err;
          cudaError_t e = launch_tc(method, dtype, gm, hp, sp, s, ctx->d_err, &nk, &err, &ran,
                                    pan ? ctx->panel[slot] : nullptr,
                                    pan ? ctx->panel_bytes[slot] : 0,
                                    pk ? ctx->pack[slot] : nullptr, pk ? ctx->pack_bytes[slot] : 0,
                                    nullptr, f);
          if (e == cudaSuccess && sp > 1) e = launch_splitk_reduce(dtype, work, sp, red, s);
          cudaEventRecord(ctx->ev[5], s);
          if (e != cudaSuccess || cudaEventSynchronize(ctx->ev[5]) != cudaSuccess) {
            cudaGetLastError();
            ok = false;
            break;
          }
          float ms = 0;
          cudaEventElapsedTime(&ms, ctx->ev[4], ctx->ev[5]);
          if (rep > 0) total += ms;  // the first run warms up
        }
        if (ok && total < best) {
          best = total;
          code = f * 100 + v;
        }
      }
    }
    if (code < 0) return false;
    if (check_device_error(ctx) != T1M_OK) return false;
    g_tune.choice[key] = code;
    g_tune.save();
  }
  *form = code / 100;
  *splits = variant(code % 100);
  return true;
}

// Main-product chunk length of a one-launch item (log2 of stages): narrow
// outputs (at most 32 columns, the long-K reductions of a sweep's second
// steps, whose outputs are sums of many terms of either sign) fold every
// stage, which keeps the truncation bias of the tensor cores' accumulation
// per chunk at 4 MMAs instead of 16; their converters fold at most 32
// columns, so the extra folds cost little.  Wider tiles keep four stages.
int group_fold_shift(int tile_n) { return tile_n <= 32 ? 0 : 2; }

// Tile choice of a one-launch item: a tensor-core width or a SIMT tile.
constexpr int kWidthSimt = 1;
bool prepare_group_tc(const GemmArgs& g, const HostPlan& hp, int splits, int width,
                      TcProblem* tp) {
  const bool simt = width == kWidthSimt;
  if (simt && hp.N > kTcSkinnyMaxN) return false;
  if (!tc_prepare(g, hp, splits, tp, simt ? 16 : width)) return false;
  tp->skinny = simt ? 1 : 0;
  tp->fold_shift = group_fold_shift(tp->tile_n);
  return true;
}

// Default family before (or without) tuning.
int heuristic_family(int dtype, const HostPlan& hp) {
  if (dtype == T1M_COMPLEX64 && hp.M >= 32 && hp.N >= 32) return kFamTC;
  return hp.N <= 16 ? kFamSimtSkinny : kFamSimt;
}

}  // namespace

struct t1m_group {
  t1m_context* ctx = nullptr;
  int dtype = 0;
  int n = 0;
  double flops = 0;
  void* vectors = nullptr;      // all scatter vectors of all items
  void* tc_dev = nullptr;       // TcProblem array
  int* done = nullptr;          // tile-completion counters, then split-K arrival counters
  int64_t fix_count = 0;        // split-K arrival counters (after the tc_count done counters)
  bool deps = false;            // the single launch resolves dependencies (cooperative)
  void* simt_dev = nullptr;     // SimtProblem arrays, per (level, family)
  void* reduce_dev = nullptr;   // SplitReduce arrays, per level
  void* work = nullptr;         // split-K partials of all split items
  struct Launch {
    int family;
    int64_t offset;   // first descriptor in tc_dev / simt_dev
    int count;
    int64_t tiles;
    int nmax = 16;    // skinny launches: column bound of the kernel (4 or 16)
  };
  std::vector<std::vector<Launch>> levels;
  bool single_tc = false;
  int64_t tc_total = 0;
  int tc_count = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int kernels = 0;
};

namespace {

int enqueue_group(t1m_group* g, cudaStream_t s) {
  t1m_context* ctx = g->ctx;
  cudaError_t e = cudaSuccess;
  int kernels = 0;
  if (g->single_tc) {
    // Counters start at zero every launch (the fix counters also reset
    // themselves in the kernel; a launch cut short by a timeout may not).
    e = cudaMemsetAsync(g->done, 0, sizeof(int) * size_t(g->tc_count + g->fix_count), s);
    if (e == cudaSuccess)
      e = tc_launch_persistent(nullptr, static_cast<const TcProblem*>(g->tc_dev), g->tc_count,
                               g->tc_total, ctx->num_sms, g->deps ? g->done : nullptr, s,
                               ctx->d_err, g->fix_count ? g->done + g->tc_count : nullptr);
    kernels = 1;
  } else {
    for (auto& lev : g->levels) {
      for (auto& l : lev) {
        if (l.tiles == 0) continue;
        if (l.family == kFamTC)
          e = tc_launch_persistent(nullptr, static_cast<const TcProblem*>(g->tc_dev) + l.offset,
                                   l.count, l.tiles, ctx->num_sms, nullptr, s, ctx->d_err);
        else if (l.family == kFamReduce)
          e = launch_splitk_reduce_group(g->dtype,
                                         static_cast<const SplitReduce*>(g->reduce_dev) + l.offset,
                                         l.count, l.tiles, s);
        else if (l.family == kFamSimtSkinny)
          e = launch_skinny_group(g->dtype, l.nmax,
                                  static_cast<const SimtProblem*>(g->simt_dev) + l.offset, l.count,
                                  l.tiles, s);
        else
          e = launch_simt_group(g->dtype, false,
                                static_cast<const SimtProblem*>(g->simt_dev) + l.offset, l.count,
                                l.tiles, s);
        ++kernels;
        if (e != cudaSuccess) break;
      }
      if (e != cudaSuccess) break;
    }
  }
  g->kernels = kernels;
  return e == cudaSuccess ? T1M_OK : cuda_fail(ctx, e, "grouped launch");
}

}  // namespace

extern "C" int t1m_group_destroy(t1m_group* g) {
  if (!g) return T1M_ERR_INVALID_ARGUMENT;
  if (g->ctx) {
    cudaSetDevice(g->ctx->device);
    cudaStreamSynchronize(g->ctx->stream);
  }
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  if (g->vectors) cudaFree(g->vectors);
  if (g->tc_dev) cudaFree(g->tc_dev);
  if (g->simt_dev) cudaFree(g->simt_dev);
  if (g->reduce_dev) cudaFree(g->reduce_dev);
  if (g->work) cudaFree(g->work);
  if (g->done) cudaFree(g->done);
  delete g;
  return T1M_OK;
}

extern "C" int t1m_group_create(t1m_context* ctx, int dtype, int n, const t1m_group_item* items,
                                uint32_t options, t1m_group** out) {
  if (!ctx || !out || n < 0 || (n > 0 && !items)) return T1M_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  const size_t es = elem_size(dtype);
  if (es == 0) return fail(ctx, T1M_ERR_INVALID_ARGUMENT, "unknown dtype");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "set device");
  std::unique_ptr<t1m_group, int (*)(t1m_group*)> g(new t1m_group(), t1m_group_destroy);
  g->ctx = ctx;
  g->dtype = dtype;
  g->n = n;

  // Plans, dependency levels and families.
  std::vector<HostPlan> plans(n);
  std::vector<int> level(n, 0), family(n, kFamSimt);
  size_t vec_elems = 0;
  for (int i = 0; i < n; ++i) {
    const t1m_group_item& it = items[i];
    if (!it.a || !it.b || !it.c || !it.labels_a || !it.labels_b || !it.labels_c)
      return fail(ctx, T1M_ERR_INVALID_ARGUMENT, "null member in group item " + std::to_string(i));
    if (it.depends_on >= i)
      return fail(ctx, T1M_ERR_INVALID_ARGUMENT, "item " + std::to_string(i) +
                                                      " depends on a later item");
    int64_t sa[64], sb[64], sc[64];
    for (const t1m_tensor* t : {it.a, it.b, it.c})
      if (t->ndim < 0 || t->ndim > 64 || (t->ndim > 0 && !t->extents))
        return fail(ctx, T1M_ERR_INVALID_ARGUMENT, "bad rank in group item " + std::to_string(i));
    if (!resolve_strides(it.a, sa) || !resolve_strides(it.b, sb) || !resolve_strides(it.c, sc))
      return fail(ctx, T1M_ERR_INVALID_ARGUMENT, "strided tensor without strides");
    std::string err;
    int st = build_plan(dtype, it.a->ndim, it.a->extents, sa, it.labels_a, it.b->ndim,
                        it.b->extents, sb, it.labels_b, it.c->ndim, it.c->extents, sc,
                        it.labels_c, &plans[i], &err);
    if (st != T1M_OK) return fail(ctx, st, "group item " + std::to_string(i) + ": " + err);
    const HostPlan& hp = plans[i];
    if (!hp.modes_b.empty())
      return fail(ctx, T1M_ERR_LABELS, "group item " + std::to_string(i) +
                                           ": batch labels (in A, B and C) are taken by "
                                           "t1m_contract, not by grouped launches");
    if (hp.M > 0 && hp.N > 0 && hp.K > 0 &&
        (!is_device_pointer(it.a->data) || !is_device_pointer(it.b->data) ||
         !is_device_pointer(it.c->data)))
      return fail(ctx, T1M_ERR_INVALID_ARGUMENT,
                  "grouped contractions take device pointers (item " + std::to_string(i) + ")");
    level[i] = it.depends_on >= 0 ? level[it.depends_on] + 1 : 0;
    family[i] = heuristic_family(dtype, hp);
    if (ctx->method == T1M_METHOD_PLAIN && family[i] == kFamTC) family[i] = kFamSimt;
    vec_elems += hp.rsA.size() + hp.csA.size() + hp.rsB.size() + hp.csB.size() + hp.rsC.size() +
                 hp.csC.size() + 6;
    g->flops += (dtype >= T1M_COMPLEX64 ? 8.0 : 2.0) * double(hp.M) * double(hp.N) * double(hp.K);
  }

  // One persistent launch (T1M_GROUP_ONE_LAUNCH): a complex64 batch runs
  // every item on the persistent tensor-core kernel, each with its own tile;
  // dependencies and split-K reductions are resolved inside the kernel.
  // Measured on the sweep batch of 1024 updates: 159 ms against 128 ms as
  // family launches per level, because the second steps (N <= 4, A streamed
  // once) run as SIMT tiles at 47 ms against 22 ms on the skinny kernel
  // (its two CTAs per SM keep 160 KB of A in flight; the persistent kernel's
  // four raw stages hold 32 KB), so the family launches stay the default.
  const bool one_launch = n > 0 && dtype == T1M_COMPLEX64 && ctx->method != T1M_METHOD_PLAIN &&
                          (options & T1M_GROUP_ONE_LAUNCH);
  // Tile per item: an output width (16, 32, 64 or 128 columns on the tensor
  // cores) or kWidthSimt (outputs of at most kTcSkinnyMaxN columns as SIMT
  // tiles of the same kernel).
  std::vector<int> width(n, 128);
  if (one_launch)
    for (int i = 0; i < n; ++i) {
      family[i] = kFamTC;
      width[i] = plans[i].N <= kTcSkinnyMaxN ? kWidthSimt : tc_default_tile_n(plans[i].N);
    }

  // Scatter vectors of every item, one allocation.
  e = cudaMalloc(&g->vectors, std::max<size_t>(vec_elems, 1) * sizeof(int64_t));
  if (e != cudaSuccess) return fail(ctx, T1M_ERR_ALLOC, "group scatter vectors");
  std::vector<int64_t> host(vec_elems);
  std::vector<GemmArgs> args(n);
  size_t off = 0;
  for (int i = 0; i < n; ++i) {
    const HostPlan& hp = plans[i];
    const t1m_group_item& it = items[i];
    const std::vector<int64_t>* vs[6] = {&hp.rsA, &hp.csA, &hp.rsB, &hp.csB, &hp.rsC, &hp.csC};
    const int64_t* dptr[6];
    for (int v = 0; v < 6; ++v) {
      std::copy(vs[v]->begin(), vs[v]->end(), host.begin() + off);
      host[off + vs[v]->size()] = 0;
      dptr[v] = static_cast<const int64_t*>(g->vectors) + off;
      off += vs[v]->size() + 1;
    }
    GemmArgs& a = args[i];
    a = GemmArgs{};
    a.A = it.a->data;
    a.B = it.b->data;
    a.C = it.c->data;
    a.M = hp.M;
    a.N = hp.N;
    a.K = hp.K;
    a.rsA = dptr[0]; a.csA = dptr[1]; a.rsB = dptr[2]; a.csB = dptr[3];
    a.rsC = dptr[4]; a.csC = dptr[5];
    a.uA_m = hp.uA_m; a.uA_k = hp.uA_k; a.uB_k = hp.uB_k; a.uB_n = hp.uB_n;
    a.uC_m = hp.uC_m; a.uC_n = hp.uC_n;
    a.alpha[0] = it.alpha[0];
    a.alpha[1] = it.alpha[1];
    a.beta[0] = it.beta[0];
    a.beta[1] = it.beta[1];
    a.flags = 0;
    if (it.flags & T1M_FLAG_ACCUMULATE) a.flags |= kFlagAccumulate;
    if (it.flags & T1M_FLAG_CONJ_A) a.flags |= kFlagConjA;
    if (it.flags & T1M_FLAG_CONJ_B) a.flags |= kFlagConjB;
    if (!(it.flags & T1M_FLAG_ACCUMULATE) && a.beta[0] == 0.0 && a.beta[1] == 0.0)
      a.flags |= kFlagBetaZero;
    a.k_per_split = std::max<int64_t>(hp.K, 1);
    a.c_split_stride = 0;
  }
  if (vec_elems) {
    e = cudaMemcpy(g->vectors, host.data(), vec_elems * sizeof(int64_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "group scatter vectors upload");
  }

  // Autotuning of a one-launch batch: per shape class, time the tile widths
  // up to the output's width once on a representative item (main kernel
  // only, with its split count, into a scratch output) and keep the fastest.
  if (one_launch && (options & T1M_GROUP_AUTOTUNE)) {
    std::lock_guard<std::mutex> lock(g_tune.mu);
    g_tune.load(ctx->device);
    bool changed = false;
    for (int i = 0; i < n; ++i) {
      const HostPlan& hp = plans[i];
      if (hp.M == 0 || hp.N == 0 || hp.K == 0) continue;
      const std::string key = "w" + shape_class(dtype, hp);
      auto it = g_tune.choice.find(key);
      if (it != g_tune.choice.end()) {
        width[i] = it->second;
        continue;
      }
      int64_t kps = 0;
      const int nsp = group_splits(dtype, kFamTC, hp, es, &kps);
      void* scratch = nullptr;
      if (cudaMalloc(&scratch, size_t(nsp) * size_t(hp.M) * size_t(hp.N) * es) != cudaSuccess)
        return fail(ctx, T1M_ERR_ALLOC, "autotune scratch");
      const GemmArgs probe = split_args(args[i], scratch, kps);
      float best = 1e30f;
      int best_w = width[i];
      // Outputs of at most kTcSkinnyMaxN columns are SIMT tiles (see the
      // forced widths below); wider ones try every width they can use.
      std::vector<int> cands;
      if (hp.N <= kTcSkinnyMaxN) cands.push_back(kWidthSimt);
      for (int w : kTcTileWidths) {
        if (hp.N <= kTcSkinnyMaxN) break;
        if (w > 16 && w / 2 >= hp.N) break;  // wider than the output needs
        cands.push_back(w);
      }
      for (int w : cands) {
        TcProblem tp;
        if (!prepare_group_tc(probe, hp, nsp, w, &tp)) continue;
        tp.dep = -1;
        float total = 0;
        bool ok = true;
        for (int rep = 0; rep < 3 && ok; ++rep) {
          cudaEventRecord(ctx->ev[4], ctx->stream);
          const cudaError_t le = tc_launch_persistent(&tp, nullptr, 1, tc_problem_tiles(tp),
                                                      ctx->num_sms, nullptr, ctx->stream,
                                                      ctx->d_err);
          cudaEventRecord(ctx->ev[5], ctx->stream);
          if (le != cudaSuccess || cudaEventSynchronize(ctx->ev[5]) != cudaSuccess) {
            cudaGetLastError();
            ok = false;
            break;
          }
          float ms = 0;
          cudaEventElapsedTime(&ms, ctx->ev[4], ctx->ev[5]);
          if (rep > 0) total += ms;  // first run warms up
        }
        if (ok && total < best) {
          best = total;
          best_w = w;
        }
      }
      cudaFree(scratch);
      if (int st = check_device_error(ctx)) return st;
      width[i] = best_w;
      g_tune.choice[key] = best_w;
      changed = true;
    }
    if (changed) g_tune.save();
  }

  // A forced tile width (T1M_GROUP_TILE_*).
  if (const uint32_t fw = options & (T1M_GROUP_TILE_16 | T1M_GROUP_TILE_32 | T1M_GROUP_TILE_64 |
                                     T1M_GROUP_TILE_128)) {
    if (fw != T1M_GROUP_TILE_16 && fw != T1M_GROUP_TILE_32 && fw != T1M_GROUP_TILE_64 &&
        fw != T1M_GROUP_TILE_128)
      return fail(ctx, T1M_ERR_INVALID_ARGUMENT, "more than one tile width option");
    // Outputs of at most kTcSkinnyMaxN columns stay SIMT tiles: a batch with
    // N = 2, 5 and 8 items on forced 16-column tensor-core tiles raised an
    // unspecified launch failure whose cause reading the code did not show
    // (N = 1 and 3 items on the same tiles, and all of them as SIMT tiles,
    // ran correctly), so narrow outputs do not take that form.
    for (int i = 0; i < n; ++i)
      if (width[i] != kWidthSimt) width[i] = static_cast<int>(fw);
  }

  // Autotuning of family launches: per shape class, time the candidate
  // families once on a representative item (into a scratch output) and keep
  // the fastest.
  if (!one_launch && (options & T1M_GROUP_AUTOTUNE)) {
    std::lock_guard<std::mutex> lock(g_tune.mu);
    g_tune.load(ctx->device);
    bool changed = false;
    for (int i = 0; i < n; ++i) {
      const HostPlan& hp = plans[i];
      if (hp.M == 0 || hp.N == 0 || hp.K == 0) continue;
      const std::string key = shape_class(dtype, hp);
      auto it = g_tune.choice.find(key);
      if (it != g_tune.choice.end()) {
        // A shape class spans N up to twice its bucket: the skinny kernel
        // only takes outputs of at most kSkinnyMaxN columns.
        if (it->second != kFamSimtSkinny || hp.N <= kSkinnyMaxN) family[i] = it->second;
        continue;
      }
      std::vector<int> cands = {kFamSimt};
      if (hp.N <= kSkinnyMaxN) cands.push_back(kFamSimtSkinny);
      if (dtype == T1M_COMPLEX64 && ctx->method != T1M_METHOD_PLAIN) cands.push_back(kFamTC);
      // Each candidate runs with its own split count (the main kernel only:
      // the reduction is the same for all of them) into a scratch output.
      size_t scratch_bytes = 0;
      for (int f : cands) {
        int64_t kps = 0;
        const int sp = group_splits(dtype, f, hp, es, &kps);
        scratch_bytes = std::max(scratch_bytes, size_t(sp) * size_t(hp.M) * size_t(hp.N) * es);
      }
      void* scratch = nullptr;
      if (cudaMalloc(&scratch, scratch_bytes) != cudaSuccess)
        return fail(ctx, T1M_ERR_ALLOC, "autotune scratch");
      void* pd = nullptr;
      if (cudaMalloc(&pd, sizeof(TcProblem) > sizeof(SimtProblem) ? sizeof(TcProblem) : sizeof(SimtProblem)) != cudaSuccess) {
        cudaFree(scratch);
        return fail(ctx, T1M_ERR_ALLOC, "autotune descriptor");
      }
      float best = 1e30f;
      int best_f = family[i];
      for (int f : cands) {
        float total = 0;
        bool ok = true;
        int64_t kps = 0;
        const int nsp = group_splits(dtype, f, hp, es, &kps);
        const GemmArgs probe = split_args(args[i], scratch, kps);
        for (int rep = 0; rep < 3 && ok; ++rep) {
          cudaEventRecord(ctx->ev[4], ctx->stream);
          cudaError_t le;
          if (f == kFamTC) {
            TcProblem tp;
            ok = tc_prepare(probe, hp, nsp, &tp);
            tp.tile_begin = 0;
            tp.dep = -1;
            le = ok ? tc_launch_persistent(&tp, nullptr, 1, tc_problem_tiles(tp), ctx->num_sms,
                                           nullptr, ctx->stream, ctx->d_err)
                    : cudaErrorInvalidValue;
          } else if (f == kFamSimtSkinny) {
            SimtProblem sp{probe, 0};
            const int nmax = hp.N <= 4 ? 4 : 16;
            if (skinny_async_ok(sp.g, hp.rsA, es, nmax)) sp.g.flags |= kFlagSkinnyAsync;
            cudaMemcpy(pd, &sp, sizeof(sp), cudaMemcpyHostToDevice);
            le = launch_skinny_group(dtype, nmax, static_cast<SimtProblem*>(pd), 1,
                                     skinny_tiles(probe, nsp, nmax), ctx->stream);
          } else {
            SimtProblem sp{probe, 0};
            cudaMemcpy(pd, &sp, sizeof(sp), cudaMemcpyHostToDevice);
            int bm, bn;
            simt_group_tile(dtype, false, &bm, &bn);
            const int64_t tiles = nsp * ((hp.M + bm - 1) / bm) * ((hp.N + bn - 1) / bn);
            le = launch_simt_group(dtype, false, static_cast<SimtProblem*>(pd), 1, tiles,
                                   ctx->stream);
          }
          cudaEventRecord(ctx->ev[5], ctx->stream);
          if (le != cudaSuccess || cudaEventSynchronize(ctx->ev[5]) != cudaSuccess) {
            cudaGetLastError();
            ok = false;
            break;
          }
          float ms = 0;
          cudaEventElapsedTime(&ms, ctx->ev[4], ctx->ev[5]);
          if (rep > 0) total += ms;  // first run warms up
        }
        if (ok && total < best) {
          best = total;
          best_f = f;
        }
      }
      cudaFree(pd);
      cudaFree(scratch);
      if (int st = check_device_error(ctx)) return st;
      family[i] = best_f;
      g_tune.choice[key] = best_f;
      changed = true;
    }
    if (changed) g_tune.save();
  }

  // Split-K per item (bounded K per tile) and the workspace of the split
  // items; if the workspace would exceed its budget the caps are relaxed.
  std::vector<int> splits(n, 1);
  std::vector<int64_t> kps(n, 0), work_off(n, -1);
  size_t work_bytes = 0;
  for (int i = 0; i < n; ++i) {
    const HostPlan& hp = plans[i];
    if (hp.M == 0 || hp.N == 0 || hp.K == 0) continue;
    splits[i] = group_splits(dtype, family[i], hp, es, &kps[i]);
    if (splits[i] > 1) {
      work_off[i] = static_cast<int64_t>(work_bytes);
      work_bytes += (size_t(splits[i]) * size_t(hp.M) * size_t(hp.N) * es + 255) & ~size_t(255);
    }
  }
  if (work_bytes > kGroupWorkBytes) {
    std::fill(splits.begin(), splits.end(), 1);
    work_bytes = 0;
  }
  bool any_split = false;
  for (int i = 0; i < n; ++i) any_split = any_split || splits[i] > 1;
  if (work_bytes) {
    e = cudaMalloc(&g->work, work_bytes);
    if (e != cudaSuccess) return fail(ctx, T1M_ERR_ALLOC, "group split-K workspace");
  }
  std::vector<GemmArgs> main_args(args);
  for (int i = 0; i < n; ++i)
    if (splits[i] > 1)
      main_args[i] = split_args(args[i], static_cast<char*>(g->work) + work_off[i], kps[i]);

  // Launch lists.  A one-launch batch (and any batch whose items all run on
  // the tensor cores) is ONE persistent launch: dependencies and split-K
  // reductions resolved in the kernel.  Otherwise per level one launch per
  // family, then one grouped split-K reduction.
  bool all_tc = n > 0;
  for (int i = 0; i < n; ++i) all_tc = all_tc && family[i] == kFamTC;
  int max_level = 0;
  for (int i = 0; i < n; ++i) max_level = std::max(max_level, level[i]);
  std::vector<TcProblem> tcs;
  std::vector<SimtProblem> simts;
  std::vector<SplitReduce> reds;
  std::vector<int> tc_index(n, -1);
  if (all_tc) {
    // Tile list order: an item that reads another item's C is placed after
    // the next independent item that follows its dependency, so its tiles
    // rarely wait on tiles still in flight (and find part of that C in L2).
    // Dependent items wait in input order; after an independent item is
    // placed, every waiting item whose dependency was placed before it
    // follows.  A dependency always precedes its dependent: it has a smaller
    // index, so it is placed first or waits ahead of it.
    std::vector<int> order, waiting;
    std::vector<int64_t> pos(n, -1);
    order.reserve(n);
    auto place = [&](int i) {
      pos[i] = static_cast<int64_t>(order.size());
      order.push_back(i);
    };
    for (int i = 0; i < n; ++i) {
      if (items[i].depends_on >= 0) {
        waiting.push_back(i);
        continue;
      }
      const int64_t here = static_cast<int64_t>(order.size());
      place(i);
      std::vector<int> keep;
      for (int w : waiting) {
        const int64_t dp = pos[items[w].depends_on];
        if (dp >= 0 && dp < here) place(w);
        else keep.push_back(w);
      }
      waiting.swap(keep);
    }
    for (int w : waiting) place(w);
    for (int i : order) {
      const HostPlan& hp = plans[i];
      TcProblem tp;
      if (!prepare_group_tc(main_args[i], hp, splits[i], width[i], &tp))
        return fail(ctx, T1M_ERR_UNSUPPORTED, "group item " + std::to_string(i) +
                                                  " cannot run on the tensor cores");
      tp.tile_begin = g->tc_total;
      tp.dep = -1;
      tp.dep_tiles = 0;
      tp.dep_wait_cycles = ctx->wait_limit_us * (ctx->clock_khz / 1000);
      if (splits[i] > 1) {
        // In-kernel split-K reduction into the item's own output.
        tp.fix_begin = g->fix_count;
        g->fix_count += int64_t(tp.tiles_m) * tp.tiles_n;
        tp.out = args[i];
      }
      if (items[i].depends_on >= 0) {
        const TcProblem& d = tcs[tc_index[items[i].depends_on]];
        tp.dep = tc_index[items[i].depends_on];
        // Only final tiles count: every output tile of the dependency once.
        tp.dep_tiles = d.tiles_m * d.tiles_n;
        // Test aid: a count the dependency never reaches.
        if (options & T1M_GROUP_INJECT_UNMET_DEPENDENCY) ++tp.dep_tiles;
        g->deps = true;
      }
      tc_index[i] = static_cast<int>(tcs.size());
      g->tc_total += tc_problem_tiles(tp);
      tcs.push_back(tp);
    }
    g->single_tc = true;
    max_level = -1;  // no level launches
  }
  g->levels.assign(max_level + 1, {});
  for (int lv = 0; lv <= max_level; ++lv) {
    for (int fam : {kFamTC, kFamSimt, kFamSimtSkinny}) {
      t1m_group::Launch L{fam, fam == kFamTC ? int64_t(tcs.size()) : int64_t(simts.size()), 0, 0};
      if (fam == kFamSimtSkinny) {
        // One kernel instance per launch: the smallest column bound that
        // covers every item of the launch.
        L.nmax = 4;
        for (int i = 0; i < n; ++i)
          if (level[i] == lv && family[i] == fam && plans[i].N > 4) L.nmax = 16;
      }
      for (int i = 0; i < n; ++i) {
        if (level[i] != lv || family[i] != fam) continue;
        const HostPlan& hp = plans[i];
        if (fam == kFamTC) {
          TcProblem tp;
          if (!tc_prepare(main_args[i], hp, splits[i], &tp))
            return fail(ctx, T1M_ERR_UNSUPPORTED, "group item " + std::to_string(i) +
                                                      " cannot run on the tensor cores");
          tp.tile_begin = L.tiles;
          tp.dep = -1;
          tp.dep_tiles = 0;
          tp.dep_wait_cycles = ctx->wait_limit_us * (ctx->clock_khz / 1000);
          tc_index[i] = static_cast<int>(tcs.size());
          const int64_t t = tc_problem_tiles(tp);
          L.tiles += t;
          g->tc_total += t;
          tcs.push_back(tp);
        } else if (fam == kFamSimtSkinny) {
          SimtProblem sp{main_args[i], L.tiles};
          if (skinny_async_ok(sp.g, hp.rsA, es, L.nmax)) sp.g.flags |= kFlagSkinnyAsync;
          L.tiles += skinny_tiles(main_args[i], splits[i], L.nmax);
          simts.push_back(sp);
        } else {
          int bm, bn;
          simt_group_tile(dtype, false, &bm, &bn);
          SimtProblem sp{main_args[i], L.tiles};
          L.tiles += splits[i] * ((hp.M + bm - 1) / bm) * ((hp.N + bn - 1) / bn);
          simts.push_back(sp);
        }
        ++L.count;
      }
      if (L.count > 0) g->levels[lv].push_back(L);
    }
    t1m_group::Launch R{kFamReduce, int64_t(reds.size()), 0, 0};
    for (int i = 0; i < n; ++i) {
      if (level[i] != lv || splits[i] <= 1) continue;
      SplitReduce r{};
      r.out = args[i];
      r.work = static_cast<char*>(g->work) + work_off[i];
      r.begin = R.tiles;
      r.splits = splits[i];
      R.tiles += plans[i].M * plans[i].N;
      reds.push_back(r);
      ++R.count;
    }
    if (R.count > 0) g->levels[lv].push_back(R);
  }
  g->tc_count = static_cast<int>(tcs.size());
  if (!tcs.empty()) {
    e = cudaMalloc(&g->tc_dev, tcs.size() * sizeof(TcProblem));
    if (e == cudaSuccess)
      e = cudaMemcpy(g->tc_dev, tcs.data(), tcs.size() * sizeof(TcProblem), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMalloc(&g->done, sizeof(int) * size_t(int64_t(tcs.size()) + g->fix_count));
    if (e == cudaSuccess)
      e = cudaMemset(g->done, 0, sizeof(int) * size_t(int64_t(tcs.size()) + g->fix_count));
    if (e != cudaSuccess) return fail(ctx, T1M_ERR_ALLOC, "group descriptors");
  }
  if (!reds.empty()) {
    e = cudaMalloc(&g->reduce_dev, reds.size() * sizeof(SplitReduce));
    if (e == cudaSuccess)
      e = cudaMemcpy(g->reduce_dev, reds.data(), reds.size() * sizeof(SplitReduce),
                     cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(ctx, T1M_ERR_ALLOC, "group descriptors");
  }
  if (!simts.empty()) {
    e = cudaMalloc(&g->simt_dev, simts.size() * sizeof(SimtProblem));
    if (e == cudaSuccess)
      e = cudaMemcpy(g->simt_dev, simts.data(), simts.size() * sizeof(SimtProblem),
                     cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(ctx, T1M_ERR_ALLOC, "group descriptors");
  }

  if (options & T1M_GROUP_GRAPH) {
    cudaStream_t cs = nullptr;
    e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "capture stream");
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    int st = T1M_OK;
    if (e == cudaSuccess) st = enqueue_group(g.get(), cs);
    cudaGraph_t graph = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess || e2 != cudaSuccess || st != T1M_OK || !graph) {
      if (graph) cudaGraphDestroy(graph);
      return st != T1M_OK ? st : cuda_fail(ctx, e != cudaSuccess ? e : e2, "graph capture");
    }
    g->graph = graph;
    e = cudaGraphInstantiate(&g->exec, graph, 0);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "graph instantiate");
  }
  *out = g.release();
  return T1M_OK;
}

extern "C" int t1m_group_launch(t1m_group* g, t1m_report* report) {
  if (!g || !g->ctx) return T1M_ERR_INVALID_ARGUMENT;
  t1m_context* ctx = g->ctx;
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  if (report) cudaEventRecord(ctx->ev[0], s);
  int st = T1M_OK;
  if (g->exec) {
    const cudaError_t e = cudaGraphLaunch(g->exec, s);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "graph launch");
    if (g->kernels == 0) g->kernels = 1;
  } else {
    st = enqueue_group(g, s);
    if (st != T1M_OK) return st;
  }
  if (report) {
    cudaEventRecord(ctx->ev[1], s);
    cudaError_t e = cudaEventSynchronize(ctx->ev[1]);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "grouped launch");
    if (int s2 = check_device_error(ctx)) return s2;
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
    std::memset(report, 0, sizeof(*report));
    report->method = T1M_METHOD_AUTO;
    report->split_k = 1;
    report->flops = g->flops;
    report->kernel_ms = ms;
    report->kernels = g->kernels;
  }
  return T1M_OK;
}
