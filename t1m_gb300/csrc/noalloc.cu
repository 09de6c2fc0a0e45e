// t1m_contract_noalloc: the contraction for callers that cannot allocate
// device memory.
//
// Some callers own every byte of device memory themselves (a host
// application with its own memory pool or a fixed memory budget), and some
// run in loops where cudaMalloc/cudaFree are not acceptable, because
// cudaFree synchronises the whole device and both can fail or stall at
// arbitrary points.  t1m_contract cannot serve them: it allocates the plan's
// scatter vectors, host staging buffers and the split-K workspace.  This entry
// point allocates nothing.  Its scratch memory (the plan's scatter vectors,
// the kernels' error word and the split-K partial products) lives in the
// file-scope array below, which every GPU that loads the library holds until
// the process exits.
//
// Limits and rules (also stated in include/t1m_capi.h):
//  * Scratch is T1M_NOALLOC_SCRATCH_BYTES (64 MiB).  A contraction whose
//    scatter vectors do not fit is rejected; the split count is reduced until
//    the partial products fit (down to no split, where C is written directly).
//  * Operands must be device pointers (host staging would need buffers).
//  * Every call shares the one array and overwrites it; it keeps the last
//    call's contents.  Calls that overlap on the GPU (other streams, other
//    host threads) race on it; the call is synchronous (it waits for its
//    stream before returning), so consecutive calls from one thread do not.
//  * The first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current); make that first call
//    before any stream capture.  The address is kept for the life of the
//    process, so calls after cudaDeviceReset are not supported.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include "internal.h"
#include "t1m_capi.h"

namespace t1m {
namespace gb300 {
cudaError_t launch_dmma(int dtype, const GemmArgs& args, int splits, cudaStream_t stream,
                        int* kernels);
void dmma_tile(int* bm, int* bn, int* bk);
}  // namespace gb300
}  // namespace t1m

namespace {

using namespace t1m::gb300;

// The scratch memory.  In host code `g_noalloc_scratch` is only a host-side
// stand-in for the symbol, never a device address: kernels get the address
// from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[T1M_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
constexpr size_t kErrBytes = 256;  // kernels' error word at offset 0

std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Once per device, with that device current: the array's device address.
int scratch_address(int device, void** out, std::string* msg) {
  if (device < 0 || device >= kMaxDevices) {
    *msg = "device ordinal out of range";
    return T1M_ERR_INVALID_ARGUMENT;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      *msg = std::string("cudaGetSymbolAddress of the scratch array failed: ") +
             cudaGetErrorString(e);
      return T1M_ERR_CUDA;
    }
    g_scratch_addr[device] = p;
  }
  *out = g_scratch_addr[device];
  return T1M_OK;
}

size_t elem_size(int dtype) {
  switch (dtype) {
    case T1M_FLOAT32: return 4;
    case T1M_FLOAT64: return 8;
    case T1M_COMPLEX64: return 8;
    case T1M_COMPLEX128: return 16;
  }
  return 0;
}

bool strides_of(const t1m_tensor* t, int64_t* out) {
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

bool on_device(const void* p) {
  cudaPointerAttributes attr{};
  if (!p || cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

size_t round_up(size_t x) { return (x + 255) & ~size_t(255); }

int finish(char* err, int32_t err_len, int status, const std::string& msg) {
  if (err && err_len > 0) {
    std::strncpy(err, msg.c_str(), static_cast<size_t>(err_len) - 1);
    err[err_len - 1] = 0;
  }
  return status;
}

}  // namespace

extern "C" int t1m_contract_noalloc(void* stream_ptr, int method, int dtype, const void* alpha,
                                    const t1m_tensor* a, const char* la, const t1m_tensor* b,
                                    const char* lb, const void* beta, const t1m_tensor* c,
                                    const char* lc, uint32_t flags, char* err,
                                    int32_t err_len) {
  if (!a || !b || !c || !la || !lb || !lc || !alpha || !beta)
    return finish(err, err_len, T1M_ERR_INVALID_ARGUMENT, "null argument");
  const size_t es = elem_size(dtype);
  if (es == 0) return finish(err, err_len, T1M_ERR_INVALID_ARGUMENT, "unknown dtype");
  for (const t1m_tensor* t : {a, b, c})
    if (t->ndim < 0 || t->ndim > 64 || (t->ndim > 0 && !t->extents) ||
        t->layout < T1M_ROW_MAJOR || t->layout > T1M_STRIDED)
      return finish(err, err_len, T1M_ERR_INVALID_ARGUMENT, "bad tensor rank, extents or layout");
  int64_t sa[64], sb[64], sc[64];
  if (!strides_of(a, sa) || !strides_of(b, sb) || !strides_of(c, sc))
    return finish(err, err_len, T1M_ERR_INVALID_ARGUMENT, "strided tensor without strides");

  HostPlan hp;
  std::string msg;
  int st = build_plan(dtype, a->ndim, a->extents, sa, la, b->ndim, b->extents, sb, lb, c->ndim,
                      c->extents, sc, lc, &hp, &msg);
  if (st != T1M_OK) return finish(err, err_len, st, msg);
  if (!hp.modes_b.empty())
    return finish(err, err_len, T1M_ERR_LABELS,
                  "batch labels (in A, B and C) are taken by t1m_contract only");
  if (hp.M == 0 || hp.N == 0) return finish(err, err_len, T1M_OK, "");
  if (!on_device(c->data) || (hp.K > 0 && (!on_device(a->data) || !on_device(b->data))))
    return finish(err, err_len, T1M_ERR_INVALID_ARGUMENT,
                  "t1m_contract_noalloc takes device pointers only (host data would need "
                  "staging buffers)");

  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return finish(err, err_len, T1M_ERR_CUDA, cudaGetErrorString(e));
  void* scratch = nullptr;
  st = scratch_address(device, &scratch, &msg);
  if (st != T1M_OK) return finish(err, err_len, st, msg);
  cudaStream_t stream = static_cast<cudaStream_t>(stream_ptr);

  // Scratch layout: error word | six scatter vectors | split-K partials.
  const std::vector<int64_t>* vs[6] = {&hp.rsA, &hp.csA, &hp.rsB, &hp.csB, &hp.rsC, &hp.csC};
  size_t vec_bytes = 0;
  for (auto* v : vs) vec_bytes += round_up((v->size() + 1) * sizeof(int64_t));
  const size_t fixed = kErrBytes + vec_bytes;
  if (fixed > T1M_NOALLOC_SCRATCH_BYTES)
    return finish(err, err_len, T1M_ERR_UNSUPPORTED,
                  "contraction too large for the " +
                      std::to_string(T1M_NOALLOC_SCRATCH_BYTES >> 20) +
                      " MiB no-allocation scratch: its scatter vectors need " +
                      std::to_string(fixed) + " bytes");
  unsigned char* base = static_cast<unsigned char*>(scratch);
  int* err_word = reinterpret_cast<int*>(base);
  const int64_t* dev_vec[6];
  size_t off = kErrBytes;
  for (int i = 0; i < 6; ++i) {
    dev_vec[i] = reinterpret_cast<const int64_t*>(base + off);
    e = cudaMemcpyAsync(base + off, vs[i]->data(), vs[i]->size() * sizeof(int64_t),
                        cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return finish(err, err_len, T1M_ERR_CUDA, cudaGetErrorString(e));
    off += round_up((vs[i]->size() + 1) * sizeof(int64_t));
  }
  // The error word must start at zero; the partials are fully overwritten.
  e = cudaMemsetAsync(err_word, 0, sizeof(int), stream);
  if (e != cudaSuccess) return finish(err, err_len, T1M_ERR_CUDA, cudaGetErrorString(e));

  // The method asked for, or t1m_contract's automatic choice (the same rule,
  // auto_method).  Its tensor-core form picks BF16x6 or 3xTF32 per operand
  // layout exactly as t1m_contract does; only the B panels and dense operand
  // packs, which would need workspace, are not used here (they change
  // speed, not results).
  const bool cplx = dtype == T1M_COMPLEX64 || dtype == T1M_COMPLEX128;
  const bool is_auto = method == T1M_METHOD_AUTO;
  if (is_auto) method = auto_method(dtype, hp);
  const bool dmma_ok = method == T1M_METHOD_DMMA && (dtype == T1M_FLOAT64 || dtype == T1M_COMPLEX128);
  if (method != T1M_METHOD_PLAIN && !dmma_ok && !tc_supported(method, dtype, hp))
    return finish(err, err_len, T1M_ERR_UNSUPPORTED, "method not available for this dtype");

  GemmArgs g{};
  g.A = a->data;
  g.B = b->data;
  g.C = c->data;
  g.M = hp.M;
  g.N = hp.N;
  g.K = hp.K;
  g.rsA = dev_vec[0]; g.csA = dev_vec[1]; g.rsB = dev_vec[2];
  g.csB = dev_vec[3]; g.rsC = dev_vec[4]; g.csC = dev_vec[5];
  g.uA_m = hp.uA_m; g.uA_k = hp.uA_k; g.uB_k = hp.uB_k; g.uB_n = hp.uB_n;
  g.uC_m = hp.uC_m; g.uC_n = hp.uC_n;
  auto read_scalar = [&](const void* p, double* o) {
    switch (dtype) {
      case T1M_FLOAT32: o[0] = *static_cast<const float*>(p); o[1] = 0; break;
      case T1M_FLOAT64: o[0] = *static_cast<const double*>(p); o[1] = 0; break;
      case T1M_COMPLEX64: o[0] = static_cast<const float*>(p)[0]; o[1] = static_cast<const float*>(p)[1]; break;
      default: o[0] = static_cast<const double*>(p)[0]; o[1] = static_cast<const double*>(p)[1]; break;
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
  g.k_per_split = std::max<int64_t>(hp.K, 1);
  g.c_split_stride = 0;

  int kernels = 0;
  if (hp.K == 0) {
    e = launch_simt(dtype, g, 1, stream, &kernels);
  } else {
    // Split count as t1m_contract's automatic choice, bounded by the scratch
    // left for the partial products.
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
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int64_t tiles = ((hp.M + bm - 1) / bm) * ((hp.N + bn - 1) / bn);
    const int64_t ksteps = (hp.K + bk - 1) / bk;
    int64_t s = 1;
    const int64_t target = int64_t(sms) * per_sm;
    if (tiles < target / 2 && ksteps >= 8)
      s = std::min<int64_t>((target + tiles - 1) / tiles, ksteps / 4);
    // The precision rule of the automatic method (accuracy_k_limit).
    const int64_t lim = is_auto ? accuracy_k_limit(method, dtype) : 0;
    if (lim > 0) s = std::max<int64_t>(s, (hp.K + lim - 1) / lim);
    s = std::max<int64_t>(1, std::min<int64_t>({s, ksteps, 4096}));
    const size_t room = T1M_NOALLOC_SCRATCH_BYTES - fixed;
    while (s > 1 && size_t(s) * size_t(hp.M) * size_t(hp.N) * es > room) --s;
    const int64_t steps_per = (ksteps + s - 1) / s;
    const int splits = static_cast<int>((ksteps + steps_per - 1) / steps_per);
    GemmArgs gm = g;
    void* partials = base + fixed;
    if (splits > 1) {
      gm.C = partials;
      gm.rsC = nullptr;
      gm.csC = nullptr;
      gm.uC_m = 1;
      gm.uC_n = hp.M;
      gm.alpha[0] = 1.0;
      gm.alpha[1] = 0.0;
      gm.beta[0] = gm.beta[1] = 0.0;
      gm.flags = (g.flags & (kFlagConjA | kFlagConjB)) | kFlagBetaZero;
      gm.k_per_split = steps_per * bk;
      gm.c_split_stride = hp.M * hp.N;
    }
    if (method == T1M_METHOD_PLAIN) {
      e = launch_simt(dtype, gm, splits, stream, &kernels);
    } else if (method == T1M_METHOD_DMMA) {
      e = launch_dmma(dtype, gm, splits, stream, &kernels);
    } else {
      std::string lerr;
      e = launch_tc(method, dtype, gm, hp, splits, stream, err_word, &kernels, &lerr, nullptr);
      if (e != cudaSuccess && !lerr.empty()) return finish(err, err_len, T1M_ERR_CUDA, lerr);
    }
    if (e == cudaSuccess && splits > 1) e = launch_splitk_reduce(dtype, partials, splits, g, stream);
  }
  if (e != cudaSuccess) return finish(err, err_len, T1M_ERR_CUDA, cudaGetErrorString(e));
  // Synchronous: the scratch is reused by the next call.
  e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return finish(err, err_len, T1M_ERR_CUDA, cudaGetErrorString(e));
  int code = 0;
  e = cudaMemcpy(&code, err_word, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return finish(err, err_len, T1M_ERR_CUDA, cudaGetErrorString(e));
  if (code != 0)
    return finish(err, err_len, T1M_ERR_KERNEL_TIMEOUT,
                  "a bounded device-side wait timed out (kernel code " + std::to_string(code) + ")");
  return finish(err, err_len, T1M_OK, "");
}
