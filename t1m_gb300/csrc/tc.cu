// Tensor-core form: complex64 block-scatter contraction on tcgen05 (sm_103a),
// 1M formulation with split-TF32 (3xTF32) compensated products.
//
// Replaces the reference's 1M five-loop GEMM (include/t1m/t1m.h:508-554) and
// its BLIS micro-kernel (bli/mappings.h:91-99).  The reference packs complex A
// into real 2x2 blocks [re -im; im re] and complex B into re/im row pairs
// (t1m.h:309-337), then runs a real GEMM of size 2M x N x 2K.  Here the same
// real GEMM runs on the 5th-generation tensor cores:
//
//  * A (1M-expanded, 2 real rows per complex row): producer warps gather
//    complex A straight from the tensor through the scatter vectors, build the
//    rows [re, -im, ...] and [im, re, ...], split each value into TF32 hi and
//    lo parts (hi = rna(x), lo = rna(x - hi)), and store both into TENSOR
//    MEMORY with tcgen05.st.  The 4x-expanded operand never exists in shared
//    or global memory.
//  * B (K-major, re/im interleaved along K, which is exactly the 1M B panel):
//    producers gather it, split hi/lo and store it into shared memory in the
//    128-byte-swizzled K-major layout the MMA descriptors read.
//  * One thread issues tcgen05.mma kind::tf32 (M = 128 real rows = 64 complex
//    rows, N = 256 complex columns, K = 8): A_hi*B_hi + A_hi*B_lo + A_lo*B_hi
//    into one FP32 accumulator in TMEM (256 columns).
//  * The epilogue reads the accumulator with tcgen05.ld; real rows 2i / 2i+1
//    are re / im of complex row i (t1m.h:425-426), paired across neighbouring
//    lanes with one shuffle, scaled by alpha/beta and scatter-written to C.
//
// Pipelining: kStages stages of (A hi/lo in TMEM, B hi/lo in shared memory),
// full/empty mbarriers between the 256 producer threads and the MMA thread;
// tcgen05.commit releases a stage when its MMAs have read it.  Every wait is
// bounded (ptx::mbar_wait); a timeout records an error code and the kernel
// leaves after freeing its tensor memory.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "internal.h"
#include "ptx.h"
#include "t1m_capi.h"

namespace t1m {
namespace gb300 {
namespace {

constexpr int kTileMc = 64;     // complex rows per CTA (MMA M = 128 real rows)
constexpr int kTileN = 256;     // complex columns per CTA (MMA N)
constexpr int kStepK = 16;      // complex K per stage = 32 TF32 = one 128 B swizzle row
constexpr int kStages = 3;
constexpr int kThreads = 384;   // warp 0: MMA + TMEM owner; warps 4..11: producers
constexpr int kProducerBase = 128;
constexpr int kProducers = 256;
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kAccCol = 0;      // accumulator: columns [0, 256)
constexpr uint32_t kAStageCol = 256; // A stage s: columns 256 + 64 s (hi 32 | lo 32)
constexpr int kBHalfBytes = kTileN * 128;       // 256 rows x 128 B
constexpr int kStageBytes = 2 * kBHalfBytes;    // hi + lo
constexpr int kBarrierBytes = 256;
constexpr int kSmemBytes = 1024 + kStages * kStageBytes + kBarrierBytes;
constexpr uint32_t kIdesc = ptx::idesc_f32acc(2u /*TF32*/, 128, kTileN);

static_assert(kAStageCol + 64 * kStages <= kTmemCols, "TMEM budget");
static_assert(kSmemBytes <= 227 * 1024, "shared memory budget");

enum : int { kErrFullWait = 1, kErrEmptyWait = 2, kErrAccWait = 3 };

__device__ __forceinline__ int64_t offs(const int64_t* v, int64_t u, int64_t i) {
  return u >= 0 ? i * u : __ldg(v + i);
}

__device__ __forceinline__ uint32_t swz128(int n, int k) {
  // Byte offset of complex element (row n, complex k) in a 128 B-swizzled
  // K-major tile of TF32 pairs: 16-byte chunk (k/2) of row n lands at chunk
  // (k/2) ^ (n % 8) of its 128-byte row; rows grouped in 1024-byte atoms.
  return static_cast<uint32_t>((n >> 3) * 1024 + (n & 7) * 128 +
                               ((((k >> 1) ^ (n & 7)) & 7) << 4) + (k & 1) * 8);
}

__device__ __forceinline__ void record_error(int* flag, int code) {
  if (flag) atomicCAS(flag, 0, code);
}

struct Split {
  uint32_t hi, lo;
};

__device__ __forceinline__ Split split_tf32(float x) {
  const float h = ptx::tf32_rna(x);
  const float l = ptx::tf32_rna(x - h);
  return {__float_as_uint(h), __float_as_uint(l)};
}

__global__ void __launch_bounds__(kThreads, 1)
tc3xtf32_contract(const GemmArgs args, int* err_flag, int b_kcontig) {
  extern __shared__ __align__(16) uint8_t smem_raw[];
  const uint32_t raw = ptx::smem_u32(smem_raw);
  const uint32_t sb = (raw + 1023u) & ~1023u;            // B stages (1024-aligned)
  uint8_t* const sb_ptr = smem_raw + (sb - raw);
  const uint32_t bars = sb + kStages * kStageBytes;
  auto full_bar = [&](int s) { return bars + 8u * s; };
  auto empty_bar = [&](int s) { return bars + 8u * (kStages + s); };
  const uint32_t acc_bar = bars + 16u * kStages;
  const uint32_t tmem_slot = acc_bar + 8u;
  volatile uint32_t* tmem_slot_ptr =
      reinterpret_cast<volatile uint32_t*>(sb_ptr + kStages * kStageBytes + 16 * kStages + 8);

  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;

  if (warp == 0) {
    ptx::tmem_alloc(tmem_slot, kTmemCols);
    ptx::tmem_relinquish();
  }
  if (tid == 32) {
    for (int s = 0; s < kStages; ++s) {
      ptx::mbar_init(full_bar(s), kProducers / 32);
      ptx::mbar_init(empty_bar(s), 1);
    }
    ptx::mbar_init(acc_bar, 1);
    ptx::fence_mbar_init();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_slot_ptr;

  const int64_t M = args.M, N = args.N, K = args.K;
  const int64_t tiles_m = (M + kTileMc - 1) / kTileMc;
  const int64_t tiles_n = (N + kTileN - 1) / kTileN;
  // Groups of 16 M-tiles sweep N so CTAs running together share B in L2.
  constexpr int64_t G = 16;
  const int64_t t = blockIdx.x;
  const int64_t group = t / (G * tiles_n);
  const int64_t first_m = group * G;
  const int64_t gsize = min(G, tiles_m - first_m);
  const int64_t tm = first_m + (t % (G * tiles_n)) % gsize;
  const int64_t tn = (t % (G * tiles_n)) / gsize;
  const int64_t m0 = tm * kTileMc, n0 = tn * kTileN;
  const int64_t ksteps = (K + kStepK - 1) / kStepK;

  if (warp == 0) {
    // ---------------------------------------------------------- MMA issue ---
    if (lane == 0) {
      bool ok = true;
      for (int64_t s = 0; s < ksteps && ok; ++s) {
        const int st = static_cast<int>(s % kStages);
        const uint32_t ph = static_cast<uint32_t>((s / kStages) & 1);
        if (!ptx::mbar_wait(full_bar(st), ph)) {
          record_error(err_flag, kErrFullWait);
          ok = false;
          break;
        }
        ptx::tc_fence_after();
        const uint32_t a_hi = tmem + kAStageCol + 64u * st;
        const uint32_t a_lo = a_hi + 32u;
        const uint32_t b_hi = sb + st * kStageBytes;
        const uint32_t b_lo = b_hi + kBHalfBytes;
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          const uint64_t dh = ptx::smem_desc_sw128(b_hi + 32u * kk);
          const uint64_t dl = ptx::smem_desc_sw128(b_lo + 32u * kk);
          const uint32_t first = (s == 0 && kk == 0) ? 0u : 1u;
          ptx::mma_tf32_ts(tmem + kAccCol, a_hi + 8u * kk, dh, kIdesc, first);
          ptx::mma_tf32_ts(tmem + kAccCol, a_hi + 8u * kk, dl, kIdesc, 1u);
          ptx::mma_tf32_ts(tmem + kAccCol, a_lo + 8u * kk, dh, kIdesc, 1u);
        }
        ptx::mma_commit(empty_bar(st));
      }
      // Signal the epilogue (also after an abort, so nobody waits forever),
      // then make sure no MMA is still writing TMEM before it is freed.
      ptx::mma_commit(acc_bar);
      if (!ptx::mbar_wait(acc_bar, 0)) record_error(err_flag, kErrAccWait);
    }
    __syncwarp();
  } else if (tid >= kProducerBase) {
    // ---------------------------------------------------------- producers ---
    const int pt = tid - kProducerBase;
    const int wg = pt >> 7;          // which half of the K-step (A) / of N (B)
    const int q = (pt >> 5) & 3;     // TMEM lane quarter of this warp
    const int rho = 32 * q + lane;   // real row = TMEM lane
    const int ci = rho >> 1;         // complex row in the tile
    const int part = rho & 1;        // 0: real row "re", 1: "im"
    const bool conjA = args.flags & kFlagConjA;
    const bool conjB = args.flags & kFlagConjB;
    const float2* __restrict__ A = static_cast<const float2*>(args.A);
    const float2* __restrict__ B = static_cast<const float2*>(args.B);

    const bool row_ok = (m0 + ci) < M;
    const int64_t rowA = row_ok ? offs(args.rsA, args.uA_m, m0 + ci) : 0;
    const int tw = pt & 127;
    // B element (n, k) handled in slot j: K-contiguous tensors walk k across
    // neighbouring threads (coalesced 128-byte column runs), others walk n.
    auto b_n = [&](int j) { return b_kcontig ? (wg * 128 + (tw >> 4) + 8 * j) : (wg * 128 + tw); };
    auto b_k = [&](int j) { return b_kcontig ? (tw & 15) : j; };

    float2 va[4], vb[16];
    auto load = [&](int64_t k0) {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int64_t kk = k0 + wg * 8 + 2 * j + part;
        float2 v = make_float2(0.f, 0.f);
        if (row_ok && kk < K) v = A[rowA + offs(args.csA, args.uA_k, kk)];
        if (conjA) v.y = -v.y;
        va[j] = v;
      }
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int64_t n = n0 + b_n(j);
        const int64_t kk = k0 + b_k(j);
        float2 v = make_float2(0.f, 0.f);
        if (n < N && kk < K) v = B[offs(args.rsB, args.uB_k, kk) + offs(args.csB, args.uB_n, n)];
        if (conjB) v.y = -v.y;
        vb[j] = v;
      }
    };

    bool ok = true;
    load(0);
    for (int64_t s = 0; s < ksteps; ++s) {
      const int st = static_cast<int>(s % kStages);
      const uint32_t ph = static_cast<uint32_t>((s / kStages) & 1);
      // A row values for this half of the step: the pair (2i, 2i+1) loaded
      // alternate k; exchange so both hold all eight.
      float2 av[8];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        float2 other;
        other.x = __shfl_xor_sync(0xffffffffu, va[j].x, 1);
        other.y = __shfl_xor_sync(0xffffffffu, va[j].y, 1);
        av[2 * j] = part ? other : va[j];
        av[2 * j + 1] = part ? va[j] : other;
      }
      float2 bv[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) bv[j] = vb[j];
      if (s + 1 < ksteps) load((s + 1) * kStepK);  // prefetch the next step

      if (!ptx::mbar_wait(empty_bar(st), ph ^ 1u)) {
        record_error(err_flag, kErrEmptyWait);
        ok = false;
        break;
      }
      ptx::tc_fence_after();
      // A -> TMEM: 1M rows, [re, -im] (part 0) or [im, re] (part 1) per k.
      uint32_t hi[16], lo[16];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float x0 = part ? av[j].y : av[j].x;
        const float x1 = part ? av[j].x : -av[j].y;
        const Split s0 = split_tf32(x0), s1 = split_tf32(x1);
        hi[2 * j] = s0.hi;
        lo[2 * j] = s0.lo;
        hi[2 * j + 1] = s1.hi;
        lo[2 * j + 1] = s1.lo;
      }
      const uint32_t a_col = tmem + (static_cast<uint32_t>(32 * q) << 16) + kAStageCol + 64u * st + 16u * wg;
      ptx::tmem_st16(a_col, hi);
      ptx::tmem_st16(a_col + 32u, lo);
      // B -> shared memory (swizzled K-major hi and lo tiles).
      uint8_t* bst = sb_ptr + st * kStageBytes;
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const Split r = split_tf32(bv[j].x), im = split_tf32(bv[j].y);
        const uint32_t off = swz128(b_n(j), b_k(j));
        *reinterpret_cast<uint2*>(bst + off) = make_uint2(r.hi, im.hi);
        *reinterpret_cast<uint2*>(bst + kBHalfBytes + off) = make_uint2(r.lo, im.lo);
      }
      ptx::tmem_wait_st();
      ptx::fence_proxy_async_smem();
      ptx::tc_fence_before();
      __syncwarp();
      if (lane == 0) ptx::mbar_arrive(full_bar(st));
    }

    // ---------------------------------------------------------- epilogue ---
    if (!ptx::mbar_wait(acc_bar, 0)) {
      record_error(err_flag, kErrAccWait);
      ok = false;
    }
    ptx::tc_fence_after();
    if (ok) {
      const bool accumulate = args.flags & kFlagAccumulate;
      const bool beta_zero = args.flags & kFlagBetaZero;
      const float ar = (float)args.alpha[0], ai = (float)args.alpha[1];
      const float br = (float)args.beta[0], bi = (float)args.beta[1];
      float2* __restrict__ Cp = static_cast<float2*>(args.C);
      const int64_t rowC = row_ok ? offs(args.rsC, args.uC_m, m0 + ci) : 0;
#pragma unroll 1
      for (int cc = 0; cc < 8; ++cc) {
        const int c0 = wg * 128 + 16 * cc;
        uint32_t r[16];
        ptx::tmem_ld16(tmem + (static_cast<uint32_t>(32 * q) << 16) + kAccCol + c0, r);
        ptx::tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const float va0 = __uint_as_float(r[2 * j]);
          const float va1 = __uint_as_float(r[2 * j + 1]);
          const float send = part ? va0 : va1;
          const float recv = __shfl_xor_sync(0xffffffffu, send, 1);
          const int col = c0 + 2 * j + part;
          const float re = part ? recv : va0;
          const float im = part ? va1 : recv;
          const int64_t n = n0 + col;
          if (row_ok && n < N) {
            float2* p = Cp + rowC + offs(args.csC, args.uC_n, n);
            const float tr = ar * re - ai * im;
            const float ti = ar * im + ai * re;
            if (accumulate) {
              const float2 o = *p;
              *p = make_float2(o.x + tr, o.y + ti);
            } else if (beta_zero) {
              *p = make_float2(tr, ti);
            } else {
              const float2 o = *p;
              *p = make_float2(tr + (br * o.x - bi * o.y), ti + (br * o.y + bi * o.x));
            }
          }
        }
      }
    }
  }

  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, kTmemCols);
  }
}

bool g_attr_set = false;

}  // namespace

bool tc_supported(int method, int dtype, const HostPlan& plan) {
  (void)plan;
  return method == T1M_METHOD_TC_3XTF32 && dtype == T1M_COMPLEX64;
}

cudaError_t launch_tc(int method, int dtype, const GemmArgs& args, const HostPlan& plan,
                      cudaStream_t stream, int* err_flag, int* kernels, std::string* err) {
  *kernels = 0;
  if (!tc_supported(method, dtype, plan)) {
    *err = "tensor-core method not available for this dtype";
    return cudaErrorNotSupported;
  }
  if (!g_attr_set) {
    cudaError_t e = cudaFuncSetAttribute(tc3xtf32_contract,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    if (e != cudaSuccess) return e;
    g_attr_set = true;
  }
  const int64_t tiles = ((args.M + kTileMc - 1) / kTileMc) * ((args.N + kTileN - 1) / kTileN);
  if (tiles == 0) return cudaSuccess;
  const int b_kcontig = (plan.uB_k == 1) ? 1 : 0;
  tc3xtf32_contract<<<static_cast<unsigned>(tiles), kThreads, kSmemBytes, stream>>>(
      args, err_flag, b_kcontig);
  *kernels = 1;
  return cudaGetLastError();
}

}  // namespace gb300
}  // namespace t1m
