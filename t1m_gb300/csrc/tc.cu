// Tensor-core form: complex64 block-scatter contraction on tcgen05 (sm_103a),
// 1M formulation with split-TF32 (3xTF32) compensated products.
//
// Replaces the reference's 1M five-loop GEMM (include/t1m/t1m.h:508-554) and
// its BLIS micro-kernel (bli/mappings.h:91-99).  The reference packs complex A
// into real 2x2 blocks [re -im; im re] and complex B into re/im row pairs
// (t1m.h:309-337), then runs a real GEMM of size 2M x N x 2K.  Here the same
// real GEMM runs on the 5th-generation tensor cores, with no packed copy of
// any tensor in HBM:
//
//  1. Loader warps bring raw complex tiles into a ring of shared-memory
//     stages.  Where the block-scatter blocks of an operand have unit stride
//     (a bundle whose 16-element blocks are contiguous runs, or which is one
//     uniform run), TMA fetches them: one cp.async.bulk.tensor per operand
//     tile, or one per 16-row block, with the coordinates taken from the
//     scatter vectors (128-byte swizzle where the innermost run is K).  Other
//     operands are gathered element by element with cp.async through the
//     scatter vectors (zero fill past the edges).
//  2. Converter warps read a raw stage, build the 1M A rows [re, -im, ...]
//     and [im, re, ...] for every complex row, split every value into TF32 hi
//     and lo parts and store A hi/lo into TENSOR MEMORY with tcgen05.st (the
//     4x-expanded A never exists in shared or global memory) and B hi/lo into
//     shared memory in the 128-byte-swizzled K-major layout the MMA
//     descriptors read (the 1M B panel is the raw interleaved re/im data).
//  3. One thread issues tcgen05.mma kind::tf32 (M = 128 real rows = 64 complex
//     rows, N = 128 complex columns, K = 8).
//
// Accuracy.  The tensor core's FP32 accumulation truncates: measured on
// GB300, every MMA instruction that accumulates into D adds a bias of about
// 2e-8 |D|, so 3 x 1024 MMAs over K = 4096 complex would cost ~6e-5 relative
// error.  Therefore
//  * the main product A_hi*B_hi goes into a short-lived CHUNK accumulator
//    (two of them, ping-pong), restarted every kFold stages (128 real K =
//    16 MMAs), and each finished chunk is folded by the converter warps into
//    FP32 registers with round-to-nearest adds (tcgen05.ld + FADD);
//  * the two correction products A_hi*B_lo + A_lo*B_hi (2^-11 of the main
//    term) accumulate in a separate TMEM accumulator for the whole K range
//    and are added once at the end.
//  The epilogue pairs real rows 2i / 2i+1 (re / im of complex row i,
//  t1m.h:425-426) across neighbouring lanes with one shuffle, applies
//  alpha/beta and scatter-writes C.
//
// Persistence and grouping.  One CTA per SM loops over a list of output
// tiles; the list may span many contractions of different shapes (a grouped
// launch: one descriptor per contraction in global memory), so a batch of
// uneven contractions runs as one launch.  All rings, chunk buffers and
// accumulators carry over from tile to tile; the MMA of a tile waits until the
// epilogue of the previous tile has read the accumulators.
//
// Synchronisation: mbarriers between loaders -> converters (raw ring),
// converters -> MMA (operand stages), MMA -> converters (tcgen05.commit on
// stage release, chunk completion and tile completion) and converters -> MMA
// (chunk and accumulator release).  Every wait is bounded (ptx::mbar_wait); a
// timeout records an error code in a device word the host checks, and the
// kernel leaves after freeing its tensor memory.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "internal.h"
#include "ptx.h"
#include "t1m_capi.h"
#include "tc.h"

namespace t1m {
namespace gb300 {
namespace {

constexpr int kTileMc = 64;     // complex rows per tile (MMA M = 128 real rows)
constexpr int kTileN = 128;     // complex columns per tile (MMA N)
constexpr int kStepK = 16;      // complex K per stage = 32 TF32 = one 128 B swizzle row
constexpr int kRaw = 4;         // raw tile stages
constexpr int kStages = 2;      // converted operand stages
constexpr int kFold = 4;        // stages per chunk accumulator (128 real K)
constexpr int kSkinnyTcN = 8;   // columns of a SIMT tile of the persistent kernel
// Longest in-kernel split-K reduction a single product takes (partials read
// per thread of the last split's CTA); longer ones use the reduction kernel.
constexpr int64_t kFixMaxLoads = 64;
static_assert(kSkinnyTcN == kTcSkinnyMaxN, "SIMT tile width");
constexpr int kThreads = 384;   // warp 0: MMA; warps 1-3: loaders; 4-11: converters
constexpr int kLoaderBase = 32;
constexpr int kLoaders = 96;
constexpr int kConvBase = 128;
constexpr int kConverters = 256;
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kChunkCol0 = 0;    // chunk accumulator 0: [0, 128)
constexpr uint32_t kChunkCol1 = 128;  // chunk accumulator 1: [128, 256)
constexpr uint32_t kCorrCol = 256;    // correction accumulator: [256, 384)
constexpr uint32_t kAStageCol = 384;  // A stage s: 384 + 64 s (hi 32 | lo 32)

constexpr int kRawABytes = kTileMc * kStepK * 8;   // 8 KB
constexpr int kRawBBytes = kTileN * kStepK * 8;    // 16 KB
constexpr int kRawBytes = kRawABytes + kRawBBytes;
constexpr int kBHalfBytes = kTileN * 128;          // B hi (or lo): 128 rows x 128 B
constexpr int kOpBytes = 2 * kBHalfBytes;
constexpr int kBarrierBytes = 256;
constexpr int kSmemBytes = 1024 + kRaw * kRawBytes + kStages * kOpBytes + kBarrierBytes;

constexpr uint32_t kRegsLaunch = 168;   // 65536 / 384, rounded down to a multiple of 8
constexpr uint32_t kRegsControl = 96;   // warpgroup 0: MMA issue + loaders
constexpr uint32_t kRegsConvert = 200;  // warpgroups 1-2: converters
static_assert(4 * kRegsControl + 8 * kRegsConvert <= 12 * kRegsLaunch, "register split");
static_assert(kAStageCol + 64 * kStages <= kTmemCols, "TMEM budget");
static_assert(kSmemBytes <= 227 * 1024, "shared memory budget");
static_assert(kRawABytes % 1024 == 0 && kRawBBytes % 1024 == 0, "TMA swizzle alignment");

enum : int {
  kErrFullWait = 1,
  kErrEmptyWait = 2,
  kErrAccWait = 3,
  kErrChunkWait = 4,
  kErrRawWait = 5,
  kErrAccEmptyWait = 6,
  kErrDepWait = 7
};

__device__ __forceinline__ int64_t offs(const int64_t* v, int64_t u, int64_t i) {
  return u >= 0 ? i * u : __ldg(v + i);
}

// Byte offset of complex element (row r, complex k) in a 128 B-swizzled tile
// of 128-byte rows: 16-byte chunk (k/2) of row r lands at chunk (k/2)^(r%8);
// rows are grouped in 1024-byte atoms.  This is both the TMA SWIZZLE_128B
// layout and the UMMA K-major SW128 layout.
__device__ __forceinline__ uint32_t swz128(int r, int k) {
  return static_cast<uint32_t>((r >> 3) * 1024 + (r & 7) * 128 +
                               ((((k >> 1) ^ (r & 7)) & 7) << 4) + (k & 1) * 8);
}

__device__ __forceinline__ void record_error(int* flag, int code) {
  if (flag) atomicCAS(flag, 0, code);
}

struct Split {
  uint32_t hi, lo;
};

// hi/lo split on the FMA pipe (Veltkamp splitting, factor 2^13 + 1): hi keeps
// the leading 11 significant bits of x rounded to nearest (exactly a TF32
// value), lo = x - hi is exact with at most 13 significant bits, of which the
// TF32 MMA uses the leading 11 (|error| <= 2^-22 |x|).  Valid for
// |x| < 2^127 / 8193; the _rn intrinsics keep the compiler from contracting
// or reassociating the three operations.
__device__ __forceinline__ Split split_tf32(float x) {
  const float c = __fmul_rn(x, 8193.0f);
  const float h = __fsub_rn(c, __fsub_rn(c, x));
  const float l = __fsub_rn(x, h);
  return {__float_as_uint(h), __float_as_uint(l)};
}

// Split-product precision of the one-tile-per-CTA kernel.
//   TF32x3: x = hi + lo (TF32), products hi*hi + hi*lo + lo*hi (kind::tf32).
//   BF16x3: x = x0 + x1 (bf16, 8 significant bits each), products
//           x0*y0 + x0*y1 + x1*y0 (kind::f16): about 16 correct bits.
//   BF16x6: x = x0 + x1 + x2, products x0*y0 + x0*y1 + x1*y0 + x1*y1 +
//           x0*y2 + x2*y0: about 24 correct bits (FP32-class).
// The bf16 forms are the split-and-sum scheme of Henry, Tang and Heinecke,
// "Leveraging the bfloat16 artificial intelligence datatype for
// higher-precision computations" (ARITH 2019).
enum : int { kPrecTF32x3 = 0, kPrecBF16x3 = 1, kPrecBF16x6 = 2 };

// Split a pair of floats (consecutive K) into P packed bf16x2 words: piece 0
// is the round-to-nearest bf16 of the value, each further piece the bf16 of
// the remainder (x - x0 is exact in FP32).  Low half = x, high half = y.
template <int P>
__device__ __forceinline__ void split_bf16(float x, float y, uint32_t& w0, uint32_t& w1,
                                           uint32_t& w2) {
  w0 = ptx::cvt_bf16x2(x, y);
  const float rx = __fsub_rn(x, __uint_as_float(w0 << 16));
  const float ry = __fsub_rn(y, __uint_as_float(w0 & 0xFFFF0000u));
  w1 = ptx::cvt_bf16x2(rx, ry);
  if (P == 3) {
    const float sx = __fsub_rn(rx, __uint_as_float(w1 << 16));
    const float sy = __fsub_rn(ry, __uint_as_float(w1 & 0xFFFF0000u));
    w2 = ptx::cvt_bf16x2(sx, sy);
  }
}

__device__ __forceinline__ float lds32(uint32_t addr) {
  float v;
  asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(addr));
  return v;
}
__device__ __forceinline__ float2 lds64(uint32_t addr) {
  float2 v;
  asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
  return v;
}
__device__ __forceinline__ float4 lds128(uint32_t addr) {
  float4 v;
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"(addr));
  return v;
}
__device__ __forceinline__ void sts64(uint32_t addr, uint32_t a, uint32_t b) {
  asm volatile("st.shared.v2.b32 [%0], {%1, %2};" ::"r"(addr), "r"(a), "r"(b) : "memory");
}
__device__ __forceinline__ void sts128(uint32_t addr, uint32_t a, uint32_t b, uint32_t c,
                                       uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c),
               "r"(d)
               : "memory");
}

// Gather loaders (96 threads, lt = 0..95): one 8-byte cp.async per complex
// element through the scatter vectors, zero fill outside the tile's valid
// rows / columns and [k0, ke).  Source addresses are formed eight at a time
// before their copies are issued, so the index loads of non-uniform bundles
// overlap instead of each waiting behind the previous cp.async.
//   A, raw layout [k][m] (512 B rows): element e = lt + 96 i, m = e % 64,
//      k = e / 64 (consecutive threads walk m: coalesced where M is unit
//      stride).
//   B, raw layout [n][k] 128 B-swizzled: thread lt always takes k = lt % 16
//      (96 is a multiple of 16), so one K offset per stage; n = lt / 16 + 6 i.
// kBatch addresses are formed per round (8 where registers allow; the
// persistent kernel's loader warps run on a reduced register budget).
template <int kBatch>
__device__ __forceinline__ void gather_a_stage(const GemmArgs& g, uint32_t dst, int lt,
                                               int64_t m0, int64_t k0, int64_t ke) {
  // Descriptor fields in registers: the cp.async statements clobber memory,
  // which would otherwise force a reload of every field per element.
  const float2* __restrict__ A = static_cast<const float2*>(g.A);
  const int64_t* __restrict__ rsA = g.rsA;
  const int64_t* __restrict__ csA = g.csA;
  const int64_t uA_m = g.uA_m, uA_k = g.uA_k, M = g.M;
  constexpr int kPer = (kTileMc * kStepK + kLoaders - 1) / kLoaders;  // 11
#pragma unroll 1
  for (int i0 = 0; i0 < kPer; i0 += kBatch) {
    const float2* src[kBatch];
    uint32_t okm = 0;
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      const int e = lt + kLoaders * (i0 + j);
      const int m = e % kTileMc, k = e / kTileMc;
      const bool in = (i0 + j < kPer) && e < kTileMc * kStepK && (m0 + m < M) && (k0 + k < ke);
      src[j] = in ? A + offs(rsA, uA_m, m0 + m) + offs(csA, uA_k, k0 + k) : A;
      okm |= in ? (1u << j) : 0u;
    }
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      const int e = lt + kLoaders * (i0 + j);
      if (i0 + j < kPer && e < kTileMc * kStepK) {
        const int m = e % kTileMc, k = e / kTileMc;
        ptx::cp_async_8(dst + static_cast<uint32_t>(k * 512 + m * 8), src[j],
                        ((okm >> j) & 1u) ? 8u : 0u);
      }
    }
  }
}

template <int kBatch>
__device__ __forceinline__ void gather_b_stage(const GemmArgs& g, uint32_t dst, int lt,
                                               int64_t n0, int64_t k0, int64_t ke,
                                               int tile_n = kTileN) {
  const float2* __restrict__ B = static_cast<const float2*>(g.B);
  const int64_t* __restrict__ csB = g.csB;
  const int64_t uB_n = g.uB_n, N = g.N;
  const int k = lt & (kStepK - 1);
  const bool kin = k0 + k < ke;
  const int64_t rk = kin ? offs(g.rsB, g.uB_k, k0 + k) : 0;
  constexpr int kStride = kLoaders / kStepK;                     // 6
  const int per = (tile_n + kStride - 1) / kStride;              // 22 for 128 columns
#pragma unroll 1
  for (int i0 = 0; i0 < per; i0 += kBatch) {
    const float2* src[kBatch];
    uint32_t okm = 0;
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      const int n = (lt >> 4) + kStride * (i0 + j);
      const bool in = kin && (i0 + j < per) && n < tile_n && (n0 + n < N);
      src[j] = in ? B + rk + offs(csB, uB_n, n0 + n) : B;
      okm |= in ? (1u << j) : 0u;
    }
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      const int n = (lt >> 4) + kStride * (i0 + j);
      if (i0 + j < per && n < tile_n)
        ptx::cp_async_8(dst + swz128(n, k), src[j], ((okm >> j) & 1u) ? 8u : 0u);
    }
  }
}

// Real (float32) gathers, 4-byte cp.async.  A raw tile [k][m]: 32 k x 128 m
// floats, 512-byte rows (consecutive threads walk m); B raw tile [n][k]:
// 128 n x 32 k floats in 128-byte swizzled rows, the same bytes as the
// complex [n][k] tile (k pairs take the place of complex elements).  B:
// thread lt always takes k = lt % 32 (96 is a multiple of 32), n = lt / 32 + 3 i.
template <int kBatch>
__device__ __forceinline__ void gather_a_stage_real(const GemmArgs& g, uint32_t dst, int lt,
                                                    int64_t m0, int64_t k0, int64_t ke) {
  const float* __restrict__ A = static_cast<const float*>(g.A);
  const int64_t* __restrict__ rsA = g.rsA;
  const int64_t* __restrict__ csA = g.csA;
  const int64_t uA_m = g.uA_m, uA_k = g.uA_k, M = g.M;
  constexpr int kElems = 128 * 32;
  constexpr int kPer = (kElems + kLoaders - 1) / kLoaders;  // 43
#pragma unroll 1
  for (int i0 = 0; i0 < kPer; i0 += kBatch) {
    const float* src[kBatch];
    uint32_t okm = 0;
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      const int e = lt + kLoaders * (i0 + j);
      const int m = e % 128, k = e / 128;
      const bool in = (i0 + j < kPer) && e < kElems && (m0 + m < M) && (k0 + k < ke);
      src[j] = in ? A + offs(rsA, uA_m, m0 + m) + offs(csA, uA_k, k0 + k) : A;
      okm |= in ? (1u << j) : 0u;
    }
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      const int e = lt + kLoaders * (i0 + j);
      if (i0 + j < kPer && e < kElems) {
        const int m = e % 128, k = e / 128;
        ptx::cp_async_4(dst + static_cast<uint32_t>(k * 512 + m * 4), src[j],
                        ((okm >> j) & 1u) ? 4u : 0u);
      }
    }
  }
}

template <int kBatch>
__device__ __forceinline__ void gather_b_stage_real(const GemmArgs& g, uint32_t dst, int lt,
                                                    int64_t n0, int64_t k0, int64_t ke) {
  const float* __restrict__ B = static_cast<const float*>(g.B);
  const int64_t* __restrict__ csB = g.csB;
  const int64_t uB_n = g.uB_n, N = g.N;
  const int k = lt & 31;
  const bool kin = k0 + k < ke;
  const int64_t rk = kin ? offs(g.rsB, g.uB_k, k0 + k) : 0;
  constexpr int kStride = kLoaders / 32;                 // 3
  constexpr int kPer = (kTileN + kStride - 1) / kStride; // 43
#pragma unroll 1
  for (int i0 = 0; i0 < kPer; i0 += kBatch) {
    const float* src[kBatch];
    uint32_t okm = 0;
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      const int n = (lt >> 5) + kStride * (i0 + j);
      const bool in = kin && (i0 + j < kPer) && n < kTileN && (n0 + n < N);
      src[j] = in ? B + rk + offs(csB, uB_n, n0 + n) : B;
      okm |= in ? (1u << j) : 0u;
    }
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      const int n = (lt >> 5) + kStride * (i0 + j);
      if (i0 + j < kPer && n < kTileN)
        ptx::cp_async_4(dst + swz128(n, k >> 1) + 4u * (k & 1), src[j],
                        ((okm >> j) & 1u) ? 4u : 0u);
    }
  }
}

// Epilogue of one converter thread: accumulator columns [col0, col0 + kCols)
// of real row 2 ci + part (part 0 holds the real parts of complex row ci,
// part 1 the imaginary parts).  Lane pairs swap halves with two shuffles per
// four columns so that each thread holds complete complex values: part 0
// writes columns 4q, 4q + 1 and part 1 columns 4q + 2, 4q + 3 of every group
// of four.  With kFlagCPairs the two values go out as one 16-byte access (a
// lane pair fills a 32-byte sector); with kFlagCCol16 one column offset is
// looked up per 16 columns.  C <- alpha*acc (+ beta*C, or + C when
// accumulating).
template <int kCols>
__device__ __forceinline__ void store_tile(const GemmArgs& g, float2* __restrict__ Cp,
                                           int64_t row, bool row_ok, int64_t n0, int col0,
                                           int part, const float (&master)[kCols],
                                           int64_t n_end = INT64_MAX) {
  const uint32_t flags = g.flags;
  const bool accumulate = flags & kFlagAccumulate;
  const bool beta_zero = flags & kFlagBetaZero;
  const bool pairs = flags & kFlagCPairs;
  const bool col16 = flags & kFlagCCol16;
  const float ar = (float)g.alpha[0], ai = (float)g.alpha[1];
  const float br = (float)g.beta[0], bi = (float)g.beta[1];
  const int64_t N = min(g.N, n_end);  // columns of this tile: [n0, N)
  const int64_t* __restrict__ csC = g.csC;
  const int64_t uC_n = g.uC_n;
  const int64_t rowC = row_ok ? offs(g.rsC, g.uC_m, row) : 0;
  float2* __restrict__ Cr = Cp + rowC;
  int64_t blk = 0;  // offset of the current 16-column block (kFlagCCol16)
#pragma unroll
  for (int q = 0; q < kCols / 4; ++q) {
    const float s0 = part ? master[4 * q] : master[4 * q + 2];
    const float s1 = part ? master[4 * q + 1] : master[4 * q + 3];
    const float r0 = __shfl_xor_sync(0xffffffffu, s0, 1);
    const float r1 = __shfl_xor_sync(0xffffffffu, s1, 1);
    const float re0 = part ? r0 : master[4 * q], im0 = part ? master[4 * q + 2] : r0;
    const float re1 = part ? r1 : master[4 * q + 1], im1 = part ? master[4 * q + 3] : r1;
    const int c = col0 + 4 * q + 2 * part;
    const int64_t n = n0 + c;
    if (col16 && (q & 3) == 0) {
      const int64_t nb = n0 + col0 + 16 * (q >> 2);
      blk = (row_ok && nb < N) ? offs(csC, uC_n, nb) : 0;
    }
    if (!row_ok || n >= N) continue;
    const int64_t on = col16 ? blk + (c - col0 - 16 * (q >> 2)) : offs(csC, uC_n, n);
    const bool second = n + 1 < N;
    const float t0r = ar * re0 - ai * im0, t0i = ar * im0 + ai * re0;
    const float t1r = ar * re1 - ai * im1, t1i = ar * im1 + ai * re1;
    if (pairs && second) {
      float4* p4 = reinterpret_cast<float4*>(Cr + on);
      if (accumulate) {
        const float4 o = *p4;
        *p4 = make_float4(o.x + t0r, o.y + t0i, o.z + t1r, o.w + t1i);
      } else if (beta_zero) {
        *p4 = make_float4(t0r, t0i, t1r, t1i);
      } else {
        const float4 o = *p4;
        *p4 = make_float4(t0r + (br * o.x - bi * o.y), t0i + (br * o.y + bi * o.x),
                          t1r + (br * o.z - bi * o.w), t1i + (br * o.w + bi * o.z));
      }
    } else {
      float2* p0 = Cr + on;
      float2* p1 = second ? Cr + (col16 ? on + 1 : offs(csC, uC_n, n + 1)) : p0;
      if (accumulate) {
        const float2 o = *p0;
        *p0 = make_float2(o.x + t0r, o.y + t0i);
        if (second) {
          const float2 o1 = *p1;
          *p1 = make_float2(o1.x + t1r, o1.y + t1i);
        }
      } else if (beta_zero) {
        *p0 = make_float2(t0r, t0i);
        if (second) *p1 = make_float2(t1r, t1i);
      } else {
        const float2 o = *p0;
        *p0 = make_float2(t0r + (br * o.x - bi * o.y), t0i + (br * o.y + bi * o.x));
        if (second) {
          const float2 o1 = *p1;
          *p1 = make_float2(t1r + (br * o1.x - bi * o1.y), t1i + (br * o1.y + bi * o1.x));
        }
      }
    }
  }
}

// Real epilogue: accumulator columns [col0, col0 + kCols) of real row `row`
// (one TMEM lane per row, no pairing).  For real problems kFlagCPairs means
// four consecutive columns contiguous and 16-byte aligned: one 16-byte store
// per four values.  kFlagCCol16 as in store_tile.
template <int kCols>
__device__ __forceinline__ void store_tile_real(const GemmArgs& g, float* __restrict__ Cp,
                                                int64_t row, bool row_ok, int64_t n0, int col0,
                                                const float (&master)[kCols]) {
  if (!row_ok) return;
  const uint32_t flags = g.flags;
  const bool accumulate = flags & kFlagAccumulate;
  const bool beta_zero = flags & kFlagBetaZero;
  const bool quads = flags & kFlagCPairs;
  const bool col16 = flags & kFlagCCol16;
  const float ar = (float)g.alpha[0], br = (float)g.beta[0];
  const int64_t N = g.N;
  const int64_t* __restrict__ csC = g.csC;
  const int64_t uC_n = g.uC_n;
  float* __restrict__ Cr = Cp + offs(g.rsC, g.uC_m, row);
  int64_t blk = 0;
#pragma unroll
  for (int q = 0; q < kCols / 4; ++q) {
    const int c = col0 + 4 * q;
    const int64_t n = n0 + c;
    if (col16 && (q & 3) == 0) {
      const int64_t nb = n0 + col0 + 16 * (q >> 2);
      blk = nb < N ? offs(csC, uC_n, nb) : 0;
    }
    if (n >= N) continue;
    const int64_t on = col16 ? blk + (c - col0 - 16 * (q >> 2)) : offs(csC, uC_n, n);
    float t[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) t[i] = ar * master[4 * q + i];
    if (quads && n + 3 < N) {
      float4* p4 = reinterpret_cast<float4*>(Cr + on);
      if (accumulate) {
        const float4 o = *p4;
        *p4 = make_float4(o.x + t[0], o.y + t[1], o.z + t[2], o.w + t[3]);
      } else if (beta_zero) {
        *p4 = make_float4(t[0], t[1], t[2], t[3]);
      } else {
        const float4 o = *p4;
        *p4 = make_float4(t[0] + br * o.x, t[1] + br * o.y, t[2] + br * o.z, t[3] + br * o.w);
      }
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        if (n + i >= N) break;
        float* p = Cr + (col16 ? on + i : (i == 0 ? on : offs(csC, uC_n, n + i)));
        if (accumulate) *p += t[i];
        else if (beta_zero) *p = t[i];
        else *p = t[i] + br * *p;
      }
    }
  }
}

// Position of one output tile in the tile list.  tn: the problem's tile
// width; out_tile: index of the output tile within its split (its fix
// counter is p->fix_begin + out_tile).
struct TileRef {
  const TcProblem* p;
  int pi;
  int tn;
  int fsh;  // log2 of the stages per main chunk (p->fold_shift)
  int64_t m0, n0, kb, ke, ksteps, out_tile;
};

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void red_release_add(int* p, int v) {
  asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Converter warps only (256 threads): named barrier 1.
__device__ __forceinline__ void converters_sync() {
  asm volatile("bar.sync 1, 256;" ::: "memory");
}

// Tiles of problem p are numbered split-major; within a split, groups of 16
// M-tiles sweep N so CTAs running together share B in L2.  Every role of a
// CTA walks its tiles in increasing order, so the problem is found by a
// forward scan from the previous tile's (`hint`): usually one load of the
// next descriptor's tile_begin, where a binary search over a batch of
// thousands of problems took a dozen dependent loads per tile and role.
__device__ __forceinline__ TileRef locate(const TcProblem* single, const TcProblem* group,
                                          int nprob, int64_t t, int& hint) {
  const TcProblem* p = single;
  int lo = 0;
  if (group) {
    lo = hint;
    while (lo + 1 < nprob && group[lo + 1].tile_begin <= t) ++lo;
    hint = lo;
    p = group + lo;
  }
  const int64_t lt = t - p->tile_begin;
  const int64_t per_split = int64_t(p->tiles_m) * p->tiles_n;
  const int64_t split = lt / per_split;
  const int64_t r = lt % per_split;
  constexpr int64_t G = 16;
  const int64_t group_idx = r / (G * p->tiles_n);
  const int64_t first_m = group_idx * G;
  const int64_t gsize = min(G, int64_t(p->tiles_m) - first_m);
  const int64_t tm = first_m + (r % (G * p->tiles_n)) % gsize;
  const int64_t tn = (r % (G * p->tiles_n)) / gsize;
  TileRef ref;
  ref.p = p;
  ref.pi = lo;
  ref.tn = p->tile_n;
  ref.fsh = p->fold_shift;
  ref.out_tile = r;
  ref.m0 = tm * kTileMc;
  ref.n0 = tn * p->tile_n;
  ref.kb = split * p->g.k_per_split;
  ref.ke = min(p->g.K, ref.kb + p->g.k_per_split);
  ref.ksteps = (ref.ke - ref.kb + kStepK - 1) / kStepK;
  return ref;
}

// In-kernel split-K reduction of one output tile (the converter warps of the
// split that arrived last, pt = 0..255): C(m, n) <- alpha * sum_s W_s(m, n)
// + beta * C(m, n) (or C + alpha * sum), the sum and the epilogue in FP64.
// The summation order is the reduction kernel's (splitk.cu): G = 2, 4 or 8
// groups, group g summing the slices g, g + G, ... in ascending order, then
// the G group sums in group order; and its epilogue expressions, so both
// paths give the same result.  The partials are the raw products written
// through p.g (dense, uniform strides, c_split_stride apart); other CTAs
// wrote them, so they are read from L2 (ld.global.cg).  Thread pt takes row
// m0 + pt % 64 and columns n0 + pt / 64, + 4, ... of the tile.
__device__ __forceinline__ double2 fix_cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __noinline__ void fix_reduce_tile(const TcProblem& p, const TileRef& tr, int pt) {
  const GemmArgs& w = p.g;
  const GemmArgs& o = p.out;
  const int64_t m = tr.m0 + (pt & 63);
  if (m >= w.M) return;
  const int64_t n_end = min(w.N, tr.n0 + tr.tn);
  const float2* __restrict__ W = static_cast<const float2*>(w.C);
  const int64_t wm = m * w.uC_m;
  const int64_t om = offs(o.rsC, o.uC_m, m);
  const int splits = p.splits;
  const int G = splits <= 2 ? 2 : splits <= 4 ? 4 : 8;
  const double2 alpha = make_double2(o.alpha[0], o.alpha[1]);
  const double2 beta = make_double2(o.beta[0], o.beta[1]);
  for (int64_t n = tr.n0 + (pt >> 6); n < n_end; n += 4) {
    const float2* src = W + wm + n * w.uC_n;
    double2 tot = make_double2(0.0, 0.0);
    for (int gi = 0; gi < G; ++gi) {
      double2 acc = make_double2(0.0, 0.0);
#pragma unroll 4
      for (int sp = gi; sp < splits; sp += G) {
        const float2 v = __ldcg(src + static_cast<int64_t>(sp) * w.c_split_stride);
        acc.x += static_cast<double>(v.x);
        acc.y += static_cast<double>(v.y);
      }
      if (gi == 0) {
        tot = acc;
      } else {
        tot.x += acc.x;
        tot.y += acc.y;
      }
    }
    float2* dst = static_cast<float2*>(o.C) + om + offs(o.csC, o.uC_n, n);
    double2 r = fix_cmul(alpha, tot);
    if (o.flags & kFlagAccumulate) {
      const float2 c = *dst;
      r.x += static_cast<double>(c.x);
      r.y += static_cast<double>(c.y);
    } else if (!(o.flags & kFlagBetaZero)) {
      const float2 c = *dst;
      const double2 bc = fix_cmul(beta, make_double2(c.x, c.y));
      r.x += bc.x;
      r.y += bc.y;
    }
    *dst = make_float2(static_cast<float>(r.x), static_cast<float>(r.y));
  }
}

__global__ void __launch_bounds__(kThreads, 1)
tc3xtf32_persistent(const __grid_constant__ TcProblem single, const TcProblem* group, int nprob,
                    int64_t total_tiles, int* done, int* err_flag, int* fix) {
  extern __shared__ __align__(16) uint8_t smem_raw[];
  __shared__ int s_fix_last;  // in-kernel split-K: this CTA's split arrived last
  // SIMT tiles: B columns of a stage, k-major, double-buffered (rows padded
  // so the four k a warp reads at once fall in different banks).
  __shared__ float2 s_skb[2][kStepK][kSkinnyTcN + 1];
  const uint32_t base = (ptx::smem_u32(smem_raw) + 1023u) & ~1023u;
  uint8_t* const base_ptr = smem_raw + (base - ptx::smem_u32(smem_raw));
  const uint32_t raw0 = base;                          // kRaw x (A 8 KB | B 16 KB)
  const uint32_t op0 = raw0 + kRaw * kRawBytes;        // kStages x (B hi | B lo)
  const uint32_t bars = op0 + kStages * kOpBytes;
  auto raw_a = [&](int r) { return raw0 + r * kRawBytes; };
  auto raw_b = [&](int r) { return raw0 + r * kRawBytes + kRawABytes; };
  auto raw_full = [&](int r) { return bars + 8u * r; };
  auto raw_empty = [&](int r) { return bars + 8u * (kRaw + r); };
  auto full_bar = [&](int s) { return bars + 8u * (2 * kRaw + s); };
  auto empty_bar = [&](int s) { return bars + 8u * (2 * kRaw + kStages + s); };
  auto chunk_full = [&](int b) { return bars + 8u * (2 * kRaw + 2 * kStages + b); };
  auto chunk_empty = [&](int b) { return bars + 8u * (2 * kRaw + 2 * kStages + 2 + b); };
  const uint32_t acc_full = bars + 8u * (2 * kRaw + 2 * kStages + 4);
  const uint32_t acc_empty = acc_full + 8u;
  const uint32_t tmem_slot = acc_empty + 8u;
  volatile uint32_t* tmem_slot_ptr = reinterpret_cast<volatile uint32_t*>(base_ptr + (tmem_slot - base));

  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;

  if (warp == 0) {
    ptx::tmem_alloc(tmem_slot, kTmemCols);
    ptx::tmem_relinquish();
  }
  if (tid == 32) {
    // Raw stages complete with one expect_tx arrival (TMA thread) plus one
    // cp.async arrival per loader thread; both are issued for every stage.
    for (int r = 0; r < kRaw; ++r) {
      ptx::mbar_init(raw_full(r), 1 + kLoaders);
      ptx::mbar_init(raw_empty(r), kConverters / 32);
    }
    for (int s = 0; s < kStages; ++s) {
      ptx::mbar_init(full_bar(s), kConverters / 32);
      ptx::mbar_init(empty_bar(s), 1);
    }
    for (int b = 0; b < 2; ++b) {
      ptx::mbar_init(chunk_full(b), 1);
      ptx::mbar_init(chunk_empty(b), kConverters / 32);
    }
    ptx::mbar_init(acc_full, 1);
    ptx::mbar_init(acc_empty, kConverters / 32);
    ptx::fence_mbar_init();
  }
  if (tid == 64 && !group) {
    if (single.amode != kAGather) ptx::tma_prefetch_desc(&single.map_a);
    if (single.bmode != kBGather) ptx::tma_prefetch_desc(&single.map_b);
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_slot_ptr;

  // Register budget: the MMA/loader warpgroup needs few registers, the two
  // converter warpgroups hold 64 accumulator floats each plus the stage data.
  // 4 warps x 96 + 8 warps x 200 registers (x 32 lanes) = 63,488 <= the
  // 384 x 168 = 64,512 the block is launched with.
  if (warp < 4)
    ptx::regs_dec<kRegsControl>();
  else
    ptx::regs_inc<kRegsConvert>();

  if (warp == 0) {
    // ---------------------------------------------------------- MMA issue ---
    if (lane == 0) {
      bool ok = true;
      int64_t op_cnt = 0, chunk_cnt = 0, tile_cnt = 0;  // tile_cnt: tensor-core tiles
      int hint = 0;
      for (int64_t t = blockIdx.x; t < total_tiles && ok; t += gridDim.x) {
        const TileRef tr = locate(&single, group, nprob, t, hint);
        // SIMT tiles (narrow outputs) are computed by the converter warps
        // alone: no MMA, no TMEM, none of this thread's barriers.
        if (tr.p->skinny) continue;
        const uint32_t idesc = ptx::idesc_f32acc(2u /*TF32*/, 128, static_cast<uint32_t>(tr.tn));
        // The previous tile's epilogue must have read the accumulators.
        if (tile_cnt > 0 && !ptx::mbar_wait(acc_empty, static_cast<uint32_t>((tile_cnt - 1) & 1))) {
          record_error(err_flag, kErrAccEmptyWait);
          ok = false;
          break;
        }
        for (int64_t s = 0; s < tr.ksteps; ++s, ++op_cnt) {
          const int st = static_cast<int>(op_cnt % kStages);
          const uint32_t ph = static_cast<uint32_t>((op_cnt / kStages) & 1);
          const int64_t fmask = (int64_t(1) << tr.fsh) - 1;
          const bool chunk_start = (s & fmask) == 0;
          if (chunk_start && s > 0) ++chunk_cnt;
          const int buf = static_cast<int>(chunk_cnt & 1);
          if (chunk_start && chunk_cnt >= 2 &&
              !ptx::mbar_wait(chunk_empty(buf), static_cast<uint32_t>(((chunk_cnt - 2) >> 1) & 1))) {
            record_error(err_flag, kErrChunkWait);
            ok = false;
            break;
          }
          if (!ptx::mbar_wait(full_bar(st), ph)) {
            record_error(err_flag, kErrFullWait);
            ok = false;
            break;
          }
          ptx::tc_fence_after();
          const uint32_t d_main = tmem + (buf ? kChunkCol1 : kChunkCol0);
          const uint32_t d_corr = tmem + kCorrCol;
          const uint32_t a_hi = tmem + kAStageCol + 64u * st;
          const uint32_t a_lo = a_hi + 32u;
          const uint32_t b_hi = op0 + st * kOpBytes;
          const uint32_t b_lo = b_hi + kBHalfBytes;
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) {
            const uint64_t dh = ptx::smem_desc_sw128(b_hi + 32u * kk);
            const uint64_t dl = ptx::smem_desc_sw128(b_lo + 32u * kk);
            ptx::mma_tf32_ts(d_main, a_hi + 8u * kk, dh, idesc, (chunk_start && kk == 0) ? 0u : 1u);
            ptx::mma_tf32_ts(d_corr, a_hi + 8u * kk, dl, idesc, (s == 0 && kk == 0) ? 0u : 1u);
            ptx::mma_tf32_ts(d_corr, a_lo + 8u * kk, dh, idesc, 1u);
          }
          ptx::mma_commit(empty_bar(st));
          if ((s & fmask) == fmask || s == tr.ksteps - 1) ptx::mma_commit(chunk_full(buf));
        }
        if (!ok) break;
        ++chunk_cnt;  // the next tile starts a fresh chunk
        ptx::mma_commit(acc_full);
        ++tile_cnt;
      }
      // Make sure no MMA is still writing TMEM before it is freed.
      if (tile_cnt > 0 && !ptx::mbar_wait(acc_full, static_cast<uint32_t>((tile_cnt - 1) & 1)))
        record_error(err_flag, kErrAccWait);
      if (!ok) {
        // Release the epilogue of a tile whose MMAs were cut short.
        ptx::mma_commit(acc_full);
      }
    }
    __syncwarp();
  } else if (tid < kConvBase) {
    // ------------------------------------------------------------ loaders ---
    const int lt = tid - kLoaderBase;  // 0..95
    int64_t raw_cnt = 0;
    int hint = 0;
    bool dep_failed = false;  // a dependency wait of this thread ran out
    for (int64_t t = blockIdx.x; t < total_tiles; t += gridDim.x) {
      const TileRef tr = locate(&single, group, nprob, t, hint);
      const TcProblem* p = tr.p;
      const GemmArgs& g = p->g;
      const int amode = p->amode, bmode = p->bmode;
      // Element offsets of the 16-row A blocks and 16-column B blocks of this
      // tile (block TMA modes), per tile; rows past the edge read row 0's
      // block (their products only reach outputs that are not written).
      int64_t rowa[4] = {0, 0, 0, 0};
      int64_t colb[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      if (lt == 0 && (amode == kAMK16 || amode == kAKM16 || amode == kAMK16K)) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int64_t m = tr.m0 + 16 * j;
          rowa[j] = m < g.M ? offs(g.rsA, g.uA_m, m) : 0;
        }
      }
      if (lt == 0 && (bmode == kBNK16 || bmode == kBKN16)) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int64_t n = tr.n0 + 16 * j;
          colb[j] = (16 * j < tr.tn && n < g.N) ? offs(g.csB, g.uB_n, n) : 0;
        }
      }
      // The B stage holds tn rows (columns of the output tile).
      const uint32_t b_bytes = static_cast<uint32_t>(tr.tn) * (kRawBBytes / kTileN);
      // Tiles fetched entirely by TMA need only the TMA thread; the other
      // loader threads skip them (the TMA thread arrives on their behalf).
      const bool gathering = amode == kAGather || bmode == kBGather;
      if (!gathering && lt != 0) {
        raw_cnt += tr.ksteps;
        continue;
      }
      bool stop = false;
      if (done && p->dep >= 0 && !dep_failed) {
        // This problem reads the C of problem p->dep: wait (bounded) until all
        // of its tiles are written, then order those generic-proxy writes
        // before this thread's TMA / cp.async reads.
        const int* ctr = done + p->dep;
        const long long budget = p->dep_wait_cycles > 0 ? p->dep_wait_cycles : ptx::kSpinBudget;
        if (ld_acquire(ctr) < p->dep_tiles) {
          const long long t0 = clock64();
          while (ld_acquire(ctr) < p->dep_tiles) {
            __nanosleep(200);
            if (clock64() - t0 > budget) {
              record_error(err_flag, kErrDepWait);
              dep_failed = true;
              break;
            }
          }
        }
        asm volatile("fence.proxy.async.global;" ::: "memory");
      }
      // After a dependency wait ran out, this thread's remaining stages of
      // dependent problems are drained rather than loaded: it still arrives
      // on every raw stage it owes, so the converters and the MMA thread run
      // their pipelines to the end (no wait of theirs runs out, every MMA
      // completes before TMEM is freed); the outputs of such a launch are
      // undefined, and the error word reports it.
      const bool drain = dep_failed && p->dep >= 0;
      for (int64_t s = 0; s < tr.ksteps && !stop; ++s, ++raw_cnt) {
        const int r = static_cast<int>(raw_cnt % kRaw);
        const uint32_t ph = static_cast<uint32_t>((raw_cnt / kRaw) & 1);
        const int64_t k0 = tr.kb + s * kStepK;
        if (!ptx::mbar_wait(raw_empty(r), ph ^ 1u)) {
          record_error(err_flag, kErrRawWait);
          stop = true;
          break;
        }
        if (drain) {
          // The arrivals a loaded stage would bring: the TMA thread's one
          // (plus the skipped loaders' on TMA-only tiles), one per gatherer.
          if (lt == 0) ptx::mbar_arrive_count(raw_full(r), gathering ? 1u : 1u + kLoaders);
          if (gathering) ptx::mbar_arrive(raw_full(r));
          continue;
        }
        if (lt == 0) {
          const uint32_t bytes = (amode != kAGather ? kRawABytes : 0) +
                                 (bmode != kBGather ? b_bytes : 0);
          ptx::mbar_arrive_expect_tx(raw_full(r), bytes);
          if (amode == kAMK)
            ptx::tma_load_2d(raw_a(r), &p->map_a, static_cast<int>(2 * tr.m0), static_cast<int>(k0), raw_full(r));
          if (amode == kAMK16)
#pragma unroll
            for (int j = 0; j < 4; ++j)
              ptx::tma_load_2d(raw_a(r) + 2048u * j, &p->map_a, static_cast<int>(2 * rowa[j]),
                               static_cast<int>(k0), raw_full(r));
          if (amode == kAKM)
            ptx::tma_load_2d(raw_a(r), &p->map_a, static_cast<int>(2 * offs(g.csA, g.uA_k, k0)),
                             static_cast<int>(tr.m0), raw_full(r));
          if (amode == kAKM16) {
            const int64_t ck = offs(g.csA, g.uA_k, k0);
#pragma unroll
            for (int j = 0; j < 4; ++j)
              ptx::tma_load_2d(raw_a(r) + 2048u * j, &p->map_a, static_cast<int>(2 * (rowa[j] + ck)),
                               0, raw_full(r));
          }
          if (bmode == kBNK)
            ptx::tma_load_2d(raw_b(r), &p->map_b, static_cast<int>(2 * offs(g.rsB, g.uB_k, k0)),
                             static_cast<int>(tr.n0), raw_full(r));
          if (amode == kAMK16K) {
            const int64_t ck = offs(g.csA, g.uA_k, k0);
#pragma unroll
            for (int j = 0; j < 4; ++j)
              ptx::tma_load_2d(raw_a(r) + 2048u * j, &p->map_a, static_cast<int>(2 * (rowa[j] + ck)),
                               0, raw_full(r));
          }
          if (bmode == kBNK16 || bmode == kBKN16) {
            const int64_t rk = offs(g.rsB, g.uB_k, k0);
#pragma unroll
            for (int j = 0; j < 8; ++j)
              if (16 * j < tr.tn)
                ptx::tma_load_2d(raw_b(r) + 2048u * j, &p->map_b,
                                 static_cast<int>(2 * (colb[j] + rk)), 0, raw_full(r));
          }
          if (bmode == kBKN)
            ptx::tma_load_2d(raw_b(r), &p->map_b, static_cast<int>(2 * tr.n0), static_cast<int>(k0), raw_full(r));
          if (!gathering) {
            ptx::mbar_arrive_count(raw_full(r), kLoaders);
            continue;
          }
        }
        if (amode == kAGather) gather_a_stage<2>(g, raw_a(r), lt, tr.m0, k0, tr.ke);
        if (bmode == kBGather) gather_b_stage<2>(g, raw_b(r), lt, tr.n0, k0, tr.ke, tr.tn);
        ptx::cp_async_arrive_noinc(raw_full(r));
      }
      if (stop) break;
    }
  } else {
    // -------------------------------------------- converters, fold, epilogue ---
    const int pt = tid - kConvBase;
    const int wg = pt >> 7;          // which half of the K-step (A) / of N (B, C)
    const int q = (pt >> 5) & 3;     // TMEM lane quarter of this warp
    const int rho = 32 * q + lane;   // real row = TMEM lane
    const int ci = rho >> 1;         // complex row in the tile
    const int part = rho & 1;        // 0: real row "re", 1: "im"
    const uint32_t lane_base = static_cast<uint32_t>(32 * q) << 16;

    float master[64];
    // Columns of the current tile (its width): accumulator columns past it
    // hold nothing of this tile and are not read.
    int cur_tn = kTileN;
    auto fold_from = [&](uint32_t col) {
#pragma unroll
      for (int cc = 0; cc < 2; ++cc) {
        if (64 * wg + 32 * cc >= cur_tn) break;  // warp-uniform
        uint32_t r[32];
        ptx::tmem_ld32_sync(tmem + lane_base + col + 64u * wg + 32u * cc, r);
#pragma unroll
        for (int j = 0; j < 32; ++j) master[32 * cc + j] += __uint_as_float(r[j]);
      }
    };

    bool ok = true;
    // Ring positions (index and phase parity) carried from tile to tile.
    uint32_t rr = 0, rph = 0, st = 0, sph = 0;
    int64_t chunk_cnt = 0, tile_cnt = 0;

    // One tile's stage loop for one (A layout, B layout) pair; the layout
    // decisions are compile-time inside, taken once per tile outside.
    //   A layouts: 0 = [k][m] rows of 512 B, 1 = four [16 k][16 m] blocks,
    //              2 = [m][k] 128 B swizzled;  B: 0 = [n][k] swizzled, 1 = [k][n],
    //              3 = eight [16 k][16 n] blocks.
    auto run_stages = [&](auto alay, auto blay, const TileRef& tr, bool conjA, bool conjB,
                          bool row_ok, int64_t chunk_base) -> bool {
      constexpr int AL = decltype(alay)::value;
      constexpr int BL = decltype(blay)::value;
      // Offsets of this thread's raw reads and operand writes.  Where they are
      // affine in the unrolled index (base + j*stride) only the base is kept,
      // so the strides become immediate offsets of the shared-memory accesses.
      uint32_t aoff_sw[4];  // [m][k] swizzled A: four 16-byte chunks
      uint32_t abase;
      if constexpr (AL == 2) {
#pragma unroll
        for (int j = 0; j < 4; ++j) aoff_sw[j] = swz128(ci, 8 * wg + 2 * j);
        abase = 0;
      } else if constexpr (AL == 1) {
        abase = static_cast<uint32_t>((ci >> 4) * 2048 + (8 * wg) * 128 + (ci & 15) * 8);
      } else {
        abase = static_cast<uint32_t>((8 * wg) * 512 + ci * 8);
      }
      constexpr uint32_t kAStep = AL == 1 ? 128u : 512u;
      // B: piece j of this thread is piece 0 plus kBStep j bytes in the raw
      // tile (and for [n][k] 4096 j in the swizzled operand tile).  In the
      // [k][n] forms piece j is k = (pt >> 6) + 4 j, columns n, n + 1.
      // The tile's B has tr.tn rows: a [k][n] stage (TMA box [16 k][tn n])
      // has rows of tn complex, and pieces past tn are neither read nor
      // converted (the MMA reads tn rows).
      constexpr bool kBRowsK = BL == 1 || BL == 3;
      const int tn = tr.tn;
      const uint32_t bpitch = static_cast<uint32_t>(tn) * 8u;
      const uint32_t kBStep = BL == 3 ? 512u : BL == 1 ? 4u * bpitch : 4096u;
      // [k][n] raw tiles: warp w takes columns 16 w .. 16 w + 15 (two per
      // lane) and k = lane % 4 (+ 4 j): per store instruction the warp's
      // 32 lanes then write 8-byte pieces into all eight 16-byte chunks of
      // the 128-byte swizzled rows (two lanes per slot, the minimum), where
      // k fixed per warp put all of them in four chunks (8-way conflicts).
      const int bn = kBRowsK ? 16 * (pt >> 5) + 2 * ((pt & 31) >> 2) : 0;
      const int bk = kBRowsK ? (pt & 3) : 0;
      const uint32_t bsrc0 =
          BL == 1 ? static_cast<uint32_t>(bk * bpitch + bn * 8)
          : BL == 3 ? static_cast<uint32_t>((bn >> 4) * 2048 + bk * 128 + (bn & 15) * 8)
                    : swz128(pt >> 3, 2 * (pt & 7));
      // Pieces j of this thread inside the tile's tn rows.
      uint32_t bmask = 0;
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (kBRowsK ? bn < tn : (pt >> 3) + 32 * j < tn) bmask |= 1u << j;
      uint32_t boff_kn[4][2];
      if constexpr (kBRowsK) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int k = bk + 4 * j, n = bn;
          boff_kn[j][0] = swz128(n, k);
          boff_kn[j][1] = swz128(n + 1, k);
        }
      }
      const int ksteps = static_cast<int>(tr.ksteps);
      for (int s = 0; s < ksteps; ++s) {
        if (!ptx::mbar_wait(raw_full(rr), rph)) {
          record_error(err_flag, kErrRawWait);
          return false;
        }
        const uint32_t ra = raw_a(rr), rb = raw_b(rr);
        float2 av[8];
        if constexpr (AL == 2) {
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const float4 v = lds128(ra + aoff_sw[j]);
            av[2 * j] = make_float2(v.x, v.y);
            av[2 * j + 1] = make_float2(v.z, v.w);
          }
        } else {
          const uint32_t a0 = ra + abase;
#pragma unroll
          for (int j = 0; j < 8; ++j) av[j] = lds64(a0 + kAStep * j);
        }
        float4 bv[4];
        const uint32_t b0 = rb + bsrc0;
#pragma unroll
        for (int j = 0; j < 4; ++j)
          bv[j] = (bmask >> j) & 1u ? lds128(b0 + kBStep * j) : make_float4(0.f, 0.f, 0.f, 0.f);
        // The raw stage is released after the conversion (below), once the
        // values read from it are consumed and behind the cross-proxy fence:
        // TMA (async proxy) refills it, and generic-proxy reads that are not
        // ordered before that by a proxy fence can observe the refill.
        const int r_cur = static_cast<int>(rr);
        if (++rr == kRaw) {
          rr = 0;
          rph ^= 1u;
        }

        if (!ptx::mbar_wait(empty_bar(st), sph ^ 1u)) {
          record_error(err_flag, kErrEmptyWait);
          return false;
        }
        ptx::tc_fence_after();
        // A -> TMEM: 1M rows, [re, -im] (part 0) or [im, re] (part 1) per k.
        uint32_t hi[16], lo[16];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          float2 v = av[j];
          if (conjA) v.y = -v.y;
          if (!row_ok) v = make_float2(0.f, 0.f);
          const float x0 = part ? v.y : v.x;
          const float x1 = part ? v.x : -v.y;
          const Split s0 = split_tf32(x0), s1 = split_tf32(x1);
          hi[2 * j] = s0.hi;
          lo[2 * j] = s0.lo;
          hi[2 * j + 1] = s1.hi;
          lo[2 * j + 1] = s1.lo;
        }
        const uint32_t a_col = tmem + lane_base + kAStageCol + 64u * st + 16u * wg;
        ptx::tmem_st16(a_col, hi);
        ptx::tmem_st16(a_col + 32u, lo);
        // B -> shared memory (swizzled K-major hi and lo tiles).
        const uint32_t ob = op0 + st * kOpBytes;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (!((bmask >> j) & 1u)) continue;
          float4 v = bv[j];
          if (conjB) {
            v.y = -v.y;
            v.w = -v.w;
          }
          const Split r0 = split_tf32(v.x), i0 = split_tf32(v.y);
          const Split r1 = split_tf32(v.z), i1 = split_tf32(v.w);
          if constexpr (kBRowsK) {
            sts64(ob + boff_kn[j][0], r0.hi, i0.hi);
            sts64(ob + boff_kn[j][1], r1.hi, i1.hi);
            sts64(ob + kBHalfBytes + boff_kn[j][0], r0.lo, i0.lo);
            sts64(ob + kBHalfBytes + boff_kn[j][1], r1.lo, i1.lo);
          } else {
            const uint32_t o = ob + bsrc0 + 4096u * j;
            sts128(o, r0.hi, i0.hi, r1.hi, i1.hi);
            sts128(o + kBHalfBytes, r0.lo, i0.lo, r1.lo, i1.lo);
          }
        }
        ptx::tmem_wait_st();
        ptx::fence_proxy_async_smem();
        ptx::tc_fence_before();
        __syncwarp();
        if (lane == 0) {
          ptx::mbar_arrive(full_bar(st));
          ptx::mbar_arrive(raw_empty(r_cur));
        }
        if (++st == kStages) {
          st = 0;
          sph ^= 1u;
        }

        // Fold the previous chunk once the first stage of the next is queued.
        if ((s & ((1 << tr.fsh) - 1)) == 0 && s >= (1 << tr.fsh)) {
          const int64_t c = chunk_base + (s >> tr.fsh) - 1;
          const int buf = static_cast<int>(c & 1);
          if (!ptx::mbar_wait(chunk_full(buf), static_cast<uint32_t>((c >> 1) & 1))) {
            record_error(err_flag, kErrChunkWait);
            return false;
          }
          ptx::tc_fence_after();
          fold_from(buf ? kChunkCol1 : kChunkCol0);
          ptx::tc_fence_before();
          __syncwarp();
          if (lane == 0) ptx::mbar_arrive(chunk_empty(buf));
        }
      }
      return true;
    };

    // SIMT tiles (TcProblem::skinny: outputs of at most kSkinnyTcN columns):
    // the converter warps compute the tile's products with FP32 FMAs straight
    // from the raw stages, which the loaders fill exactly as for tensor-core
    // tiles; the MMA thread skips the tile.  Thread pt takes row pt / 4 of
    // the tile and k = kq, kq + 4, kq + 8, kq + 12 of every stage (kq =
    // pt % 4); per stage the B columns are first copied into s_skb (k-major,
    // conjugated), and each stage's products are summed on their own before
    // they are added to the running sums (shorter FP32 sums, smaller error).
    // The four threads of a row then add their sums (shuffles) and the first
    // writes the row.  Returns false when a wait ran out.
    uint32_t sk_cnt = 0;  // SIMT stages processed (s_skb buffer parity)
    int hint = 0;
    auto run_skinny = [&](const TileRef& tr, int alay, int blay, bool conjA, bool conjB,
                          float2* __restrict__ Cp) -> bool {
      const GemmArgs& g = tr.p->g;
      const int r = pt >> 2, kq = pt & 3;
      const int ncols = static_cast<int>(min(g.N - tr.n0, static_cast<int64_t>(kSkinnyTcN)));
      uint32_t aoff[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int k = kq + 4 * i;
        aoff[i] = alay == 2 ? swz128(r, k)
                  : alay == 1 ? static_cast<uint32_t>((r >> 4) * 2048 + k * 128 + (r & 15) * 8)
                              : static_cast<uint32_t>(k * 512 + r * 8);
      }
      // B element copied by this thread (pt < 16 x kSkinnyTcN): k = pt / N', n = pt % N'.
      const int bk = pt / kSkinnyTcN, bn = pt % kSkinnyTcN;
      const bool bcopy = pt < kStepK * kSkinnyTcN;
      const uint32_t boff =
          blay == 1 ? static_cast<uint32_t>(bk * tr.tn * 8 + bn * 8)
          : blay == 3 ? static_cast<uint32_t>((bn >> 4) * 2048 + bk * 128 + (bn & 15) * 8)
                      : swz128(bn, bk);
      float acc[2 * kSkinnyTcN];
#pragma unroll
      for (int j = 0; j < 2 * kSkinnyTcN; ++j) acc[j] = 0.f;
      const int ksteps = static_cast<int>(tr.ksteps);
      for (int s = 0; s < ksteps; ++s) {
        if (!ptx::mbar_wait(raw_full(rr), rph)) {
          record_error(err_flag, kErrRawWait);
          return false;
        }
        const uint32_t ra = raw_a(rr), rb = raw_b(rr);
        const int r_cur = static_cast<int>(rr);
        if (++rr == kRaw) {
          rr = 0;
          rph ^= 1u;
        }
        // Buffers alternate over all SIMT stages of this CTA (also across
        // tiles): a buffer is rewritten only after the barrier that follows
        // its last reads.
        float2 (*bs)[kSkinnyTcN + 1] = s_skb[sk_cnt++ & 1];
        if (bcopy) {
          float2 b = bn < ncols ? lds64(rb + boff) : make_float2(0.f, 0.f);
          if (conjB) b.y = -b.y;
          bs[bk][bn] = b;
        }
        float2 a[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          a[i] = lds64(ra + aoff[i]);
          if (conjA) a[i].y = -a[i].y;
        }
        converters_sync();  // this stage's B copy is complete
        float sacc[2 * kSkinnyTcN];
#pragma unroll
        for (int j = 0; j < 2 * kSkinnyTcN; ++j) sacc[j] = 0.f;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
#pragma unroll
          for (int n = 0; n < kSkinnyTcN; ++n) {
            if (n >= ncols) break;
            const float2 b = bs[kq + 4 * i][n];
            sacc[2 * n] = fmaf(a[i].x, b.x, fmaf(-a[i].y, b.y, sacc[2 * n]));
            sacc[2 * n + 1] = fmaf(a[i].x, b.y, fmaf(a[i].y, b.x, sacc[2 * n + 1]));
          }
        }
#pragma unroll
        for (int j = 0; j < 2 * kSkinnyTcN; ++j) acc[j] += sacc[j];
        // The stage's values are consumed: release it to the next TMA fill
        // behind the cross-proxy fence.
        ptx::fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) ptx::mbar_arrive(raw_empty(r_cur));
      }
#pragma unroll
      for (int j = 0; j < 2 * kSkinnyTcN; ++j) {
        acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], 1);
        acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], 2);
      }
      const int64_t m = tr.m0 + r;
      if (kq == 0 && m < g.M) {
        const bool accumulate = g.flags & kFlagAccumulate;
        const bool beta_zero = g.flags & kFlagBetaZero;
        const float ar = (float)g.alpha[0], ai = (float)g.alpha[1];
        const float br = (float)g.beta[0], bi = (float)g.beta[1];
        float2* __restrict__ Cr = Cp + offs(g.rsC, g.uC_m, m);
#pragma unroll
        for (int n = 0; n < kSkinnyTcN; ++n) {
          if (n >= ncols) break;
          const float re = acc[2 * n], im = acc[2 * n + 1];
          const float tr_ = ar * re - ai * im, ti = ar * im + ai * re;
          float2* c = Cr + offs(g.csC, g.uC_n, tr.n0 + n);
          if (accumulate) {
            const float2 o = *c;
            *c = make_float2(o.x + tr_, o.y + ti);
          } else if (beta_zero) {
            *c = make_float2(tr_, ti);
          } else {
            const float2 o = *c;
            *c = make_float2(tr_ + (br * o.x - bi * o.y), ti + (br * o.y + bi * o.x));
          }
        }
      }
      return true;
    };

    for (int64_t t = blockIdx.x; t < total_tiles && ok; t += gridDim.x) {
      const TileRef tr = locate(&single, group, nprob, t, hint);
      const TcProblem* p = tr.p;
      const GemmArgs& g = p->g;
      const int amode = p->amode, bmode = p->bmode;
      const bool conjA = g.flags & kFlagConjA;
      const bool conjB = g.flags & kFlagConjB;
      const bool row_ok = (tr.m0 + ci) < g.M;
      const int alay = (amode == kAKM || amode == kAKM16) ? 2
                       : (amode == kAMK16 || amode == kAMK16K) ? 1 : 0;
      const int blay = bmode == kBKN ? 1 : (bmode == kBKN16 ? 3 : 0);
      const int64_t split = tr.kb / g.k_per_split;
      float2* __restrict__ Cp = static_cast<float2*>(g.C) + split * g.c_split_stride;
      if (p->skinny) {
        ok = run_skinny(tr, alay, blay, conjA, conjB, Cp);
        if (!ok) break;
      } else {
        cur_tn = tr.tn;
#pragma unroll
        for (int j = 0; j < 64; ++j) master[j] = 0.f;
        const int64_t chunk_base = chunk_cnt;
        using I0 = std::integral_constant<int, 0>;
        using I1 = std::integral_constant<int, 1>;
        using I2 = std::integral_constant<int, 2>;
        using I3 = std::integral_constant<int, 3>;
        switch (alay * 4 + blay) {
          case 0: ok = run_stages(I0{}, I0{}, tr, conjA, conjB, row_ok, chunk_base); break;
          case 1: ok = run_stages(I0{}, I1{}, tr, conjA, conjB, row_ok, chunk_base); break;
          case 3: ok = run_stages(I0{}, I3{}, tr, conjA, conjB, row_ok, chunk_base); break;
          case 4: ok = run_stages(I1{}, I0{}, tr, conjA, conjB, row_ok, chunk_base); break;
          case 5: ok = run_stages(I1{}, I1{}, tr, conjA, conjB, row_ok, chunk_base); break;
          case 7: ok = run_stages(I1{}, I3{}, tr, conjA, conjB, row_ok, chunk_base); break;
          case 8: ok = run_stages(I2{}, I0{}, tr, conjA, conjB, row_ok, chunk_base); break;
          case 9: ok = run_stages(I2{}, I1{}, tr, conjA, conjB, row_ok, chunk_base); break;
          default: ok = run_stages(I2{}, I3{}, tr, conjA, conjB, row_ok, chunk_base); break;
        }
        if (!ok) break;

        // -------------------------------------------------------- epilogue ---
        if (!ptx::mbar_wait(acc_full, static_cast<uint32_t>(tile_cnt & 1))) {
          record_error(err_flag, kErrAccWait);
          ok = false;
          break;
        }
        ptx::tc_fence_after();
        // The last chunk of the tile was not folded in the loop; then the
        // corrections.  After these reads the accumulators are free again.
        const int64_t c_last = chunk_base + (tr.ksteps > 0 ? (tr.ksteps - 1) >> tr.fsh : 0);
        const int buf_last = static_cast<int>(c_last & 1);
        // An empty K range (K = 0) leaves the accumulators unwritten: nothing
        // is folded (C = beta C), but the arrivals below keep the barrier
        // phases of both sides in step (the MMA thread counts a chunk too).
        if (tr.ksteps > 0) {
          fold_from(buf_last ? kChunkCol1 : kChunkCol0);
          fold_from(kCorrCol);
        }
        ptx::tc_fence_before();
        __syncwarp();
        if (lane == 0) {
          ptx::mbar_arrive(chunk_empty(buf_last));
          ptx::mbar_arrive(acc_empty);
        }
        chunk_cnt = c_last + 1;
        ++tile_cnt;

        if (64 * wg < tr.tn)
          store_tile<64>(g, Cp, tr.m0 + ci, row_ok, tr.n0, wg * 64, part, master,
                         tr.n0 + tr.tn);
      }
      bool final_tile = true;
      if (fix && p->fix_begin >= 0) {
        // In-kernel split-K reduction.  Every converter's partial stores
        // are made visible device-wide before the one arrival of this split;
        // the split that arrives last (all others' partials written) sums
        // the output tile over all splits.
        __threadfence();
        converters_sync();
        if (pt == 0) {
          int* ctr = fix + p->fix_begin + tr.out_tile;
          const int last = atomicAdd(ctr, 1) == p->splits - 1;
          if (last) *ctr = 0;  // every split has arrived: ready for the next launch
          s_fix_last = last;
          __threadfence();
        }
        converters_sync();
        final_tile = s_fix_last != 0;
        if (final_tile) fix_reduce_tile(*p, tr, pt);
      }
      if (done && final_tile) {
        // Publish the tile: every converter's stores, then one release-add.
        converters_sync();
        if (pt == 0) {
          __threadfence();
          red_release_add(done + tr.pi, 1);
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

// ---------------------------------------------------------- B panels ---
// B split once for all M tiles: row n of the panel array holds, per stage of
// 32 real k (16 complex k), kBufs rows of 128 bytes, the bytes the converters
// would write into the operand stage for column n before the 128-byte swizzle
// (which the TMA load of a panel stage applies):
//   3xTF32: [hi of the 32 values] [lo]
//   BF16x3: [piece 0 (32 bf16) | piece 1]
//   BF16x6: [piece 0 | piece 1] [piece 2 | zeros]
// Values in k order: re, im (conjugated under kFlagConjB) of each complex k,
// or the real k; zero past K.  The pieces are the converters' (same split
// functions), so a product is bit-identical with or without panels.
// One thread per (column, stage); stages fastest when B has unit K stride
// (contiguous reads and writes), columns fastest otherwise (reads coalesced
// across columns).
template <int Prec, bool kReal>
__global__ void __launch_bounds__(256)
split_b_panels(const GemmArgs g, uint4* __restrict__ out, int64_t nstages, int k_fastest) {
  constexpr int kBufs = Prec == kPrecBF16x3 ? 1 : 2;
  const int64_t idx = static_cast<int64_t>(blockIdx.x) * 256 + threadIdx.x;
  if (idx >= g.N * nstages) return;
  const int64_t n = k_fastest ? idx / nstages : idx % g.N;
  const int64_t s = k_fastest ? idx % nstages : idx / g.N;
  const int64_t cn = offs(g.csB, g.uB_n, n);
  float v[32];
  // A full stage of a unit-K-stride column, 16-byte aligned, is read as eight
  // 16-byte loads; otherwise element by element through the K offsets.
  if constexpr (kReal) {
    const float* __restrict__ B = static_cast<const float*>(g.B);
    const float* col = B + cn + 32 * s;
    if (g.uB_k == 1 && 32 * s + 32 <= g.K && (reinterpret_cast<uintptr_t>(col) & 15u) == 0) {
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float4 q = reinterpret_cast<const float4*>(col)[j];
        v[4 * j] = q.x;
        v[4 * j + 1] = q.y;
        v[4 * j + 2] = q.z;
        v[4 * j + 3] = q.w;
      }
    } else {
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int64_t k = 32 * s + j;
        v[j] = k < g.K ? B[cn + offs(g.rsB, g.uB_k, k)] : 0.f;
      }
    }
  } else {
    const float2* __restrict__ B = static_cast<const float2*>(g.B);
    const bool conj = g.flags & kFlagConjB;
    const float2* col = B + cn + 16 * s;
    if (g.uB_k == 1 && 16 * s + 16 <= g.K && (reinterpret_cast<uintptr_t>(col) & 15u) == 0) {
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float4 q = reinterpret_cast<const float4*>(col)[j];
        v[4 * j] = q.x;
        v[4 * j + 1] = q.y;
        v[4 * j + 2] = q.z;
        v[4 * j + 3] = q.w;
      }
    } else {
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int64_t k = 16 * s + j;
        const float2 x = k < g.K ? B[cn + offs(g.rsB, g.uB_k, k)] : make_float2(0.f, 0.f);
        v[2 * j] = x.x;
        v[2 * j + 1] = x.y;
      }
    }
    if (conj) {
#pragma unroll
      for (int j = 0; j < 16; ++j) v[2 * j + 1] = -v[2 * j + 1];
    }
  }
  uint4* __restrict__ row = out + (n * nstages + s) * (8 * kBufs);
  if constexpr (Prec == kPrecTF32x3) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const Split a = split_tf32(v[4 * q]), b = split_tf32(v[4 * q + 1]);
      const Split c = split_tf32(v[4 * q + 2]), d = split_tf32(v[4 * q + 3]);
      row[q] = make_uint4(a.hi, b.hi, c.hi, d.hi);
      row[8 + q] = make_uint4(a.lo, b.lo, c.lo, d.lo);
    }
  } else {
    constexpr int kPieces = Prec == kPrecBF16x6 ? 3 : 2;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      uint32_t w[4][3];
#pragma unroll
      for (int i = 0; i < 4; ++i)
        split_bf16<kPieces>(v[8 * q + 2 * i], v[8 * q + 2 * i + 1], w[i][0], w[i][1], w[i][2]);
      row[q] = make_uint4(w[0][0], w[1][0], w[2][0], w[3][0]);
      row[4 + q] = make_uint4(w[0][1], w[1][1], w[2][1], w[3][1]);
      if (kPieces == 3) {
        row[8 + q] = make_uint4(w[0][2], w[1][2], w[2][2], w[3][2]);
        row[12 + q] = make_uint4(0u, 0u, 0u, 0u);
      }
    }
  }
}

// --------------------------------------------- one tile per CTA variant ---
// For a single contraction whose operands are a uniform 2-D view or gathered,
// this non-persistent form (one output tile per CTA, operand modes as template
// parameters) measured faster than the persistent kernel on GB300 (2.81 ms vs
// 3.06-3.10 ms for complex64 4096^3), so single contractions use it when their
// fetch modes allow; the persistent kernel serves grouped launches and the
// per-16-row block TMA modes.
enum : int { kTmaMK = 0, kTmaKM = 1, kGatherMK = 2 };
// B modes: raw tiles by TMA ([n][k] or [k][n]) or gathered, each split by the
// converters; or kPanelNK, B split once beforehand into panels
// (split_b_panels) whose stages TMA loads straight into the operand ring.
enum : int { kTmaNK = 0, kTmaKN = 1, kGatherNK = 2, kPanelNK = 3 };
// Operand stages of the panel form: TMA fills them, so the ring is deeper
// than the converter-written one (which is bounded by the A stages in TMEM).
constexpr int kPanelStages = 4;

struct TmaMaps {
  CUtensorMap a;
  CUtensorMap b;
};

// Prec selects the split products (kPrec*).  The bf16 forms keep the same
// tiles, stages and accumulators; per stage (32 real K) they issue two K = 16
// kind::f16 MMAs per product, A pieces packed two per TMEM column (16 columns
// each) and B pieces in 64-byte halves of the 128-byte swizzled rows (pieces
// 0 | 1 in the first B buffer, piece 2 in the second).
// Converter warpgroups of the one-tile kernel.  Two (8 warps, 384 threads in
// all, 64 accumulator columns per converter thread) measured faster on GB300
// than four (16 warps, 640 threads, 32 columns each: 180 vs 198 TFLOP/s at
// complex64 4096^3, 3xTF32), whose 96-register budget and doubled per-stage
// barrier traffic outweigh the extra warps to interleave.
constexpr int kCW1 = 2;
constexpr int kConverters1 = 128 * kCW1;
constexpr int kThreads1 = kConvBase + kConverters1;
constexpr int kAK1 = kStepK / kCW1;                          // complex k of A per thread
constexpr int kMC1 = kTileN / kCW1;                          // accumulator columns per thread
constexpr int kBP1 = (kTileN * kStepK / 2) / kConverters1;   // 16-byte B pieces per thread
constexpr int kB16P1 = (kTileN * kStepK / 4) / kConverters1; // bf16 B chunks per thread
static_assert(kAK1 % 4 == 0 && kMC1 % 32 == 0 && kBP1 >= 1 && kB16P1 >= 1, "converter split");

// Real float32 (kReal): the same GEMM without the 1M expansion.  A tile is
// 128 real rows (one TMEM lane each), K is staged 32 reals per stage (the
// same 128-byte swizzle rows), the raw A stage doubles to 16 KB, B's raw
// bytes are the complex layout's (k pairs for complex elements), and the
// epilogue writes one real row per thread.
// CTA pairs (kPair): each CTA holds half of the B tile (64 columns), raw and
// converted, so its B stages are half as large.
// Both forms keep the same TMEM layout and pipeline: two chunk
// accumulators (ping-pong), the corrections, two converted A stages.  A
// 4-stage A ring with a single chunk accumulator measured slower in both
// (the MMA thread then waits for each fold before a chunk's main products).
constexpr int kBarrierBytes1 = 256;
// MMA issue by two threads (different warps) for 3xTF32: one issues the main
// products into the chunk accumulators, the other the correction products
// into their accumulator.  Each accumulator still sees one thread's products
// in a fixed order (results unchanged, bit for bit).  Measured at complex64
// 4096^3 (pairs): 3xTF32 200 -> 208 TFLOP/s; BF16x6 218 -> 202 and BF16x3
// 293 -> 286, so the bf16 forms keep one issuer.  A thread issuing MMAs
// stalls while the tensor pipe's queue is full, so the split helps only
// where its own issue work is the longer part.  Needs a free warp: loaders
// that gather use all three loader warps.
template <int Prec>
constexpr bool split_mma_issue() {
  return Prec == kPrecTF32x3;
}
template <bool kReal, bool kPanel, bool kPair = false>
constexpr int smem_bytes_1() {
  return 1024 +
         kRaw * ((kReal ? 16384 : kRawABytes) + (kPanel ? 0 : (kPair ? kRawBBytes / 2 : kRawBBytes))) +
         (kPanel ? kPanelStages : kStages) * (kPair ? kOpBytes / 2 : kOpBytes) + kBarrierBytes1;
}

// kPair: clusters of two CTAs sharing one tcgen05.mma.cta_group::2 per
// product (M = 256 real rows = 128 complex rows per pair, N = 128).  Each CTA
// loads and converts its own 64 complex rows of A into its own TMEM, as in
// the one-CTA form, but only its half of the B tile (64 columns), and the
// pair's MMAs read B half from each CTA: per SM, half the B bytes staged,
// converted and read by the tensor cores per flop.  One thread of the even
// CTA issues every MMA; the converters of both CTAs arrive on its barriers,
// and its commits arrive on the barriers of both.
template <int AMode, int BMode, int Prec, bool kReal, bool kPair>
__global__ void __launch_bounds__(kThreads1, 1)
tc1m_contract(const GemmArgs args, const __grid_constant__ TmaMaps maps, int* err_flag) {
  constexpr bool kBF16 = Prec != kPrecTF32x3;
  // Stages per main chunk: the truncation bias of the tensor cores' FP32
  // accumulation grows with the accumulating MMAs per chunk, so chunks hold
  // 16 main-product MMAs: 8 stages of 2 kind::f16 MMAs (K = 16) or 4 of 4
  // kind::tf32 MMAs (K = 8).  Measured at complex64 4096^3: BF16x6 folding
  // every 8 stages 221.5 -> 225.5 TFLOP/s, error 2.8e-7 -> 3.3e-7 (log-uniform
  // set 3.2e-7 -> 3.6e-7); 3xTF32 at 8 stages rose to 6.9e-7, so it keeps 4.
  constexpr int kFoldT = kBF16 ? 2 * kFold : kFold;
  constexpr int kPieces = Prec == kPrecBF16x6 ? 3 : 2;
  // MMA M: 128 real rows per CTA, 256 for a pair.
  constexpr uint32_t kIdescT = ptx::idesc_f32acc(kBF16 ? 1u /*BF16*/ : 2u /*TF32*/,
                                                 kPair ? 256u : 128u, kTileN);
  constexpr bool kTmaA = AMode != kGatherMK;
  constexpr bool kPanel = BMode == kPanelNK;
  constexpr bool kTmaB = BMode == kTmaNK || BMode == kTmaKN;
  constexpr bool kGather = !kTmaA || BMode == kGatherNK;
  constexpr int kOpStages = kPanel ? kPanelStages : kStages;
  constexpr int kPanelBufs = Prec == kPrecBF16x3 ? 1 : 2;
  constexpr int kRowsT = kReal ? 128 : kTileMc;        // C rows per tile
  constexpr int kStepKE = kReal ? 32 : kStepK;         // K elements per stage
  constexpr int kCx = kReal ? 1 : 2;                   // floats per element (TMA coordinates)
  constexpr int kRawABytesT = kReal ? 16384 : kRawABytes;
  // B columns this CTA loads and converts, and the sizes that follow.
  constexpr int kNCta = kPair ? kTileN / 2 : kTileN;
  constexpr int kRawBBytesT = kNCta * kStepK * 8;
  constexpr int kBHalfT = kNCta * 128;      // one converted B buffer (hi, lo or 2 pieces)
  constexpr int kOpBytesT = 2 * kBHalfT;
  constexpr int kBPT = (kNCta * kStepK / 2) / kConverters1;    // 16-byte TF32 B pieces per thread
  constexpr int kB16PT = (kNCta * kStepK / 4) / kConverters1;  // bf16 B chunks per thread
  static_assert(kBPT >= 1 && kB16PT >= 1, "B conversion split");
  static_assert(!kPair || (!kReal && !kPanel && kTmaA && kTmaB),
                "CTA pairs take complex operands loaded by TMA");
  // Arrivals on the barriers the MMA thread waits for: the converter warps
  // of this CTA, or of both CTAs of a pair.
  constexpr uint32_t kConvArrivals = (kPair ? 2u : 1u) * (kConverters1 / 32);
  constexpr int kRawBytesT = kRawABytesT + (kPanel ? 0 : kRawBBytesT);
  // Arrivals per raw stage: one expect_tx arrive from the TMA thread, one
  // cp.async completion arrive per gather thread.
  constexpr uint32_t kRawArrivals = (kTmaA || kTmaB ? 1u : 0u) + (kGather ? kLoaders : 0u);
  constexpr uint32_t kTmaBytes = (kTmaA ? kRawABytesT : 0) + (kTmaB ? kRawBBytesT : 0);

  extern __shared__ __align__(16) uint8_t smem_raw[];
  const uint32_t base = (ptx::smem_u32(smem_raw) + 1023u) & ~1023u;
  uint8_t* const base_ptr = smem_raw + (base - ptx::smem_u32(smem_raw));
  const uint32_t raw0 = base;                          // kRaw x (A | B)
  const uint32_t op0 = raw0 + kRaw * kRawBytesT;       // kOpStages x (B hi | B lo)
  const uint32_t bars = op0 + kOpStages * kOpBytesT;
  auto raw_a = [&](int r) { return raw0 + r * kRawBytesT; };
  auto raw_b = [&](int r) { return raw0 + r * kRawBytesT + kRawABytesT; };
  auto raw_full = [&](int r) { return bars + 8u * r; };
  auto raw_empty = [&](int r) { return bars + 8u * (kRaw + r); };
  auto full_bar = [&](int s) { return bars + 8u * (2 * kRaw + s); };
  auto empty_bar = [&](int s) { return bars + 8u * (2 * kRaw + kStages + s); };
  auto chunk_full = [&](int b) { return bars + 8u * (2 * kRaw + 2 * kStages + b); };
  auto chunk_empty = [&](int b) { return bars + 8u * (2 * kRaw + 2 * kStages + 2 + b); };
  const uint32_t acc_bar = bars + 8u * (2 * kRaw + 2 * kStages + 4);
  const uint32_t tmem_slot = acc_bar + 8u;
  // Panel stages: filled by TMA (one expect_tx arrive), emptied by an MMA commit.
  auto pfull = [&](int i) { return acc_bar + 16u + 8u * i; };
  auto pempty = [&](int i) { return acc_bar + 16u + 8u * (kPanelStages + i); };
  static_assert(8 * (2 * kRaw + 2 * kStages + 5 + 1 + 2 * kPanelStages) <= kBarrierBytes1,
                "barrier area");
  volatile uint32_t* tmem_slot_ptr = reinterpret_cast<volatile uint32_t*>(base_ptr + (tmem_slot - base));

  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const uint32_t rank = kPair ? ptx::cluster_ctarank() : 0u;

  if (warp == 0) {
    if constexpr (kPair) {
      ptx::tmem_alloc2(tmem_slot, kTmemCols);
      ptx::tmem_relinquish2();
    } else {
      ptx::tmem_alloc(tmem_slot, kTmemCols);
      ptx::tmem_relinquish();
    }
  }
  if (tid == 32) {
    // Barriers the MMA issuers commit to count one commit per issuer.
    constexpr uint32_t kIssuers = (split_mma_issue<Prec>() && !kGather) ? 2u : 1u;
    if (kPanel) {
      for (int i = 0; i < kPanelStages; ++i) {
        ptx::mbar_init(pfull(i), 1);
        ptx::mbar_init(pempty(i), kIssuers);
      }
    }
    for (int r = 0; r < kRaw; ++r) {
      ptx::mbar_init(raw_full(r), kRawArrivals);
      ptx::mbar_init(raw_empty(r), kConverters1 / 32);
    }
    for (int s = 0; s < kStages; ++s) {
      ptx::mbar_init(full_bar(s), kConvArrivals);
      ptx::mbar_init(empty_bar(s), kIssuers);
    }
    for (int b = 0; b < 2; ++b) {
      ptx::mbar_init(chunk_full(b), 1);
      ptx::mbar_init(chunk_empty(b), kConvArrivals);
    }
    ptx::mbar_init(acc_bar, kIssuers);
    ptx::fence_mbar_init();
  }
  if (tid == 64) {
    if (kTmaA) ptx::tma_prefetch_desc(&maps.a);
    if (kTmaB) ptx::tma_prefetch_desc(&maps.b);
  }
  // A pair starts once both CTAs have their barriers and TMEM.
  ptx::tc_fence_before();
  if constexpr (kPair) ptx::cluster_sync(); else __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_slot_ptr;
  // Waits of the MMA thread (for a pair, the converters of both CTAs arrive
  // on them), its MMAs and commits.
  auto wait_conv = [&](uint32_t bar, uint32_t ph) { return ptx::mbar_wait(bar, ph); };
  auto mma_tf = [&](uint32_t d, uint32_t a, uint64_t b, uint32_t acc) {
    if constexpr (kPair) ptx::mma_tf32_ts2(d, a, b, kIdescT, acc);
    else ptx::mma_tf32_ts(d, a, b, kIdescT, acc);
  };
  auto mma_bf = [&](uint32_t d, uint32_t a, uint64_t b, uint32_t acc) {
    if constexpr (kPair) ptx::mma_f16_ts2(d, a, b, kIdescT, acc);
    else ptx::mma_f16_ts(d, a, b, kIdescT, acc);
  };
  auto commit = [&](uint32_t bar) {
    if constexpr (kPair) ptx::mma_commit2(bar);
    else ptx::mma_commit(bar);
  };
  // Converter arrivals on the MMA thread's barriers (the even CTA's for a pair).
  auto arrive_mma = [&](uint32_t bar) {
    if constexpr (kPair) ptx::mbar_arrive_cluster(ptx::mapa(bar, 0));
    else ptx::mbar_arrive(bar);
  };

  const int64_t M = args.M, N = args.N;
  // Split-K: this CTA row covers K range [kb, K) (kb a multiple of kStepK).
  const int64_t kb = static_cast<int64_t>(blockIdx.y) * args.k_per_split;
  const int64_t K = min(args.K, kb + args.k_per_split);
  // Output tiles: kRowsT rows per CTA, two CTAs' rows per pair.
  constexpr int kRowsTile = kPair ? 2 * kRowsT : kRowsT;
  const int64_t tiles_m = (M + kRowsTile - 1) / kRowsTile;
  const int64_t tiles_n = (N + kTileN - 1) / kTileN;
  // Groups of 16 M-tiles of 64 rows (8 pair tiles) sweep N so CTAs running
  // together share B in L2.
  constexpr int64_t G = kPair ? 8 : 16;
  const int64_t t = kPair ? (blockIdx.x >> 1) : blockIdx.x;
  const int64_t group = t / (G * tiles_n);
  const int64_t first_m = group * G;
  const int64_t gsize = min(G, tiles_m - first_m);
  const int64_t tm = first_m + (t % (G * tiles_n)) % gsize;
  const int64_t tn = (t % (G * tiles_n)) / gsize;
  const int64_t m0 = tm * kRowsTile + rank * kRowsT, n0 = tn * kTileN;
  const int64_t nb0 = n0 + rank * kNCta;  // first B column this CTA loads
  const int64_t ksteps = (K - kb + kStepKE - 1) / kStepKE;

  // Threads issuing MMAs: lane 0 of warp 0 (main products, or all), and with
  // a split issue lane 0 of warp 3 (correction products).
  constexpr bool kSplitIssue = split_mma_issue<Prec>() && !kGather;
  if (warp == 0 || (kSplitIssue && warp == 3)) {
    // ---------------------------------------------------------- MMA issue ---
    const bool issue_main = warp == 0;
    const bool issue_corr = !kSplitIssue || warp == 3;
    if (lane == 0 && rank == 0) {
      // Descriptors: the 14-bit start-address field of a shared-memory
      // descriptor is address >> 4, so a descriptor at a byte offset is the
      // base descriptor plus offset >> 4.
      const uint64_t desc0 = ptx::smem_desc_sw128(op0);
      const uint32_t d_corr = tmem + kCorrCol;
      for (int64_t s = 0; s < ksteps; ++s) {
        const int st = static_cast<int>(s % kStages);
        const uint32_t ph = static_cast<uint32_t>((s / kStages) & 1);
        const int64_t c = s / kFoldT;
        const int buf = static_cast<int>(c & 1);
        const bool chunk_start = (s % kFoldT) == 0;
        if (issue_main && chunk_start && c >= 2 &&
            !wait_conv(chunk_empty(buf), static_cast<uint32_t>(((c - 2) >> 1) & 1))) {
          record_error(err_flag, kErrChunkWait);
          break;
        }
        if (!wait_conv(full_bar(st), ph)) {
          record_error(err_flag, kErrFullWait);
          break;
        }
        const int sb = kPanel ? static_cast<int>(s % kPanelStages) : st;
        if (kPanel && !ptx::mbar_wait(pfull(sb), static_cast<uint32_t>((s / kPanelStages) & 1))) {
          record_error(err_flag, kErrFullWait);
          break;
        }
        ptx::tc_fence_after();
        const uint32_t d_main = tmem + (buf ? kChunkCol1 : kChunkCol0);
        const uint32_t a_st = tmem + kAStageCol + 64u * st;
        const uint64_t db = desc0 + static_cast<uint64_t>((sb * kOpBytesT) >> 4);
        // One stage: TF32x3 (kind::tf32, K = 8): 4 x (hi.hi -> main, hi.lo +
        // lo.hi -> corrections).  bf16 (kind::f16, K = 16): A piece p at 16
        // TMEM columns +16p, B piece p in 64-byte half (p & 1) of B buffer
        // (p >> 1); 2 x (x0y0 -> main, x0y1 + x1y0 [+ x1y1 + x0y2 + x2y0] ->
        // corrections).
        auto bd = [&](int p, int kk) {
          return db + static_cast<uint64_t>(((p >> 1) * kBHalfT + 64 * (p & 1) + 32 * kk) >> 4);
        };
        constexpr int kKK = kBF16 ? 2 : 4;
        if (issue_main) {
#pragma unroll
          for (int kk = 0; kk < kKK; ++kk) {
            const uint32_t acc = (chunk_start && kk == 0) ? 0u : 1u;
            if constexpr (!kBF16) mma_tf(d_main, a_st + 8u * kk, db + 2u * kk, acc);
            else mma_bf(d_main, a_st + 8u * kk, bd(0, kk), acc);
          }
        }
        if (issue_corr) {
#pragma unroll
          for (int kk = 0; kk < kKK; ++kk) {
            const uint32_t first = (s == 0 && kk == 0) ? 0u : 1u;
            if constexpr (!kBF16) {
              const uint64_t dh = db + 2u * kk;
              const uint64_t dl = db + static_cast<uint64_t>((kBHalfT + 32 * kk) >> 4);
              mma_tf(d_corr, a_st + 8u * kk, dl, first);
              mma_tf(d_corr, a_st + 32u + 8u * kk, dh, 1u);
            } else {
              const uint32_t ak = a_st + 8u * kk;
              mma_bf(d_corr, ak, bd(1, kk), first);
              mma_bf(d_corr, ak + 16u, bd(0, kk), 1u);
              if (kPieces == 3) {
                mma_bf(d_corr, ak + 16u, bd(1, kk), 1u);
                mma_bf(d_corr, ak, bd(2, kk), 1u);
                mma_bf(d_corr, ak + 32u, bd(0, kk), 1u);
              }
            }
          }
        }
        commit(empty_bar(st));
        if (kPanel) commit(pempty(sb));
        if (issue_main && ((s % kFoldT) == kFoldT - 1 || s == ksteps - 1)) commit(chunk_full(buf));
      }
      // Signal the epilogue (also after an abort, so nobody waits forever),
      // then make sure no MMA is still writing TMEM before it is freed.
      commit(acc_bar);
      if (!ptx::mbar_wait(acc_bar, 0)) record_error(err_flag, kErrAccWait);
    }
    __syncwarp();
  } else if (tid < kConvBase) {
    // ------------------------------------------------------------ loaders ---
    const int lt = tid - kLoaderBase;  // 0..95
    // Gather work of this thread: fixed rows / columns, K walked per stage.
    for (int64_t s = 0; s < ksteps; ++s) {
      const int r = static_cast<int>(s % kRaw);
      const uint32_t ph = static_cast<uint32_t>((s / kRaw) & 1);
      const int64_t k0 = kb + s * kStepKE;
      if (kGather || lt == 0) {
        if (!ptx::mbar_wait(raw_empty(r), ph ^ 1u)) {
          record_error(err_flag, kErrRawWait);
          break;
        }
      }
      if ((kTmaA || kTmaB) && lt == 0) {
        ptx::mbar_arrive_expect_tx(raw_full(r), kTmaBytes);
        if (AMode == kTmaMK)
          ptx::tma_load_2d(raw_a(r), &maps.a, static_cast<int>(kCx * m0), static_cast<int>(k0), raw_full(r));
        if (AMode == kTmaKM)
          ptx::tma_load_2d(raw_a(r), &maps.a, static_cast<int>(kCx * k0), static_cast<int>(m0), raw_full(r));
        if (BMode == kTmaNK)
          ptx::tma_load_2d(raw_b(r), &maps.b, static_cast<int>(kCx * k0), static_cast<int>(nb0), raw_full(r));
        if (BMode == kTmaKN)
          ptx::tma_load_2d(raw_b(r), &maps.b, static_cast<int>(kCx * nb0), static_cast<int>(k0), raw_full(r));
      }
      if (kGather) {
        if constexpr (kReal) {
          if (AMode == kGatherMK) gather_a_stage_real<8>(args, raw_a(r), lt, m0, k0, K);
          if (BMode == kGatherNK) gather_b_stage_real<8>(args, raw_b(r), lt, n0, k0, K);
        } else {
          if (AMode == kGatherMK) gather_a_stage<8>(args, raw_a(r), lt, m0, k0, K);
          if (BMode == kGatherNK) gather_b_stage<8>(args, raw_b(r), lt, n0, k0, K);
        }
        ptx::cp_async_arrive_noinc(raw_full(r));
      }
      if (kPanel && lt == 0) {
        // B panel stage: kPanelBufs 128-byte rows per column, the operand
        // stage's bytes before the swizzle (the TMA load applies it).
        const int sb = static_cast<int>(s % kPanelStages);
        if (!ptx::mbar_wait(pempty(sb), static_cast<uint32_t>(((s / kPanelStages) & 1) ^ 1))) {
          record_error(err_flag, kErrRawWait);
          break;
        }
        const int x = static_cast<int>((kb / kStepKE + s) * kPanelBufs * 64);
        ptx::mbar_arrive_expect_tx(pfull(sb), static_cast<uint32_t>(kPanelBufs * kBHalfT));
        ptx::tma_load_2d(op0 + sb * kOpBytesT, &maps.b, x, static_cast<int>(n0), pfull(sb));
        if (kPanelBufs == 2)
          ptx::tma_load_2d(op0 + sb * kOpBytesT + kBHalfT, &maps.b, x + 64, static_cast<int>(n0),
                           pfull(sb));
      }
    }
  } else {
    // -------------------------------------------- converters, fold, epilogue ---
    // kCW1 warpgroups: warpgroup wg converts complex k [kAK1 wg, kAK1 (wg + 1))
    // of every staged A row and a 1/kCW1 share of the B tile, and folds and
    // writes accumulator columns [kMC1 wg, kMC1 (wg + 1)) of its TMEM lanes.
    const int pt = tid - kConvBase;
    const int wg = pt >> 7;
    const int q = (pt >> 5) & 3;     // TMEM lane quarter of this warp
    const int rho = 32 * q + lane;   // real row = TMEM lane
    const int ci = rho >> 1;         // complex row in the tile
    const int part = rho & 1;        // 0: real row "re", 1: "im"
    const uint32_t lane_base = static_cast<uint32_t>(32 * q) << 16;
    const bool conjA = args.flags & kFlagConjA;
    const bool conjB = args.flags & kFlagConjB;
    // C row of this thread: complex row ci, or (real) the lane's own row.
    const int crow = kReal ? rho : ci;
    const bool row_ok = (m0 + crow) < M;

    float master[kMC1];
#pragma unroll
    for (int j = 0; j < kMC1; ++j) master[j] = 0.f;

    // Fold chunk accumulator at column `col` into the FP32 master registers
    // (round-to-nearest adds): this thread's lane, kMC1 columns.
    auto fold_from = [&](uint32_t col) {
#pragma unroll
      for (int cc = 0; cc < kMC1 / 32; ++cc) {
        uint32_t r[32];
        ptx::tmem_ld32_sync(tmem + lane_base + col + kMC1 * wg + 32u * cc, r);
#pragma unroll
        for (int j = 0; j < 32; ++j) master[32 * cc + j] += __uint_as_float(r[j]);
      }
    };

    // Loop-invariant shared-memory offsets of this thread's raw reads and
    // operand writes.
    // Real A: the same 8-byte units of the swizzled [m][k] rows (k pairs),
    // row = the lane; [k][m] rows of 128 floats.
    uint32_t aoff[kAK1];
#pragma unroll
    for (int j = 0; j < kAK1; ++j)
      aoff[j] = (AMode == kTmaKM) ? swz128(crow, kAK1 * wg + 2 * (j >> 1))
                                  : static_cast<uint32_t>((kAK1 * wg + j) * 512 + ci * 8);
    const uint32_t areal = static_cast<uint32_t>(2 * kAK1 * wg * 512 + rho * 4);
    // TF32 B: piece j of this thread (id = pt + kConverters1 j) is two complex
    // k of one column ([n][k] tiles) or one k of two columns ([k][n] tile).
    uint32_t bsrc[kBPT], boff[kBPT][2];
#pragma unroll
    for (int j = 0; j < kBPT; ++j) {
      const int id = pt + kConverters1 * j;
      if (BMode == kTmaKN) {
        // k: complex k, or (real) the k pair 2k, 2k + 1 (rows of kNCta
        // complex or 128 real values).  Warp task w = id / 32 takes k =
        // 4 (w % 4) + lane % 4 and columns 16 (w / 4) + 2 (lane / 4), + 1:
        // the warp's 8-byte stores then fill all eight 16-byte chunks of the
        // swizzled rows (two lanes per slot) instead of four (k fixed per
        // warp: 8-way bank conflicts).
        const int w = id >> 5, l = id & 31;
        const int k = 4 * (w & 3) + (l & 3), n = 16 * (w >> 2) + 2 * (l >> 2);
        bsrc[j] = kReal ? static_cast<uint32_t>(2 * k * 512 + n * 4)
                        : static_cast<uint32_t>(k * kNCta * 8 + n * 8);
        boff[j][0] = swz128(n, k);
        boff[j][1] = swz128(n + 1, k);
      } else {
        const int n = id >> 3, kp = id & 7;
        bsrc[j] = swz128(n, 2 * kp);
        boff[j][0] = bsrc[j];
        boff[j][1] = 0;
      }
    }
    // bf16 B: id = pt + kConverters1 j covers column n = id & 127 and complex
    // k 4 kq .. 4 kq + 3 (kq = id >> 7): two 16-byte raw reads (one per k
    // pair) in the swizzled [n][k] tiles, four 8-byte reads in the [k][n]
    // tile; one 16-byte chunk (8 bf16) per piece, chunk kq (+4 for odd
    // pieces) of row n.  Consecutive lanes take consecutive n: no bank
    // conflicts.
    uint32_t b16src[kB16PT], b16row[kB16PT], b16chunk[kB16PT];
#pragma unroll
    for (int j = 0; j < kB16PT; ++j) {
      const int id = pt + kConverters1 * j;
      const int n = id % kNCta, kq = id / kNCta;
      b16src[j] = (BMode == kTmaKN)
                      ? (kReal ? static_cast<uint32_t>(8 * kq * 512 + n * 4)
                               : static_cast<uint32_t>(4 * kq * kNCta * 8 + n * 8))
                      : swz128(n, 4 * kq);
      b16row[j] = static_cast<uint32_t>((n >> 3) * 1024 + (n & 7) * 128);
      b16chunk[j] = static_cast<uint32_t>(kq ^ (n & 7));
    }
    constexpr int kBV = kBPT > 2 * kB16PT ? kBPT : 2 * kB16PT;

    bool ok = true;
    int r = 0, st = 0;
    uint32_t rph = 0, ph = 0;
    for (int64_t s = 0; s < ksteps; ++s) {
      if (!ptx::mbar_wait(raw_full(r), rph)) {
        record_error(err_flag, kErrRawWait);
        ok = false;
        break;
      }
      // A: kAK1 complex k (this warpgroup's share of the step) of row ci.
      const uint32_t ra = raw_a(r);
      [[maybe_unused]] const uint32_t rb = raw_b(r);
      // Complex: av[j] = (re, im) of complex k.  Real: av[j] = values of the
      // k pair 2j, 2j + 1 of the lane's row.
      float2 av[kAK1];
      if (AMode == kTmaKM) {
#pragma unroll
        for (int j = 0; j < kAK1 / 2; ++j) {
          const float4 v = lds128(ra + aoff[2 * j]);
          av[2 * j] = make_float2(v.x, v.y);
          av[2 * j + 1] = make_float2(v.z, v.w);
        }
      } else if constexpr (kReal) {
#pragma unroll
        for (int j = 0; j < kAK1; ++j)
          av[j] = make_float2(lds32(ra + areal + 1024u * j), lds32(ra + areal + 1024u * j + 512u));
      } else {
#pragma unroll
        for (int j = 0; j < kAK1; ++j) av[j] = lds64(ra + aoff[j]);
      }
      // B: this thread's 16-byte pieces (two complex each) of the raw tile
      // (none with panels: B arrives split).
      float4 bv[kBV];
      if constexpr (kPanel) {
      } else if constexpr (!kBF16) {
#pragma unroll
        for (int j = 0; j < kBPT; ++j) {
          if (kReal && BMode == kTmaKN) {
            // Columns n, n + 1 of rows 2k, 2k + 1: pair (2k, 2k + 1) of each column.
            const float2 t0 = lds64(rb + bsrc[j]), t1 = lds64(rb + bsrc[j] + 512u);
            bv[j] = make_float4(t0.x, t1.x, t0.y, t1.y);
          } else {
            bv[j] = lds128(rb + bsrc[j]);
          }
        }
      } else {
#pragma unroll
        for (int j = 0; j < kB16PT; ++j) {
          if (kReal && BMode == kTmaKN) {
            // Column n, real k 8 kq .. 8 kq + 7 (rows of 128 floats).
            float v[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) v[i] = lds32(rb + b16src[j] + 512u * i);
            bv[2 * j] = make_float4(v[0], v[1], v[2], v[3]);
            bv[2 * j + 1] = make_float4(v[4], v[5], v[6], v[7]);
          } else if (BMode == kTmaKN) {
            constexpr uint32_t kRow = kNCta * 8;  // one k row of the raw [k][n] tile
            const float2 t0 = lds64(rb + b16src[j]), t1 = lds64(rb + b16src[j] + kRow);
            const float2 t2 = lds64(rb + b16src[j] + 2 * kRow), t3 = lds64(rb + b16src[j] + 3 * kRow);
            bv[2 * j] = make_float4(t0.x, t0.y, t1.x, t1.y);
            bv[2 * j + 1] = make_float4(t2.x, t2.y, t3.x, t3.y);
          } else {
            // k pair 2kq + 1 sits in the neighbouring 16-byte chunk (bit 4).
            bv[2 * j] = lds128(rb + b16src[j]);
            bv[2 * j + 1] = lds128(rb + (b16src[j] ^ 16u));
          }
        }
      }
      // The raw stage is released after the conversion (below), once the
      // values read from it are consumed and behind the cross-proxy fence:
      // TMA (async proxy) refills it, and generic-proxy reads that are not
      // ordered before that by a proxy fence can observe the refill.

      // A: the 1M rows of this thread's kAK1 complex k, [re, -im] (part 0) or
      // [im, re] (part 1), real: the pair as is; rows past M arrive as zeros
      // (TMA out-of-bounds fill, gather zero fill).  Split into registers
      // before the operand wait: only the stores follow it, which shortens
      // the round trip from an MMA stage's release to the next stage's
      // arrival (two A stages fit in TMEM, so that round trip must finish
      // within one stage of MMAs).
      uint32_t w[3][kAK1];                  // bf16: piece p of pair j
      uint32_t hi[2 * kAK1], lo[2 * kAK1];  // TF32: hi / lo of each value
#pragma unroll
      for (int j = 0; j < kAK1; ++j) {
        float2 v = av[j];
        if (conjA) v.y = -v.y;
        const float x0 = kReal ? v.x : (part ? v.y : v.x);
        const float x1 = kReal ? v.y : (part ? v.x : -v.y);
        if constexpr (kBF16) {
          split_bf16<kPieces>(x0, x1, w[0][j], w[1][j], w[2][j]);
        } else {
          const Split s0 = split_tf32(x0), s1 = split_tf32(x1);
          hi[2 * j] = s0.hi;
          lo[2 * j] = s0.lo;
          hi[2 * j + 1] = s1.hi;
          lo[2 * j + 1] = s1.lo;
        }
      }

      if (!ptx::mbar_wait(empty_bar(st), ph ^ 1u)) {
        record_error(err_flag, kErrEmptyWait);
        ok = false;
        break;
      }
      ptx::tc_fence_after();
      [[maybe_unused]] const uint32_t ob = op0 + st * kOpBytesT;
      if constexpr (kBF16) {
        // A -> TMEM: kPieces bf16x2 words per pair, piece p at columns +16p.
        const uint32_t a_col = tmem + lane_base + kAStageCol + 64u * st + kAK1 * wg;
#pragma unroll
        for (int p = 0; p < kPieces; ++p) ptx::tmem_st_n<kAK1>(a_col + 16u * p, w[p]);
        // B -> shared memory: 4 complex k of column n, re/im interleaved.
#pragma unroll
        for (int j = 0; j < (kPanel ? 0 : kB16PT); ++j) {
          float4 v0 = bv[2 * j], v1 = bv[2 * j + 1];
          if (conjB) {
            v0.y = -v0.y;
            v0.w = -v0.w;
            v1.y = -v1.y;
            v1.w = -v1.w;
          }
          uint32_t qw[4][3];
          split_bf16<kPieces>(v0.x, v0.y, qw[0][0], qw[0][1], qw[0][2]);
          split_bf16<kPieces>(v0.z, v0.w, qw[1][0], qw[1][1], qw[1][2]);
          split_bf16<kPieces>(v1.x, v1.y, qw[2][0], qw[2][1], qw[2][2]);
          split_bf16<kPieces>(v1.z, v1.w, qw[3][0], qw[3][1], qw[3][2]);
#pragma unroll
          for (int p = 0; p < kPieces; ++p)
            sts128(ob + (p >> 1) * kBHalfT + b16row[j] + ((b16chunk[j] ^ (4u * (p & 1))) << 4),
                   qw[0][p], qw[1][p], qw[2][p], qw[3][p]);
        }
      } else {
        // A -> TMEM: hi and lo of each value.
        const uint32_t a_col = tmem + lane_base + kAStageCol + 64u * st + 2 * kAK1 * wg;
        ptx::tmem_st_n<2 * kAK1>(a_col, hi);
        ptx::tmem_st_n<2 * kAK1>(a_col + 32u, lo);
        // B -> shared memory (swizzled K-major hi and lo tiles).
#pragma unroll
        for (int j = 0; j < (kPanel ? 0 : kBPT); ++j) {
          float4 v = bv[j];
          if (conjB) {
            v.y = -v.y;
            v.w = -v.w;
          }
          const Split r0 = split_tf32(v.x), i0 = split_tf32(v.y);
          const Split r1 = split_tf32(v.z), i1 = split_tf32(v.w);
          if (BMode == kTmaKN) {
            sts64(ob + boff[j][0], r0.hi, i0.hi);
            sts64(ob + boff[j][1], r1.hi, i1.hi);
            sts64(ob + kBHalfT + boff[j][0], r0.lo, i0.lo);
            sts64(ob + kBHalfT + boff[j][1], r1.lo, i1.lo);
          } else {
            sts128(ob + boff[j][0], r0.hi, i0.hi, r1.hi, i1.hi);
            sts128(ob + kBHalfT + boff[j][0], r0.lo, i0.lo, r1.lo, i1.lo);
          }
        }
      }
      ptx::tmem_wait_st();
      ptx::fence_proxy_async_smem();
      ptx::tc_fence_before();
      __syncwarp();
      if (lane == 0) {
        arrive_mma(full_bar(st));
        ptx::mbar_arrive(raw_empty(r));
      }

      // Fold chunk c at stage 4 (c + 1) + 1: the operand wait above already
      // covered the MMAs of stage 4 c + 3 (the chunk's last), so the chunk
      // wait does not stall the next conversion.  The chunk's buffer is next
      // written by chunk c + 2, from stage 4 (c + 2).
      if ((s % kFoldT) == 1 && s > kFoldT) {
        const int64_t c = s / kFoldT - 1;
        const int buf = static_cast<int>(c & 1);
        if (!ptx::mbar_wait(chunk_full(buf), static_cast<uint32_t>((c >> 1) & 1))) {
          record_error(err_flag, kErrChunkWait);
          ok = false;
          break;
        }
        ptx::tc_fence_after();
        fold_from(buf ? kChunkCol1 : kChunkCol0);
        ptx::tc_fence_before();
        __syncwarp();
        if (lane == 0) arrive_mma(chunk_empty(buf));
      }
      if (++r == kRaw) {
        r = 0;
        rph ^= 1u;
      }
      if (++st == kStages) {
        st = 0;
        ph ^= 1u;
      }
    }

    // ---------------------------------------------------------- epilogue ---
    if (!ptx::mbar_wait(acc_bar, 0)) {
      record_error(err_flag, kErrAccWait);
      ok = false;
    }
    ptx::tc_fence_after();
    if (ok) {
      // Chunks the loop did not fold: the last, and the one before it when
      // the last has a single stage; then add the corrections.
      const int64_t c_last = (ksteps - 1) / kFoldT;
      if (c_last >= 1 && ksteps < kFoldT * c_last + 2)
        fold_from(((c_last - 1) & 1) ? kChunkCol1 : kChunkCol0);
      fold_from((c_last & 1) ? kChunkCol1 : kChunkCol0);
      fold_from(kCorrCol);
      if constexpr (kReal) {
        float* __restrict__ Cp =
            static_cast<float*>(args.C) + static_cast<int64_t>(blockIdx.y) * args.c_split_stride;
        store_tile_real<kMC1>(args, Cp, m0 + rho, row_ok, n0, wg * kMC1, master);
      } else {
        float2* __restrict__ Cp =
            static_cast<float2*>(args.C) + static_cast<int64_t>(blockIdx.y) * args.c_split_stride;
        store_tile<kMC1>(args, Cp, m0 + ci, row_ok, n0, wg * kMC1, part, master);
      }
    }
  }

  // A pair frees its TMEM together, once the MMAs (waited for by the even
  // CTA's MMA thread) and every cross-CTA arrival are done.
  ptx::tc_fence_before();
  if constexpr (kPair) ptx::cluster_sync(); else __syncthreads();
  if (warp == 0) {
    ptx::tc_fence_after();
    if constexpr (kPair) ptx::tmem_dealloc2(tmem, kTmemCols);
    else ptx::tmem_dealloc(tmem, kTmemCols);
  }
}

// ------------------------------------------------------ operand pieces ---
// CTA pairs over operands split into bf16 pieces beforehand.
//
// A pre-pass (split_pieces) writes, for every complex row m of A, the two 1M
// rows [re, -im, ...] and [im, re, ...] and, for every column n of B, the row
// [re, im, ...] of its complex k (K fastest, real k = 2k + part), each value
// split into P bf16 pieces exactly as tc1m_contract's converters split them
// (split_bf16, conjugation first): P arrays per operand, rows `pitch`
// elements apart.  The pair kernel then runs without converters: TMA loads
// all pieces of a stage (3-D boxes: 64 real k x rows x P) into 128-byte
// swizzled K-major shared memory, and one thread of the even CTA issues
// tcgen05.mma.cta_group::2 with both operands read from shared memory.
// Per accumulator its MMAs run in tc1m_contract's order (main product into
// the chunk accumulators, a chunk every 16 MMAs of K = 16; corrections x0y1,
// x1y0 [, x1y1, x0y2, x2y0] per K = 16 step into their own accumulator), so
// the two forms give the same result bit for bit.
//
// The split happens once per operand element instead of once per tile that
// reads it; the price is the pieces in device memory: 2 x 2 x 2P bytes per
// complex element of A (the 1M rows) and 2 x 2P per element of B, written
// and read back once by TMA per tile.
constexpr int kPcStepK = 64;                   // real k per stage: one 128-byte row per piece
constexpr int kPcABytes = 128 * 128;           // one A piece of a stage: 128 real rows
constexpr int kPcBBytes = (kTileN / 2) * 128;  // one B piece: this CTA's 64 columns
constexpr int kPcFold = 4;                     // stages per main chunk (16 MMAs of K = 16)
constexpr int kPcBarrierBytes = 256;
template <int P>
constexpr int pc_stage_bytes() {
  return P * (kPcABytes + kPcBBytes);
}
// Stages in the ring: as many as 227 KB hold (72 KB each for three pieces).
template <int P>
constexpr int pc_stages() {
  return P == 3 ? 3 : 4;
}
template <int P>
constexpr int pc_smem_bytes() {
  return 1024 + pc_stages<P>() * pc_stage_bytes<P>() + kPcBarrierBytes;
}

// Pieces of one operand for a block of 32 rows x 32 complex k (256 threads):
// the block reads its tile along whichever direction has unit stride
// (through the offset vectors otherwise) and writes 16 bytes per piece and
// output row per thread (4 complex k).  Blocks [0, blocks_a) cover A,
// the rest B.  Rows past M or N are not written (the tensor maps end
// there); complex k in [K, K rounded up to 4) are written as zeros.
template <int P>
__global__ void __launch_bounds__(256)
split_pieces(const GemmArgs g, uint16_t* __restrict__ pa, uint16_t* __restrict__ pb,
             int64_t pitch, int64_t plane_a, int64_t plane_b, int64_t blocks_a, int64_t tiles_k) {
  __shared__ float2 tile[32][33];
  const bool is_a = blockIdx.x < blocks_a;
  const int64_t bid = is_a ? blockIdx.x : blockIdx.x - blocks_a;
  const int64_t r0 = (bid / tiles_k) * 32, k0 = (bid % tiles_k) * 32;
  const int64_t R = is_a ? g.M : g.N, K = g.K;
  const float2* __restrict__ src = static_cast<const float2*>(is_a ? g.A : g.B);
  const int64_t* rs = is_a ? g.rsA : g.csB;
  const int64_t* ks = is_a ? g.csA : g.rsB;
  const int64_t ur = is_a ? g.uA_m : g.uB_n;
  const int64_t uk = is_a ? g.uA_k : g.uB_k;
  const bool row_fast = ur == 1 && uk != 1;
  const int t = threadIdx.x;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = row_fast ? (t & 31) : (t >> 5) + 8 * i;
    const int k = row_fast ? (t >> 5) + 8 * i : (t & 31);
    float2 v = make_float2(0.f, 0.f);
    if (r0 + r < R && k0 + k < K) v = src[offs(rs, ur, r0 + r) + offs(ks, uk, k0 + k)];
    tile[r][k] = v;
  }
  __syncthreads();
  const int r = t >> 3, kq = 4 * (t & 7);
  if (r0 + r >= R || k0 + kq >= K) return;
  const bool conj = g.flags & (is_a ? kFlagConjA : kFlagConjB);
  float2 v[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    v[j] = tile[r][kq + j];
    if (conj) v[j].y = -v[j].y;
  }
  const int64_t col = 2 * (k0 + kq);
  uint32_t w[3][4];
  if (is_a) {
#pragma unroll
    for (int part = 0; part < 2; ++part) {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float x0 = part ? v[j].y : v[j].x;
        const float x1 = part ? v[j].x : -v[j].y;
        split_bf16<P>(x0, x1, w[0][j], w[1][j], w[2][j]);
      }
      uint16_t* row = pa + (2 * (r0 + r) + part) * pitch + col;
#pragma unroll
      for (int p = 0; p < P; ++p)
        *reinterpret_cast<uint4*>(row + p * plane_a) = make_uint4(w[p][0], w[p][1], w[p][2], w[p][3]);
    }
  } else {
#pragma unroll
    for (int j = 0; j < 4; ++j) split_bf16<P>(v[j].x, v[j].y, w[0][j], w[1][j], w[2][j]);
    uint16_t* row = pb + (r0 + r) * pitch + col;
#pragma unroll
    for (int p = 0; p < P; ++p)
      *reinterpret_cast<uint4*>(row + p * plane_b) = make_uint4(w[p][0], w[p][1], w[p][2], w[p][3]);
  }
}

// The pair kernel over pieces.  Warps: 0 TMEM allocation and (even CTA, one
// lane) MMA issue; 1 TMA (one lane per CTA); 2 (odd CTA, one lane) relays
// the arrival of its stage to the even CTA's MMA thread; 4-11 fold the chunk
// accumulators and write C (two warpgroups of 64 columns each, one TMEM lane
// per thread), as tc1m_contract's converters do.
template <int Prec>
__global__ void __launch_bounds__(kThreads1, 1)
tc1m_pieces(const GemmArgs args, const __grid_constant__ TmaMaps maps, int* err_flag) {
  constexpr int P = Prec == kPrecBF16x6 ? 3 : 2;
  constexpr int S = pc_stages<P>();
  constexpr int kStageB = pc_stage_bytes<P>();
  constexpr uint32_t kIdescP = ptx::idesc_f32acc(1u /*BF16*/, 256u, kTileN);
  static_assert(8 * (3 * S + 6) <= kPcBarrierBytes, "barrier area");
  static_assert(kStageB % 1024 == 0 && kPcBBytes % 1024 == 0, "swizzle atoms");

  extern __shared__ __align__(16) uint8_t smem_raw[];
  const uint32_t base = (ptx::smem_u32(smem_raw) + 1023u) & ~1023u;
  uint8_t* const base_ptr = smem_raw + (base - ptx::smem_u32(smem_raw));
  const uint32_t bars = base + S * kStageB;
  auto full_bar = [&](int s) { return bars + 8u * s; };
  auto peer_bar = [&](int s) { return bars + 8u * (S + s); };
  auto empty_bar = [&](int s) { return bars + 8u * (2 * S + s); };
  auto chunk_full = [&](int b) { return bars + 8u * (3 * S + b); };
  auto chunk_empty = [&](int b) { return bars + 8u * (3 * S + 2 + b); };
  const uint32_t acc_bar = bars + 8u * (3 * S + 4);
  const uint32_t tmem_slot = acc_bar + 8u;
  volatile uint32_t* tmem_slot_ptr =
      reinterpret_cast<volatile uint32_t*>(base_ptr + (tmem_slot - base));

  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const uint32_t rank = ptx::cluster_ctarank();
  if (warp == 0) {
    ptx::tmem_alloc2(tmem_slot, kTmemCols);
    ptx::tmem_relinquish2();
  }
  if (tid == 32) {
    for (int s = 0; s < S; ++s) {
      ptx::mbar_init(full_bar(s), 1);
      ptx::mbar_init(peer_bar(s), 1);
      ptx::mbar_init(empty_bar(s), 1);
    }
    for (int b = 0; b < 2; ++b) {
      ptx::mbar_init(chunk_full(b), 1);
      ptx::mbar_init(chunk_empty(b), 2 * (kConverters1 / 32));
    }
    ptx::mbar_init(acc_bar, 1);
    ptx::fence_mbar_init();
  }
  if (tid == 64) {
    ptx::tma_prefetch_desc(&maps.a);
    ptx::tma_prefetch_desc(&maps.b);
  }
  ptx::tc_fence_before();
  ptx::cluster_sync();
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_slot_ptr;

  // Tiles as in tc1m_contract's pair form: groups of 8 pair tiles along M
  // sweep N; split-K rows over blockIdx.y.
  const int64_t M = args.M, N = args.N;
  const int64_t kb = static_cast<int64_t>(blockIdx.y) * args.k_per_split;
  const int64_t K = min(args.K, kb + args.k_per_split);
  constexpr int kRowsTile = 2 * kTileMc;
  const int64_t tiles_m = (M + kRowsTile - 1) / kRowsTile;
  const int64_t tiles_n = (N + kTileN - 1) / kTileN;
  constexpr int64_t G = 8;
  const int64_t t = blockIdx.x >> 1;
  const int64_t group = t / (G * tiles_n);
  const int64_t first_m = group * G;
  const int64_t gsize = min(G, tiles_m - first_m);
  const int64_t tm = first_m + (t % (G * tiles_n)) % gsize;
  const int64_t tn = (t % (G * tiles_n)) / gsize;
  const int64_t m0 = tm * kRowsTile + rank * kTileMc, n0 = tn * kTileN;
  // Stages of 64 real k over this CTA row's real K range [2 kb, 2 K).
  const int64_t ksteps = (2 * (K - kb) + kPcStepK - 1) / kPcStepK;

  if (warp == 0) {
    // ---------------------------------------------------------- MMA issue ---
    if (lane == 0 && rank == 0) {
      const uint64_t desc0 = ptx::smem_desc_sw128(base);
      const uint32_t d_corr = tmem + kCorrCol;
      for (int64_t s = 0; s < ksteps; ++s) {
        const int st = static_cast<int>(s % S);
        const uint32_t ph = static_cast<uint32_t>((s / S) & 1);
        const int64_t c = s / kPcFold;
        const int buf = static_cast<int>(c & 1);
        const bool chunk_start = (s % kPcFold) == 0;
        if (chunk_start && c >= 2 &&
            !ptx::mbar_wait(chunk_empty(buf), static_cast<uint32_t>(((c - 2) >> 1) & 1))) {
          record_error(err_flag, kErrChunkWait);
          break;
        }
        if (!ptx::mbar_wait(full_bar(st), ph) || !ptx::mbar_wait(peer_bar(st), ph)) {
          record_error(err_flag, kErrFullWait);
          break;
        }
        ptx::tc_fence_after();
        const uint32_t d_main = tmem + (buf ? kChunkCol1 : kChunkCol0);
        const uint64_t ds = desc0 + static_cast<uint64_t>((st * kStageB) >> 4);
        // K = 16 steps of this stage inside the CTA row's K range: a split
        // may end half way through a stage (its K a multiple of 16 complex);
        // the rest of the box belongs to the next split.  Past the end of K
        // the box is zero-filled.
        const int64_t rem = 2 * (K - kb) - kPcStepK * s;
        const int nkk = rem >= kPcStepK ? 4 : static_cast<int>((rem + 15) / 16);
        // Piece p, K = 16 step kk: A at +p x 16 KB, B after the A pieces at
        // +p x 8 KB, each +32 bytes per step inside the 128-byte rows.
        auto da = [&](int p, int kk) {
          return ds + static_cast<uint64_t>((p * kPcABytes + 32 * kk) >> 4);
        };
        auto db = [&](int p, int kk) {
          return ds + static_cast<uint64_t>((P * kPcABytes + p * kPcBBytes + 32 * kk) >> 4);
        };
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
          if (kk < nkk)
            ptx::mma_f16_ss2(d_main, da(0, kk), db(0, kk), kIdescP,
                             (chunk_start && kk == 0) ? 0u : 1u);
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          if (kk >= nkk) break;
          ptx::mma_f16_ss2(d_corr, da(0, kk), db(1, kk), kIdescP, (s == 0 && kk == 0) ? 0u : 1u);
          ptx::mma_f16_ss2(d_corr, da(1, kk), db(0, kk), kIdescP, 1u);
          if (P == 3) {
            ptx::mma_f16_ss2(d_corr, da(1, kk), db(1, kk), kIdescP, 1u);
            ptx::mma_f16_ss2(d_corr, da(0, kk), db(2, kk), kIdescP, 1u);
            ptx::mma_f16_ss2(d_corr, da(2, kk), db(0, kk), kIdescP, 1u);
          }
        }
        ptx::mma_commit2(empty_bar(st));
        if ((s % kPcFold) == kPcFold - 1 || s == ksteps - 1) ptx::mma_commit2(chunk_full(buf));
      }
      // Signal the epilogue (also after an abort), then make sure no MMA is
      // still writing TMEM before it is freed.
      ptx::mma_commit2(acc_bar);
      if (!ptx::mbar_wait(acc_bar, 0)) record_error(err_flag, kErrAccWait);
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---------------------------------------------------------------- TMA ---
    if (lane == 0) {
      const int a_row = static_cast<int>(2 * m0);                   // 1M rows of this CTA
      const int b_row = static_cast<int>(n0 + rank * (kTileN / 2));  // its B columns
      for (int64_t s = 0; s < ksteps; ++s) {
        const int st = static_cast<int>(s % S);
        const uint32_t ph = static_cast<uint32_t>((s / S) & 1);
        if (!ptx::mbar_wait(empty_bar(st), ph ^ 1u)) {
          record_error(err_flag, kErrRawWait);
          break;
        }
        const uint32_t dst = base + st * kStageB;
        const int k0 = static_cast<int>(2 * kb + kPcStepK * s);
        ptx::mbar_arrive_expect_tx(full_bar(st), static_cast<uint32_t>(kStageB));
        ptx::tma_load_3d(dst, &maps.a, k0, a_row, 0, full_bar(st));
        ptx::tma_load_3d(dst + P * kPcABytes, &maps.b, k0, b_row, 0, full_bar(st));
      }
    }
    __syncwarp();
  } else if (warp == 2) {
    // -------------------------------------------------------------- relay ---
    if (lane == 0 && rank == 1) {
      for (int64_t s = 0; s < ksteps; ++s) {
        const int st = static_cast<int>(s % S);
        if (!ptx::mbar_wait(full_bar(st), static_cast<uint32_t>((s / S) & 1))) {
          record_error(err_flag, kErrFullWait);
          break;
        }
        ptx::mbar_arrive_cluster(ptx::mapa(peer_bar(st), 0));
      }
    }
    __syncwarp();
  } else if (tid >= kConvBase) {
    // ------------------------------------------------- fold and epilogue ---
    const int pt = tid - kConvBase;
    const int wg = pt >> 7;
    const int q = (pt >> 5) & 3;
    const int rho = 32 * q + lane;
    const int ci = rho >> 1;
    const int part = rho & 1;
    const uint32_t lane_base = static_cast<uint32_t>(32 * q) << 16;
    const bool row_ok = (m0 + ci) < M;
    float master[kMC1];
#pragma unroll
    for (int j = 0; j < kMC1; ++j) master[j] = 0.f;
    auto fold_from = [&](uint32_t col) {
#pragma unroll
      for (int cc = 0; cc < kMC1 / 32; ++cc) {
        uint32_t r[32];
        ptx::tmem_ld32_sync(tmem + lane_base + col + kMC1 * wg + 32u * cc, r);
#pragma unroll
        for (int j = 0; j < 32; ++j) master[32 * cc + j] += __uint_as_float(r[j]);
      }
    };
    bool ok = true;
    const int64_t nchunks = (ksteps + kPcFold - 1) / kPcFold;
    for (int64_t c = 0; c + 1 < nchunks; ++c) {
      const int buf = static_cast<int>(c & 1);
      if (!ptx::mbar_wait(chunk_full(buf), static_cast<uint32_t>((c >> 1) & 1))) {
        record_error(err_flag, kErrChunkWait);
        ok = false;
        break;
      }
      ptx::tc_fence_after();
      fold_from(buf ? kChunkCol1 : kChunkCol0);
      ptx::tc_fence_before();
      __syncwarp();
      if (lane == 0) ptx::mbar_arrive_cluster(ptx::mapa(chunk_empty(buf), 0));
    }
    if (!ptx::mbar_wait(acc_bar, 0)) {
      record_error(err_flag, kErrAccWait);
      ok = false;
    }
    ptx::tc_fence_after();
    if (ok) {
      fold_from(((nchunks - 1) & 1) ? kChunkCol1 : kChunkCol0);
      fold_from(kCorrCol);
      float2* __restrict__ Cp =
          static_cast<float2*>(args.C) + static_cast<int64_t>(blockIdx.y) * args.c_split_stride;
      store_tile<kMC1>(args, Cp, m0 + ci, row_ok, n0, wg * kMC1, part, master);
    }
  }

  ptx::tc_fence_before();
  ptx::cluster_sync();
  if (warp == 0) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc2(tmem, kTmemCols);
  }
}

// ------------------------------------------------------------------ host ---
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// 2-D map over complex64 data viewed as floats: dim0 = 2*inner floats (unit
// stride), dim1 = outer with `outer_stride` complex elements.
bool make_map(CUtensorMap* map, const void* base, int64_t inner, int64_t outer,
              int64_t outer_stride, uint32_t box_inner_floats, uint32_t box_outer, bool swizzle) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  if (reinterpret_cast<uintptr_t>(base) % 16 != 0) return false;
  if (outer > 1 && ((outer_stride * 8) % 16 != 0 || outer_stride <= 0)) return false;
  if (2 * inner >= (int64_t(1) << 31) || outer >= (int64_t(1) << 31) || inner <= 0 || outer <= 0)
    return false;
  cuuint64_t dims[2] = {static_cast<cuuint64_t>(2 * inner), static_cast<cuuint64_t>(outer)};
  cuuint64_t strides[1] = {static_cast<cuuint64_t>(outer > 1 ? outer_stride * 8 : 16)};
  cuuint32_t box[2] = {box_inner_floats, box_outer};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides,
                  box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  swizzle ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// Every 16-aligned block of the scatter vector is a unit-stride run starting
// at an even offset (16-byte aligned complex64): the block-scatter condition
// for one TMA box per block.
bool unit_blocks16(const std::vector<int64_t>& v, int64_t n) {
  for (int64_t b = 0; b < n; b += 16) {
    if (v[b] & 1) return false;
    const int64_t e = std::min<int64_t>(n, b + 16);
    for (int64_t i = b + 1; i < e; ++i)
      if (v[i] != v[b] + (i - b)) return false;
  }
  return true;
}

template <int AMode, int BMode, int Prec, bool kReal, bool kPair = false>
cudaError_t launch_modes(const GemmArgs& args, const TmaMaps& maps, cudaStream_t stream,
                         int* err_flag, dim3 tiles) {
  constexpr int kSmem = smem_bytes_1<kReal, BMode == kPanelNK, kPair>();
  static_assert(kSmem <= 227 * 1024, "shared memory budget");
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(tc1m_contract<AMode, BMode, Prec, kReal, kPair>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  if constexpr (kPair) {
    // Clusters of two CTAs along x (tiles.x counts CTAs: two per pair tile).
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = tiles;
    cfg.blockDim = dim3(kThreads1);
    cfg.dynamicSmemBytes = kSmem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, tc1m_contract<AMode, BMode, Prec, kReal, true>, args, maps,
                              err_flag);
  } else {
    tc1m_contract<AMode, BMode, Prec, kReal, false><<<tiles, kThreads1, kSmem, stream>>>(
        args, maps, err_flag);
    return cudaGetLastError();
  }
}

// CTA pairs: complex operands both loaded by TMA ([k][m] or [m][k] A,
// [n][k] or [k][n] B); tiles.x = 2 x pair tiles.
template <int Prec>
cudaError_t launch_pair(int amode, int bmode, const GemmArgs& args, const TmaMaps& maps,
                        cudaStream_t stream, int* err_flag, dim3 tiles) {
  if (amode == kTmaMK) {
    if (bmode == kTmaNK)
      return launch_modes<kTmaMK, kTmaNK, Prec, false, true>(args, maps, stream, err_flag, tiles);
    return launch_modes<kTmaMK, kTmaKN, Prec, false, true>(args, maps, stream, err_flag, tiles);
  }
  if (bmode == kTmaNK)
    return launch_modes<kTmaKM, kTmaNK, Prec, false, true>(args, maps, stream, err_flag, tiles);
  return launch_modes<kTmaKM, kTmaKN, Prec, false, true>(args, maps, stream, err_flag, tiles);
}

cudaError_t launch_pair_prec(int method, int amode, int bmode, const GemmArgs& args,
                             const TmaMaps& maps, cudaStream_t stream, int* err_flag, dim3 tiles) {
  switch (method) {
    case T1M_METHOD_TC_BF16X3:
      return launch_pair<kPrecBF16x3>(amode, bmode, args, maps, stream, err_flag, tiles);
    case T1M_METHOD_TC_BF16X6:
      return launch_pair<kPrecBF16x6>(amode, bmode, args, maps, stream, err_flag, tiles);
    default:
      return launch_pair<kPrecTF32x3>(amode, bmode, args, maps, stream, err_flag, tiles);
  }
}

// Operand pieces: row pitch in bf16 elements (real K rounded up to 16 bytes).
int64_t pieces_pitch(int64_t K) { return (2 * K + 7) / 8 * 8; }

// 3-D map over P piece arrays (`plane` elements apart) of `rows` rows of
// `kreal` bf16 (`pitch` apart), loaded as boxes of 64 k x box_rows x P with
// the 128-byte swizzle.
bool make_map_pieces(CUtensorMap* map, const void* base, int64_t kreal, int64_t rows,
                     int64_t pitch, int64_t plane, int pieces, uint32_t box_rows) {
  EncodeTiledFn fn = encode_fn();
  if (!fn || reinterpret_cast<uintptr_t>(base) % 16 != 0) return false;
  if (kreal <= 0 || rows <= 0 || kreal >= (int64_t(1) << 31) || rows >= (int64_t(1) << 31))
    return false;
  cuuint64_t dims[3] = {static_cast<cuuint64_t>(kreal), static_cast<cuuint64_t>(rows),
                        static_cast<cuuint64_t>(pieces)};
  cuuint64_t strides[2] = {static_cast<cuuint64_t>(pitch * 2),
                           static_cast<cuuint64_t>(plane * 2)};
  cuuint32_t box[3] = {static_cast<cuuint32_t>(kPcStepK), box_rows, static_cast<cuuint32_t>(pieces)};
  cuuint32_t estr[3] = {1, 1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 3, const_cast<void*>(base), dims, strides, box,
            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The pieces of A and B not in `ready` (one launch, counted in *kernels;
// into ws, A's first), then the pair kernel over them: tiles.x = 2 x pair
// tiles, tiles.y = splits.
template <int Prec>
cudaError_t launch_pieces_prec(const GemmArgs& g, void* ws, const PiecesReady* ready, dim3 tiles,
                               cudaStream_t stream, int* err_flag, int* kernels,
                               cudaEvent_t* main_ev) {
  constexpr int P = Prec == kPrecBF16x6 ? 3 : 2;
  const int64_t pitch = pieces_pitch(g.K);
  const bool ra = ready && ready->a, rb = ready && ready->b;
  const int64_t plane_a = ra ? ready->a_plane : 2 * g.M * pitch;
  const int64_t plane_b = rb ? ready->b_plane : g.N * pitch;
  uint16_t* const w = static_cast<uint16_t*>(ws);
  uint16_t* pa = ra ? static_cast<uint16_t*>(const_cast<void*>(ready->a)) : w;
  uint16_t* pb = rb ? static_cast<uint16_t*>(const_cast<void*>(ready->b)) : w + (ra ? 0 : P * plane_a);
  TmaMaps maps;
  if (!make_map_pieces(&maps.a, pa, 2 * g.K, 2 * g.M, pitch, plane_a, P, 128) ||
      !make_map_pieces(&maps.b, pb, 2 * g.K, g.N, pitch, plane_b, P, kTileN / 2))
    return cudaErrorInvalidConfiguration;
  const int64_t tiles_k = (g.K + 31) / 32;
  const int64_t blocks_a = ra ? 0 : (g.M + 31) / 32 * tiles_k;
  const int64_t blocks_b = rb ? 0 : (g.N + 31) / 32 * tiles_k;
  if (blocks_a + blocks_b >= (int64_t(1) << 31)) return cudaErrorInvalidConfiguration;
  cudaError_t e;
  if (blocks_a + blocks_b > 0) {
    split_pieces<P><<<static_cast<unsigned>(blocks_a + blocks_b), 256, 0, stream>>>(
        g, pa, pb, pitch, plane_a, plane_b, blocks_a, tiles_k);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    ++*kernels;
  }
  constexpr int kSmem = pc_smem_bytes<P>();
  static_assert(kSmem <= 227 * 1024, "shared memory budget");
  static bool attr_set = false;
  if (!attr_set) {
    e = cudaFuncSetAttribute(tc1m_pieces<Prec>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = tiles;
  cfg.blockDim = dim3(kThreads1);
  cfg.dynamicSmemBytes = kSmem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (main_ev) cudaEventRecord(main_ev[0], stream);
  e = cudaLaunchKernelEx(&cfg, tc1m_pieces<Prec>, g, maps, err_flag);
  if (main_ev) cudaEventRecord(main_ev[1], stream);
  return e;
}

template <int AMode, int Prec, bool kReal>
cudaError_t launch_b(int bmode, const GemmArgs& args, const TmaMaps& maps, cudaStream_t stream,
                     int* err_flag, dim3 tiles) {
  switch (bmode) {
    case kTmaNK: return launch_modes<AMode, kTmaNK, Prec, kReal>(args, maps, stream, err_flag, tiles);
    case kTmaKN: return launch_modes<AMode, kTmaKN, Prec, kReal>(args, maps, stream, err_flag, tiles);
    case kPanelNK: return launch_modes<AMode, kPanelNK, Prec, kReal>(args, maps, stream, err_flag, tiles);
    default: return launch_modes<AMode, kGatherNK, Prec, kReal>(args, maps, stream, err_flag, tiles);
  }
}

template <int Prec, bool kReal>
cudaError_t launch_a(int amode, int bmode, const GemmArgs& args, const TmaMaps& maps,
                     cudaStream_t stream, int* err_flag, dim3 tiles) {
  switch (amode) {
    case kTmaMK: return launch_b<kTmaMK, Prec, kReal>(bmode, args, maps, stream, err_flag, tiles);
    case kTmaKM: return launch_b<kTmaKM, Prec, kReal>(bmode, args, maps, stream, err_flag, tiles);
    default: return launch_b<kGatherMK, Prec, kReal>(bmode, args, maps, stream, err_flag, tiles);
  }
}

template <bool kReal>
cudaError_t launch_prec(int method, int amode, int bmode, const GemmArgs& args,
                        const TmaMaps& maps, cudaStream_t stream, int* err_flag, dim3 tiles) {
  switch (method) {
    case T1M_METHOD_TC_BF16X3:
      return launch_a<kPrecBF16x3, kReal>(amode, bmode, args, maps, stream, err_flag, tiles);
    case T1M_METHOD_TC_BF16X6:
      return launch_a<kPrecBF16x6, kReal>(amode, bmode, args, maps, stream, err_flag, tiles);
    default:
      return launch_a<kPrecTF32x3, kReal>(amode, bmode, args, maps, stream, err_flag, tiles);
  }
}

// B panels pay off when enough M tiles share them (each M tile otherwise
// splits B itself; a panel costs a read of B and a write and read of the
// panel array, two or three times B's bytes).
constexpr int64_t kPanelMinTilesM = 4;

int64_t panel_stages(bool real, int64_t K) { return (K + (real ? 32 : 16) - 1) / (real ? 32 : 16); }

// Map over the panel array: rows n, each nstages x bufs x 128 bytes,
// loaded as 64 x 128 boxes of 16-bit units with the 128-byte swizzle.
bool make_map_panel(CUtensorMap* map, const void* base, int64_t nstages, int bufs, int64_t N) {
  EncodeTiledFn fn = encode_fn();
  if (!fn || reinterpret_cast<uintptr_t>(base) % 16 != 0) return false;
  const int64_t units = nstages * bufs * 64;
  if (units >= (int64_t(1) << 31) || N >= (int64_t(1) << 31) || N <= 0) return false;
  cuuint64_t dims[2] = {static_cast<cuuint64_t>(units), static_cast<cuuint64_t>(N)};
  cuuint64_t strides[1] = {static_cast<cuuint64_t>(units * 2)};
  cuuint32_t box[2] = {64, static_cast<cuuint32_t>(kTileN)};
  cuuint32_t estr[2] = {1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, const_cast<void*>(base), dims, strides, box,
            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <bool kReal>
cudaError_t launch_panels(int method, const GemmArgs& g, void* out, int64_t nstages,
                          cudaStream_t stream) {
  const int64_t threads = g.N * nstages;
  const unsigned blocks = static_cast<unsigned>((threads + 255) / 256);
  uint4* o = static_cast<uint4*>(out);
  const int kf = g.uB_k == 1 ? 1 : 0;
  switch (method) {
    case T1M_METHOD_TC_BF16X3:
      split_b_panels<kPrecBF16x3, kReal><<<blocks, 256, 0, stream>>>(g, o, nstages, kf);
      break;
    case T1M_METHOD_TC_BF16X6:
      split_b_panels<kPrecBF16x6, kReal><<<blocks, 256, 0, stream>>>(g, o, nstages, kf);
      break;
    default:
      split_b_panels<kPrecTF32x3, kReal><<<blocks, 256, 0, stream>>>(g, o, nstages, kf);
  }
  return cudaGetLastError();
}

// 2-D map over float32 data: dim0 = inner floats (unit stride), dim1 =
// outer with `outer_stride` floats.
bool make_map_f32(CUtensorMap* map, const void* base, int64_t inner, int64_t outer,
                  int64_t outer_stride, uint32_t box_inner, uint32_t box_outer, bool swizzle);

// Real float32 problems on the one-tile kernel: uniform-view TMA modes or
// gathers (no per-block maps), epilogue flags for 4-column stores.
bool tc_prepare_real(const GemmArgs& g, const HostPlan& plan, int splits, int* amode,
                     int* bmode, TmaMaps* maps, GemmArgs* out);

// Rows of every 16-aligned block of `rows` step by one common stride *stride
// (the same for all blocks, a 16-byte multiple), and every block start plus
// every 16-block start of `runs` is even (16-byte aligned complex64): the
// block-scatter condition of the KM16 / NK16 modes.
// The row coordinate of these boxes is always 0..15 and TMA bounds-checks
// coordinates, not addresses, so every block must be a full block of valid
// rows: n must be a multiple of 16.
bool common_block_stride16(const std::vector<int64_t>& rows, const std::vector<int64_t>& runs,
                           int64_t n, int64_t* stride) {
  if (n < 16 || n % 16 != 0) return false;
  int64_t s = -1;
  for (int64_t b = 0; b < n; b += 16) {
    if (rows[b] & 1) return false;
    const int64_t e = std::min<int64_t>(n, b + 16);
    for (int64_t i = b + 1; i < e; ++i) {
      const int64_t d = rows[i] - rows[i - 1];
      if (s < 0) s = d;
      if (d != s) return false;
    }
  }
  if (s <= 0 || (s * 8) % 16 != 0) return false;
  for (size_t k = 0; k + 1 < runs.size(); k += 16)
    if (runs[k] & 1) return false;
  *stride = s;
  return true;
}

// Epilogue store flags of a problem (kFlagCPairs, kFlagCCol16) from C's row
// and column offsets: the uniform strides where the arguments carry them (a
// uniform bundle, the dense split-K workspace), else the plan's vectors.
uint32_t c_store_flags(const GemmArgs& g, const HostPlan& plan) {
  auto col = [&](int64_t n) { return g.uC_n >= 0 ? n * g.uC_n : plan.csC[n]; };
  auto row = [&](int64_t m) { return g.uC_m >= 0 ? m * g.uC_m : plan.rsC[m]; };
  uint32_t f = 0;
  bool col16 = true;
  if (g.uC_n >= 0) {
    col16 = g.uC_n == 1 || g.N <= 1;
  } else {
    for (int64_t b = 0; b < g.N && col16; b += 16)
      for (int64_t i = b + 1; i < std::min<int64_t>(g.N, b + 16); ++i)
        if (col(i) != col(b) + (i - b)) {
          col16 = false;
          break;
        }
  }
  if (col16) f |= kFlagCCol16;
  bool pairs = reinterpret_cast<uintptr_t>(g.C) % 16 == 0;
  if (pairs) {
    if (g.uC_m >= 0) {
      pairs = g.uC_m % 2 == 0 || g.M <= 1;
    } else {
      for (int64_t m = 0; m < g.M && pairs; ++m) pairs = row(m) % 2 == 0;
    }
  }
  if (pairs) {
    if (g.uC_n >= 0) {
      pairs = g.uC_n == 1;
    } else {
      for (int64_t n = 0; n + 1 < g.N && pairs; n += 2)
        pairs = col(n) % 2 == 0 && col(n + 1) == col(n) + 1;
    }
  }
  if (pairs) f |= kFlagCPairs;
  return f;
}

bool make_map_f32(CUtensorMap* map, const void* base, int64_t inner, int64_t outer,
                  int64_t outer_stride, uint32_t box_inner, uint32_t box_outer, bool swizzle) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  if (reinterpret_cast<uintptr_t>(base) % 16 != 0) return false;
  if (outer > 1 && ((outer_stride * 4) % 16 != 0 || outer_stride <= 0)) return false;
  if (inner >= (int64_t(1) << 31) || outer >= (int64_t(1) << 31) || inner <= 0 || outer <= 0)
    return false;
  cuuint64_t dims[2] = {static_cast<cuuint64_t>(inner), static_cast<cuuint64_t>(outer)};
  cuuint64_t strides[1] = {static_cast<cuuint64_t>(outer > 1 ? outer_stride * 4 : 16)};
  cuuint32_t box[2] = {box_inner, box_outer};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides,
                  box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  swizzle ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// Real epilogue flags: kFlagCCol16 as for complex; kFlagCPairs for four
// consecutive columns contiguous with 16-byte aligned starts.
uint32_t c_store_flags_real(const GemmArgs& g, const HostPlan& plan) {
  auto col = [&](int64_t n) { return g.uC_n >= 0 ? n * g.uC_n : plan.csC[n]; };
  auto row = [&](int64_t m) { return g.uC_m >= 0 ? m * g.uC_m : plan.rsC[m]; };
  uint32_t f = 0;
  bool col16 = true;
  if (g.uC_n >= 0) {
    col16 = g.uC_n == 1 || g.N <= 1;
  } else {
    for (int64_t b = 0; b < g.N && col16; b += 16)
      for (int64_t i = b + 1; i < std::min<int64_t>(g.N, b + 16); ++i)
        if (col(i) != col(b) + (i - b)) {
          col16 = false;
          break;
        }
  }
  if (col16) f |= kFlagCCol16;
  bool quads = reinterpret_cast<uintptr_t>(g.C) % 16 == 0;
  if (quads) {
    if (g.uC_m >= 0) {
      quads = g.uC_m % 4 == 0 || g.M <= 1;
    } else {
      for (int64_t m = 0; m < g.M && quads; ++m) quads = row(m) % 4 == 0;
    }
  }
  if (quads) {
    if (g.uC_n >= 0) {
      quads = g.uC_n == 1;
    } else {
      for (int64_t n = 0; n + 3 < g.N && quads; n += 4)
        quads = col(n) % 4 == 0 && col(n + 1) == col(n) + 1 && col(n + 2) == col(n) + 2 &&
                col(n + 3) == col(n) + 3;
    }
  }
  if (quads) f |= kFlagCPairs;
  return f;
}

bool tc_prepare_real(const GemmArgs& g, const HostPlan& plan, int splits, int* amode,
                     int* bmode, TmaMaps* maps, GemmArgs* out) {
  constexpr int kStepKR = 32;
  if (splits < 1 || (splits > 1 && g.k_per_split % kStepKR != 0)) return false;
  if (g.M >= (int64_t(1) << 31) / 128 || g.N >= (int64_t(1) << 31) / kTileN) return false;
  *out = g;
  out->flags = (g.flags & ~(kFlagCPairs | kFlagCCol16 | kFlagConjA | kFlagConjB)) |
               c_store_flags_real(g, plan);
  std::memset(static_cast<void*>(maps), 0, sizeof(*maps));
  *amode = kGatherMK;
  if (plan.uA_m == 1 && plan.uA_k >= 0 &&
      make_map_f32(&maps->a, g.A, g.M, g.K, plan.uA_k, 128, kStepKR, false))
    *amode = kTmaMK;
  else if (plan.uA_k == 1 && plan.uA_m >= 0 &&
           make_map_f32(&maps->a, g.A, g.K, g.M, plan.uA_m, kStepKR, 128, true))
    *amode = kTmaKM;
  *bmode = kGatherNK;
  if (plan.uB_k == 1 && plan.uB_n >= 0 &&
      make_map_f32(&maps->b, g.B, g.K, g.N, plan.uB_n, kStepKR, kTileN, true))
    *bmode = kTmaNK;
  else if (plan.uB_n == 1 && plan.uB_k >= 0 &&
           make_map_f32(&maps->b, g.B, g.N, g.K, plan.uB_k, kTileN, kStepKR, false))
    *bmode = kTmaKN;
  return true;
}

std::mutex g_attr_mutex;
bool g_attr_set = false;

}  // namespace

void tc_tile(int dtype, int* bm, int* bn, int* bk) {
  const bool real = dtype == T1M_FLOAT32;
  *bm = real ? 128 : kTileMc;
  *bn = kTileN;
  *bk = real ? 32 : kStepK;
}

bool tc_supported(int method, int dtype, const HostPlan& plan) {
  (void)plan;
  return (method == T1M_METHOD_TC_3XTF32 || method == T1M_METHOD_TC_BF16X3 ||
          method == T1M_METHOD_TC_BF16X6 || method == kMethodTcAuto) &&
         (dtype == T1M_COMPLEX64 || dtype == T1M_FLOAT32);
}

// The layout checks over the scatter vectors depend only on the plan and the
// length checked (slabs of a pipelined product check shorter prefixes), so
// they are memoised in the plan.
enum : int {
  kChkUnitRsA = 1, kChkUnitCsA, kChkUnitRsB, kChkUnitCsB,
  kChkStrideRsA, kChkStrideCsA, kChkStrideCsB, kChkStrideRsB
};
constexpr int64_t kNoStride = INT64_MIN;

bool unit16(const HostPlan& plan, int which, const std::vector<int64_t>& v, int64_t n) {
  const auto key = std::make_pair(which, n);
  const auto it = plan.memo.find(key);
  if (it != plan.memo.end()) return it->second != 0;
  const bool r = unit_blocks16(v, n);
  plan.memo[key] = r ? 1 : 0;
  return r;
}

bool stride16(const HostPlan& plan, int which, const std::vector<int64_t>& rows,
              const std::vector<int64_t>& runs, int64_t n, int64_t* stride) {
  const auto key = std::make_pair(which, n);
  const auto it = plan.memo.find(key);
  if (it != plan.memo.end()) {
    if (it->second == kNoStride) return false;
    *stride = it->second;
    return true;
  }
  const bool r = common_block_stride16(rows, runs, n, stride);
  plan.memo[key] = r ? *stride : kNoStride;
  return r;
}

int tc_default_tile_n(int64_t N) {
  // Time per stage of 16 complex k and tile of the persistent kernel,
  // measured over the sweep batch's first steps with every width forced
  // (16, 32, 64, 128 columns: 5.4, 2.9, 1.6 and 1 times the 128-column
  // time for 8, 4, 2 and 1 tiles): the A side (loads, 1M split, TMEM
  // stores) dominates and does not shrink with the width.  Modelled as
  // 1000 + 3.5 x width clocks.
  int best = kTileN;
  double best_cost = 1e300;
  for (int w : kTcTileWidths) {
    const double cost = double((N + w - 1) / w) * (1000.0 + 3.5 * w);
    if (cost < best_cost) {
      best_cost = cost;
      best = w;
    }
  }
  return best;
}

bool tc_prepare(const GemmArgs& g, const HostPlan& plan, int splits, TcProblem* p, int tile_n) {
  std::memset(static_cast<void*>(p), 0, sizeof(*p));
  if (tile_n == 0) tile_n = tc_default_tile_n(g.N);
  if (tile_n != 16 && tile_n != 32 && tile_n != 64 && tile_n != 128) return false;
  p->g = g;
  p->g.flags = (g.flags & ~(kFlagCPairs | kFlagCCol16)) | c_store_flags(g, plan);
  p->tile_n = tile_n;
  p->fold_shift = 2;  // kFold = 4 stages per main chunk
  p->skinny = 0;
  p->fix_begin = -1;
  p->tiles_m = static_cast<int32_t>((g.M + kTileMc - 1) / kTileMc);
  p->tiles_n = static_cast<int32_t>((g.N + tile_n - 1) / tile_n);
  p->splits = splits;
  if (splits < 1 || (splits > 1 && g.k_per_split % kStepK != 0)) return false;
  if (g.M >= (int64_t(1) << 31) / kTileMc || g.N >= (int64_t(1) << 31) / kTileN) return false;
  // A: TMA over a uniform 2-D view, TMA per unit-stride 16-row block, or gather.
  p->amode = kAGather;
  if (plan.uA_m == 1 && plan.uA_k >= 0 &&
      make_map(&p->map_a, g.A, g.M, g.K, plan.uA_k, 2 * kTileMc, kStepK, false))
    p->amode = kAMK;
  else if (plan.uA_k == 1 && plan.uA_m >= 0 &&
           make_map(&p->map_a, g.A, g.K, g.M, plan.uA_m, 2 * kStepK, kTileMc, true))
    p->amode = kAKM;
  else if (plan.uA_k >= 0 && unit16(plan, kChkUnitRsA, plan.rsA, g.M) &&
           make_map(&p->map_a, g.A, plan.spanA, g.K, plan.uA_k, 32, kStepK, false)) {
    p->amode = kAMK16;
    p->block_maps |= 1;
  } else if (plan.uA_m >= 0 && g.K % kStepK == 0 && unit16(plan, kChkUnitCsA, plan.csA, g.K) &&
             make_map(&p->map_a, g.A, plan.spanA, g.M, plan.uA_m, 2 * kStepK, kTileMc, true)) {
    p->amode = kAKM;
    p->block_maps |= 1;
  } else if (int64_t sm = 0; g.K % kStepK == 0 && unit16(plan, kChkUnitCsA, plan.csA, g.K) &&
                             stride16(plan, kChkStrideRsA, plan.rsA, plan.csA, g.M, &sm) &&
                             make_map(&p->map_a, g.A, plan.spanA, 16, sm, 2 * kStepK, 16, true)) {
    p->amode = kAKM16;
    p->block_maps |= 1;
  } else if (int64_t sk = 0; g.M % 16 == 0 && unit16(plan, kChkUnitRsA, plan.rsA, g.M) &&
                             stride16(plan, kChkStrideCsA, plan.csA, plan.rsA, g.K, &sk) &&
                             make_map(&p->map_a, g.A, plan.spanA, 16, sk, 32, 16, false)) {
    p->amode = kAMK16K;
    p->block_maps |= 1;
  }
  // B: TMA over a uniform 2-D view or per unit-stride 16-element K block, or gather.
  p->bmode = kBGather;
  // B boxes are tile_n rows (columns of the output tile) high.
  const uint32_t tn = static_cast<uint32_t>(tile_n);
  if (plan.uB_k == 1 && plan.uB_n >= 0 &&
      make_map(&p->map_b, g.B, g.K, g.N, plan.uB_n, 2 * kStepK, tn, true))
    p->bmode = kBNK;
  else if (plan.uB_n == 1 && plan.uB_k >= 0 &&
           make_map(&p->map_b, g.B, g.N, g.K, plan.uB_k, 2 * tn, kStepK, false))
    p->bmode = kBKN;
  else if (plan.uB_n >= 0 && g.K % kStepK == 0 && unit16(plan, kChkUnitRsB, plan.rsB, g.K) &&
           make_map(&p->map_b, g.B, plan.spanB, g.N, plan.uB_n, 2 * kStepK, tn, true)) {
    p->bmode = kBNK;
    p->block_maps |= 2;
  } else if (int64_t sn = 0; g.K % kStepK == 0 && unit16(plan, kChkUnitRsB, plan.rsB, g.K) &&
                             stride16(plan, kChkStrideCsB, plan.csB, plan.rsB, g.N, &sn) &&
                             make_map(&p->map_b, g.B, plan.spanB, 16, sn, 2 * kStepK, 16, true)) {
    p->bmode = kBNK16;
    p->block_maps |= 2;
  } else if (int64_t sk = 0; g.N % 16 == 0 && unit16(plan, kChkUnitCsB, plan.csB, g.N) &&
                             stride16(plan, kChkStrideRsB, plan.rsB, plan.csB, g.K, &sk) &&
                             make_map(&p->map_b, g.B, plan.spanB, 16, sk, 32, 16, false)) {
    p->bmode = kBKN16;
    p->block_maps |= 2;
  }
  return true;
}

int64_t tc_problem_tiles(const TcProblem& p) {
  return int64_t(p.tiles_m) * p.tiles_n * p.splits;
}

cudaError_t tc_launch_persistent(const TcProblem* single, const TcProblem* dev_group, int nprob,
                                 int64_t total_tiles, int num_sms, int* done,
                                 cudaStream_t stream, int* err_flag, int* fix) {
  {
    std::lock_guard<std::mutex> lock(g_attr_mutex);
    if (!g_attr_set) {
      cudaError_t e = cudaFuncSetAttribute(tc3xtf32_persistent,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
      if (e != cudaSuccess) return e;
      g_attr_set = true;
    }
  }
  if (total_tiles <= 0) return cudaSuccess;
  const int64_t grid = std::min<int64_t>(total_tiles, std::max(1, num_sms));
  TcProblem dummy;
  if (!single) {
    std::memset(static_cast<void*>(&dummy), 0, sizeof(dummy));
    single = &dummy;
  }
  if (done) {
    // Tiles wait on tiles of other CTAs: all CTAs must be resident.
    void* params[] = {const_cast<TcProblem*>(single), &dev_group, &nprob, &total_tiles, &done,
                      &err_flag, &fix};
    return cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(tc3xtf32_persistent),
                                       dim3(static_cast<unsigned>(grid)), dim3(kThreads), params,
                                       kSmemBytes, stream);
  }
  tc3xtf32_persistent<<<static_cast<unsigned>(grid), kThreads, kSmemBytes, stream>>>(
      *single, dev_group, nprob, total_tiles, done, err_flag, fix);
  return cudaGetLastError();
}

// Operands gathered element by element are packed first (pack.cu) when they
// hold at least this many bytes; below it the extra pass is not repaid.
constexpr size_t kPackMinBytes = size_t(4) << 20;

// k-step, in the plan's K order, of an operand's unit-stride K mode (> 1); 0
// when its unit-stride mode is a row mode; -1 when it has none, or when that
// mode is the first K mode (its k runs are contiguous already).
int64_t pack_step(const std::vector<Mode>& kmodes, bool second, const std::vector<Mode>& rmodes) {
  int64_t step = 1;
  for (const Mode& m : kmodes) {
    if ((second ? m.s1 : m.s0) == 1 && m.extent > 1) return step > 1 ? step : -1;
    step *= m.extent;
  }
  for (const Mode& m : rmodes)
    if (m.s0 == 1 && m.extent > 1) return 0;
  return -1;
}

// An operand without a uniform view that has a unit-stride direction may be
// gathered element by element.
bool gather_prone(int64_t u_row, int64_t u_k) {
  return !(u_row == 1 && u_k >= 0) && !(u_k == 1 && u_row >= 0);
}

size_t tc_pack_bytes(int dtype, const HostPlan& plan) {
  if (dtype != T1M_COMPLEX64 && dtype != T1M_FLOAT32) return 0;
  const size_t es = dtype == T1M_FLOAT32 ? 4 : 8;
  const size_t pitch = static_cast<size_t>(pack_pitch(dtype, plan.K));
  size_t b = 0;
  if (gather_prone(plan.uA_m, plan.uA_k) &&
      static_cast<size_t>(plan.M) * static_cast<size_t>(plan.K) * es >= kPackMinBytes)
    b += static_cast<size_t>(plan.M) * pitch * es;
  if (gather_prone(plan.uB_n, plan.uB_k) &&
      static_cast<size_t>(plan.N) * static_cast<size_t>(plan.K) * es >= kPackMinBytes)
    b += static_cast<size_t>(plan.N) * pitch * es;
  return b;
}

size_t tc_pieces_bytes(int dtype, int method, int64_t M, int64_t N, int64_t K,
                       const PiecesReady* ready) {
  if (dtype != T1M_COMPLEX64 || M <= kTileMc || N <= 0 || K <= 0) return 0;
  if (method != T1M_METHOD_TC_BF16X3 && method != T1M_METHOD_TC_BF16X6 && method != kMethodTcAuto)
    return 0;
  const size_t pieces = method == T1M_METHOD_TC_BF16X3 ? 2 : 3;
  const int64_t rows = (ready && ready->a ? 0 : 2 * M) + (ready && ready->b ? 0 : N);
  return pieces * static_cast<size_t>(rows) * static_cast<size_t>(pieces_pitch(K)) * 2u;
}

int64_t tc_pieces_pitch(int64_t K) { return pieces_pitch(K); }

cudaError_t tc_split_operand(int pieces, bool operand_a, const GemmArgs& g, void* out,
                             int64_t plane, cudaStream_t s) {
  const int64_t pitch = pieces_pitch(g.K);
  const int64_t tiles_k = (g.K + 31) / 32;
  const int64_t blocks = ((operand_a ? g.M : g.N) + 31) / 32 * tiles_k;
  if (blocks <= 0) return cudaSuccess;
  if (blocks >= (int64_t(1) << 31)) return cudaErrorInvalidConfiguration;
  uint16_t* o = static_cast<uint16_t*>(out);
  const unsigned grid = static_cast<unsigned>(blocks);
  // B alone: no A blocks (blocks_a = 0), B's arrays at o.
  const int64_t ba = operand_a ? blocks : 0;
  if (pieces == 2)
    split_pieces<2><<<grid, 256, 0, s>>>(g, o, o, pitch, plane, plane, ba, tiles_k);
  else
    split_pieces<3><<<grid, 256, 0, s>>>(g, o, o, pitch, plane, plane, ba, tiles_k);
  return cudaGetLastError();
}

size_t tc_panel_bytes(int dtype, int64_t M, int64_t N, int64_t K) {
  const bool real = dtype == T1M_FLOAT32;
  if ((dtype != T1M_COMPLEX64 && !real) || M <= 0 || N <= 0 || K <= 0) return 0;
  const int64_t rows = real ? 128 : kTileMc;
  if ((M + rows - 1) / rows < kPanelMinTilesM) return 0;
  return static_cast<size_t>(N) * static_cast<size_t>(panel_stages(real, K)) * 256u;
}

// Method of the pieces form for a product, 0 where it does not run: the
// bf16 methods (the automatic method as BF16x6) with two or more 64-row M
// tiles; any operand layout for T1M_TILE_PIECES (the split pass reads through
// the scatter vectors), for T1M_TILE_AUTO where both operands load by TMA
// (where CTA pairs would otherwise run).
static int pieces_method(int method, int form, const TcProblem& p) {
  if (p.tiles_m < 2) return 0;
  const int pm = method == kMethodTcAuto ? T1M_METHOD_TC_BF16X6 : method;
  if (pm != T1M_METHOD_TC_BF16X3 && pm != T1M_METHOD_TC_BF16X6) return 0;
  if (form == T1M_TILE_PIECES) return pm;
  if (form != T1M_TILE_AUTO) return 0;
  const bool a_block = (p.block_maps & 1) || p.amode == kAMK16;
  const bool b_block = (p.block_maps & 2) != 0;
  const bool tma_a = !a_block && (p.amode == kAMK || p.amode == kAKM);
  const bool tma_b = !b_block && (p.bmode == kBNK || p.bmode == kBKN);
  return tma_a && tma_b ? pm : 0;
}

int tc_pieces_count(int method, int dtype, const GemmArgs& g, const HostPlan& plan, int form) {
  if (dtype != T1M_COMPLEX64 || !tc_supported(method, dtype, plan)) return 0;
  TcProblem p;
  if (!tc_prepare(g, plan, 1, &p)) return 0;
  const int pm = pieces_method(method, form, p);
  return pm == T1M_METHOD_TC_BF16X3 ? 2 : pm == T1M_METHOD_TC_BF16X6 ? 3 : 0;
}

cudaError_t launch_tc(int method, int dtype, const GemmArgs& args, const HostPlan& plan,
                      int splits, cudaStream_t stream, int* err_flag, int* kernels,
                      std::string* err, int* used_method, void* panel, size_t panel_bytes,
                      void* pack, size_t pack_bytes, int* path, int form,
                      const PiecesReady* ready, cudaEvent_t* main_ev, TcFix* fix) {
  *kernels = 0;
  auto mark = [&](int i) {
    if (main_ev) cudaEventRecord(main_ev[i], stream);
  };
  if (used_method) *used_method = method;
  if (path) *path = 0;
  // The report's path code: fetch modes in TcProblem's numbering, B panels
  // as T1M_PATH_B_PANELS, kernel form and packed operands as flag bits.
  auto set_path = [&](int am, int bm, bool persistent, bool pa, bool pb) {
    if (path)
      *path = T1M_PATH_TC | am | (bm << 4) | (persistent ? T1M_PATH_PERSISTENT : 0) |
              (pa ? T1M_PATH_A_PACKED : 0) | (pb ? T1M_PATH_B_PACKED : 0);
  };
  auto one_tile_a = [](int am) { return am == kTmaMK ? kAMK : am == kTmaKM ? kAKM : kAGather; };
  auto one_tile_b = [](int bm) {
    return bm == kTmaNK ? kBNK : bm == kTmaKN ? kBKN : bm == kPanelNK ? T1M_PATH_B_PANELS : kBGather;
  };
  if (!tc_supported(method, dtype, plan)) {
    *err = "tensor-core method not available for this dtype";
    return cudaErrorNotSupported;
  }
  if (args.M == 0 || args.N == 0) return cudaSuccess;
  const bool real = dtype == T1M_FLOAT32;
  // B panels: enough M tiles share B and the workspace holds them.  They are
  // used where they measured faster on GB300: for 3xTF32 (199 vs 192
  // TFLOP/s at complex64 4096^3; its converters split B into twice the
  // bytes of bf16 pieces) and for B that would otherwise be gathered.  The
  // bf16 methods with a TMA-loadable B keep the in-kernel split (204 vs 197
  // TFLOP/s with panels: the panel pass is not repaid there).
  const size_t need = tc_panel_bytes(dtype, args.M, args.N, args.K);
  const bool panels_ok = panel && need > 0 && panel_bytes >= need;
  auto want_panels = [&](bool b_gathered) {
    return panels_ok && (b_gathered || method == T1M_METHOD_TC_3XTF32);
  };
  const int64_t nstages = panel_stages(real, args.K);
  // Split B into the panels and point the kernel's B map at them.
  auto use_panels = [&](const GemmArgs& g, TmaMaps* maps, int* bm) -> cudaError_t {
    const int bufs = method == T1M_METHOD_TC_BF16X3 ? 1 : 2;
    if (!make_map_panel(&maps->b, panel, nstages, bufs, args.N)) return cudaSuccess;
    const cudaError_t e = real ? launch_panels<true>(method, g, panel, nstages, stream)
                               : launch_panels<false>(method, g, panel, nstages, stream);
    if (e == cudaSuccess) {
      *bm = kPanelNK;
      ++*kernels;
    }
    return e;
  };
  // Dense repacks of operands the kernels would gather element by element:
  // *ga / *hp become the problem with the packed operands (uniform, unit K
  // stride, rows `pitch` apart), loaded by TMA.  A is packed when large; B
  // when large and the panels (which gather B in their own pass) are not
  // used.
  const size_t es = real ? 4 : 8;
  const int64_t pitch = pack_pitch(dtype, args.K);
  const bool a_big = static_cast<size_t>(args.M) * static_cast<size_t>(args.K) * es >= kPackMinBytes;
  const bool b_big = static_cast<size_t>(args.N) * static_cast<size_t>(args.K) * es >= kPackMinBytes;
  auto pack_operands = [&](bool pa, bool pb, GemmArgs* ga, const HostPlan** hp) -> cudaError_t {
    const size_t bytes = (static_cast<size_t>(pa ? args.M : 0) + (pb ? args.N : 0)) *
                         static_cast<size_t>(pitch) * es;
    if (!pack || bytes == 0 || pack_bytes < bytes) return cudaSuccess;
    // The plan of the packed problem: uniform, unit K stride, rows `pitch`
    // apart for each packed operand (built once per plan and kept in it).
    std::shared_ptr<HostPlan>& slot = plan.packed[(pa ? 1 : 0) | (pb ? 2 : 0)];
    if (!slot) {
      auto q = std::make_shared<HostPlan>(plan);
      q->memo.clear();
      for (auto& x : q->packed) x.reset();
      if (pa) {
        q->uA_m = pitch;
        q->uA_k = 1;
        for (int64_t i = 0; i < plan.M; ++i) q->rsA[i] = i * pitch;
        for (int64_t i = 0; i < plan.K; ++i) q->csA[i] = i;
        q->spanA = plan.M * pitch;
      }
      if (pb) {
        q->uB_n = pitch;
        q->uB_k = 1;
        for (int64_t i = 0; i < plan.N; ++i) q->csB[i] = i * pitch;
        for (int64_t i = 0; i < plan.K; ++i) q->rsB[i] = i;
        q->spanB = plan.N * pitch;
      }
      slot = std::move(q);
    }
    *hp = slot.get();
    char* dst = static_cast<char*>(pack);
    if (pa) {
      const cudaError_t e = launch_pack(dtype, args.A, args.rsA, args.uA_m, args.csA, args.uA_k,
                                        args.M, args.K, pack_step(plan.modes_k, false, plan.modes_m),
                                        dst, pitch, stream);
      if (e != cudaSuccess) return e;
      ga->A = dst;
      ga->rsA = ga->csA = nullptr;
      ga->uA_m = pitch;
      ga->uA_k = 1;
      dst += static_cast<size_t>(args.M) * static_cast<size_t>(pitch) * es;
      ++*kernels;
    }
    if (pb) {
      const cudaError_t e = launch_pack(dtype, args.B, args.csB, args.uB_n, args.rsB, args.uB_k,
                                        args.N, args.K, pack_step(plan.modes_k, true, plan.modes_n),
                                        dst, pitch, stream);
      if (e != cudaSuccess) return e;
      ga->B = dst;
      ga->rsB = ga->csB = nullptr;
      ga->uB_n = pitch;
      ga->uB_k = 1;
      ++*kernels;
    }
    return cudaSuccess;
  };
  GemmArgs packed_args = args;
  const HostPlan* packed_plan = &plan;
  if (real) {
    // Real float32: the one-tile kernel with uniform-view TMA, gathers or panels.
    int am = kGatherMK, bm = kGatherNK;
    TmaMaps maps;
    GemmArgs gr;
    if (!tc_prepare_real(args, plan, splits, &am, &bm, &maps, &gr))
      return cudaErrorInvalidConfiguration;
    const bool pa = am == kGatherMK && a_big;
    const bool pb = bm == kGatherNK && b_big && !panels_ok;
    if (pa || pb) {
      const int before = *kernels;
      if (const cudaError_t e = pack_operands(pa, pb, &packed_args, &packed_plan)) return e;
      if (*kernels != before &&
          !tc_prepare_real(packed_args, *packed_plan, splits, &am, &bm, &maps, &gr))
        return cudaErrorInvalidConfiguration;
    }
    if (method == kMethodTcAuto)
      method = (am != kGatherMK && (bm != kGatherNK || panels_ok)) ? T1M_METHOD_TC_BF16X6
                                                                    : T1M_METHOD_TC_3XTF32;
    if (used_method) *used_method = method;
    if (want_panels(bm == kGatherNK))
      if (const cudaError_t e = use_panels(gr, &maps, &bm)) return e;
    const dim3 grid(static_cast<unsigned>(((args.M + 127) / 128) * ((args.N + kTileN - 1) / kTileN)),
                    static_cast<unsigned>(splits));
    mark(0);
    const cudaError_t e = launch_prec<true>(method, am, bm, gr, maps, stream, err_flag, grid);
    mark(1);
    if (e == cudaSuccess) ++*kernels;
    set_path(one_tile_a(am), one_tile_b(bm), false, packed_args.A != args.A,
             packed_args.B != args.B);
    return e;
  }
  TcProblem p;
  if (!tc_prepare(args, plan, splits, &p)) return cudaErrorInvalidConfiguration;
  if (const int pm = pieces_method(method, form, p)) {
    // Operand pieces: split once (the operands not in `ready`) into the
    // panel workspace, then CTA pairs with both MMA operands in shared
    // memory.  Without the workspace the product takes the forms below.
    const size_t need = tc_pieces_bytes(dtype, pm, args.M, args.N, args.K, ready);
    if (need == 0 || (panel && panel_bytes >= need)) {
      if (used_method) *used_method = pm;
      const int64_t pair_m = (p.g.M + 2 * kTileMc - 1) / (2 * kTileMc);
      const dim3 pgrid(static_cast<unsigned>(2 * pair_m * p.tiles_n),
                       static_cast<unsigned>(splits));
      const cudaError_t e =
          pm == T1M_METHOD_TC_BF16X3
              ? launch_pieces_prec<kPrecBF16x3>(p.g, panel, ready, pgrid, stream, err_flag, kernels,
                                                main_ev)
              : launch_pieces_prec<kPrecBF16x6>(p.g, panel, ready, pgrid, stream, err_flag, kernels,
                                                main_ev);
      if (e == cudaSuccess) ++*kernels;
      set_path(p.amode, p.bmode, false, false, false);
      if (path && e == cudaSuccess) *path |= T1M_PATH_PAIR | T1M_PATH_PIECES;
      return e;
    }
  }
  {
    // A per-16-row block-TMA operand A is packed as well when that puts the
    // product on the one-tile kernel (B by TMA or by panels): the block form
    // of the persistent kernel measured 3440 clocks per stage against 1450
    // (abcd,ebfd->aecf at extents 32: 113 -> 79 us).  A block-mode B is left
    // to the persistent kernel: without panels (few M tiles) the packed form
    // measured slower (abcd,dbea->ec: 66 -> 75 us).
    const bool a_blk = (p.block_maps & 1) != 0 || p.amode == kAMK16;
    const bool b_blk = (p.block_maps & 2) != 0;
    const bool pa = a_big && (p.amode == kAGather || (a_blk && (panels_ok || !b_blk)));
    const bool pb = p.bmode == kBGather && b_big && !panels_ok;
    if (pa || pb) {
      const int before = *kernels;
      if (const cudaError_t e = pack_operands(pa, pb, &packed_args, &packed_plan)) return e;
      if (*kernels != before && !tc_prepare(packed_args, *packed_plan, splits, &p))
        return cudaErrorInvalidConfiguration;
    }
  }
  p.tile_begin = 0;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  p.dep = -1;
  const bool a_block = (p.block_maps & 1) || p.amode == kAMK16;
  const bool b_block = (p.block_maps & 2) != 0;
  if (method == kMethodTcAuto) {
    // BF16x6 measured faster than 3xTF32 (203 vs 193-198 TFLOP/s at complex64
    // 4096^3) and more accurate in the one-tile kernel with TMA operands;
    // block-TMA layouts stay on the persistent 3xTF32 kernel.
    const bool tma_a = !a_block && p.amode != kAGather;
    const bool tma_b = panels_ok || (!b_block && p.bmode != kBGather);
    method = (tma_a && tma_b) ? T1M_METHOD_TC_BF16X6 : T1M_METHOD_TC_3XTF32;
    if (used_method) *used_method = method;
  }
  const bool bf16 = method != T1M_METHOD_TC_3XTF32;
  const bool b_gathered = b_block || p.bmode == kBGather;
  const bool panels = want_panels(b_gathered);
  cudaError_t e;
  if (bf16 || (!a_block && (!b_block || panels))) {
    // Uniform, gathered or panel operands: the one-tile-per-CTA form.  The
    // bf16 forms exist only here: an operand that needs a per-block map is
    // gathered instead.
    TmaMaps maps;
    maps.a = p.map_a;
    maps.b = p.map_b;
    const dim3 grid(static_cast<unsigned>(int64_t(p.tiles_m) * p.tiles_n),
                    static_cast<unsigned>(splits));
    const int am = (!a_block && p.amode == kAMK) ? kTmaMK
                   : (!a_block && p.amode == kAKM) ? kTmaKM : kGatherMK;
    int bm = (!b_block && p.bmode == kBNK) ? kTmaNK
             : (!b_block && p.bmode == kBKN) ? kTmaKN : kGatherNK;
    // CTA pairs where both operands load by TMA and there are at least two
    // 64-row M tiles: B is then split in-kernel, half per CTA, instead of by
    // a panel pass.  Their B map takes 64-column boxes.
    bool pair = form != T1M_TILE_ONE && am != kGatherMK && bm != kGatherNK && p.tiles_m >= 2;
    TmaMaps pmaps;
    if (pair) {
      pmaps.a = p.map_a;
      pair = bm == kTmaNK ? make_map(&pmaps.b, p.g.B, p.g.K, p.g.N, packed_plan->uB_n, 2 * kStepK,
                                     kTileN / 2, true)
                          : make_map(&pmaps.b, p.g.B, p.g.N, p.g.K, packed_plan->uB_k, kTileN,
                                     kStepK, false);
    }
    if (pair) {
      const int64_t pair_m = (p.g.M + 2 * kTileMc - 1) / (2 * kTileMc);
      const dim3 pgrid(static_cast<unsigned>(2 * pair_m * p.tiles_n), static_cast<unsigned>(splits));
      mark(0);
      e = launch_pair_prec(method, am, bm, p.g, pmaps, stream, err_flag, pgrid);
      mark(1);
      set_path(one_tile_a(am), one_tile_b(bm), false, packed_args.A != args.A, false);
      if (path && e == cudaSuccess) *path |= T1M_PATH_PAIR;
    } else {
      if (panels)
        if ((e = use_panels(p.g, &maps, &bm)) != cudaSuccess) return e;
      mark(0);
      e = launch_prec<false>(method, am, bm, p.g, maps, stream, err_flag, grid);
      mark(1);
      set_path(one_tile_a(am), one_tile_b(bm), false, packed_args.A != args.A,
               packed_args.B != args.B);
    }
  } else {
    // The persistent kernel takes narrower output tiles where the output
    // has few columns (abcd,dbea->ec: N = 64 in one 64-column tile instead
    // of half a 128-column tile).
    // Outputs of at most kTcSkinnyMaxN columns keep the 128-column tile:
    // 16-column tensor-core tiles for such outputs (N = 2, 5, 8) raised an
    // unspecified launch failure in a grouped launch, cause not found, so
    // they are not run.
    if (const int w = p.g.N > kTcSkinnyMaxN ? tc_default_tile_n(p.g.N) : p.tile_n;
        w != p.tile_n) {
      TcProblem q;
      if (tc_prepare(packed_args, *packed_plan, splits, &q, w)) p = q;
    }
    p.tile_begin = 0;
    p.dep = -1;
    // A split product is reduced in the kernel (the last split of each
    // output tile sums all partials in FP64 and applies the epilogue)
    // instead of by a reduction launch.
    // Only where that reduction is short: the last split's 256 threads read
    // ceil(width / 4) x splits partials each, dependent on one CTA per output
    // tile; abcd,dbea->ec (2 output tiles of 64 columns, 75 splits: 1200
    // partials per thread) took 464 us that way against 70 us with the
    // reduction kernel spread over the GPU.
    const int64_t fix_loads = (std::min<int64_t>(p.tile_n, p.g.N) + 3) / 4 * splits;
    int* fix_ctr = nullptr;
    if (fix && fix->ctr && fix->out && splits > 1 && fix_loads <= kFixMaxLoads &&
        int64_t(p.tiles_m) * p.tiles_n <= fix->cap) {
      p.fix_begin = 0;
      p.out = *fix->out;
      fix_ctr = fix->ctr;
      fix->reduced = true;
    }
    mark(0);
    e = tc_launch_persistent(&p, nullptr, 1, tc_problem_tiles(p), sms, nullptr, stream, err_flag,
                             fix_ctr);
    mark(1);
    set_path(p.amode, p.bmode, true, packed_args.A != args.A, packed_args.B != args.B);
  }
  if (e == cudaSuccess) ++*kernels;
  return e;
}

}  // namespace gb300
}  // namespace t1m
