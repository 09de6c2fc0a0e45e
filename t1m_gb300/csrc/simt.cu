// Plain GPU form: SIMT FP32 / FP64 block-scatter contraction kernels.
//
// This replaces the reference's BLIS five-loop GEMM (include/t1m/t1m.h:432-557)
// for the plain method.  One CTA computes a BM x BN tile of the matricised C;
// A and B tiles are gathered straight from the tensors through the scatter
// vectors (no packed copy in HBM), staged in shared memory, and multiplied with
// FMA.  For complex types each complex multiply-add is the 1M real product
// pair (re*re - im*im, re*im + im*re, t1m.h:309-337) done in registers.
// The epilogue scatter-writes C with alpha/beta (reference semantics
// C += alpha*A*B under kFlagAccumulate, t1m.h:406-430).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "internal.h"

namespace t1m {
namespace gb300 {
namespace {

template <class T> struct Scalar;
template <> struct Scalar<float> {
  using real = float;
  static constexpr bool cplx = false;
};
template <> struct Scalar<double> {
  using real = double;
  static constexpr bool cplx = false;
};
template <> struct Scalar<float2> {
  using real = float;
  static constexpr bool cplx = true;
};
template <> struct Scalar<double2> {
  using real = double;
  static constexpr bool cplx = true;
};

template <class T> __device__ __forceinline__ T zero();
template <> __device__ __forceinline__ float zero<float>() { return 0.f; }
template <> __device__ __forceinline__ double zero<double>() { return 0.0; }
template <> __device__ __forceinline__ float2 zero<float2>() { return make_float2(0.f, 0.f); }
template <> __device__ __forceinline__ double2 zero<double2>() { return make_double2(0.0, 0.0); }

__device__ __forceinline__ float conj_if(float v, bool) { return v; }
__device__ __forceinline__ double conj_if(double v, bool) { return v; }
__device__ __forceinline__ float2 conj_if(float2 v, bool c) { if (c) v.y = -v.y; return v; }
__device__ __forceinline__ double2 conj_if(double2 v, bool c) { if (c) v.y = -v.y; return v; }

// acc += a * b
__device__ __forceinline__ void mac(float& acc, float a, float b) { acc = fmaf(a, b, acc); }
__device__ __forceinline__ void mac(double& acc, double a, double b) { acc = fma(a, b, acc); }
__device__ __forceinline__ void mac(float2& acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.y, b.x, acc.y);
  acc.y = fmaf(a.x, b.y, acc.y);
}
__device__ __forceinline__ void mac(double2& acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.y, b.x, acc.y);
  acc.y = fma(a.x, b.y, acc.y);
}

template <class T> __device__ __forceinline__ T scal(const double* s);
template <> __device__ __forceinline__ float scal<float>(const double* s) { return (float)s[0]; }
template <> __device__ __forceinline__ double scal<double>(const double* s) { return s[0]; }
template <> __device__ __forceinline__ float2 scal<float2>(const double* s) { return make_float2((float)s[0], (float)s[1]); }
template <> __device__ __forceinline__ double2 scal<double2>(const double* s) { return make_double2(s[0], s[1]); }

__device__ __forceinline__ float mul(float a, float b) { return a * b; }
__device__ __forceinline__ double mul(double a, double b) { return a * b; }
__device__ __forceinline__ float2 mul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 mul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float add(float a, float b) { return a + b; }
__device__ __forceinline__ double add(double a, double b) { return a + b; }
__device__ __forceinline__ float2 add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 add(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }

__device__ __forceinline__ int64_t offs(const int64_t* v, int64_t u, int64_t i) {
  return u >= 0 ? i * u : __ldg(v + i);
}

constexpr int kThreads = 256;

// Global -> shared copy of one element (4, 8 or 16 bytes) that does not pass
// through registers; src_bytes 0 writes zeros (operands past the tile edge).
template <int kBytes>
__device__ __forceinline__ void cp_async_elem(void* dst, const void* src, bool in) {
  const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst));
  const uint32_t n = in ? kBytes : 0u;
  if constexpr (kBytes == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(n)
                 : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(d), "l"(src),
                 "n"(kBytes), "r"(n)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit_group() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// 16 x 16 threads; thread (tx, ty) owns rows ty*TM .. ty*TM+TM-1 of the tile
// and columns tx + 16*j (j < TN), so shared-memory reads of B are
// consecutive across a half-warp and reads of A are broadcasts.
// Grouped launches: blockIdx.x indexes the concatenated tile lists of
// group[0..nprob) (sorted by tile_begin); otherwise it is a tile of args0.
template <class T, int TM, int TN, int BK, bool kGroup>
__global__ void __launch_bounds__(kThreads, 2)
simt_contract(const GemmArgs args0, const SimtProblem* group, int nprob) {
  constexpr int BM = 16 * TM;
  constexpr int BN = 16 * TN;
  int64_t tile = blockIdx.x;
  // The contraction of this CTA: a shared-memory copy of its descriptor for
  // grouped launches, the parameter space otherwise.
  __shared__ GemmArgs group_args;
  if constexpr (kGroup) {
    int lo = 0, hi = nprob - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (group[mid].tile_begin <= tile) lo = mid; else hi = mid - 1;
    }
    tile -= group[lo].tile_begin;
    if (threadIdx.x == 0) group_args = group[lo].g;
    __syncthreads();
  }
  const GemmArgs& args = kGroup ? group_args : args0;
  constexpr int A_PER = BM * BK / kThreads;
  constexpr int B_PER = BN * BK / kThreads;
  static_assert(A_PER * kThreads == BM * BK, "A tile not divisible");
  static_assert(B_PER * kThreads == BN * BK, "B tile not divisible");

  // Rows padded by 32 bytes: tile stores that walk k across threads (a
  // K-contiguous operand) then spread over the banks instead of hitting one.
  // kStages tiles in flight: global -> shared copies by cp.async (no register
  // staging, so the FMA loop never waits on a global load), zero-filled past
  // the edges.
  constexpr int kPad = 32 / sizeof(T);
  // Three stages where they fit the 48 KB of static shared memory and the
  // registers (the grouped float instance spills with three), else two.
  constexpr int kStageBytes = BK * (BM + BN + 2 * kPad) * static_cast<int>(sizeof(T));
  constexpr int kStages =
      (3 * kStageBytes <= 40 * 1024 && !(kGroup && sizeof(T) == 4)) ? 3 : 2;
  __shared__ __align__(16) T As[kStages][BK][BM + kPad];
  __shared__ __align__(16) T Bs[kStages][BK][BN + kPad];
  __shared__ int64_t rowA[BM];
  __shared__ int64_t colB[BN];

  const T* __restrict__ A = static_cast<const T*>(args.A);
  const T* __restrict__ B = static_cast<const T*>(args.B);
  const int64_t M = args.M, N = args.N;
  const int64_t tiles_m = (M + BM - 1) / BM;
  const int64_t tiles_n = (N + BN - 1) / BN;
  // Split-K: this CTA covers K range [kb, K); a split writes its partial
  // product to its own slice of the workspace.  The split is blockIdx.y for
  // single launches; grouped launches number a problem's tiles split-major.
  int64_t split = blockIdx.y;
  if constexpr (kGroup) {
    split = tile / (tiles_m * tiles_n);
    tile -= split * tiles_m * tiles_n;
  }
  const int64_t kb = split * args.k_per_split;
  const int64_t K = min(args.K, kb + args.k_per_split);
  T* __restrict__ C = static_cast<T*>(args.C) + split * args.c_split_stride;
  const bool conjA = args.flags & kFlagConjA;
  const bool conjB = args.flags & kFlagConjB;

  // Tile order: groups of 8 M-tiles sweep N so neighbouring CTAs share B.
  const int64_t t = tile;
  constexpr int64_t G = 8;
  const int64_t first_m = (t / (G * tiles_n)) * G;
  const int64_t gsize = min(G, tiles_m - first_m);
  const int64_t tm = first_m + (t % (G * tiles_n)) % gsize;
  const int64_t tn = (t % (G * tiles_n)) / gsize;
  const int64_t m0 = tm * BM, n0 = tn * BN;

  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;

  for (int i = tid; i < BM; i += kThreads)
    rowA[i] = (m0 + i < M) ? offs(args.rsA, args.uA_m, m0 + i) : 0;
  for (int i = tid; i < BN; i += kThreads)
    colB[i] = (n0 + i < N) ? offs(args.csB, args.uB_n, n0 + i) : 0;
  __syncthreads();

  // Thread -> element maps of the tile loads: the unit-stride direction of
  // each operand is the fast thread direction (coalesced gathers).
  const bool a_kfast = (args.uA_k == 1);
  const bool b_kfast = (args.uB_k == 1) || (args.uB_n != 1);

  auto issue_tiles = [&](int64_t k0, int buf) {
#pragma unroll
    for (int p = 0; p < A_PER; ++p) {
      const int idx = tid + p * kThreads;
      const int m = a_kfast ? idx / BK : idx % BM;
      const int k = a_kfast ? idx % BK : idx / BM;
      const bool in = m0 + m < M && k0 + k < K;
      const T* src = in ? A + rowA[m] + offs(args.csA, args.uA_k, k0 + k) : A;
      cp_async_elem<sizeof(T)>(&As[buf][k][m], src, in);
    }
#pragma unroll
    for (int p = 0; p < B_PER; ++p) {
      const int idx = tid + p * kThreads;
      const int n = b_kfast ? idx / BK : idx % BN;
      const int k = b_kfast ? idx % BK : idx / BN;
      const bool in = n0 + n < N && k0 + k < K;
      const T* src = in ? B + offs(args.rsB, args.uB_k, k0 + k) + colB[n] : B;
      cp_async_elem<sizeof(T)>(&Bs[buf][k][n], src, in);
    }
  };
  // Conjugation (complex types, rare: the adjoint) in shared memory, once
  // per element of a landed stage, so the FMA loop stays free of it.
  auto conj_stage = [&](int buf) {
    if constexpr (Scalar<T>::cplx) {
      if (conjA)
        for (int e = tid; e < BK * BM; e += kThreads) {
          T& v = As[buf][e / BM][e % BM];
          v.y = -v.y;
        }
      if (conjB)
        for (int e = tid; e < BK * BN; e += kThreads) {
          T& v = Bs[buf][e / BN][e % BN];
          v.y = -v.y;
        }
      if (conjA || conjB) __syncthreads();
    }
  };

  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = zero<T>();

  const int64_t ksteps = (K - kb + BK - 1) / BK;
  // Prologue: the first kStages - 1 stages in flight (one commit group each,
  // empty groups past the end keep the group count aligned).
#pragma unroll
  for (int st = 0; st < kStages - 1; ++st) {
    if (st < ksteps) issue_tiles(kb + st * BK, st);
    cp_async_commit_group();
  }
  for (int64_t s = 0; s < ksteps; ++s) {
    const int buf = static_cast<int>(s % kStages);
    cp_async_wait_group<kStages - 2>();  // stage s has landed (this thread's copies)
    __syncthreads();                     // ... and every thread's; stage s - 1 is consumed
    conj_stage(buf);
    // Refill the slot of stage s - 1 with stage s + kStages - 1.
    const int64_t nxt = s + kStages - 1;
    if (nxt < ksteps) issue_tiles(kb + nxt * BK, static_cast<int>(nxt % kStages));
    cp_async_commit_group();
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      T a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[buf][k][ty * TM + i];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = Bs[buf][k][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) mac(acc[i][j], a[i], b[j]);
    }
  }
  cp_async_wait_group<0>();

  // Epilogue: scatter-write C with alpha/beta.
  const T alpha = scal<T>(args.alpha);
  const T beta = scal<T>(args.beta);
  const bool accumulate = args.flags & kFlagAccumulate;
  const bool beta_zero = args.flags & kFlagBetaZero;
  int64_t colC[TN];
#pragma unroll
  for (int j = 0; j < TN; ++j) {
    const int64_t n = n0 + tx + 16 * j;
    colC[j] = n < N ? offs(args.csC, args.uC_n, n) : 0;
  }
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int64_t m = m0 + ty * TM + i;
    if (m >= M) continue;
    const int64_t r = offs(args.rsC, args.uC_m, m);
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int64_t n = n0 + tx + 16 * j;
      if (n >= N) continue;
      T* p = C + r + colC[j];
      const T ab = mul(alpha, acc[i][j]);
      if (accumulate)
        *p = add(*p, ab);
      else if (beta_zero)
        *p = ab;
      else
        *p = add(ab, mul(beta, *p));
    }
  }
}

template <class T, int TM, int TN, int BK>
cudaError_t launch(const GemmArgs& args, int splits, cudaStream_t stream) {
  constexpr int BM = 16 * TM, BN = 16 * TN;
  const int64_t tiles = ((args.M + BM - 1) / BM) * ((args.N + BN - 1) / BN);
  if (tiles == 0) return cudaSuccess;
  if (tiles > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  if (splits < 1 || splits > 65535) return cudaErrorInvalidConfiguration;
  const dim3 grid(static_cast<unsigned>(tiles), static_cast<unsigned>(splits));
  simt_contract<T, TM, TN, BK, false><<<grid, kThreads, 0, stream>>>(args, nullptr, 0);
  return cudaGetLastError();
}

template <class T, int TM, int TN, int BK>
cudaError_t launch_group(const SimtProblem* dev, int nprob, int64_t total_tiles,
                         cudaStream_t stream) {
  if (total_tiles <= 0) return cudaSuccess;
  if (total_tiles > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  GemmArgs none{};
  simt_contract<T, TM, TN, BK, true><<<static_cast<unsigned>(total_tiles), kThreads, 0, stream>>>(
      none, dev, nprob);
  return cudaGetLastError();
}

// ------------------------------------------------------------- skinny ---
// Outputs of at most NMAX columns (the second step of a sweep update,
// xsyb,ytb->xst with t <= 4, or any GEMV-like contraction): the work streams A
// once, so instead of a square tile a CTA takes a block of rows and one K
// chunk.  The chunk's B (all N columns, zero-padded to NMAX) is staged in
// shared memory, transposed so lanes read consecutive k; A rows are read along
// their unit-stride direction:
//   K unit stride: one warp per row (16 / NMAX rows per warp), lanes over k
//     (256-byte coalesced reads), lane partial sums reduced across the warp;
//   otherwise: one thread per row, k in order (coalesced across threads where
//     M is unit stride), the chunk's K offsets staged in shared memory.
// Tiles are numbered split-major per problem; a split writes its partial
// product to its workspace slice exactly like the other kernels.
__device__ __forceinline__ float shfl_xor(float v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ double shfl_xor(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ float2 shfl_xor(float2 v, int m) {
  return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}
__device__ __forceinline__ double2 shfl_xor(double2 v, int m) {
  return make_double2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}

template <class T>
__device__ __forceinline__ void skinny_store(const GemmArgs& g, T* C, int64_t m, int64_t n, T v) {
  T* p = C + offs(g.rsC, g.uC_m, m) + offs(g.csC, g.uC_n, n);
  const T ab = mul(scal<T>(g.alpha), v);
  if (g.flags & kFlagAccumulate)
    *p = add(*p, ab);
  else if (g.flags & kFlagBetaZero)
    *p = ab;
  else
    *p = add(ab, mul(scal<T>(g.beta), *p));
}

template <class T, int NMAX, bool KUNIT>
__device__ __forceinline__ void skinny_body(const GemmArgs& g, int64_t tile, T (*Bs)[2048 / NMAX],
                                            int64_t* ks) {
  constexpr int KB = 2048 / NMAX;            // k per shared-memory chunk
  constexpr int RW = KUNIT ? 16 / NMAX : 1;  // rows per warp (K unit) / per thread
  constexpr int BMr = skinny_rows(KUNIT, NMAX);
  const int64_t M = g.M, N = g.N, K = g.K;
  const int64_t tiles_m = (M + BMr - 1) / BMr;
  const int64_t split = tile / tiles_m;
  const int64_t m0 = (tile - split * tiles_m) * BMr;
  const int64_t kb = split * g.k_per_split;
  const int64_t ke = min(K, kb + g.k_per_split);
  T* __restrict__ C = static_cast<T*>(g.C) + split * g.c_split_stride;
  const T* __restrict__ A = static_cast<const T*>(g.A);
  const T* __restrict__ B = static_cast<const T*>(g.B);
  const bool conjA = g.flags & kFlagConjA;
  const bool conjB = g.flags & kFlagConjB;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  // Rows of this thread (K unit: this warp's rows; otherwise: one row).
  int64_t rowoff[RW];
  bool rowok[RW];
#pragma unroll
  for (int r = 0; r < RW; ++r) {
    const int64_t m = KUNIT ? m0 + warp * RW + r : m0 + tid;
    rowok[r] = m < M;
    rowoff[r] = rowok[r] ? offs(g.rsA, g.uA_m, m) : 0;
  }
  T acc[RW][NMAX];
#pragma unroll
  for (int r = 0; r < RW; ++r)
#pragma unroll
    for (int n = 0; n < NMAX; ++n) acc[r][n] = zero<T>();

  for (int64_t k0 = kb; k0 < ke; k0 += KB) {
    const int kn = static_cast<int>(min(static_cast<int64_t>(KB), ke - k0));
    __syncthreads();  // the previous chunk is consumed
    for (int e = tid; e < KB * NMAX; e += kThreads) {
      const int n = e / KB, kk = e % KB;
      T v = zero<T>();
      if (n < N && kk < kn)
        v = conj_if(B[offs(g.rsB, g.uB_k, k0 + kk) + offs(g.csB, g.uB_n, n)], conjB);
      Bs[n][kk] = v;
    }
    if (!KUNIT)
      for (int kk = tid; kk < kn; kk += kThreads) ks[kk] = offs(g.csA, g.uA_k, k0 + kk);
    __syncthreads();
    // kU k-steps of every row are loaded before any of them is used, so
    // each thread keeps kU x RW loads in flight (the kernel is bound by the
    // latency of streaming A).
    constexpr int kU = 4;
    if (KUNIT) {
      for (int kk0 = lane; kk0 < kn; kk0 += 32 * kU) {
        T a[kU][RW];
#pragma unroll
        for (int u = 0; u < kU; ++u)
#pragma unroll
          for (int r = 0; r < RW; ++r) {
            const int kk = kk0 + 32 * u;
            a[u][r] = (rowok[r] && kk < kn) ? conj_if(A[rowoff[r] + k0 + kk], conjA) : zero<T>();
          }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const int kk = kk0 + 32 * u;
          if (kk >= kn) break;
#pragma unroll
          for (int r = 0; r < RW; ++r)
#pragma unroll
            for (int n = 0; n < NMAX; ++n) mac(acc[r][n], a[u][r], Bs[n][kk]);
        }
      }
    } else if (rowok[0]) {
      for (int kk0 = 0; kk0 < kn; kk0 += kU) {
        T a[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u)
          a[u] = kk0 + u < kn ? conj_if(A[rowoff[0] + ks[kk0 + u]], conjA) : zero<T>();
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          if (kk0 + u >= kn) break;
#pragma unroll
          for (int n = 0; n < NMAX; ++n) mac(acc[0][n], a[u], Bs[n][kk0 + u]);
        }
      }
    }
  }

  if (KUNIT) {
#pragma unroll
    for (int r = 0; r < RW; ++r) {
#pragma unroll
      for (int n = 0; n < NMAX; ++n) {
        T v = acc[r][n];
#pragma unroll
        for (int d = 16; d >= 1; d >>= 1) v = add(v, shfl_xor(v, d));
        acc[r][n] = v;
      }
      const int64_t m = m0 + warp * RW + r;
      if (lane == 0 && rowok[r])
#pragma unroll
        for (int n = 0; n < NMAX; ++n)
          if (n < N) skinny_store(g, C, m, n, acc[r][n]);
    }
  } else if (rowok[0]) {
#pragma unroll
    for (int n = 0; n < NMAX; ++n)
      if (n < N) skinny_store(g, C, m0 + tid, n, acc[0][n]);
  }
}

// Asynchronous form (kFlagSkinnyAsync, N <= 4, 8-byte elements, unit K
// stride): the CTA's 32 rows stream through a ring of kSkStages shared-memory
// stages of 64 k with cp.async (16 bytes per copy, zero fill past the edges),
// so the loads in flight no longer depend on registers; B's whole K chunk
// (at most kSkinnyAsyncMaxK) is staged once, after the first A stages are
// issued.  Warp w reduces rows 4w..4w+3, lanes over k as in skinny_body.
// Five stages of 16 KB with two CTAs per SM keep up to 128 KB of A in flight
// per SM; the sweep's second steps (59.8 GB of A per batch) read at 2.8 TB/s,
// about as with three stages: the per-tile B staging and the short K chunks
// (at most kSkinnyAsyncMaxK per tile) bound them.
constexpr int kSkStages = 5;
constexpr int kSkKS = 64;  // k per stage
constexpr size_t kSkAsyncSmem =
    size_t(kSkStages) * 32 * kSkKS * 8 + size_t(4) * kSkinnyAsyncMaxK * 8;  // 112 KB
// Shared memory of the generic skinny body (B chunk and its K offsets).
template <class T, int NMAX>
constexpr size_t skinny_generic_smem() {
  return size_t(NMAX) * (2048 / NMAX) * sizeof(T) + size_t(2048 / NMAX) * sizeof(int64_t);
}

__device__ __forceinline__ void cp_async_16(uint32_t dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src),
               "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <class T>
__device__ __forceinline__ void skinny_async_body(const GemmArgs& g, int64_t tile,
                                                  unsigned char* dsmem) {
  static_assert(sizeof(T) == 8, "8-byte elements");
  constexpr int NMAX = 4, RW = 4;
  T (*ring)[32][kSkKS] = reinterpret_cast<T (*)[32][kSkKS]>(dsmem);
  T (*Bs)[kSkinnyAsyncMaxK] =
      reinterpret_cast<T (*)[kSkinnyAsyncMaxK]>(dsmem + size_t(kSkStages) * 32 * kSkKS * 8);
  const int64_t M = g.M, N = g.N, K = g.K;
  const int64_t tiles_m = (M + 31) / 32;
  const int64_t split = tile / tiles_m;
  const int64_t m0 = (tile - split * tiles_m) * 32;
  const int64_t kb = split * g.k_per_split;
  const int64_t ke = min(K, kb + g.k_per_split);
  const int kn = static_cast<int>(ke - kb);
  const int nst = (kn + kSkKS - 1) / kSkKS;
  T* __restrict__ C = static_cast<T*>(g.C) + split * g.c_split_stride;
  const T* __restrict__ A = static_cast<const T*>(g.A);
  const T* __restrict__ B = static_cast<const T*>(g.B);
  const bool conjA = g.flags & kFlagConjA;
  const bool conjB = g.flags & kFlagConjB;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  // Copies of this thread: 16-byte chunk c = tid + 256 i of a stage, row
  // c / 32, elements 2 (c % 32) and 2 (c % 32) + 1.
  int64_t rowoff[4];
  bool rok[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = (tid >> 5) + 8 * i;
    rok[i] = m0 + r < M;
    rowoff[i] = rok[i] ? offs(g.rsA, g.uA_m, m0 + r) : 0;
  }
  const int kk2 = 2 * (tid & 31);
  auto issue = [&](int s) {
    const int slot = s % kSkStages;
    const int64_t k0 = kb + int64_t(s) * kSkKS;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = (tid >> 5) + 8 * i;
      const int64_t k = k0 + kk2;
      const bool in = rok[i] && k < ke;
      const uint32_t bytes = in ? static_cast<uint32_t>(min(static_cast<int64_t>(2), ke - k) * 8) : 0u;
      const T* src = in ? A + rowoff[i] + k : A;
      cp_async_16(static_cast<uint32_t>(__cvta_generic_to_shared(&ring[slot][r][kk2])), src, bytes);
    }
    cp_async_commit();
  };
#pragma unroll
  for (int s = 0; s < kSkStages - 1; ++s) {
    if (s < nst) issue(s);
    else cp_async_commit();
  }
  // B chunk, zero-padded to NMAX columns and to whole stages, while the
  // first A stages are in flight (visible at the first stage's barrier).
  for (int e = tid; e < NMAX * nst * kSkKS; e += kThreads) {
    const int n = e / (nst * kSkKS), kk = e % (nst * kSkKS);
    T v = zero<T>();
    if (n < N && kk < kn)
      v = conj_if(B[offs(g.rsB, g.uB_k, kb + kk) + offs(g.csB, g.uB_n, n)], conjB);
    Bs[n][kk] = v;
  }
  T acc[RW][NMAX];
#pragma unroll
  for (int r = 0; r < RW; ++r)
#pragma unroll
    for (int n = 0; n < NMAX; ++n) acc[r][n] = zero<T>();
  for (int s = 0; s < nst; ++s) {
    cp_async_wait<kSkStages - 2>();
    __syncthreads();  // stage s visible to all; the slot refilled below is free
    const int slot = s % kSkStages;
#pragma unroll
    for (int u = 0; u < kSkKS / 32; ++u) {
      const int kk = lane + 32 * u;
#pragma unroll
      for (int r = 0; r < RW; ++r) {
        const T a = conj_if(ring[slot][warp * RW + r][kk], conjA);
#pragma unroll
        for (int n = 0; n < NMAX; ++n) mac(acc[r][n], a, Bs[n][s * kSkKS + kk]);
      }
    }
    if (s + kSkStages - 1 < nst) issue(s + kSkStages - 1);
    else cp_async_commit();
  }
  cp_async_wait<0>();
#pragma unroll
  for (int r = 0; r < RW; ++r) {
#pragma unroll
    for (int n = 0; n < NMAX; ++n) {
      T v = acc[r][n];
#pragma unroll
      for (int d = 16; d >= 1; d >>= 1) v = add(v, shfl_xor(v, d));
      acc[r][n] = v;
    }
    const int64_t m = m0 + warp * RW + r;
    if (lane == 0 && m < M)
#pragma unroll
      for (int n = 0; n < NMAX; ++n)
        if (n < N) skinny_store(g, C, m, n, acc[r][n]);
  }
}

template <class T, int NMAX>
__global__ void __launch_bounds__(kThreads)
skinny_contract(const SimtProblem* group, int nprob) {
  __shared__ GemmArgs ga;
  // One dynamic area serves either body: the asynchronous ring and B chunk,
  // or the generic body's B chunk and K offsets.
  extern __shared__ __align__(16) unsigned char skinny_dsmem[];
  T (*Bs)[2048 / NMAX] = reinterpret_cast<T (*)[2048 / NMAX]>(skinny_dsmem);
  int64_t* ks = reinterpret_cast<int64_t*>(skinny_dsmem + size_t(NMAX) * (2048 / NMAX) * sizeof(T));
  int64_t tile = blockIdx.x;
  int lo = 0, hi = nprob - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (group[mid].tile_begin <= tile) lo = mid; else hi = mid - 1;
  }
  tile -= group[lo].tile_begin;
  if (threadIdx.x == 0) ga = group[lo].g;
  __syncthreads();
  if constexpr (NMAX == 4 && sizeof(T) == 8) {
    if (ga.flags & kFlagSkinnyAsync) {
      skinny_async_body<T>(ga, tile, skinny_dsmem);
      return;
    }
  }
  if (ga.uA_k == 1)
    skinny_body<T, NMAX, true>(ga, tile, Bs, ks);
  else
    skinny_body<T, NMAX, false>(ga, tile, Bs, ks);
}

template <class T, int NMAX>
cudaError_t launch_skinny(const SimtProblem* dev, int nprob, int64_t total_tiles,
                          cudaStream_t stream) {
  if (total_tiles <= 0) return cudaSuccess;
  if (total_tiles > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  // The asynchronous form's ring and B chunk exist only in the instances
  // that can run it; the generic body's arrays share the same area.
  constexpr size_t kGen = skinny_generic_smem<T, NMAX>();
  constexpr size_t kDyn = (NMAX == 4 && sizeof(T) == 8 && kSkAsyncSmem > kGen) ? kSkAsyncSmem : kGen;
  if constexpr (kDyn > 48 * 1024) {
    static bool attr_set = false;
    if (!attr_set) {
      const cudaError_t e = cudaFuncSetAttribute(
          skinny_contract<T, NMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kDyn));
      if (e != cudaSuccess) return e;
      attr_set = true;
    }
  }
  skinny_contract<T, NMAX><<<static_cast<unsigned>(total_tiles), kThreads, kDyn, stream>>>(
      dev, nprob);
  return cudaGetLastError();
}

template <int NMAX>
cudaError_t launch_skinny_dtype(int dtype, const SimtProblem* dev, int nprob, int64_t tiles,
                                cudaStream_t stream) {
  switch (dtype) {
    case 0: return launch_skinny<float, NMAX>(dev, nprob, tiles, stream);
    case 1: return launch_skinny<double, NMAX>(dev, nprob, tiles, stream);
    case 2: return launch_skinny<float2, NMAX>(dev, nprob, tiles, stream);
    case 3: return launch_skinny<double2, NMAX>(dev, nprob, tiles, stream);
  }
  return cudaErrorInvalidValue;
}

}  // namespace

bool skinny_async_ok(const GemmArgs& g, const std::vector<int64_t>& rsA, size_t elem, int nmax) {
  if (nmax != 4 || elem != 8 || g.uA_k != 1 || g.N > 4) return false;
  if (reinterpret_cast<uintptr_t>(g.A) % 16 != 0) return false;
  if (std::min<int64_t>(g.K, g.k_per_split) > kSkinnyAsyncMaxK) return false;
  if (g.k_per_split % 2 != 0 && g.k_per_split < g.K) return false;  // split starts stay even
  if (g.uA_m >= 0) return g.uA_m % 2 == 0 || g.M <= 1;
  for (int64_t m = 0; m < g.M; ++m)
    if (rsA[m] % 2 != 0) return false;
  return true;
}

int64_t skinny_tiles(const GemmArgs& g, int splits, int nmax) {
  const int64_t rows = skinny_rows(g.uA_k == 1, nmax);
  return int64_t(splits) * ((g.M + rows - 1) / rows);
}

cudaError_t launch_skinny_group(int dtype, int nmax, const SimtProblem* dev, int nprob,
                                int64_t total_tiles, cudaStream_t stream) {
  return nmax <= 4 ? launch_skinny_dtype<4>(dtype, dev, nprob, total_tiles, stream)
                   : launch_skinny_dtype<16>(dtype, dev, nprob, total_tiles, stream);
}

void simt_group_tile(int dtype, bool skinny, int* bm, int* bn) {
  if (skinny) {
    *bm = 128;
    *bn = 16;
    return;
  }
  int bk;
  simt_tile(dtype, bm, bn, &bk);
}

cudaError_t launch_simt_group(int dtype, bool skinny, const SimtProblem* dev, int nprob,
                              int64_t total_tiles, cudaStream_t stream) {
  if (skinny) {
    switch (dtype) {
      case 0: return launch_group<float, 8, 1, 16>(dev, nprob, total_tiles, stream);
      case 1: return launch_group<double, 8, 1, 16>(dev, nprob, total_tiles, stream);
      case 2: return launch_group<float2, 8, 1, 16>(dev, nprob, total_tiles, stream);
      case 3: return launch_group<double2, 8, 1, 16>(dev, nprob, total_tiles, stream);
    }
    return cudaErrorInvalidValue;
  }
  switch (dtype) {
    case 0: return launch_group<float, 8, 8, 8>(dev, nprob, total_tiles, stream);
    case 1: return launch_group<double, 8, 4, 8>(dev, nprob, total_tiles, stream);
    case 2: return launch_group<float2, 4, 8, 8>(dev, nprob, total_tiles, stream);
    case 3: return launch_group<double2, 4, 4, 8>(dev, nprob, total_tiles, stream);
  }
  return cudaErrorInvalidValue;
}

void simt_tile(int dtype, int* bm, int* bn, int* bk) {
  switch (dtype) {
    case 0: *bm = 128; *bn = 128; break;
    case 1: *bm = 128; *bn = 64; break;
    case 2: *bm = 64; *bn = 128; break;
    default: *bm = 64; *bn = 64; break;
  }
  *bk = 8;
}

cudaError_t launch_simt(int dtype, const GemmArgs& args, int splits, cudaStream_t stream,
                        int* kernels) {
  *kernels = 1;
  switch (dtype) {
    case 0: return launch<float, 8, 8, 8>(args, splits, stream);
    case 1: return launch<double, 8, 4, 8>(args, splits, stream);
    case 2: return launch<float2, 4, 8, 8>(args, splits, stream);
    case 3: return launch<double2, 4, 4, 8>(args, splits, stream);
  }
  return cudaErrorInvalidValue;
}

}  // namespace gb300
}  // namespace t1m
