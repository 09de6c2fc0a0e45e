// complex128 / float64 contraction on the FP64 tensor-core MMA (DMMA,
// mma.sync.m8n8k4.f64), the FP64 counterpart of the tensor-core form.
//
// Replaces the reference's double-precision five-loop GEMM with the BLIS
// dgemm micro-kernel (include/t1m/t1m.h:508-554, bli/mappings.h:95-97).  Each
// complex 8x8 output block accumulates four real MMAs per k-step of 4:
// Cre += Are*Bre - Aim*Bim and Cim += Are*Bim + Aim*Bre (the products of the
// 1M real expansion, t1m.h:309-337, kept as separate real/imaginary planes).
// Tiles are gathered straight from the tensors through the scatter vectors,
// double-buffered in shared memory; accumulation and the alpha/beta epilogue
// are FP64 throughout.
#include <cuda_runtime.h>

#include <cstdint>

#include "internal.h"

namespace t1m {
namespace gb300 {
namespace {

constexpr int kThreads = 128;  // 4 warps, 2 x 2
constexpr int kWarpM = 16;     // complex rows per warp (2 blocks of 8)
constexpr int kWarpN = 32;     // complex columns per warp (4 blocks of 8)
constexpr int kBM = 2 * kWarpM;
constexpr int kBN = 2 * kWarpN;
constexpr int kBK = 8;         // complex K per stage (2 MMA k-steps)

__device__ __forceinline__ int64_t offs(const int64_t* v, int64_t u, int64_t i) {
  return u >= 0 ? i * u : __ldg(v + i);
}

// d (2 doubles) += a (1) * b (1) on an 8x8x4 FP64 tile (one warp).
__device__ __forceinline__ void dmma(double (&d)[2], double a, double b) {
  asm volatile(
      "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
      : "+d"(d[0]), "+d"(d[1])
      : "d"(a), "d"(b));
}

template <bool kComplex>
__global__ void __launch_bounds__(kThreads)
dmma_contract(const GemmArgs args) {
  using T = typename std::conditional<kComplex, double2, double>::type;
  constexpr int kAPer = kBM * kBK / kThreads;  // 2
  constexpr int kBPer = kBN * kBK / kThreads;  // 4
  __shared__ __align__(16) T As[2][kBK][kBM + 2];
  __shared__ __align__(16) T Bs[2][kBK][kBN + 2];

  const int64_t M = args.M, N = args.N;
  const int64_t kb = static_cast<int64_t>(blockIdx.y) * args.k_per_split;
  const int64_t K = min(args.K, kb + args.k_per_split);
  const T* __restrict__ A = static_cast<const T*>(args.A);
  const T* __restrict__ B = static_cast<const T*>(args.B);
  T* __restrict__ C = static_cast<T*>(args.C) + static_cast<int64_t>(blockIdx.y) * args.c_split_stride;
  const bool conjA = args.flags & kFlagConjA;
  const bool conjB = args.flags & kFlagConjB;

  const int64_t tiles_m = (M + kBM - 1) / kBM;
  const int64_t tiles_n = (N + kBN - 1) / kBN;
  constexpr int64_t G = 8;
  const int64_t t = blockIdx.x;
  const int64_t group = t / (G * tiles_n);
  const int64_t first_m = group * G;
  const int64_t gsize = min(G, tiles_m - first_m);
  const int64_t m0 = (first_m + (t % (G * tiles_n)) % gsize) * kBM;
  const int64_t n0 = ((t % (G * tiles_n)) / gsize) * kBN;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp & 1) * kWarpM, wn = (warp >> 1) * kWarpN;
  const bool a_kfast = (args.uA_k == 1);
  const bool b_kfast = (args.uB_k == 1) || (args.uB_n != 1);

  T ra[kAPer], rb[kBPer];
  auto load = [&](int64_t k0) {
#pragma unroll
    for (int p = 0; p < kAPer; ++p) {
      const int idx = tid + p * kThreads;
      const int m = a_kfast ? idx / kBK : idx % kBM;
      const int k = a_kfast ? idx % kBK : idx / kBM;
      T v{};
      if (m0 + m < M && k0 + k < K)
        v = A[offs(args.rsA, args.uA_m, m0 + m) + offs(args.csA, args.uA_k, k0 + k)];
      if constexpr (kComplex) {
        if (conjA) v.y = -v.y;
      }
      ra[p] = v;
    }
#pragma unroll
    for (int p = 0; p < kBPer; ++p) {
      const int idx = tid + p * kThreads;
      const int n = b_kfast ? idx / kBK : idx % kBN;
      const int k = b_kfast ? idx % kBK : idx / kBN;
      T v{};
      if (n0 + n < N && k0 + k < K)
        v = B[offs(args.rsB, args.uB_k, k0 + k) + offs(args.csB, args.uB_n, n0 + n)];
      if constexpr (kComplex) {
        if (conjB) v.y = -v.y;
      }
      rb[p] = v;
    }
  };
  auto store = [&](int buf) {
#pragma unroll
    for (int p = 0; p < kAPer; ++p) {
      const int idx = tid + p * kThreads;
      const int m = a_kfast ? idx / kBK : idx % kBM;
      const int k = a_kfast ? idx % kBK : idx / kBM;
      As[buf][k][m] = ra[p];
    }
#pragma unroll
    for (int p = 0; p < kBPer; ++p) {
      const int idx = tid + p * kThreads;
      const int n = b_kfast ? idx / kBK : idx % kBN;
      const int k = b_kfast ? idx % kBK : idx / kBN;
      Bs[buf][k][n] = rb[p];
    }
  };

  // Accumulators: [row block][col block][re/im][2].
  double acc_re[2][4][2], acc_im[2][4][2];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int e = 0; e < 2; ++e) acc_re[i][j][e] = acc_im[i][j][e] = 0.0;

  const int64_t ksteps = (K - kb + kBK - 1) / kBK;
  if (ksteps > 0) {
    load(kb);
    store(0);
  }
  __syncthreads();
  const int fr = lane >> 2, fk = lane & 3;  // fragment row/col and k index
  for (int64_t s = 0; s < ksteps; ++s) {
    const int buf = static_cast<int>(s & 1);
    if (s + 1 < ksteps) load(kb + (s + 1) * kBK);
#pragma unroll
    for (int k4 = 0; k4 < kBK; k4 += 4) {
      double are[2], aim[2], bre[4], bim[4];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const T v = As[buf][k4 + fk][wm + 8 * i + fr];
        if constexpr (kComplex) {
          are[i] = v.x;
          aim[i] = v.y;
        } else {
          are[i] = v;
          aim[i] = 0.0;
        }
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const T v = Bs[buf][k4 + fk][wn + 8 * j + fr];
        if constexpr (kComplex) {
          bre[j] = v.x;
          bim[j] = v.y;
        } else {
          bre[j] = v;
          bim[j] = 0.0;
        }
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          dmma(acc_re[i][j], are[i], bre[j]);
          if constexpr (kComplex) {
            dmma(acc_re[i][j], -aim[i], bim[j]);
            dmma(acc_im[i][j], are[i], bim[j]);
            dmma(acc_im[i][j], aim[i], bre[j]);
          }
        }
    }
    if (s + 1 < ksteps) store(buf ^ 1);
    __syncthreads();
  }

  // Epilogue: element (row fr, cols 2*fk, 2*fk+1) of each 8x8 block.
  const double2 alpha = make_double2(args.alpha[0], args.alpha[1]);
  const double2 beta = make_double2(args.beta[0], args.beta[1]);
  const bool accumulate = args.flags & kFlagAccumulate;
  const bool beta_zero = args.flags & kFlagBetaZero;
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int64_t m = m0 + wm + 8 * i + fr;
    if (m >= M) continue;
    const int64_t rc = offs(args.rsC, args.uC_m, m);
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int64_t n = n0 + wn + 8 * j + 2 * fk + e;
        if (n >= N) continue;
        T* p = C + rc + offs(args.csC, args.uC_n, n);
        const double vr = acc_re[i][j][e], vi = acc_im[i][j][e];
        double tr = alpha.x * vr - alpha.y * vi, ti = alpha.x * vi + alpha.y * vr;
        if constexpr (kComplex) {
          if (accumulate) {
            const double2 o = *p;
            tr += o.x;
            ti += o.y;
          } else if (!beta_zero) {
            const double2 o = *p;
            tr += beta.x * o.x - beta.y * o.y;
            ti += beta.x * o.y + beta.y * o.x;
          }
          *p = make_double2(tr, ti);
        } else {
          if (accumulate)
            tr += *p;
          else if (!beta_zero)
            tr += beta.x * *p;
          *p = tr;
        }
      }
  }
}

}  // namespace

void dmma_tile(int* bm, int* bn, int* bk) {
  *bm = kBM;
  *bn = kBN;
  *bk = kBK;
}

cudaError_t launch_dmma(int dtype, const GemmArgs& args, int splits, cudaStream_t stream,
                        int* kernels) {
  *kernels = 0;
  const int64_t tiles = ((args.M + kBM - 1) / kBM) * ((args.N + kBN - 1) / kBN);
  if (tiles == 0) return cudaSuccess;
  if (tiles > 0x7fffffffLL || splits < 1 || splits > 65535) return cudaErrorInvalidConfiguration;
  const dim3 grid(static_cast<unsigned>(tiles), static_cast<unsigned>(splits));
  if (dtype == 3)
    dmma_contract<true><<<grid, kThreads, 0, stream>>>(args);
  else if (dtype == 1)
    dmma_contract<false><<<grid, kThreads, 0, stream>>>(args);
  else
    return cudaErrorInvalidValue;
  *kernels = 1;
  return cudaGetLastError();
}

}  // namespace gb300
}  // namespace t1m
