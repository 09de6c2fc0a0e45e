// Split-K reduction: C <- alpha * sum_s W[s] + beta * C (or C + alpha*sum under
// the reference's accumulate semantics), summed in FP64.
//
// The reference streams K in KC-sized chunks and scatter-adds every chunk's
// micro-tile into C (include/t1m/t1m.h:512-548).  Here, when a contraction has
// too few output tiles to fill the GPU (skinny M*N, long K) the K range is
// split across CTA rows; each split writes its partial product, dense and m
// fastest, into a workspace slice, and this kernel sums the slices in double
// precision and applies the epilogue through C's scatter vectors.  The FP64
// sum also keeps long contractions accurate: each partial only accumulates
// K/splits terms in FP32.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "internal.h"

namespace t1m {
namespace gb300 {
namespace {

__device__ __forceinline__ int64_t offs(const int64_t* v, int64_t u, int64_t i) {
  return u >= 0 ? i * u : __ldg(v + i);
}

template <class W> struct Wide;
template <> struct Wide<float> {
  static constexpr bool cplx = false;
};
template <> struct Wide<double> {
  static constexpr bool cplx = false;
};
template <> struct Wide<float2> {
  static constexpr bool cplx = true;
};
template <> struct Wide<double2> {
  static constexpr bool cplx = true;
};

__device__ __forceinline__ double2 widen(float v) { return make_double2(v, 0.0); }
__device__ __forceinline__ double2 widen(double v) { return make_double2(v, 0.0); }
__device__ __forceinline__ double2 widen(float2 v) { return make_double2(v.x, v.y); }
__device__ __forceinline__ double2 widen(double2 v) { return v; }

__device__ __forceinline__ void narrow(double2 v, float* p) { *p = static_cast<float>(v.x); }
__device__ __forceinline__ void narrow(double2 v, double* p) { *p = v.x; }
__device__ __forceinline__ void narrow(double2 v, float2* p) {
  *p = make_float2(static_cast<float>(v.x), static_cast<float>(v.y));
}
__device__ __forceinline__ void narrow(double2 v, double2* p) { *p = v; }

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Epilogue of one output element: C <- alpha*acc + beta*C (or C + alpha*acc).
template <class T>
__device__ __forceinline__ void finish(const GemmArgs& out, int64_t e, double2 acc) {
  const int64_t M = out.M;
  const int64_t m = e % M, n = e / M;
  T* p = static_cast<T*>(out.C) + offs(out.rsC, out.uC_m, m) + offs(out.csC, out.uC_n, n);
  double2 r = cmul(make_double2(out.alpha[0], out.alpha[1]), acc);
  if (out.flags & kFlagAccumulate) {
    const double2 o = widen(*p);
    r.x += o.x;
    r.y += o.y;
  } else if (!(out.flags & kFlagBetaZero)) {
    const double2 o = cmul(make_double2(out.beta[0], out.beta[1]), widen(*p));
    r.x += o.x;
    r.y += o.y;
  }
  narrow(r, p);
}

// A block of 8 warps reduces chunks of 32 consecutive outputs.  The G warps
// of a chunk (G = 2, 4 or 8 split groups) each sum the slices s = g, g + G,
// ... in ascending order, every slice read as one coalesced 32-element row;
// the first warp of the chunk adds the G partial sums in group order (a fixed
// order: the result does not depend on the launch shape), and applies the
// epilogue.  With fewer groups a block takes 8 / G chunks per step, so short
// split lists keep every warp busy.
template <class T>
__global__ void __launch_bounds__(256)
splitk_reduce(const T* __restrict__ work, int splits, int G, const GemmArgs out) {
  __shared__ double2 part[8][32];
  const int64_t MN = out.M * out.N;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = warp % G, sub = warp / G, per = 8 / G;
  const int64_t nchunks = (MN + 31) / 32;
  for (int64_t c0 = static_cast<int64_t>(blockIdx.x) * per; c0 < nchunks;
       c0 += static_cast<int64_t>(gridDim.x) * per) {
    const int64_t c = c0 + sub, e = c * 32 + lane;
    const bool live = c < nchunks && e < MN;
    double2 acc = make_double2(0.0, 0.0);
    if (live) {
#pragma unroll 4
      for (int s = g; s < splits; s += G) {
        const double2 v = widen(work[s * MN + e]);
        acc.x += v.x;
        acc.y += v.y;
      }
    }
    part[warp][lane] = acc;
    __syncthreads();
    if (g == 0 && live) {
      double2 tot = part[warp][lane];
      for (int j = 1; j < G; ++j) {
        tot.x += part[warp + j][lane].x;
        tot.y += part[warp + j][lane].y;
      }
      finish<T>(out, e, tot);
    }
    __syncthreads();
  }
}

// Grouped form: output element idx of the launch belongs to the problem with
// the last begin <= idx (binary search over the descriptors); 8 split groups
// per chunk of 32 outputs, as above.
template <class T>
__global__ void __launch_bounds__(256)
splitk_reduce_group(const SplitReduce* __restrict__ probs, int n, int64_t total) {
  __shared__ double2 part[8][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t nchunks = (total + 31) / 32;
  for (int64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const int64_t idx = c * 32 + lane;
    const bool live = idx < total;
    int lo = 0;
    double2 acc = make_double2(0.0, 0.0);
    if (live) {
      int hi = n - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (probs[mid].begin <= idx) lo = mid; else hi = mid - 1;
      }
      const SplitReduce& pr = probs[lo];
      const int64_t MN = pr.out.M * pr.out.N, e = idx - pr.begin;
      const T* __restrict__ work = static_cast<const T*>(pr.work);
#pragma unroll 4
      for (int s = warp; s < pr.splits; s += 8) {
        const double2 v = widen(work[s * MN + e]);
        acc.x += v.x;
        acc.y += v.y;
      }
    }
    part[warp][lane] = acc;
    __syncthreads();
    if (warp == 0 && live) {
      double2 tot = part[0][lane];
      for (int j = 1; j < 8; ++j) {
        tot.x += part[j][lane].x;
        tot.y += part[j][lane].y;
      }
      finish<T>(probs[lo].out, idx - probs[lo].begin, tot);
    }
    __syncthreads();
  }
}

template <class T>
cudaError_t launch_group(const SplitReduce* dev, int n, int64_t total, cudaStream_t stream) {
  if (total <= 0 || n <= 0) return cudaSuccess;
  const int64_t blocks = std::min<int64_t>((total + 31) / 32, 152 * 8);
  splitk_reduce_group<T><<<static_cast<unsigned>(blocks), 256, 0, stream>>>(dev, n, total);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch(const void* work, int splits, const GemmArgs& out, cudaStream_t stream) {
  const int64_t mn = out.M * out.N;
  if (mn == 0) return cudaSuccess;
  const int G = splits <= 2 ? 2 : splits <= 4 ? 4 : 8;
  const int64_t chunks = (mn + 31) / 32;
  const int64_t blocks = std::min<int64_t>((chunks + 8 / G - 1) / (8 / G), 152 * 8);
  splitk_reduce<T><<<static_cast<unsigned>(blocks), 256, 0, stream>>>(
      static_cast<const T*>(work), splits, G, out);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_splitk_reduce(int dtype, const void* work, int splits, const GemmArgs& out,
                                 cudaStream_t stream) {
  switch (dtype) {
    case 0: return launch<float>(work, splits, out, stream);
    case 1: return launch<double>(work, splits, out, stream);
    case 2: return launch<float2>(work, splits, out, stream);
    case 3: return launch<double2>(work, splits, out, stream);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_splitk_reduce_group(int dtype, const SplitReduce* dev, int n, int64_t total,
                                       cudaStream_t stream) {
  switch (dtype) {
    case 0: return launch_group<float>(dev, n, total, stream);
    case 1: return launch_group<double>(dev, n, total, stream);
    case 2: return launch_group<float2>(dev, n, total, stream);
    case 3: return launch_group<double2>(dev, n, total, stream);
  }
  return cudaErrorInvalidValue;
}

}  // namespace gb300
}  // namespace t1m
