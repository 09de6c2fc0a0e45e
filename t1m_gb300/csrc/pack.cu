// Dense repack of a gathered operand for the tensor-core kernels.
//
// An operand whose matricised view has neither a uniform unit-stride K nor a
// uniform row stride is gathered element by element inside the GEMM kernels
// (one 8-byte cp.async per complex element through the scatter vectors),
// which is latency-bound on GB300: one request and one 32-byte sector per
// element, a few hundred requests in flight per SM.  Where the operand is
// large, it is packed first into a dense [rows][k] array in the plan's K
// order (rows = M for A, N for B), which the kernels then load by TMA.  This
// is the packing the reference's BLIS back end does for every micro-panel
// (t1m.h:309-336), done once per operand instead of per block, and at the
// full occupancy of a standalone pass.
//
// dst[r * pitch + k] = src[ro(r) + ko(k)] for r < R, k < K, where ro / ko are
// the operand's row and K offsets (scatter vectors, or uniform strides).
// Reads are coalesced along the source's unit-stride direction through a
// 32 x 32 shared-memory tile, writes along k:
//   S > 0:  the source's unit-stride mode is a K mode whose k-step in the
//           plan's K order is S (k = k_lo + S * k_hi, source contiguous in k_hi);
//   S == 0: the source's unit-stride mode is a row mode (source contiguous in r);
//   S < 0:  no unit-stride mode: one thread per element, k fastest.
#include <cuda_runtime.h>

#include <cstdint>

#include "internal.h"
#include "t1m_capi.h"

namespace t1m {
namespace gb300 {
namespace {

__device__ __forceinline__ int64_t poffs(const int64_t* v, int64_t u, int64_t i) {
  return u >= 0 ? i * u : v[i];
}

template <typename T>
__global__ void __launch_bounds__(256)
pack_tiled(const T* __restrict__ src, const int64_t* __restrict__ ro, int64_t ur,
           const int64_t* __restrict__ ko, int64_t uk, int64_t R, int64_t K, int64_t S,
           T* __restrict__ dst, int64_t pitch, int64_t tiles_a, int64_t tiles_b) {
  __shared__ T tile[32][33];
  // Source offsets of the tile's 32 + 32 index values, loaded once per tile:
  // offsets are linear in the mode indices and S spans whole modes, so
  // ko(k_lo + S k_hi) = ko(k_lo) + ko(S k_hi) (and src(r, k) = ro(r) + ko(k)).
  __shared__ int64_t off_a[32], off_b[32];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 8 warps
  // Tile coordinates: S > 0: (row r, k_hi tile ta, k_lo tile tb);
  // S == 0: (row tile ta, k tile tb).
  int64_t t = blockIdx.x;
  const int64_t tb = t % tiles_b;
  t /= tiles_b;
  const int64_t ta = t % tiles_a;
  const int64_t r0 = t / tiles_a;
  if (S > 0) {
    const int64_t nhi = K / S;  // S is a product of leading K extents
    if (threadIdx.x < 32) {
      const int64_t khi = ta * 32 + threadIdx.x;
      off_a[threadIdx.x] = khi < nhi ? poffs(ko, uk, S * khi) : 0;
    } else if (threadIdx.x < 64) {
      const int64_t klo = tb * 32 + threadIdx.x - 32;
      off_b[threadIdx.x - 32] = klo < S ? poffs(ko, uk, klo) : 0;
    }
    __syncthreads();
    const int64_t rbase = poffs(ro, ur, r0);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int64_t klo = tb * 32 + ty + 8 * i, khi = ta * 32 + tx;
      if (klo < S && khi < nhi) tile[ty + 8 * i][tx] = src[rbase + off_b[ty + 8 * i] + off_a[tx]];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int64_t klo = tb * 32 + tx, khi = ta * 32 + ty + 8 * i;
      if (klo < S && khi < nhi) dst[r0 * pitch + klo + S * khi] = tile[tx][ty + 8 * i];
    }
  } else {
    if (threadIdx.x < 32) {
      const int64_t r = ta * 32 + threadIdx.x;
      off_a[threadIdx.x] = r < R ? poffs(ro, ur, r) : 0;
    } else if (threadIdx.x < 64) {
      const int64_t k = tb * 32 + threadIdx.x - 32;
      off_b[threadIdx.x - 32] = k < K ? poffs(ko, uk, k) : 0;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int64_t r = ta * 32 + tx, k = tb * 32 + ty + 8 * i;
      if (r < R && k < K) tile[ty + 8 * i][tx] = src[off_a[tx] + off_b[ty + 8 * i]];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int64_t k = tb * 32 + tx, r = ta * 32 + ty + 8 * i;
      if (r < R && k < K) dst[r * pitch + k] = tile[tx][ty + 8 * i];
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(256)
pack_elementwise(const T* __restrict__ src, const int64_t* __restrict__ ro, int64_t ur,
                 const int64_t* __restrict__ ko, int64_t uk, int64_t R, int64_t K,
                 T* __restrict__ dst, int64_t pitch) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * 256 + threadIdx.x;
  if (i >= R * K) return;
  const int64_t r = i / K, k = i % K;
  dst[r * pitch + k] = src[poffs(ro, ur, r) + poffs(ko, uk, k)];
}

template <typename T>
cudaError_t launch_pack_t(const void* src, const int64_t* ro, int64_t ur, const int64_t* ko,
                          int64_t uk, int64_t R, int64_t K, int64_t S, void* dst, int64_t pitch,
                          cudaStream_t stream) {
  const T* s = static_cast<const T*>(src);
  T* d = static_cast<T*>(dst);
  if (S < 0) {
    const int64_t blocks = (R * K + 255) / 256;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    pack_elementwise<T><<<static_cast<unsigned>(blocks), 256, 0, stream>>>(s, ro, ur, ko, uk, R,
                                                                          K, d, pitch);
    return cudaGetLastError();
  }
  int64_t ta, tb, rows;
  if (S > 0) {
    ta = ((K + S - 1) / S + 31) / 32;  // k_hi tiles
    tb = (S + 31) / 32;                // k_lo tiles
    rows = R;
  } else {
    ta = (R + 31) / 32;
    tb = (K + 31) / 32;
    rows = 1;
  }
  const int64_t blocks = rows * ta * tb;
  if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  pack_tiled<T><<<static_cast<unsigned>(blocks), 256, 0, stream>>>(s, ro, ur, ko, uk, R, K, S, d,
                                                                  pitch, ta, tb);
  return cudaGetLastError();
}

}  // namespace

int64_t pack_pitch(int dtype, int64_t K) {
  const int64_t per16 = dtype == T1M_FLOAT32 ? 4 : 2;  // elements per 16 bytes
  return (K + per16 - 1) / per16 * per16;
}

cudaError_t launch_pack(int dtype, const void* src, const int64_t* ro, int64_t ur,
                        const int64_t* ko, int64_t uk, int64_t R, int64_t K, int64_t S,
                        void* dst, int64_t pitch, cudaStream_t stream) {
  if (R <= 0 || K <= 0) return cudaSuccess;
  if (dtype == T1M_FLOAT32)
    return launch_pack_t<float>(src, ro, ur, ko, uk, R, K, S, dst, pitch, stream);
  return launch_pack_t<float2>(src, ro, ur, ko, uk, R, K, S, dst, pitch, stream);
}

}  // namespace gb300
}  // namespace t1m
