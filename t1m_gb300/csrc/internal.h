// Internal declarations shared by the host plan builder, the C-ABI and the
// kernels of libt1m_cuda.so.  Nothing here is part of the public ABI.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

namespace t1m {
namespace gb300 {

// One mode of a bundle as seen by the two tensors that share it.
//   M bundle: s0 = stride in A, s1 = stride in C
//   N bundle: s0 = stride in B, s1 = stride in C
//   K bundle: s0 = stride in A, s1 = stride in B
struct Mode {
  int64_t extent;
  int64_t s0;
  int64_t s1;
  char label;
};

// Host-side description of one contraction after label analysis.
// Element (m, n) of the matricised problem lives at
//   A: rsA[m] + csA[k]   B: rsB[k] + csB[n]   C: rsC[m] + csC[n]
// (the reference's rscat/cscat vectors, t1m.h:141-174, in element units).
// A batch (Hadamard) mode: a label of A, B and C alike.  The contraction is
// one independent product per batch index (no reference counterpart: the
// reference leaves such labels undefined).
struct BatchMode {
  int64_t extent, sa, sb, sc;
  char label;
};

struct HostPlan {
  int dtype = 0;
  int64_t M = 0, N = 0, K = 0;
  std::vector<Mode> modes_m, modes_n, modes_k;
  std::vector<BatchMode> modes_b;  // first mode fastest
  int64_t batch = 1;               // product of the batch extents
  std::vector<int64_t> rsA, csA, rsB, csB, rsC, csC;
  // Uniform stride of each scatter vector, or -1 when it is not an arithmetic
  // progression (the block-scatter "constant stride" of t1m.h:179-205 taken
  // over the whole vector).
  int64_t uA_m = -1, uA_k = -1, uB_k = -1, uB_n = -1, uC_m = -1, uC_n = -1;
  // Number of elements each tensor spans in memory (1 + sum (e-1)*s).
  int64_t spanA = 0, spanB = 0, spanC = 0;
  // Derived once per plan (the context caches plans across calls): results
  // of the tensor-core path's layout checks over the scatter vectors, keyed
  // by check and length, and the plans with densely packed operands (index
  // 1: A packed, 2: B packed, 3: both).
  mutable std::map<std::pair<int, int64_t>, int64_t> memo;
  mutable std::shared_ptr<HostPlan> packed[4];
};

// Element offsets of batch index `bi` (mixed radix over modes_b, first mode
// fastest) in A, B and C.
inline void batch_offsets(const HostPlan& hp, int64_t bi, int64_t* oa, int64_t* ob,
                          int64_t* oc) {
  *oa = *ob = *oc = 0;
  for (const BatchMode& m : hp.modes_b) {
    const int64_t i = bi % m.extent;
    bi /= m.extent;
    *oa += i * m.sa;
    *ob += i * m.sb;
    *oc += i * m.sc;
  }
}

// Validate labels/extents/strides and build the plan.  Returns a t1m_status
// and fills *err with a message on failure.
int build_plan(int dtype, int na, const int64_t* ea, const int64_t* sa,
               const char* la, int nb, const int64_t* eb, const int64_t* sb,
               const char* lb, int nc, const int64_t* ec, const int64_t* sc,
               const char* lc, HostPlan* plan, std::string* err);

// Device-resident copy of a plan's scatter vectors (one allocation).
struct DevicePlan {
  void* block = nullptr;
  size_t bytes = 0;
  const int64_t *rsA = nullptr, *csA = nullptr, *rsB = nullptr, *csB = nullptr,
                *rsC = nullptr, *csC = nullptr;
};

// Kernel arguments of one contraction launch (plain or tensor-core).
struct GemmArgs {
  const void* A;
  const void* B;
  void* C;
  int64_t M, N, K;
  const int64_t *rsA, *csA, *rsB, *csB, *rsC, *csC;
  int64_t uA_m, uA_k, uB_k, uB_n, uC_m, uC_n;
  double alpha[2];
  double beta[2];
  uint32_t flags;  // kFlag* below
  // Split-K: CTA row blockIdx.y handles K range [y*k_per_split, ...) and, when
  // c_split_stride != 0, writes its partial product to C + y*c_split_stride.
  int64_t k_per_split;
  int64_t c_split_stride;
};

constexpr uint32_t kFlagAccumulate = 1u;  // C += alpha*AB (beta ignored)
constexpr uint32_t kFlagConjA = 2u;
constexpr uint32_t kFlagConjB = 4u;
constexpr uint32_t kFlagBetaZero = 16u;  // BLAS semantics with beta == 0
// Epilogue store forms of the tensor-core kernels (set by tc_prepare):
// C columns pairwise contiguous and every pair 16-byte aligned (one 16-byte
// store per two complex values), and C column offsets unit stride inside
// every 16-column block (one offset lookup per 16 columns).
constexpr uint32_t kFlagCPairs = 32u;
constexpr uint32_t kFlagCCol16 = 64u;
// Skinny kernel: A streams through a cp.async shared-memory pipeline (set by
// the host where A has unit K stride, 8-byte elements, 16-byte aligned rows,
// a K chunk of at most kSkinnyAsyncMaxK and N <= 4).
constexpr uint32_t kFlagSkinnyAsync = 128u;
constexpr int kSkinnyAsyncMaxK = 1024;

// Internal method id: tensor cores, precision chosen per problem by the
// launcher (BF16x6 where the one-tile kernel fetches both operands by TMA,
// 3xTF32 elsewhere); the report carries the method that ran.
constexpr int kMethodTcAuto = 100;

// Method of T1M_METHOD_AUTO for a planned contraction (capi.cu): the tensor
// cores (kMethodTcAuto) for complex64 with M*N*K >= 2^18 and float32 with
// M*N*K >= 2^20, else the plain kernel.  t1m_contract and
// t1m_contract_noalloc share it.
int auto_method(int dtype, const HostPlan& plan);

// Precision rule of T1M_METHOD_AUTO: the longest K range (elements of the
// contracted bundle) one FP32-accumulated partial product may cover so that
// its relative error against FP64 stays below 1e-6 (0: no limit, the FP64
// paths).  Longer contractions are split along K and the partials summed,
// with the epilogue, in FP64 (the split-K reduction).
//  * plain FP32: sequential FMA accumulation, error ~3.1e-8 sqrt(terms)
//    (measured 2.8e-6 at 8192 real terms): 256 real terms per partial, i.e.
//    K <= 128 complex or 256 real;
//  * tensor cores: the correction accumulator truncates ~2e-8 per MMA over
//    the whole range (4e-7 at K = 4096 complex): K <= 4096 complex or 8192
//    real.
int64_t accuracy_k_limit(int method, int dtype);

// Launchers.  Return cudaError_t of the launch.
// simt.cu: plain FP32/FP64 kernel; `splits` CTA rows along K.
cudaError_t launch_simt(int dtype, const GemmArgs& args, int splits, cudaStream_t stream,
                        int* kernels);
// Output tile sizes of the plain kernel for a dtype (for split decisions).
void simt_tile(int dtype, int* bm, int* bn, int* bk);

// One contraction of a grouped plain launch (device array, sorted by
// tile_begin).  Its tiles are numbered split-major: g.k_per_split and
// g.c_split_stride describe split-K exactly as for a single launch, and the
// problem owns splits x tiles of the launch's tile list.
struct SimtProblem {
  GemmArgs g;
  int64_t tile_begin;
};
// Tile of a grouped plain launch: the regular tile, or a skinny one (128 x 16)
// for contractions with few output columns.
void simt_group_tile(int dtype, bool skinny, int* bm, int* bn);
cudaError_t launch_simt_group(int dtype, bool skinny, const SimtProblem* dev, int nprob,
                              int64_t total_tiles, cudaStream_t stream);

// Skinny grouped launches (simt.cu): outputs of at most `nmax` (4 or 16)
// columns, bound by reading A once.  Rows per CTA: one warp per row (16 / nmax
// rows per warp, 8 warps) when A has unit K stride, else one thread per row.
constexpr int kSkinnyMaxN = 16;
__host__ __device__ constexpr int skinny_rows(bool k_unit, int nmax) {
  return k_unit ? 8 * (16 / nmax) : 256;
}
// kFlagSkinnyAsync for an item of a skinny launch of column bound nmax
// (rs: the plan's A row offsets; uniform stride uA_m where >= 0).
bool skinny_async_ok(const GemmArgs& g, const std::vector<int64_t>& rsA, size_t elem, int nmax);
// Tiles of one skinny problem: splits x ceil(M / rows).
int64_t skinny_tiles(const GemmArgs& g, int splits, int nmax);
cudaError_t launch_skinny_group(int dtype, int nmax, const SimtProblem* dev, int nprob,
                                int64_t total_tiles, cudaStream_t stream);

// splitk.cu: C <- alpha * sum_s W[s] + beta*C (or C + alpha*sum) with the sum
// in FP64.  W holds `splits` dense M x N partials, m fastest, of the dtype.
cudaError_t launch_splitk_reduce(int dtype, const void* work, int splits, const GemmArgs& out,
                                 cudaStream_t stream);

// Grouped split-K reduction: one launch over the outputs of many split
// contractions (device array sorted by begin = prefix sum of M*N).
struct SplitReduce {
  GemmArgs out;       // C, its scatter vectors and the epilogue
  const void* work;   // splits dense M x N partials, m fastest
  int64_t begin;      // first output element of this problem in the launch
  int32_t splits;
  int32_t pad;
};
cudaError_t launch_splitk_reduce_group(int dtype, const SplitReduce* dev, int n,
                                       int64_t total, cudaStream_t stream);

// Operand pieces already in device memory (the host-buffer pipeline splits
// its resident operand once for all slabs): P bf16 arrays per operand, rows
// tc_pieces_pitch(K) elements apart, `*_plane` elements between arrays; A's
// rows are the 1M rows (two per complex row), B's one per column.  Null
// pointers: the product splits that operand itself.
struct PiecesReady {
  const void* a = nullptr;
  int64_t a_plane = 0;
  const void* b = nullptr;
  int64_t b_plane = 0;
};

// tc.cu: one contraction on the tensor cores (complex64 / float32, split
// methods).  `panel` (panel_bytes) is workspace for B split once into
// panels, at least tc_panel_bytes(dtype, M, N, K) bytes, or null.
// `pack` (pack_bytes) is workspace for operands repacked densely
// (tc_pack_bytes), or null.
// `path` (may be null) receives the product's T1M_PATH_* code (t1m_capi.h).
// `main_ev` (may be null): two events recorded on `stream` right before and
// after the launch of the product's main kernel (after its split, pack and
// panel passes).
// In-kernel split-K reduction of a split product on the persistent kernel:
// `ctr` (cap zeroed ints) for the arrival counters, `out` the product's own
// arguments (C, alpha, beta, flags); launch_tc sets `reduced` when the kernel
// applied the epilogue itself (no reduction kernel needed).
struct TcFix {
  int* ctr;
  int64_t cap;
  const GemmArgs* out;
  bool reduced;
};
cudaError_t launch_tc(int method, int dtype, const GemmArgs& args, const HostPlan& plan,
                      int splits, cudaStream_t stream, int* err_flag, int* kernels,
                      std::string* err, int* used_method, void* panel = nullptr,
                      size_t panel_bytes = 0, void* pack = nullptr, size_t pack_bytes = 0,
                      int* path = nullptr, int form = 0 /* T1M_TILE_* */,
                      const PiecesReady* ready = nullptr, cudaEvent_t* main_ev = nullptr,
                      TcFix* fix = nullptr);
// Panel workspace a product would use (0: panels not used at this size).
size_t tc_panel_bytes(int dtype, int64_t M, int64_t N, int64_t K);
// Bytes of the operand pieces of the T1M_TILE_PIECES form (held in the panel
// workspace), 0 where that form does not apply.  kMethodTcAuto counts the
// BF16x6 pieces.  With `ready`, only the operands it does not hold.
size_t tc_pieces_bytes(int dtype, int method, int64_t M, int64_t N, int64_t K,
                       const PiecesReady* ready = nullptr);
int64_t tc_pieces_pitch(int64_t K);
// Pieces per element (2 or 3) the product would be split into by launch_tc
// with this method and tile form, 0 if it would not run as pieces.
int tc_pieces_count(int method, int dtype, const GemmArgs& g, const HostPlan& plan, int form);
// Split operand A (the 1M rows of its M rows) or B (its N rows) of g into
// `pieces` arrays at `out`, `plane` elements apart (one launch on s).
cudaError_t tc_split_operand(int pieces, bool operand_a, const GemmArgs& g, void* out,
                             int64_t plane, cudaStream_t s);
// Pack workspace a product may use (0: neither operand would be packed).
size_t tc_pack_bytes(int dtype, const HostPlan& plan);

// pack.cu: dst[r * pitch + k] = src[ro(r) + ko(k)] (complex64 or float32),
// reads coalesced along the source's unit-stride direction: a K mode of
// k-step S (S > 0), a row mode (S == 0), or none (S < 0).
int64_t pack_pitch(int dtype, int64_t K);
cudaError_t launch_pack(int dtype, const void* src, const int64_t* ro, int64_t ur,
                        const int64_t* ko, int64_t uk, int64_t R, int64_t K, int64_t S,
                        void* dst, int64_t pitch, cudaStream_t stream);
bool tc_supported(int method, int dtype, const HostPlan& plan);
void tc_tile(int dtype, int* bm, int* bn, int* bk);

}  // namespace gb300
}  // namespace t1m
