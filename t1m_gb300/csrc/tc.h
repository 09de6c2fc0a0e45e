// Problem descriptor of the persistent tensor-core kernel (tc.cu), shared with
// the grouped-launch host code (grouped.cu).
#pragma once

#include <cuda.h>

#include <cstdint>
#include <string>

#include "internal.h"

namespace t1m {
namespace gb300 {

// Operand fetch modes (see tc.cu).
//   A: gather [k][m];  MK: one TMA box [k][64 m] (M unit stride, uniform K);
//      MK16: four TMA boxes [16 k][16 m], one per unit-stride 16-row block;
//      KM: one TMA box [64 m][16 k] with 128 B swizzle (K unit stride, or
//      unit-stride 16-element K blocks and uniform M)
//   B: gather [n][k] swizzled;  NK: one TMA box [128 n][16 k] with 128 B
//      swizzle (K unit stride, or unit-stride 16-element K blocks);
//      KN: one TMA box [16 k][128 n] (N unit stride)
//   A KM16 / B NK16: K runs in unit-stride 16-element blocks and rows that
//      step by one common stride inside every 16-row block: one TMA box
//      [16 rows][16 k] (128 B swizzle) per 16-row block, its coordinate the
//      block's element offset; same shared-memory layouts as KM / NK.
//   A MK16K / B KN16: the transposed case (adjoint operands): rows (M or N)
//      in unit-stride 16-element blocks, K stepping by one common stride
//      inside every 16-element K block: one box [16 k][16 rows] per 16-row
//      block and K step, coordinate = row block offset + K block offset.
//      A keeps the MK16 layout; B lands as eight [16 k][16 n] blocks.
enum : int32_t { kAGather = 0, kAMK = 1, kAMK16 = 2, kAKM = 3, kAKM16 = 4, kAMK16K = 5 };
enum : int32_t { kBGather = 0, kBNK = 1, kBKN = 2, kBNK16 = 3, kBKN16 = 4 };

struct TcProblem {
  CUtensorMap map_a;
  CUtensorMap map_b;
  GemmArgs g;
  int32_t amode, bmode;
  int32_t tiles_m, tiles_n, splits;
  // Grouped launches: problem whose C this one reads (-1: none), and its tile
  // count; the loaders of this problem wait until that many of its tiles have
  // been written.
  int32_t dep;
  int32_t dep_tiles;
  // Bit 0: A's map is a per-16-element block map (coordinates from the
  // scatter vector); bit 1: the same for B.
  int32_t block_maps;
  int64_t tile_begin;  // first tile of this problem in the launch's tile list
  // Bound, in SM clock cycles, on the wait for the dependency's tiles (0:
  // the kernels' default of about two seconds).
  int64_t dep_wait_cycles;
  // Output tile width in complex (or real) columns: the MMA N and the height
  // of the B stage, one of 16, 32, 64, 128 (kTcTileWidths).  Narrow outputs
  // (the second step of a sweep update, N <= 4) take a 16-column tile
  // instead of computing a 128-column tile of which most is empty.
  int32_t tile_n;
  // Stages per main-product chunk accumulator, as a power of two (default
  // 2: four stages, 16 accumulating MMAs).  The tensor cores' FP32
  // accumulation truncates, with a bias of about 2e-8 of the accumulator per
  // accumulating MMA, so shorter chunks (folded into FP32 registers with
  // round-to-nearest adds) keep outputs that are sums of many terms of
  // either sign accurate.
  int32_t fold_shift;
  // In-kernel split-K reduction (grouped launches): when fix_begin >= 0 the
  // splits write raw partial products through g (a dense workspace, as for
  // the separate reduction) and count their arrivals on fix counters
  // fix_begin + output tile; the split that arrives last sums all partials
  // of its output tile in FP64, in split order, and applies the epilogue of
  // `out` (the item's C, alpha, beta and flags).  Only those final tiles
  // count towards the problem's tile-completion counter.
  int64_t fix_begin;
  GemmArgs out;
  // SIMT tile (tile_n 16, N <= 8): the converter warps compute the products
  // with FP32 FMAs from the raw stages and the MMA thread skips the tile.  A
  // narrow output streams A once; on the tensor cores its 1M split of A
  // would bound it (measured on the sweep batch's second steps: 57 ms as
  // 16-column tensor-core tiles, against 22 ms on the skinny kernel).
  int32_t skinny;
  int32_t pad2_;
};

// Widest output a SIMT tile of the persistent kernel takes.
constexpr int kTcSkinnyMaxN = 8;

// Output tile widths of the persistent kernel.
constexpr int kTcTileWidths[4] = {16, 32, 64, 128};
// Tile width for an output of N columns when none is given: the cheapest
// under a per-stage cost model of the persistent kernel (A side fixed, B
// side and MMA proportional to the width), so narrow outputs get narrow
// tiles and wide outputs 128 columns.
int tc_default_tile_n(int64_t N);

// Fill a descriptor (fetch modes, tensor maps, tile counts).  False if the
// problem cannot run on this kernel.
// `tile_n`: output tile width (one of kTcTileWidths), 0 = tc_default_tile_n.
bool tc_prepare(const GemmArgs& g, const HostPlan& plan, int splits, TcProblem* p,
                int tile_n = 128);
int64_t tc_problem_tiles(const TcProblem& p);
// One persistent launch over `total_tiles` tiles of `single` (dev_group null)
// or of the device array dev_group[0..nprob) (sorted by tile_begin, every
// dependency's tiles before its dependents').  `done` (grouped launches with
// dependencies) holds one zeroed tile-completion counter per problem; such
// launches are cooperative so all CTAs are resident.
// `fix` holds the zeroed split-K arrival counters of problems with
// fix_begin >= 0 (null when there are none).
cudaError_t tc_launch_persistent(const TcProblem* single, const TcProblem* dev_group, int nprob,
                                 int64_t total_tiles, int num_sms, int* done,
                                 cudaStream_t stream, int* err_flag, int* fix = nullptr);

}  // namespace gb300
}  // namespace t1m
