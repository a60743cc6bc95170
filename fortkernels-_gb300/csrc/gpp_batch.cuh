// Batched GPP: many instances in one persistent work queue per pass.
#pragma once

#include "sigma_internal.cuh"

namespace sigma {

// Tile shapes of the FP64 main pass (bands x columns per item).  Tiles 0-2
// belong to the per-band-frequency kernel, tiles 3-6 to the shared-frequency
// kernel (sch_fp64y_item; 64 x 16 is the single-instance plan's item); a
// batch runs one kernel for all its instances (two CTAs per SM when every
// instance takes a tile of 12 outputs per thread: 32 x 32 or 64 x 16).
enum GppTile {
  kTile32x32 = 0, kTile16x64 = 1, kTile64x16 = 2,
  kTileY64x32 = 3, kTileY32x64 = 4, kTileY32x32 = 5, kTileY64x16 = 6, kTileCount = 7
};
__host__ __device__ constexpr int tile_bn(int t) {
  return (t == kTile16x64) ? 16 : ((t == kTile64x16 || t == kTileY64x32 || t == kTileY64x16) ? 64 : 32);
}
__host__ __device__ constexpr int tile_bp(int t) {
  return (t == kTile16x64 || t == kTileY32x64) ? 64 : ((t == kTile64x16 || t == kTileY64x16) ? 16 : 32);
}
__host__ __device__ constexpr bool tile_shared(int t) { return t >= kTileY64x32; }

// One pass over every instance: items of instance i are the global items
// [item_off[i], item_off[i+1]) of a single device counter.
struct GppBatchView {
  const GppDev* dev;
  const GppWork* work;
  const MixedPrep* prep;
  const int* item_off;   // [n_inst + 1]
  const int* tile;       // [n_inst] GppTile (FP64 main pass)
  int n_inst;
  int total;
  int* counter;
};

// The instance that owns global item g: the last one whose offset is <= g.
__device__ __forceinline__ int batch_owner(const int* off, int n, int g) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= g) lo = mid; else hi = mid - 1;
  }
  return lo;
}

cudaError_t launch_sch_fp64_batch(const GppBatchView& b, int grid, cudaStream_t s);
cudaError_t launch_ssx_fp64_batch(const GppBatchView& b, int grid, cudaStream_t s);
cudaError_t launch_sch_mixed_batch(const GppBatchView& b, int grid, cudaStream_t s);
cudaError_t launch_ssx_mixed_batch(const GppBatchView& b, int grid, bool all_shared_wx, cudaStream_t s);
cudaError_t launch_sch_fp64y_batch(const GppBatchView& b, int grid, bool small, cudaStream_t s);
// Mixed main pass with one frequency set per instance: items of 2*kBN bands x
// 2*kBPM columns (the pre-pass must cover twice the items' block counts).
cudaError_t launch_sch_mixedy_batch(const GppBatchView& b, int grid, cudaStream_t s);
int sch_batch_blocks_per_sm_mixedy();
int sch_batch_blocks_per_sm_fp64();
int sch_batch_blocks_per_sm_fp64y(bool small);
int ssx_batch_blocks_per_sm_fp64();
int sch_batch_blocks_per_sm_mixed();
int ssx_batch_blocks_per_sm_mixed();

}  // namespace sigma
