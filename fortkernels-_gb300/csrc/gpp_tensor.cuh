// Tensor-core GPP form (SIGMA_PREC_TENSOR): the factor pass and the batched
// (grouped) contraction of many instances.
#pragma once

#include "sigma_internal.cuh"
#include "ff_ozaki.cuh"

namespace sigma {

constexpr int kFacCols = 16;        // columns (my_igp) per factor tile
constexpr int kFacK = 32;           // g-vectors per factor tile (one K tile of the contraction)
constexpr int kFusedBands = 8;      // occupied bands whose ssx sums the factor pass takes

// One instance of the factor pass.  Items are (g-vector segment, column
// block); an item writes the contraction's A slices of its tiles and, for
// the occupied bands, the ssx partial sums of its columns over its
// g-vectors into ssx.partial in the reduction's layout (band block, column
// block, segment).  Each item also writes its share of the contraction's
// other operands (B slices of aqsn, epilogue factors of aqsm): memory-bound
// work spread through the compute-bound pass instead of two launches.
struct FactorJob {
  GppDev p;
  unsigned char* a_tiles;  // OzakiPrep::a_tiles of the instance's contraction
  int kt;                  // K tiles per real / imaginary half
  int ncb;                 // column blocks of kFacCols columns
  int n_seg, seg_tiles;    // g-vector segments per column block, K tiles per segment
  int item_off;            // first global item of the job
  GppWork ssx;             // ssx partial layout (bn kSsxBN, n_col_blocks ncb, n_splits n_seg)
  FfDev d;                 // the contraction's operands (aqsn, aqsm, column weight)
  OzakiPrep oz;            // its slice images and epilogue factor table
  long long b_per_item, w_per_item;  // B-slice / epilogue-factor elements per main item
};

// Sizes the factor items of one instance whose share of a launch over
// `grid` CTAs is `share` (its fraction of the launch's (column, g-vector)
// elements; about 12 items per CTA over the launch) and fills the ssx work
// layout (partial pointer and item_off left to the caller).
void factor_job_size(FactorJob& j, const GppDev& p, int kt, int grid, double share);
// The contraction's operands of the job (B slices, epilogue factors) as the
// items' shares; d and oz of the instance's contraction plan.
void factor_job_operands(FactorJob& j, const FfDev& d, const OzakiPrep& oz);
size_t factor_ssx_partial_bytes(const FactorJob& j);
// Items of the job: the (segment, column block) items and those that zero
// the padding rows of the last row block.
int factor_job_items(const FactorJob& j);
// resident blocks per SM for a launch whose instances have at most
// max_nvband occupied bands (its shared memory grows with them)
int factor_blocks_per_sm(int max_nvband);
// Whether the fused pass covers the occupied bands of this instance.
inline bool factor_fuses_ssx(int nvband) { return nvband <= kFusedBands; }

// The factor pass over jobs[0 .. n_jobs) (device array; job i's items are
// [item_off, item_off + factor_job_items)), `total` items in all.
cudaError_t launch_factor_pass(const FactorJob* jobs, int n_jobs, int total, int grid, int max_nvband,
                               cudaStream_t s);
// One instance, the job passed by value (item_off 0).
cudaError_t launch_factor_pass(const FactorJob& job, int grid, cudaStream_t s);

}  // namespace sigma
