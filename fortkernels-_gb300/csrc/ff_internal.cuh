// Internal declarations of the FF schDt contraction.
#pragma once

#include "sigma_internal.cuh"

namespace sigma {

// Rows of the contraction are (ifreq, my_igp) pairs; each frequency's
// columns are padded to a multiple of kFfRows so that a row block never
// straddles two frequencies.  Work items are (row block, band block, K split).
constexpr int kFfRows = 64;    // complex rows (my_igp of one frequency) per tile
constexpr int kFfCols = 64;    // complex columns (bands) per tile

struct FfDev {
  int nb, nc, ng, nf;
  int ngp;                 // padded columns per frequency
  const double2* epsr;     // [nf][ng][nc]
  const double2* aqsn;     // [nb][nc]
  const double2* aqsm;     // [nb][nc]
  const int* igp_of;       // [ng]; -1 marks a column left out of the sum
  // Optional column weight: the epilogue multiplies tempz by
  // vfac * vcoul[igp] * conj(aqsm[n1][igp]) when vcoul is set (static
  // remainders), by conj(aqsm[n1][igp]) alone otherwise (schDt).
  const double* vcoul;
  double vfac;
  // Optional FP32 operand [nf][ng][nc] used instead of epsr (the tensor-core
  // form rounds its operand to FP32 before slicing it)
  const float2* epsr32 = nullptr;
  // Optional second output of the split-BF16 form: the same sum with the
  // extra column factor vfac2 * vcoul2[igp]
  const double* vcoul2 = nullptr;
  double vfac2 = 1.0;
};

// Column weight of the contraction epilogue (0 for a column left out).
__device__ __forceinline__ double ff_column_weight(const FfDev& p, int igp) {
  if (igp < 0) return 0.0;
  return p.vcoul ? p.vfac * p.vcoul[igp] : 1.0;
}

struct FfWork {
  int n_row_blocks;        // nf * ngp / kFfRows
  int n_col_blocks;        // ceil(nb / kFfCols)
  int n_splits, split_len; // K splits (split_len a multiple of the K tile)
  int n_items;
  int* counter;
  double2* partial;        // [row block][col block][split][kFfCols]
  int* status;
};

// item -> (row block, band block, split); band blocks vary fastest so that
// resident CTAs share the big I_epsR operand through L2.
struct FfItem {
  int rb, cb, s;
  size_t pidx;
};
__device__ __forceinline__ FfItem ff_decode(const FfWork& w, int item) {
  FfItem t;
  t.cb = item % w.n_col_blocks;
  const int r = item / w.n_col_blocks;
  t.s = r % w.n_splits;
  t.rb = r / w.n_splits;
  t.pidx = ((size_t)t.rb * w.n_col_blocks + t.cb) * w.n_splits + t.s;
  return t;
}

cudaError_t launch_ff_fp64(const FfDev& p, const FfWork& w, int grid, cudaStream_t s);
int ff_fp64_blocks_per_sm();
cudaError_t launch_ff_reduce(const FfDev& p, const FfWork& w, double2* schdt, cudaStream_t s);

}  // namespace sigma
