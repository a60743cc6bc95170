// Deterministic cross-block reduction of the GPP partial sums.
//
// The reference sums per-thread partial arrays after its band loop
// (BGW-Kernels/gppKer.cpp:431-439) in an order that changes with OpenMP's
// dynamic schedule.  Here every partial has a fixed slot, and the sums run in
// a fixed order with Neumaier-compensated FP64 accumulation: one warp per
// (band, frequency) sums the column blocks and g-vector splits, then one
// warp per frequency sums the bands.  Results are identical run to run.
#include "sigma_internal.cuh"

namespace sigma {
namespace {


struct ReduceArgs {
  int sch_rows;       // bands whose sums come from sch partials (0: acht_n1 already holds them)
  const double2* sch_partial;
  int sch_ncb, sch_splits, sch_bn;
  const double2* ssx_partial;
  int ssx_ncb, ssx_splits;
  int nb, nvband;
  double2* acht_n1;  // [nb][3]
  double2* asx_n1;   // [nvband][3]
};

__global__ void reduce_bands_kernel(ReduceArgs a) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int n_sch = a.sch_rows * kNW, n_ssx = a.nvband * kNW;
  if (warp >= n_sch + n_ssx) return;
  const bool is_sch = warp < n_sch;
  const int e = is_sch ? warp : warp - n_sch;
  const int n1 = e / kNW, iw = e % kNW;
  const int bn = is_sch ? a.sch_bn : kSsxBN;
  const int ncb = is_sch ? a.sch_ncb : a.ssx_ncb;
  const int ns = is_sch ? a.sch_splits : a.ssx_splits;
  const double2* part = is_sch ? a.sch_partial : a.ssx_partial;
  const int bb = n1 / bn, bl = n1 % bn;
  Comp sx, sy;
  const int count = ncb * ns;
  for (int q = lane; q < count; q += 32) {
    const size_t item = (size_t)bb * count + q;  // (bb * ncb + cb) * ns + s
    const double2 v = part[item * bn * kNW + bl * kNW + iw];
    sx.add(v.x);
    sy.add(v.y);
  }
  const double rx = warp_sum_comp(sx), ry = warp_sum_comp(sy);
  if (lane == 0) {
    if (is_sch)
      a.acht_n1[e] = make_double2(rx, ry);
    else
      a.asx_n1[e] = make_double2(rx, ry);
  }
}

__global__ void reduce_total_kernel(const double2* acht_n1, const double2* asx_n1, int nb,
                                    int nvband, double2* achtemp, double2* asxtemp,
                                    double2* acht_n1_loc) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp < 2 * kNW) {
    const bool ach = warp < kNW;
    const int iw = ach ? warp : warp - kNW;
    const double2* src = ach ? acht_n1 : asx_n1;
    const int n = ach ? nb : nvband;
    Comp sx, sy;
    for (int n1 = lane; n1 < n; n1 += 32) {
      const double2 v = src[n1 * kNW + iw];
      sx.add(v.x);
      sy.add(v.y);
    }
    const double rx = warp_sum_comp(sx), ry = warp_sum_comp(sy);
    if (lane == 0) (ach ? achtemp : asxtemp)[iw] = make_double2(rx, ry);
  }
  if (acht_n1_loc)
    for (int n1 = threadIdx.x; n1 < nb; n1 += blockDim.x) acht_n1_loc[n1] = acht_n1[n1 * kNW + 2];
}

}  // namespace

cudaError_t launch_gpp_reduce(const GppWork& sch, const GppWork& ssx, int nb, double2* acht_n1,
                              double2* achtemp, double2* asxtemp, double2* acht_n1_loc,
                              cudaStream_t s) {
  ReduceArgs a;
  a.sch_rows = sch.partial ? nb : 0;
  a.sch_partial = sch.partial;
  a.sch_ncb = sch.n_col_blocks;
  a.sch_splits = sch.n_splits;
  a.sch_bn = sch.bn;
  a.ssx_partial = ssx.partial;
  a.ssx_ncb = ssx.n_col_blocks;
  a.ssx_splits = ssx.n_splits;
  a.nb = nb;
  a.nvband = ssx.band_count;
  a.acht_n1 = acht_n1;
  a.asx_n1 = acht_n1 + (size_t)nb * kNW;
  const int warps = (a.sch_rows + a.nvband) * kNW;
  const int threads = 256;
  const int blocks = (warps * 32 + threads - 1) / threads;
  if (blocks > 0) {
    reduce_bands_kernel<<<blocks, threads, 0, s>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  reduce_total_kernel<<<1, 256, 0, s>>>(acht_n1, a.asx_n1, nb, a.nvband, achtemp, asxtemp,
                                        acht_n1_loc);
  return cudaGetLastError();
}

}  // namespace sigma
