// Deterministic cross-block reduction of the GPP partial sums.
//
// The reference sums per-thread partial arrays after its band loop
// (BGW-Kernels/gppKer.cpp:431-439) in an order that changes with OpenMP's
// dynamic schedule.  Here every partial has a fixed slot, and the sums run in
// a fixed order with Neumaier-compensated FP64 accumulation: one block per
// (band, frequency) sums the column blocks and g-vector splits (each thread
// a fixed strided subset, then a fixed butterfly per warp and the warps in
// order), then one warp per frequency sums the bands.  Results are
// identical run to run.
#include "sigma_internal.cuh"

namespace sigma {
namespace {


constexpr int kRowThreads = 256;

// Row `row` of the band-sum stage (one block).
__device__ __forceinline__ void reduce_bands_row(const ReduceArgs& a, int row) {
  __shared__ double s_x[kRowThreads / 32], s_y[kRowThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int n_sch = a.sch_rows * kNW;
  const bool is_sch = row < n_sch;
  const int e = is_sch ? row : row - n_sch;
  const int n1 = e / kNW, iw = e % kNW;
  const int bn = is_sch ? a.sch_bn : kSsxBN;
  const int ncb = is_sch ? a.sch_ncb : a.ssx_ncb;
  const int ns = is_sch ? a.sch_splits : a.ssx_splits;
  const double2* part = is_sch ? a.sch_partial : a.ssx_partial;
  const int bb = n1 / bn, bl = n1 % bn;
  Comp sx, sy;
  const int count = ncb * ns;
  for (int q = threadIdx.x; q < count; q += kRowThreads) {
    const size_t item = (size_t)bb * count + q;  // (bb * ncb + cb) * ns + s
    const double2 v = part[item * bn * kNW + bl * kNW + iw];
    sx.add(v.x);
    sy.add(v.y);
  }
  const double rx = warp_sum_comp(sx), ry = warp_sum_comp(sy);
  if (lane == 0) {
    s_x[warp] = rx;
    s_y[warp] = ry;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    Comp tx, ty;
    for (int w = 0; w < kRowThreads / 32; ++w) {
      tx.add(s_x[w]);
      ty.add(s_y[w]);
    }
    if (is_sch)
      a.acht_n1[e] = make_double2(tx.value(), ty.value());
    else
      a.asx_n1[e] = make_double2(tx.value(), ty.value());
  }
}

__global__ void __launch_bounds__(kRowThreads) reduce_bands_kernel(ReduceArgs a) {
  reduce_bands_row(a, blockIdx.x);
}

__device__ __forceinline__ void reduce_total_block(const double2* acht_n1, const double2* asx_n1, int nb,
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

__global__ void reduce_total_kernel(const double2* acht_n1, const double2* asx_n1, int nb,
                                    int nvband, double2* achtemp, double2* asxtemp,
                                    double2* acht_n1_loc) {
  reduce_total_block(acht_n1, asx_n1, nb, nvband, achtemp, asxtemp, acht_n1_loc);
}

// Group forms over many instances: blocks row_off .. + (sch_rows + nvband) * 3
// of each job, then one block per job.
__global__ void __launch_bounds__(kRowThreads) reduce_bands_group_kernel(const ReduceJob* jobs, int n) {
  const int row = blockIdx.x;
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].row_off <= row) lo = mid; else hi = mid - 1;
  }
  reduce_bands_row(jobs[lo].a, row - jobs[lo].row_off);
}

__global__ void reduce_total_group_kernel(const ReduceJob* jobs) {
  const ReduceJob& j = jobs[blockIdx.x];
  reduce_total_block(j.a.acht_n1, j.a.asx_n1, j.a.nb, j.a.nvband, j.achtemp, j.asxtemp, j.acht_n1_loc);
}

}  // namespace

ReduceJob gpp_reduce_job(const GppWork& sch, const GppWork& ssx, int nb, double2* acht_n1, double2* achtemp,
                         double2* asxtemp, double2* acht_n1_loc, int row_off) {
  ReduceJob j{};
  ReduceArgs& a = j.a;
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
  j.achtemp = achtemp;
  j.asxtemp = asxtemp;
  j.acht_n1_loc = acht_n1_loc;
  j.row_off = row_off;
  return j;
}

int gpp_reduce_job_rows(const ReduceJob& j) { return (j.a.sch_rows + j.a.nvband) * kNW; }

cudaError_t launch_gpp_reduce_group(const ReduceJob* jobs, int n, int total_rows, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (total_rows > 0) {
    reduce_bands_group_kernel<<<total_rows, kRowThreads, 0, s>>>(jobs, n);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  reduce_total_group_kernel<<<n, 256, 0, s>>>(jobs);
  return cudaGetLastError();
}

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
  const int rows = (a.sch_rows + a.nvband) * kNW;
  if (rows > 0) {
    reduce_bands_kernel<<<rows, kRowThreads, 0, s>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  reduce_total_kernel<<<1, 256, 0, s>>>(acht_n1, a.asx_n1, nb, a.nvband, achtemp, asxtemp,
                                        acht_n1_loc);
  return cudaGetLastError();
}

}  // namespace sigma
