// Tensor-core form of the GPP main pass (precision SIGMA_PREC_TENSOR).
//
// With one frequency set for every band, a term factors as
//   scha = conj(aqsm[n1][igp]) * aqsn[n1][ig] * Y_iw[my_igp][ig],
//   Y_iw = I_eps wtilde conj(wdiff) / |wdiff|^2   (0 when the pole guard
//                                                  drops the term),
// so the band sum is the FF contraction with the three frequencies as
// "frequency slabs" and the column weight 0.5 vcoul[igp]:
//   acht_n1[n1][iw] = sum_my_igp 0.5 vcoul[igp] conj(aqsm[n1][igp])
//                       * sum_ig aqsn[n1][ig] Y_iw[my_igp][ig].
// This file forms Y in FP64 (guard decisions exactly as the FP64 path takes
// them); the contraction runs on the split-BF16 tcgen05 kernel of the FF
// path (ff_ozaki.cu), whose partial sums come back in FP64.
#include "sigma_internal.cuh"

namespace sigma {
namespace {

__global__ void __launch_bounds__(256) gpp_y_factor_kernel(GppDev p, double2* y) {
  const long long total = (long long)p.ng * p.nc;
  const double wx0 = p.wx[0], wx1 = p.wx[1], wx2 = p.wx[2];
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const double2 wt = p.wt[t];
    const double2 ie = p.ieps[t];
    const double2 g = make_double2(fma(ie.x, wt.x, -ie.y * wt.y), fma(ie.x, wt.y, ie.y * wt.x));
    const double b = wt.y, b2 = guard_b2(b);
    const double thr = guard_thr(wt.x, b2);
    auto factor = [&](double wx) {
      const double c = __dsub_rn(wx, wt.x);
      const double wv = fma(c, c, b2);
      const double r = gt_nonneg(wv, thr) ? rcp_f64_seed32(wv) : 0.0;
      const double zr = c * r, zi = b * r;
      return make_double2(fma(g.x, zr, -g.y * zi), fma(g.x, zi, g.y * zr));
    };
    y[t] = factor(wx0);
    y[total + t] = factor(wx1);
    y[2 * total + t] = factor(wx2);
  }
}

}  // namespace

cudaError_t launch_gpp_y_factor(const GppDev& p, double2* y, cudaStream_t s) {
  gpp_y_factor_kernel<<<152 * 8, 256, 0, s>>>(p, y);
  return cudaGetLastError();
}

}  // namespace sigma
