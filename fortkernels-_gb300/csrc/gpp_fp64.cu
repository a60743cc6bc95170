// GPP sigma sum, plain FP64 path (sm_103a).
//
// Replaces the band / column / g-vector / frequency loop nest of
// BGW-Kernels/gppKer.cpp:303-439.  Work is cut into items (32 bands x 32
// columns x one g-vector split); a persistent grid takes items from a device
// counter, stages the columns' wtilde / I_eps and the bands' aqsn through
// shared memory with coalesced 16-byte loads, and every thread evaluates a
// 2 x 2 (band x column) register tile over the three frequencies.
//
// GB300 runs FP64 at 1/64 of its FP32 rate, so the term is rewritten to
// spend as few FP64 pipe instructions as possible (8 per term plus 6 per
// band/column/g-vector shared by the three frequencies; the reciprocal is an
// FP32 hardware seed refined by one FP64 Newton step, rcp_f64_seed32):
//   scha / conj(aqsm[n1][igp]) = aqsn * I_eps * wtilde * conj(wdiff) / |wdiff|^2
//                              = R * (c + i b) * r,   R = aqsn * (I_eps * wtilde),
//   c = wx - Re wtilde, b = Im wtilde, r = 1 / (c^2 + b^2).
// conj(aqsm[n1][igp]), 0.5 and vcoul[igp] are applied once per column after
// the g-vector sum.  The pole guard is a compare against a per-(column,
// g-vector) threshold on the integer pipe and a select of r (exact poles give
// r = inf and are dropped by the select, never multiplied).
#include "sigma_internal.cuh"

namespace sigma {
namespace {

constexpr int kPad = 1;
constexpr int kTN = 2, kTP = 2;  // register tile: bands x columns per thread

struct SchSmem {
  double a[kCK][kBP + kPad];
  double b[kCK][kBP + kPad];
  double b2[kCK][kBP + kPad];
  double thr[kCK][kBP + kPad];
  double2 g[kCK][kBP + kPad];
  double2 n[kCK][kBN + kPad];
};
static_assert(sizeof(double2) * kBN * kNW * kBP <= sizeof(SchSmem), "epilogue reuses staging memory");
static_assert(sizeof(SchSmem) <= 100 * 1024, "two CTAs per SM");

__device__ __forceinline__ double2 cmul(double2 x, double2 y) {
  return make_double2(fma(x.x, y.x, -__dmul_rn(x.y, y.y)), fma(x.x, y.y, __dmul_rn(x.y, y.x)));
}

__global__ void __launch_bounds__(kThreads, 2) sch_fp64_kernel(GppDev p, GppWork w) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SchSmem& sm = *reinterpret_cast<SchSmem*>(smem_raw);
  __shared__ int s_item;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int band_end = w.band_begin + w.band_count;

  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(w.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= w.n_items) break;
    const ItemCoord ic = decode_item(w, item);
    const int split = ic.s, cb = ic.cb, bb = ic.bb;
    const int n1_0 = w.band_begin + bb * kBN;
    const int p0 = cb * kBP;
    const int ig_begin = split * w.split_len;
    const int ig_end = min(ig_begin + w.split_len, p.nc);

    double wxr[kTN][kNW];
#pragma unroll
    for (int i = 0; i < kTN; ++i) {
      const int n1 = n1_0 + ty + 16 * i;
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw)
        wxr[i][iw] = n1 < band_end ? p.wx[(size_t)n1 * p.wx_stride + iw] : 0.0;
    }
    double2 acc[kTN][kTP][kNW];
#pragma unroll
    for (int i = 0; i < kTN; ++i)
#pragma unroll
      for (int j = 0; j < kTP; ++j)
#pragma unroll
        for (int iw = 0; iw < kNW; ++iw) acc[i][j][iw] = make_double2(0.0, 0.0);

    for (int ig0 = ig_begin; ig0 < ig_end; ig0 += kCK) {
      __syncthreads();
      for (int e = tid; e < kCK * kBP; e += kThreads) {
        const int k = e % kCK, pl = e / kCK;
        const int ig = ig0 + k, my_igp = p0 + pl;
        double a = 0.0, b = 0.0, b2 = 0.0, thr = __longlong_as_double(0x7ff0000000000000LL);
        double2 g = make_double2(0.0, 0.0);
        if (ig < ig_end && my_igp < p.ng) {
          const size_t off = (size_t)my_igp * p.nc + ig;
          const double2 wt = p.wt[off];
          const double2 ie = p.ieps[off];
          a = wt.x;
          b = wt.y;
          b2 = guard_b2(b);
          thr = guard_thr(a, b2);
          g = cmul(ie, wt);
        }
        sm.a[k][pl] = a;
        sm.b[k][pl] = b;
        sm.b2[k][pl] = b2;
        sm.thr[k][pl] = thr;
        sm.g[k][pl] = g;
      }
      for (int e = tid; e < kCK * kBN; e += kThreads) {
        const int k = e % kCK, bl = e / kCK;
        const int ig = ig0 + k, n1 = n1_0 + bl;
        double2 v = make_double2(0.0, 0.0);
        if (ig < ig_end && n1 < band_end) v = p.aqsn[(size_t)n1 * p.nc + ig];
        sm.n[k][bl] = v;
      }
      __syncthreads();

#pragma unroll 2
      for (int k = 0; k < kCK; ++k) {
        double a[kTP], b[kTP], b2[kTP], thr[kTP];
        double2 g[kTP], nn[kTN];
#pragma unroll
        for (int j = 0; j < kTP; ++j) {
          const int pl = tx + 16 * j;
          a[j] = sm.a[k][pl];
          b[j] = sm.b[k][pl];
          b2[j] = sm.b2[k][pl];
          thr[j] = sm.thr[k][pl];
          g[j] = sm.g[k][pl];
        }
#pragma unroll
        for (int i = 0; i < kTN; ++i) nn[i] = sm.n[k][ty + 16 * i];
#pragma unroll
        for (int i = 0; i < kTN; ++i)
#pragma unroll
          for (int j = 0; j < kTP; ++j) {
            const double2 R = cmul(nn[i], g[j]);
            const double bRre = __dmul_rn(b[j], R.x), bRim = __dmul_rn(b[j], R.y);
#pragma unroll
            for (int iw = 0; iw < kNW; ++iw) {
              const double c = __dsub_rn(wxr[i][iw], a[j]);
              const double wv = fma(c, c, b2[j]);
              double r = rcp_f64_seed32(wv);
              r = gt_nonneg(wv, thr[j]) ? r : 0.0;
              const double ure = fma(R.x, c, -bRim);
              const double uim = fma(R.y, c, bRre);
              acc[i][j][iw].x = fma(ure, r, acc[i][j][iw].x);
              acc[i][j][iw].y = fma(uim, r, acc[i][j][iw].y);
            }
          }
      }
    }

    // epilogue: x conj(aqsm[n1][igp]) * 0.5 * vcoul[igp], then a fixed-order
    // sum over the tile's columns
    __syncthreads();
    double2(*red)[kNW][kBP] = reinterpret_cast<double2(*)[kNW][kBP]>(smem_raw);
#pragma unroll
    for (int i = 0; i < kTN; ++i)
#pragma unroll
      for (int j = 0; j < kTP; ++j) {
        const int bl = ty + 16 * i, pl = tx + 16 * j;
        const int n1 = n1_0 + bl, my_igp = p0 + pl;
        const int igp = my_igp < p.ng ? p.igp_of[my_igp] : -1;
        if (n1 < band_end && igp >= 0) {
          const double2 am = p.aqsm[(size_t)n1 * p.nc + igp];
          const double2 m = make_double2(am.x, -am.y);
          const double f = 0.5 * p.vcoul[igp];
#pragma unroll
          for (int iw = 0; iw < kNW; ++iw) {
            const double2 v = cmul(acc[i][j][iw], m);
            red[bl][iw][pl] = make_double2(v.x * f, v.y * f);
          }
        } else {
#pragma unroll
          for (int iw = 0; iw < kNW; ++iw) red[bl][iw][pl] = make_double2(0.0, 0.0);
        }
      }
    __syncthreads();
    if (tid < kBN * kNW) {
      const int bl = tid / kNW, iw = tid % kNW;
      double sx = 0.0, sy = 0.0;
      for (int pl = 0; pl < kBP; ++pl) {
        sx += red[bl][iw][pl].x;
        sy += red[bl][iw][pl].y;
      }
      w.partial[ic.pidx * kBN * kNW + tid] = make_double2(sx, sy);
    }
  }
}

// ---------------------------------------------------------------- occupied bands
// Screened exchange of the occupied bands (ssxt_scht_solver branches,
// BGW-Kernels/gppKer.cpp:38-58):
//   kept term:                 ssx = Omega2 / wx^2,            Omega2 = wtilde^2 I_eps
//   dropped, |delw|^2 > to1:   ssx = -I_eps wtilde / (2 (wtilde + wx))
//                              (= -Omega2 conj(cden) delw / |cden|^2, cden = 4 wtilde^2 (delw + 1/2))
//   otherwise (incl. exact poles, where the reference's delw is NaN): 0
// and asxtemp[iw] += occ vcoul[igp] conj(aqsm[n1][igp]) sum_ig aqsn[n1][ig] ssx.
constexpr int kSsxBP = 256;    // columns per item, one per thread
constexpr int kSsxCK = 8;      // g-vectors per staged chunk

struct SsxSmem {
  double a[kSsxCK][kSsxBP];
  double b[kSsxCK][kSsxBP];
  double2 g[kSsxCK][kSsxBP];
  double2 om[kSsxCK][kSsxBP];
  double2 n[kSsxCK][kSsxBN];
};
static_assert(sizeof(SsxSmem) <= 200 * 1024, "shared memory budget");

__global__ void __launch_bounds__(kThreads) ssx_fp64_kernel(GppDev p, GppWork w) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SsxSmem& sm = *reinterpret_cast<SsxSmem*>(smem_raw);
  __shared__ int s_item;
  __shared__ double2 s_red[kSsxBN][kNW][kThreads / 32];
  __shared__ double s_wx[kSsxBN][kNW], s_iwx2[kSsxBN][kNW];
  const int tid = threadIdx.x;
  const int band_end = w.band_begin + w.band_count;

  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(w.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= w.n_items) break;
    const ItemCoord ic = decode_item(w, item);
    const int split = ic.s, cb = ic.cb, bb = ic.bb;
    const int n1_0 = w.band_begin + bb * kSsxBN;
    const int nbl = min(kSsxBN, band_end - n1_0);
    const int p0 = cb * kSsxBP;
    const int ig_begin = split * w.split_len;
    const int ig_end = min(ig_begin + w.split_len, p.nc);
    if (tid < kSsxBN * kNW) {
      const int i = tid / kNW, iw = tid % kNW;
      const double wx = i < nbl ? p.wx[(size_t)(n1_0 + i) * p.wx_stride + iw] : 1.0;
      s_wx[i][iw] = wx;
      s_iwx2[i][iw] = rcp_f64(wx * wx);
    }

    double2 acc[kSsxBN][kNW];
#pragma unroll
    for (int i = 0; i < kSsxBN; ++i)
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) acc[i][iw] = make_double2(0.0, 0.0);

    for (int ig0 = ig_begin; ig0 < ig_end; ig0 += kSsxCK) {
      __syncthreads();
      for (int e = tid; e < kSsxCK * kSsxBP; e += kThreads) {
        const int k = e % kSsxCK, pl = e / kSsxCK;
        const int ig = ig0 + k, my_igp = p0 + pl;
        double2 wt = make_double2(0.0, 0.0), ie = make_double2(0.0, 0.0);
        if (ig < ig_end && my_igp < p.ng) {
          const size_t off = (size_t)my_igp * p.nc + ig;
          wt = p.wt[off];
          ie = p.ieps[off];
        }
        sm.a[k][pl] = wt.x;
        sm.b[k][pl] = wt.y;
        sm.g[k][pl] = cmul(ie, wt);
        sm.om[k][pl] = cmul(cmul(wt, wt), ie);
      }
      for (int e = tid; e < kSsxCK * kSsxBN; e += kThreads) {
        const int k = e % kSsxCK, bl = e / kSsxCK;
        const int ig = ig0 + k, n1 = n1_0 + bl;
        double2 v = make_double2(0.0, 0.0);
        if (ig < ig_end && n1 < band_end) v = p.aqsn[(size_t)n1 * p.nc + ig];
        sm.n[k][bl] = v;
      }
      __syncthreads();

      for (int k = 0; k < kSsxCK; ++k) {
        const double a = sm.a[k][tid], b = sm.b[k][tid];
        const double2 g = sm.g[k][tid], om = sm.om[k][tid];
        const double b2 = guard_b2(b);
        const double thr = guard_thr(a, b2), thr2 = guard_thr2(a, b2);
#pragma unroll
        for (int i = 0; i < kSsxBN; ++i) {
          if (i < nbl) {
            const double2 an = sm.n[k][i];
#pragma unroll
            for (int iw = 0; iw < kNW; ++iw) {
              const double wx = s_wx[i][iw];
              const double wv = guard_w(wx, a, b2);
              const bool keep = gt_nonneg(wv, thr);
              const bool br2 = !keep && gt_nonneg(wv, 0.0) && gt_nonneg(thr2, wv);
              // branch 1: Omega2 / wx^2
              const double iwx2 = s_iwx2[i][iw];
              const double2 s1 = make_double2(om.x * iwx2, om.y * iwx2);
              // branch 2: -G conj(z) / (2 |z|^2), z = wtilde + wx
              const double zr = a + wx;
              const double q = -0.5 * rcp_f64(fma(zr, zr, b2));
              const double2 s2 =
                  make_double2(fma(g.x, zr, g.y * b) * q, fma(g.y, zr, -g.x * b) * q);
              const double2 s = keep ? s1 : (br2 ? s2 : make_double2(0.0, 0.0));
              acc[i][iw].x = fma(an.x, s.x, fma(-an.y, s.y, acc[i][iw].x));
              acc[i][iw].y = fma(an.x, s.y, fma(an.y, s.x, acc[i][iw].y));
            }
          }
        }
      }
    }

    // epilogue: x conj(aqsm[n1][igp]) * occ * vcoul[igp]; fixed-order sum over
    // the item's columns (warp shuffles, then warps in order)
    const int my_igp = p0 + tid;
    const int igp = my_igp < p.ng ? p.igp_of[my_igp] : -1;
    const int lane = tid & 31, warp = tid >> 5;
    for (int i = 0; i < kSsxBN; ++i)
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) {
        double2 v = make_double2(0.0, 0.0);
        if (i < nbl && igp >= 0) {
          const double2 am = p.aqsm[(size_t)(n1_0 + i) * p.nc + igp];
          const double f = p.occ * p.vcoul[igp];
          v = cmul(acc[i][iw], make_double2(am.x, -am.y));
          v.x *= f;
          v.y *= f;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
          v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
        }
        if (lane == 0) s_red[i][iw][warp] = v;
      }
    __syncthreads();
    if (tid < kSsxBN * kNW) {
      const int i = tid / kNW, iw = tid % kNW;
      double sx = 0.0, sy = 0.0;
      for (int q = 0; q < kThreads / 32; ++q) {
        sx += s_red[i][iw][q].x;
        sy += s_red[i][iw][q].y;
      }
      w.partial[ic.pidx * kSsxBN * kNW + tid] = make_double2(sx, sy);
    }
  }
}

}  // namespace

int sch_blocks_per_sm_fp64() {
  int n = 0;
  cudaFuncSetAttribute(sch_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(SchSmem));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sch_fp64_kernel, kThreads, sizeof(SchSmem));
  return n > 0 ? n : 1;
}

int ssx_blocks_per_sm_fp64() {
  int n = 0;
  cudaFuncSetAttribute(ssx_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(SsxSmem));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ssx_fp64_kernel, kThreads, sizeof(SsxSmem));
  return n > 0 ? n : 1;
}

cudaError_t launch_sch_fp64(const GppDev& p, const GppWork& w, int grid, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(sch_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       sizeof(SchSmem));
  if (e != cudaSuccess) return e;
  sch_fp64_kernel<<<grid, kThreads, sizeof(SchSmem), s>>>(p, w);
  return cudaGetLastError();
}

cudaError_t launch_ssx_fp64(const GppDev& p, const GppWork& w, int grid, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(ssx_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       sizeof(SsxSmem));
  if (e != cudaSuccess) return e;
  ssx_fp64_kernel<<<grid, kThreads, sizeof(SsxSmem), s>>>(p, w);
  return cudaGetLastError();
}

}  // namespace sigma
