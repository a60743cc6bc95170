// GPP sigma sum, mixed-precision path (sm_103a).
//
// Same work decomposition and term algebra as the FP64 path (gpp_fp64.cu),
// with the bulk arithmetic in FP32:
//   * wtilde's real part is staged as an FP32 (hi, lo) pair and wx likewise,
//     so c = wx - Re wtilde = (wx_hi - a_hi) + (wx_lo - a_lo) keeps ~2^-24
//     relative accuracy even when wx and Re wtilde nearly cancel;
//   * 1/|wdiff|^2 is the FP32 hardware reciprocal refined by one
//     Newton-Raphson step;
//   * each thread sums 16 g-vectors in FP32, then folds that run into a
//     float-float (TwoSum) accumulator; partials leave the tile in FP64 and
//     are reduced with compensated FP64 sums (gpp_reduce.cu).
// The pole guard must take exactly the FP64 path's decision: a term whose
// FP32 |wdiff|^2 lands within 2^-19 (relative) of its threshold is re-decided
// from the FP64 inputs with the FP64 path's own expressions (guard_w /
// guard_thr).  Such terms are rare (~1e-6 of them on the production value
// ranges), so the re-check runs in a warp-uniform fix-up after each
// g-vector step.
#include "sigma_internal.cuh"

namespace sigma {
namespace {

constexpr int kPad = 1;
constexpr int kTN = 2, kTP = 2;
constexpr int kRun = 16;  // g-vectors summed in FP32 before the float-float fold

struct __align__(16) ColF {
  float ahi, alo, b, b2;
  float tlo, thi, gx, gy;
};

struct SchSmemF {
  ColF col[kCK][kBP + kPad];
  float2 n[kCK][kBN + kPad];
};
constexpr size_t kSchSmemBytes =
    sizeof(SchSmemF) > sizeof(double2) * kBN * kNW * kBP ? sizeof(SchSmemF)
                                                         : sizeof(double2) * kBN * kNW * kBP;

__device__ __forceinline__ double2 cmul(double2 x, double2 y) {
  return make_double2(fma(x.x, y.x, -__dmul_rn(x.y, y.y)), fma(x.x, y.y, __dmul_rn(x.y, y.x)));
}
__device__ __forceinline__ float2 cmulf(float2 x, float2 y) {
  return make_float2(fmaf(x.x, y.x, -x.y * y.y), fmaf(x.x, y.y, x.y * y.x));
}

__device__ __forceinline__ void split_f(double v, float& hi, float& lo) {
  hi = __double2float_rn(v);
  lo = __double2float_rn(v - (double)hi);
}

// Exact FP64 keep/drop decision of term (column my_igp, g-vector ig, frequency wx).
__device__ __noinline__ bool keep_exact(const GppDev& p, int my_igp, int ig, double wx) {
  const double2 wt = p.wt[(size_t)my_igp * p.nc + ig];
  const double b2 = guard_b2(wt.y);
  return gt_nonneg(guard_w(wx, wt.x, b2), guard_thr(wt.x, b2));
}

__global__ void __launch_bounds__(kThreads, 2) sch_mixed_kernel(GppDev p, GppWork w) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SchSmemF& sm = *reinterpret_cast<SchSmemF*>(smem_raw);
  __shared__ int s_item;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int band_end = w.band_begin + w.band_count;
  const float band_lo = 1.0f - kGuardBand, band_hi = 1.0f + kGuardBand;

  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(w.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= w.n_items) break;
    const int split = item % w.n_splits;
    const int cb = (item / w.n_splits) % w.n_col_blocks;
    const int bb = item / (w.n_splits * w.n_col_blocks);
    const int n1_0 = w.band_begin + bb * kBN;
    const int p0 = cb * kBP;
    const int ig_begin = split * w.split_len;
    const int ig_end = min(ig_begin + w.split_len, p.nc);

    float wxh[kTN][kNW], wxl[kTN][kNW];
#pragma unroll
    for (int i = 0; i < kTN; ++i) {
      const int n1 = n1_0 + ty + 16 * i;
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) {
        const double wx = n1 < band_end ? p.wx[(size_t)n1 * p.wx_stride + iw] : 0.0;
        split_f(wx, wxh[i][iw], wxl[i][iw]);
      }
    }
    float2 acc[kTN][kTP][kNW];
    float2 hi[kTN][kTP][kNW], lo[kTN][kTP][kNW];
#pragma unroll
    for (int i = 0; i < kTN; ++i)
#pragma unroll
      for (int j = 0; j < kTP; ++j)
#pragma unroll
        for (int iw = 0; iw < kNW; ++iw) {
          acc[i][j][iw] = make_float2(0.f, 0.f);
          hi[i][j][iw] = make_float2(0.f, 0.f);
          lo[i][j][iw] = make_float2(0.f, 0.f);
        }

    for (int ig0 = ig_begin; ig0 < ig_end; ig0 += kCK) {
      __syncthreads();
      for (int e = tid; e < kCK * kBP; e += kThreads) {
        const int k = e % kCK, pl = e / kCK;
        const int ig = ig0 + k, my_igp = p0 + pl;
        ColF c;
        c.ahi = c.alo = c.b = c.b2 = c.gx = c.gy = 0.f;
        c.tlo = c.thi = __int_as_float(0x7f800000);
        if (ig < ig_end && my_igp < p.ng) {
          const size_t off = (size_t)my_igp * p.nc + ig;
          const double2 wt = p.wt[off];
          const double2 ie = p.ieps[off];
          const double b2 = guard_b2(wt.y);
          const float thr = __double2float_rn(guard_thr(wt.x, b2));
          split_f(wt.x, c.ahi, c.alo);
          c.b = __double2float_rn(wt.y);
          c.b2 = __double2float_rn(b2);
          c.tlo = thr * band_lo;
          c.thi = thr * band_hi;
          const double2 g = cmul(ie, wt);
          c.gx = __double2float_rn(g.x);
          c.gy = __double2float_rn(g.y);
        }
        sm.col[k][pl] = c;
      }
      for (int e = tid; e < kCK * kBN; e += kThreads) {
        const int k = e % kCK, bl = e / kCK;
        const int ig = ig0 + k, n1 = n1_0 + bl;
        float2 v = make_float2(0.f, 0.f);
        if (ig < ig_end && n1 < band_end) {
          const double2 d = p.aqsn[(size_t)n1 * p.nc + ig];
          v = make_float2(__double2float_rn(d.x), __double2float_rn(d.y));
        }
        sm.n[k][bl] = v;
      }
      __syncthreads();

#pragma unroll 1
      for (int kr = 0; kr < kCK; kr += kRun) {
#pragma unroll 4
        for (int k = kr; k < kr + kRun; ++k) {
          ColF col[kTP];
          float2 nn[kTN];
#pragma unroll
          for (int j = 0; j < kTP; ++j) col[j] = sm.col[k][tx + 16 * j];
#pragma unroll
          for (int i = 0; i < kTN; ++i) nn[i] = sm.n[k][ty + 16 * i];
          bool unc = false;
#pragma unroll
          for (int i = 0; i < kTN; ++i)
#pragma unroll
            for (int j = 0; j < kTP; ++j) {
              const float2 R = cmulf(nn[i], make_float2(col[j].gx, col[j].gy));
              const float bRre = col[j].b * R.x, bRim = col[j].b * R.y;
#pragma unroll
              for (int iw = 0; iw < kNW; ++iw) {
                const float c = (wxh[i][iw] - col[j].ahi) + (wxl[i][iw] - col[j].alo);
                const float wv = fmaf(c, c, col[j].b2);
                const float r = rcp_f32(wv);
                const bool keep = wv > col[j].thi;
                unc |= (wv > col[j].tlo) && !keep;
                const float rm = keep ? r : 0.f;
                const float ure = fmaf(R.x, c, -bRim);
                const float uim = fmaf(R.y, c, bRre);
                acc[i][j][iw].x = fmaf(ure, rm, acc[i][j][iw].x);
                acc[i][j][iw].y = fmaf(uim, rm, acc[i][j][iw].y);
              }
            }
          if (__any_sync(0xffffffffu, unc)) {
            // Terms near a threshold were dropped above; add back the ones the
            // FP64 decision keeps.
#pragma unroll
            for (int i = 0; i < kTN; ++i)
#pragma unroll
              for (int j = 0; j < kTP; ++j) {
                const int n1 = n1_0 + ty + 16 * i, my_igp = p0 + tx + 16 * j, ig = ig0 + k;
                const float2 R = cmulf(nn[i], make_float2(col[j].gx, col[j].gy));
                const float bRre = col[j].b * R.x, bRim = col[j].b * R.y;
#pragma unroll
                for (int iw = 0; iw < kNW; ++iw) {
                  const float c = (wxh[i][iw] - col[j].ahi) + (wxl[i][iw] - col[j].alo);
                  const float wv = fmaf(c, c, col[j].b2);
                  if (wv > col[j].tlo && !(wv > col[j].thi) && n1 < band_end &&
                      my_igp < p.ng && ig < ig_end &&
                      keep_exact(p, my_igp, ig, p.wx[(size_t)n1 * p.wx_stride + iw])) {
                    const float r = rcp_f32(wv);
                    acc[i][j][iw].x = fmaf(fmaf(R.x, c, -bRim), r, acc[i][j][iw].x);
                    acc[i][j][iw].y = fmaf(fmaf(R.y, c, bRre), r, acc[i][j][iw].y);
                  }
                }
              }
          }
        }
        // fold the FP32 run into the float-float accumulators
#pragma unroll
        for (int i = 0; i < kTN; ++i)
#pragma unroll
          for (int j = 0; j < kTP; ++j)
#pragma unroll
            for (int iw = 0; iw < kNW; ++iw) {
              float s, e;
              two_sum_f(hi[i][j][iw].x, acc[i][j][iw].x, s, e);
              hi[i][j][iw].x = s;
              lo[i][j][iw].x += e;
              two_sum_f(hi[i][j][iw].y, acc[i][j][iw].y, s, e);
              hi[i][j][iw].y = s;
              lo[i][j][iw].y += e;
              acc[i][j][iw] = make_float2(0.f, 0.f);
            }
      }
    }

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
            const double2 s = make_double2((double)hi[i][j][iw].x + (double)lo[i][j][iw].x,
                                           (double)hi[i][j][iw].y + (double)lo[i][j][iw].y);
            const double2 v = cmul(s, m);
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
      Comp sx, sy;
      for (int pl = 0; pl < kBP; ++pl) {
        sx.add(red[bl][iw][pl].x);
        sy.add(red[bl][iw][pl].y);
      }
      w.partial[(size_t)item * kBN * kNW + tid] = make_double2(sx.value(), sy.value());
    }
  }
}

// ---------------------------------------------------------------- occupied bands
// FP32 form of ssx_fp64_kernel.  The three branch decisions (keep, the
// |delw|^2 > to1 test, and the exact-pole test |wdiff|^2 > 0) fall back to the
// FP64 expressions whenever FP32 |wdiff|^2 is near the corresponding threshold.
constexpr int kSsxBN = 8;
constexpr int kSsxBP = 256;

struct __align__(16) ColS {
  float ahi, alo, b, b2;
  float thr, thr2, gx, gy;
  float ox, oy, pad0, pad1;
};

struct SsxSmemF {
  ColS col[kCK][kSsxBP];
  float2 n[kCK][kSsxBN];
};

// FP64 branch of one occupied-band term: 0 dropped, 1 kept, 2 second branch.
__device__ __noinline__ int ssx_branch_exact(const GppDev& p, int my_igp, int ig, double wx) {
  const double2 wt = p.wt[(size_t)my_igp * p.nc + ig];
  const double b2 = guard_b2(wt.y);
  const double wv = guard_w(wx, wt.x, b2);
  if (gt_nonneg(wv, guard_thr(wt.x, b2))) return 1;
  if (gt_nonneg(wv, 0.0) && gt_nonneg(guard_thr2(wt.x, b2), wv)) return 2;
  return 0;
}

__global__ void __launch_bounds__(kThreads) ssx_mixed_kernel(GppDev p, GppWork w) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SsxSmemF& sm = *reinterpret_cast<SsxSmemF*>(smem_raw);
  __shared__ int s_item;
  __shared__ double2 s_red[kSsxBN][kNW][kThreads / 32];
  __shared__ float s_wxh[kSsxBN][kNW], s_wxl[kSsxBN][kNW], s_iwx2[kSsxBN][kNW];
  __shared__ double s_wx[kSsxBN][kNW];
  const int tid = threadIdx.x;
  const int band_end = w.band_begin + w.band_count;
  const float blo = 1.0f - kGuardBand, bhi = 1.0f + kGuardBand;

  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(w.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= w.n_items) break;
    const int split = item % w.n_splits;
    const int cb = (item / w.n_splits) % w.n_col_blocks;
    const int bb = item / (w.n_splits * w.n_col_blocks);
    const int n1_0 = w.band_begin + bb * kSsxBN;
    const int nbl = min(kSsxBN, band_end - n1_0);
    const int p0 = cb * kSsxBP;
    const int ig_begin = split * w.split_len;
    const int ig_end = min(ig_begin + w.split_len, p.nc);
    if (tid < kSsxBN * kNW) {
      const int i = tid / kNW, iw = tid % kNW;
      const double wx = i < nbl ? p.wx[(size_t)(n1_0 + i) * p.wx_stride + iw] : 1.0;
      s_wx[i][iw] = wx;
      split_f(wx, s_wxh[i][iw], s_wxl[i][iw]);
      s_iwx2[i][iw] = __double2float_rn(rcp_f64(wx * wx));
    }

    float2 acc[kSsxBN][kNW];
#pragma unroll
    for (int i = 0; i < kSsxBN; ++i)
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) acc[i][iw] = make_float2(0.f, 0.f);
    double2 accd[kSsxBN][kNW];
#pragma unroll
    for (int i = 0; i < kSsxBN; ++i)
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) accd[i][iw] = make_double2(0.0, 0.0);

    for (int ig0 = ig_begin; ig0 < ig_end; ig0 += kCK) {
      __syncthreads();
      for (int e = tid; e < kCK * kSsxBP; e += kThreads) {
        const int k = e % kCK, pl = e / kCK;
        const int ig = ig0 + k, my_igp = p0 + pl;
        ColS c;
        c.ahi = c.alo = c.b = c.b2 = c.gx = c.gy = c.ox = c.oy = c.pad0 = c.pad1 = 0.f;
        c.thr = __int_as_float(0x7f800000);
        c.thr2 = 0.f;
        if (ig < ig_end && my_igp < p.ng) {
          const size_t off = (size_t)my_igp * p.nc + ig;
          const double2 wt = p.wt[off];
          const double2 ie = p.ieps[off];
          const double b2 = guard_b2(wt.y);
          split_f(wt.x, c.ahi, c.alo);
          c.b = __double2float_rn(wt.y);
          c.b2 = __double2float_rn(b2);
          c.thr = __double2float_rn(guard_thr(wt.x, b2));
          c.thr2 = __double2float_rn(guard_thr2(wt.x, b2));
          const double2 g = cmul(ie, wt), om = cmul(cmul(wt, wt), ie);
          c.gx = __double2float_rn(g.x);
          c.gy = __double2float_rn(g.y);
          c.ox = __double2float_rn(om.x);
          c.oy = __double2float_rn(om.y);
        }
        sm.col[k][pl] = c;
      }
      for (int e = tid; e < kCK * kSsxBN; e += kThreads) {
        const int k = e % kCK, bl = e / kCK;
        const int ig = ig0 + k, n1 = n1_0 + bl;
        float2 v = make_float2(0.f, 0.f);
        if (ig < ig_end && n1 < band_end) {
          const double2 d = p.aqsn[(size_t)n1 * p.nc + ig];
          v = make_float2(__double2float_rn(d.x), __double2float_rn(d.y));
        }
        sm.n[k][bl] = v;
      }
      __syncthreads();

      for (int k = 0; k < kCK; ++k) {
        const ColS col = sm.col[k][tid];
#pragma unroll
        for (int i = 0; i < kSsxBN; ++i) {
          if (i < nbl) {
            const float2 an = sm.n[k][i];
#pragma unroll
            for (int iw = 0; iw < kNW; ++iw) {
              const float c = (s_wxh[i][iw] - col.ahi) + (s_wxl[i][iw] - col.alo);
              const float wv = fmaf(c, c, col.b2);
              int br;
              const bool near = (wv > col.thr * blo && wv <= col.thr * bhi) ||
                                (wv >= col.thr2 * blo && wv < col.thr2 * bhi) ||
                                wv < 1e-30f;
              if (near) {
                br = (p0 + tid < p.ng && ig0 + k < ig_end)
                         ? ssx_branch_exact(p, p0 + tid, ig0 + k, s_wx[i][iw])
                         : 0;
              } else {
                br = wv > col.thr ? 1 : (wv < col.thr2 ? 2 : 0);
              }
              float2 s = make_float2(0.f, 0.f);
              if (br == 1) {
                s = make_float2(col.ox * s_iwx2[i][iw], col.oy * s_iwx2[i][iw]);
              } else if (br == 2) {
                const float zr = (s_wxh[i][iw] + col.ahi) + (s_wxl[i][iw] + col.alo);
                const float q = -0.5f * rcp_f32(fmaf(zr, zr, col.b2));
                s = make_float2(fmaf(col.gx, zr, col.gy * col.b) * q,
                                fmaf(col.gy, zr, -col.gx * col.b) * q);
              }
              acc[i][iw].x = fmaf(an.x, s.x, fmaf(-an.y, s.y, acc[i][iw].x));
              acc[i][iw].y = fmaf(an.x, s.y, fmaf(an.y, s.x, acc[i][iw].y));
            }
          }
        }
      }
      // fold the chunk's FP32 sums into FP64 (32 g-vectors per run)
#pragma unroll
      for (int i = 0; i < kSsxBN; ++i)
        if (i < nbl) {
#pragma unroll
          for (int iw = 0; iw < kNW; ++iw) {
            accd[i][iw].x += (double)acc[i][iw].x;
            accd[i][iw].y += (double)acc[i][iw].y;
            acc[i][iw] = make_float2(0.f, 0.f);
          }
        }
    }

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
          v = cmul(accd[i][iw], make_double2(am.x, -am.y));
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
      Comp sx, sy;
      for (int q = 0; q < kThreads / 32; ++q) {
        sx.add(s_red[i][iw][q].x);
        sy.add(s_red[i][iw][q].y);
      }
      w.partial[(size_t)item * kSsxBN * kNW + tid] = make_double2(sx.value(), sy.value());
    }
  }
}

}  // namespace

int sch_blocks_per_sm_mixed() {
  int n = 0;
  cudaFuncSetAttribute(sch_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSchSmemBytes);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sch_mixed_kernel, kThreads, kSchSmemBytes);
  return n > 0 ? n : 1;
}

int ssx_blocks_per_sm_mixed() {
  int n = 0;
  cudaFuncSetAttribute(ssx_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(SsxSmemF));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ssx_mixed_kernel, kThreads, sizeof(SsxSmemF));
  return n > 0 ? n : 1;
}

cudaError_t launch_sch_mixed(const GppDev& p, const GppWork& w, int grid, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(sch_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       kSchSmemBytes);
  if (e != cudaSuccess) return e;
  sch_mixed_kernel<<<grid, kThreads, kSchSmemBytes, s>>>(p, w);
  return cudaGetLastError();
}

cudaError_t launch_ssx_mixed(const GppDev& p, const GppWork& w, int grid, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(ssx_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       sizeof(SsxSmemF));
  if (e != cudaSuccess) return e;
  ssx_mixed_kernel<<<grid, kThreads, sizeof(SsxSmemF), s>>>(p, w);
  return cudaGetLastError();
}

}  // namespace sigma
