// GPP sigma sum, mixed-precision path (sm_103a).
//
// Same term algebra as the FP64 path (gpp_fp64.cu), with the bulk arithmetic
// in FP32:
//   * a pre-pass turns each (column, g-vector) into FP32 operands once per
//     execution: Re wtilde as an FP32 (hi, lo) pair so that
//     c = wx - Re wtilde = (wx_hi - a_hi) + (wx_lo - a_lo) keeps ~2^-24
//     relative accuracy when wx and Re wtilde nearly cancel; Im wtilde;
//     G = I_eps * wtilde; and the pole-guard threshold.  aqsn is converted
//     too.  The layouts are tile-interleaved so that the main kernel stages a
//     chunk with three TMA bulk copies (cp.async.bulk) into a double-buffered
//     shared-memory ring, completion tracked by mbarriers;
//   * 1/|wdiff|^2 is the FP32 hardware reciprocal refined by one
//     Newton-Raphson step;
//   * each thread sums 8 g-vectors in FP32, then folds that run into a
//     float-float (TwoSum) accumulator; partials leave the tile in FP64 and
//     are reduced with compensated FP64 sums (gpp_reduce.cu).
// The pole guard must take exactly the FP64 path's decision: a term whose
// FP32 |wdiff|^2 lands within 2^-19 (relative) of its threshold is re-decided
// from the FP64 inputs with the FP64 path's own expressions (guard_w /
// guard_thr).  Such terms are rare (~1e-6 of them on the production value
// ranges), so the re-check runs in a warp-uniform fix-up after each
// g-vector step.
#include "sigma_internal.cuh"
#include "floatfloat.cuh"
#include "ff_ozaki.cuh"
#include "gpp_batch.cuh"

namespace sigma {
namespace {

constexpr int kTN = 2;    // bands per thread (one column per thread)
constexpr int kRun = 8;   // g-vectors summed in FP32 before the float-float fold
constexpr uint32_t kChunkBytes =
    kCK * kBPM * sizeof(float4) + kCK * kBPM * sizeof(float2) + kCK * kBN * sizeof(float2);

struct __align__(16) Stage {
  float4 a[kCK][kBPM];
  float2 b[kCK][kBPM];
  float2 n[kCK][kBN];
};
struct __align__(16) SchSmemM {
  Stage st[2];
  double2 red[kNW][kBPM][kBN];
  unsigned long long bar[2];
};
static_assert(sizeof(Stage) == kChunkBytes, "one chunk is one contiguous copy per operand");
static_assert(sizeof(SchSmemM) <= 72 * 1024, "three CTAs per SM");

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

// ---- TMA bulk copies and mbarriers (PTX ISA: cp.async.bulk, mbarrier)
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes,
                                          unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// Bounded waits (sigma_tma.cuh): mbar_wait gives up once the launch's status
// word is set or after its poll bound (recording SIGMA_ERR_TIMEOUT);
// mbar_wait_own waits for a copy this CTA issued itself, whatever the status.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, uint32_t parity, int* status) {
  return tma::mbar_wait(smem_u32(bar), parity, status);
}
__device__ __forceinline__ void mbar_wait_own(unsigned long long* bar, uint32_t parity) {
  tma::mbar_wait_own(smem_u32(bar), parity);
}

// After a failed wait at chunk c: the copies of chunk c (parity `pc` on
// bar[c & 1]) and, when issued, of chunk c + 1 (parity `pn` on the other
// barrier) may still be landing; the issuing thread waits for both before
// the CTA leaves, so no copy writes shared memory after it is released.
__device__ __forceinline__ void drain_chunks(unsigned long long* bar, int c, int n_chunks, uint32_t pc,
                                             uint32_t pn) {
  mbar_wait_own(&bar[c & 1], pc);
  if (c + 1 < n_chunks) mbar_wait_own(&bar[(c + 1) & 1], pn);
}

// Issues the three bulk copies of chunk (cb, bb, ig0) into stage `st`.
__device__ __forceinline__ void issue_chunk(const MixedPrep& m, int cb, int bb, int ig0, Stage& st,
                                            unsigned long long* bar) {
  mbar_expect_tx(bar, kChunkBytes);
  const size_t col_off = ((size_t)cb * m.nc_pad + ig0) * kBPM;
  const size_t band_off = ((size_t)bb * m.nc_pad + ig0) * kBN;
  bulk_load(&st.a[0][0], m.colA + col_off, sizeof(st.a), bar);
  bulk_load(&st.b[0][0], m.colB + col_off, sizeof(st.b), bar);
  bulk_load(&st.n[0][0], m.band + band_off, sizeof(st.n), bar);
}

// Exact FP64 keep/drop decision of term (column my_igp, g-vector ig, frequency wx).
__device__ __forceinline__ bool keep_exact(const GppDev& p, int my_igp, int ig, double wx) {
  const double2 wt = p.wt[(size_t)my_igp * p.nc + ig];
  const double b2 = guard_b2(wt.y);
  return keep_nonneg(guard_w(wx, wt.x, b2), guard_thr(wt.x, b2));
}

// ---- pre-pass: FP32 operands in tile-interleaved layouts
// With one frequency set for every band (wx_stride 0) the fourth operand
// is a bit mask of the terms kept for frequency iw (bit iw), decided exactly
// as the FP64 path decides; otherwise it is the FP32 threshold and the main
// kernel decides per term.
__global__ void __launch_bounds__(256) prep_cols_kernel(GppDev p, MixedPrep m, int n_col_blocks) {
  __shared__ float4 ta[32][kBPM + 1];
  __shared__ float2 tb[32][kBPM + 1];
  __shared__ float2 tc[32][kBPM + 1];
  const int tid = threadIdx.x;
  const bool shared_wx = p.wx_stride == 0;
  float wxh[kNW], wxl[kNW];
#pragma unroll
  for (int iw = 0; iw < kNW; ++iw) split_f(p.wx[iw], wxh[iw], wxl[iw]);
  const long long tiles = (long long)n_col_blocks * (m.nc_pad / 32);
  for (long long t = blockIdx.x; t < tiles; t += gridDim.x) {
    const int cb = (int)(t / (m.nc_pad / 32));
    const int ig0 = (int)(t % (m.nc_pad / 32)) * 32;
    __syncthreads();
    for (int e = tid; e < 32 * kBPM; e += 256) {
      const int pl = e / 32, k = e % 32;  // reads run along g-vectors
      const int my_igp = cb * kBPM + pl, ig = ig0 + k;
      float4 a = make_float4(0.f, 0.f, 0.f, __int_as_float(0x7f800000));
      float2 g = make_float2(0.f, 0.f), om = make_float2(0.f, 0.f);
      if (shared_wx) a.w = __uint_as_float(0u);  // padding: no term kept
      if (my_igp < p.ng && ig < p.nc) {
        const size_t off = (size_t)my_igp * p.nc + ig;
        const double2 wt = p.wt[off];
        const double2 ie = p.ieps[off];
        const double b2 = guard_b2(wt.y);
        split_f(wt.x, a.x, a.y);
        a.z = __double2float_rn(wt.y);
        const double thr = guard_thr(wt.x, b2);
        if (shared_wx) {
          // keep/drop of the three frequencies, decided once per (column,
          // g-vector): FP32 when clear of the threshold, FP64 otherwise.
          // With occupied bands, bits 3..5 also hold the second branch of
          // their ssx term (dropped, and |wdiff|^2 below |wtilde|^2 / to1),
          // decided the same way.
          const float t32 = __double2float_rn(thr);
          const double thr2 = p.nvband > 0 ? guard_thr2(wt.x, b2) : 0.0;
          const float t2_32 = __double2float_rn(thr2);
          const float bb = a.z * a.z;
          unsigned mask = 0u;
#pragma unroll
          for (int iw = 0; iw < kNW; ++iw) {
            const float c = (wxh[iw] - a.x) + (wxl[iw] - a.y);
            const float wv = fmaf(c, c, bb);
            bool keep;
            if (wv > t32 * (1.0f + kGuardBand))
              keep = true;
            else if (wv <= t32 * (1.0f - kGuardBand))
              keep = false;
            else
              keep = keep_nonneg(guard_w(p.wx[iw], wt.x, b2), thr);
            mask |= keep ? (1u << iw) : 0u;
            if (p.nvband > 0 && !keep) {
              bool second;
              if (wv > 1e-30f && wv < t2_32 * (1.0f - kGuardBand))
                second = true;
              else if (wv >= t2_32 * (1.0f + kGuardBand))
                second = false;
              else {
                const double w64 = guard_w(p.wx[iw], wt.x, b2);
                second = gt_nonneg(w64, 0.0) && gt_nonneg(thr2, w64);
              }
              mask |= second ? (8u << iw) : 0u;
            }
          }
          a.w = __uint_as_float(mask);
        } else {
          a.w = __double2float_rn(thr);
        }
        const double2 gg = cmul(ie, wt);
        g = make_float2(__double2float_rn(gg.x), __double2float_rn(gg.y));
        if (m.colC) {
          const double2 o2 = cmul(wt, gg);  // Omega2 = wtilde^2 I_eps
          om = make_float2(__double2float_rn(o2.x), __double2float_rn(o2.y));
        }
      }
      ta[k][pl] = a;
      tb[k][pl] = g;
      tc[k][pl] = om;
    }
    __syncthreads();
    for (int e = tid; e < 32 * kBPM; e += 256) {
      const int k = e / kBPM, pl = e % kBPM;  // writes run along columns
      const size_t o = ((size_t)cb * m.nc_pad + ig0 + k) * kBPM + pl;
      m.colA[o] = ta[k][pl];
      m.colB[o] = tb[k][pl];
      if (m.colC) m.colC[o] = tc[k][pl];
    }
  }
}

// Tensor form (precision SIGMA_PREC_TENSOR).  With one frequency set for
// every band a term factors as
//   scha = conj(aqsm[n1][igp]) * aqsn[n1][ig] * Y_iw[my_igp][ig],
// so the band sum is the FF contraction (ff_ozaki.cu) with the three
// frequencies as slabs and the column weight 0.5 vcoul[igp].  The contraction
// rounds its operand to FP32 before splitting it into BF16 slices, so this
// pass forms the factors
//   Y[iw][my_igp][ig] = G (c + i b) / (c^2 + b^2)   (0 when the guard drops it)
//                     = (wx G - |wtilde|^2 I_eps) / (c^2 + b^2)
// rounded to FP32, computed in float-float arithmetic (pairs of FP32 values,
// ~2^-44 relative) from exact splits of the FP64 inputs, on the FP32 pipe
// instead of GB300's 1/64-rate FP64 pipe, and writes them directly as the
// contraction's A slices (oz.a_tiles set).  Keep and second-branch decisions
// are taken in float-float and re-taken with the FP64 path's own expressions
// within 2^-30 of a threshold.  In the same pass (same inputs) it writes the
// pre-pass operands of the occupied-band kernel (colA with the exact keep
// and second-branch bits, colB = G, colC = Omega2) when m.colA is set; with
// no slices it writes those operands alone (the mixed form's pre-pass for
// one frequency set).  Tiles of kBPM columns x 32 g-vectors staged in shared
// memory, from which the operand and slice writes run.

__global__ void __launch_bounds__(256) tensor_factors_kernel(GppDev p, MixedPrep m, int n_col_blocks,
                                                             OzakiPrep oz) {
  __shared__ float4 ta[32][kBPM + 1];
  __shared__ float2 tb[32][kBPM + 1];
  __shared__ float2 tc[32][kBPM + 1];
  __shared__ float2 ty[kNW][kBPM][33];  // the tile's factors for the slice writes
  const bool slices = oz.a_tiles != nullptr;
  const int tid = threadIdx.x;
  FF wx[kNW];
#pragma unroll
  for (int iw = 0; iw < kNW; ++iw) wx[iw] = ff_of(p.wx[iw]);
  const bool ops = m.colA != nullptr;
  const FF quarter{0.25f, 0.f};
  const long long tiles = (long long)n_col_blocks * (m.nc_pad / 32);
  for (long long t = blockIdx.x; t < tiles; t += gridDim.x) {
    const int cb = (int)(t / (m.nc_pad / 32));
    const int ig0 = (int)(t % (m.nc_pad / 32)) * 32;
    __syncthreads();
#pragma unroll 2
    for (int e = tid; e < 32 * kBPM; e += 256) {
      const int pl = e / 32, k = e % 32;  // reads and factor writes run along g-vectors
      const int my_igp = cb * kBPM + pl, ig = ig0 + k;
      float4 av = make_float4(0.f, 0.f, 0.f, __uint_as_float(0u));
      float2 g32 = make_float2(0.f, 0.f), om = make_float2(0.f, 0.f);
      float2 yt[kNW] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
      if (my_igp < p.ng && ig < p.nc) {
        const size_t off = (size_t)my_igp * p.nc + ig;
        const double2 wt = p.wt[off];
        const double2 ie = p.ieps[off];
        const FF a = ff_of(wt.x), b = ff_of(wt.y), er = ff_of(ie.x), ei = ff_of(ie.y);
        const FF gx = ff_add(ff_mul(er, a), ff_neg(ff_mul(ei, b)));
        const FF gy = ff_add(ff_mul(er, b), ff_mul(ei, a));
        const FF b2 = ff_mul(b, b);
        const FF s2 = ff_add(ff_mul(a, a), b2);            // |wtilde|^2
        const FF s_big = ff_mul(s2, FF{1e6f, 0.f});        // |wtilde|^2 / to1 (1e6 exact)
        // G (c + i b) = wx G - G conj(wtilde) = wx G - |wtilde|^2 I_eps
        const FF sex = ff_mul(s2, er), sey = ff_mul(s2, ei);
        unsigned mask = 0u;
#pragma unroll
        for (int iw = 0; iw < kNW; ++iw) {
          const FF c = ff_add(wx[iw], ff_neg(a));
          const FF wv = ff_add(ff_mul(c, c), b2);
          // keep: |wdiff|^2 > max(0.25, |wtilde|^2 * 4e-6), i.e. both
          // wv > 0.25 and wv * 250000 > |wtilde|^2 (250000 exact in FP32)
          bool n1, n2;
          const bool k1 = ff_gt_fast(wv, quarter, n1);
          const bool k2 = ff_gt_fast(ff_mul(wv, FF{250000.f, 0.f}), s2, n2);
          bool keep = k1 && k2;
          if (n1 || n2) keep = keep_fp64(p.wx[iw], wt.x, wt.y);  // within 2^-30 of a threshold
          if (slices) {
            float2 yv = make_float2(0.f, 0.f);
            if (keep) {
              const FF r = ff_rcp(wv);
              yv = make_float2(ff_mul_round(ff_add(ff_mul(wx[iw], gx), ff_neg(sex)), r),
                               ff_mul_round(ff_add(ff_mul(wx[iw], gy), ff_neg(sey)), r));
            }
            yt[iw] = yv;
          }
          mask |= keep ? (1u << iw) : 0u;
          if (ops && p.nvband > 0 && !keep) {
            // second branch: 0 < |wdiff|^2 < |wtilde|^2 / to1
            bool n3;
            bool second = wv.hi > 0.f && ff_gt_fast(s_big, wv, n3);
            if (n3 || wv.hi < 1e-30f) second = second_fp64(p.wx[iw], wt.x, wt.y);
            mask |= second ? (8u << iw) : 0u;
          }
        }
        if (ops) {
          av = make_float4(a.hi, a.lo, ff_round(b), __uint_as_float(mask));
          g32 = make_float2(ff_round(gx), ff_round(gy));
          if (m.colC) {  // Omega2 = wtilde G
            om = make_float2(ff_round(ff_add(ff_mul(a, gx), ff_neg(ff_mul(b, gy)))),
                             ff_round(ff_add(ff_mul(a, gy), ff_mul(b, gx))));
          }
        }
      }
      ta[k][pl] = av;
      tb[k][pl] = g32;
      tc[k][pl] = om;
      if (slices) {
#pragma unroll
        for (int iw = 0; iw < kNW; ++iw) ty[iw][pl][k] = yt[iw];
      }
    }
    if (!ops && !slices) continue;
    __syncthreads();
    if (ops) {
      for (int e = tid; e < 32 * kBPM; e += 256) {
        const int k = e / kBPM, pl = e % kBPM;  // operand writes run along columns
        const size_t o = ((size_t)cb * m.nc_pad + ig0 + k) * kBPM + pl;
        m.colA[o] = ta[k][pl];
        m.colB[o] = tb[k][pl];
        if (m.colC) m.colC[o] = tc[k][pl];
      }
    }
    if (slices) {
      // split-BF16 slices of the contraction's A rows (iw, column), 8
      // g-vectors per chunk; consecutive threads fill one 8-row group
      for (int c = tid; c < kNW * kBPM * 4; c += 256) {
        const int ch = c % 4, pl = (c / 4) % kBPM, iw = c / (4 * kBPM);
        const int col = cb * kBPM + pl;
        if (col >= p.ng) continue;
        float re[8], im[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const float2 v = ty[iw][pl][ch * 8 + j];
          re[j] = v.x;
          im[j] = v.y;
        }
        oz_put_a(oz, iw * p.ng + col, ig0 + ch * 8, re, im);
      }
    }
  }
}

__global__ void __launch_bounds__(256) prep_bands_kernel(GppDev p, MixedPrep m, int band_begin,
                                                         int band_count, int n_band_blocks) {
  __shared__ float2 tn[32][kBN + 1];
  const int tid = threadIdx.x;
  const long long tiles = (long long)n_band_blocks * (m.nc_pad / 32);
  for (long long t = blockIdx.x; t < tiles; t += gridDim.x) {
    const int bb = (int)(t / (m.nc_pad / 32));
    const int ig0 = (int)(t % (m.nc_pad / 32)) * 32;
    __syncthreads();
    for (int e = tid; e < 32 * kBN; e += 256) {
      const int bl = e / 32, k = e % 32;
      const int n1 = band_begin + bb * kBN + bl, ig = ig0 + k;
      float2 v = make_float2(0.f, 0.f);
      if (bb * kBN + bl < band_count && ig < p.nc) {
        const double2 d = p.aqsn[(size_t)n1 * p.nc + ig];
        v = make_float2(__double2float_rn(d.x), __double2float_rn(d.y));
      }
      tn[k][bl] = v;
    }
    __syncthreads();
    for (int e = tid; e < 32 * kBN; e += 256) {
      const int k = e / kBN, bl = e % kBN;
      m.band[((size_t)bb * m.nc_pad + ig0 + k) * kBN + bl] = tn[k][bl];
    }
  }
}

// ---- main pass
// The terms of one staged chunk (kCK g-vectors) for the thread's 2 bands x 1
// column x 3 frequencies, folded into the float-float accumulators every
// kRun g-vectors.  kMask: the keep decisions come as a per-(column,
// g-vector) bit mask from the pre-pass; otherwise each term compares its FP32
// |wdiff|^2 with the threshold and near-threshold terms are re-decided in
// FP64.  kWxl: the frequencies are not exact in FP32 and carry a low part.
template <bool kMask, bool kWxl>
__device__ __forceinline__ void chunk_terms(const Stage& st, int pl, int ty, const float (&wxh)[kTN][kNW],
                                            const float (&wxl)[kTN][kNW], float2 (&acc)[kTN][kNW],
                                            float2 (&hi)[kTN][kNW], float2 (&lo)[kTN][kNW],
                                            const GppDev& p, int n1_0, int my_igp, int ig0,
                                            int ig_end, int band_end) {
  const float band_lo = 1.0f - kGuardBand, band_hi = 1.0f + kGuardBand;
#pragma unroll 1
  for (int kr = 0; kr < kCK; kr += kRun) {
#pragma unroll 2
    for (int k = kr; k < kr + kRun; ++k) {
      const float4 a = st.a[k][pl];
      const float2 g = st.b[k][pl];
      float2 nn[kTN];
#pragma unroll
      for (int i = 0; i < kTN; ++i) nn[i] = st.n[k][ty + 16 * i];
      const float b2 = a.z * a.z;
      if constexpr (kMask) {
        const unsigned mask = __float_as_uint(a.w);
#pragma unroll
        for (int i = 0; i < kTN; ++i) {
          const float2 R = cmulf(nn[i], g);
          const float bRre = a.z * R.x, bRim = a.z * R.y;
#pragma unroll
          for (int iw = 0; iw < kNW; ++iw) {
            const float c = kWxl ? (wxh[i][iw] - a.x) + (wxl[i][iw] - a.y) : (wxh[i][iw] - a.x) - a.y;
            const float r = rcp_f32(fmaf(c, c, b2));
            const float rm = (mask & (1u << iw)) ? r : 0.f;
            acc[i][iw].x = fmaf(fmaf(R.x, c, -bRim), rm, acc[i][iw].x);
            acc[i][iw].y = fmaf(fmaf(R.y, c, bRre), rm, acc[i][iw].y);
          }
        }
      } else {
        const float thi = a.w * band_hi, tlo = a.w * band_lo;
        bool unc = false;
#pragma unroll
        for (int i = 0; i < kTN; ++i) {
          const float2 R = cmulf(nn[i], g);
          const float bRre = a.z * R.x, bRim = a.z * R.y;
#pragma unroll
          for (int iw = 0; iw < kNW; ++iw) {
            const float c = (wxh[i][iw] - a.x) + (wxl[i][iw] - a.y);
            const float wv = fmaf(c, c, b2);
            const float r = rcp_f32(wv);
            const bool keep = wv > thi;
            unc |= (wv > tlo) && !keep;
            const float rm = keep ? r : 0.f;
            acc[i][iw].x = fmaf(fmaf(R.x, c, -bRim), rm, acc[i][iw].x);
            acc[i][iw].y = fmaf(fmaf(R.y, c, bRre), rm, acc[i][iw].y);
          }
        }
        if (__any_sync(0xffffffffu, unc)) {
          // Terms near a threshold were dropped above; add back the ones the
          // FP64 decision keeps.
          const int ig = ig0 + k;
#pragma unroll
          for (int i = 0; i < kTN; ++i) {
            const int n1 = n1_0 + ty + 16 * i;
            const float2 R = cmulf(nn[i], g);
            const float bRre = a.z * R.x, bRim = a.z * R.y;
#pragma unroll
            for (int iw = 0; iw < kNW; ++iw) {
              const float c = (wxh[i][iw] - a.x) + (wxl[i][iw] - a.y);
              const float wv = fmaf(c, c, b2);
              if (wv > tlo && !(wv > thi) && n1 < band_end && my_igp < p.ng && ig < ig_end &&
                  keep_exact(p, my_igp, ig, p.wx[(size_t)n1 * p.wx_stride + iw])) {
                const float r = rcp_f32(wv);
                acc[i][iw].x = fmaf(fmaf(R.x, c, -bRim), r, acc[i][iw].x);
                acc[i][iw].y = fmaf(fmaf(R.y, c, bRre), r, acc[i][iw].y);
              }
            }
          }
        }
      }
    }
    // fold the FP32 run into the float-float accumulators
#pragma unroll
    for (int i = 0; i < kTN; ++i)
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) {
        float sum, err;
        two_sum_f(hi[i][iw].x, acc[i][iw].x, sum, err);
        hi[i][iw].x = sum;
        lo[i][iw].x += err;
        two_sum_f(hi[i][iw].y, acc[i][iw].y, sum, err);
        hi[i][iw].y = sum;
        lo[i][iw].y += err;
        acc[i][iw] = make_float2(0.f, 0.f);
      }
  }
}

// One work item of the main pass (TMA ring barriers and their phases persist
// across the items a CTA takes).  False (the same in every thread) when a
// copy wait gave up; the CTA then takes no further item.
__device__ __forceinline__ bool sch_mixed_item(const GppDev& p, const GppWork& w, const MixedPrep& m,
                                               int item, SchSmemM& sm, int tid, uint32_t& phase0,
                                               uint32_t& phase1) {
  const int tx = tid & 15, ty = tid >> 4;
  const int band_end = w.band_begin + w.band_count;
  const bool shared_wx = p.wx_stride == 0;
  const ItemCoord ic = decode_item(w, item);
  const int n1_0 = w.band_begin + ic.bb * kBN;
  const int ig_begin = ic.s * w.split_len;
  const int ig_end = min(ig_begin + w.split_len, p.nc);
  const int n_chunks = (ig_end - ig_begin + kCK - 1) / kCK;
  const int pl = tx;
  const int my_igp = ic.cb * kBPM + pl;

  float wxh[kTN][kNW], wxl[kTN][kNW];
  bool exact = true;
#pragma unroll
  for (int i = 0; i < kTN; ++i) {
    const int n1 = n1_0 + ty + 16 * i;
#pragma unroll
    for (int iw = 0; iw < kNW; ++iw) {
      const double wx = n1 < band_end ? p.wx[(size_t)n1 * p.wx_stride + iw] : 0.0;
      split_f(wx, wxh[i][iw], wxl[i][iw]);
      exact = exact && wxl[i][iw] == 0.f;
    }
  }
  const bool wx_exact = __syncthreads_and(exact) != 0;  // every frequency exact in FP32
  float2 acc[kTN][kNW], hi[kTN][kNW], lo[kTN][kNW];
#pragma unroll
  for (int i = 0; i < kTN; ++i)
#pragma unroll
    for (int iw = 0; iw < kNW; ++iw) {
      acc[i][iw] = make_float2(0.f, 0.f);
      hi[i][iw] = make_float2(0.f, 0.f);
      lo[i][iw] = make_float2(0.f, 0.f);
    }

  if (tid == 0) issue_chunk(m, ic.cb, ic.bb, ig_begin, sm.st[0], &sm.bar[0]);
  for (int c = 0; c < n_chunks; ++c) {
    const int buf = c & 1;
    const int ig0 = ig_begin + c * kCK;
    if (tid == 0 && c + 1 < n_chunks)
      issue_chunk(m, ic.cb, ic.bb, ig0 + kCK, sm.st[buf ^ 1], &sm.bar[buf ^ 1]);
    const uint32_t pc = buf ? phase1 : phase0, pn = buf ? phase0 : phase1;
    const bool ok = mbar_wait(&sm.bar[buf], pc, m.status);
    if (buf == 0) phase0 ^= 1; else phase1 ^= 1;
    const Stage& st = sm.st[buf];
    if (shared_wx) {
      if (wx_exact)
        chunk_terms<true, false>(st, pl, ty, wxh, wxl, acc, hi, lo, p, n1_0, my_igp, ig0, ig_end, band_end);
      else
        chunk_terms<true, true>(st, pl, ty, wxh, wxl, acc, hi, lo, p, n1_0, my_igp, ig0, ig_end, band_end);
    } else {
      chunk_terms<false, true>(st, pl, ty, wxh, wxl, acc, hi, lo, p, n1_0, my_igp, ig0, ig_end, band_end);
    }
    // every thread is done with this stage before it is refilled
    if (__syncthreads_or(!ok)) {
      if (tid == 0) drain_chunks(sm.bar, c, n_chunks, pc, pn);
      return false;
    }
  }

  // epilogue: x conj(aqsm[n1][igp]) * 0.5 * vcoul[igp] in FP64, then a
  // fixed-order compensated sum over the tile's columns
  const int igp = my_igp < p.ng ? p.igp_of[my_igp] : -1;
#pragma unroll
  for (int i = 0; i < kTN; ++i) {
    const int bl = ty + 16 * i;
    const int n1 = n1_0 + bl;
    if (n1 < band_end && igp >= 0) {
      const double2 am = p.aqsm[(size_t)n1 * p.nc + igp];
      const double2 mm = make_double2(am.x, -am.y);
      const double f = 0.5 * p.vcoul[igp];
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) {
        const double2 sv = make_double2((double)hi[i][iw].x + (double)lo[i][iw].x,
                                        (double)hi[i][iw].y + (double)lo[i][iw].y);
        const double2 v = cmul(sv, mm);
        sm.red[iw][pl][bl] = make_double2(v.x * f, v.y * f);
      }
    } else {
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) sm.red[iw][pl][bl] = make_double2(0.0, 0.0);
    }
  }
  __syncthreads();
  if (tid < kBN * kNW) {
    const int iw = tid / kBN, bl = tid % kBN;
    Comp sx, sy;
    for (int q = 0; q < kBPM; ++q) {
      sx.add(sm.red[iw][q][bl].x);
      sy.add(sm.red[iw][q][bl].y);
    }
    w.partial[ic.pidx * kBN * kNW + bl * kNW + iw] = make_double2(sx.value(), sy.value());
  }
  return true;
}

__global__ void __launch_bounds__(kThreads, 3) sch_mixed_kernel(GppDev p, GppWork w, MixedPrep m) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  SchSmemM& sm = *reinterpret_cast<SchSmemM*>(smem_raw);
  __shared__ int s_item;
  const int tid = threadIdx.x;
  if (tid == 0) {
    mbar_init(&sm.bar[0], 1);
    mbar_init(&sm.bar[1], 1);
    mbar_fence_init();
  }
  uint32_t phase0 = 0, phase1 = 0;
  for (;;) {
    __syncthreads();
    // no further items once a wait of this launch gave up
    if (tid == 0) s_item = tma::status_set(m.status) ? w.n_items : atomicAdd(w.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= w.n_items) break;
    if (!sch_mixed_item(p, w, m, item, sm, tid, phase0, phase1)) break;
  }
}

__global__ void __launch_bounds__(kThreads, 3) sch_mixed_batch_kernel(GppBatchView b) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  SchSmemM& sm = *reinterpret_cast<SchSmemM*>(smem_raw);
  __shared__ int s_item;
  const int tid = threadIdx.x;
  if (tid == 0) {
    mbar_init(&sm.bar[0], 1);
    mbar_init(&sm.bar[1], 1);
    mbar_fence_init();
  }
  uint32_t phase0 = 0, phase1 = 0;
  for (;;) {
    __syncthreads();
    // no further items once a wait of this launch gave up (one status word per batch)
    if (tid == 0) s_item = tma::status_set(b.prep[0].status) ? b.total : atomicAdd(b.counter, 1);
    __syncthreads();
    const int g = s_item;
    if (g >= b.total) break;
    const int inst = batch_owner(b.item_off, b.n_inst, g);
    if (!sch_mixed_item(b.dev[inst], b.work[inst], b.prep[inst], g - b.item_off[inst], sm, tid, phase0,
                        phase1))
      break;
  }
}

}  // namespace

namespace {

// ---------------------------------------------------------------- shared-frequency main pass
// With one frequency set for every band the factor Y_iw = G (c + i b) r of a
// (column, g-vector) is the same for every band (the FP64 path's
// sch_fp64y_kernel uses the same algebra).  sch_mixedy forms Y once per
// staged chunk in FP32 from the pre-pass operands and the exact keep masks,
// and the band sum becomes an FP32 complex GEMM: items of 64 bands x 32
// columns (two pre-pass blocks each way), 16 x 16 threads with 4 bands x 2
// columns x 3 frequencies each, runs of kRun g-vectors folded into
// float-float accumulators as in the per-band kernel.
constexpr int kYBN = 2 * kBN, kYBP = 2 * kBPM;  // 64 bands x 32 columns
constexpr uint32_t kYChunkBytes = 2 * kChunkBytes;

struct __align__(16) StageY {
  float4 a[2][kCK][kBPM];
  float2 b[2][kCK][kBPM];
  float2 n[2][kCK][kBN];
};
struct __align__(16) SchSmemY {
  StageY st[2];
  float2 y[kCK][kNW][kYBP];
  unsigned long long bar[2];
};
static_assert(sizeof(StageY) == kYChunkBytes, "six bulk copies per chunk");

// band_halves: pre-pass band blocks of the item that hold bands (1 for a
// last block of at most kBN bands, whose second block is not copied)
__device__ __forceinline__ void issue_chunk_y(const MixedPrep& m, int cb, int bb, int ig0, int band_halves,
                                              StageY& st, unsigned long long* bar) {
  mbar_expect_tx(bar, kYChunkBytes - (uint32_t)(2 - band_halves) * (uint32_t)sizeof(st.n[0]));
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const size_t col_off = ((size_t)(2 * cb + h) * m.nc_pad + ig0) * kBPM;
    const size_t band_off = ((size_t)(2 * bb + h) * m.nc_pad + ig0) * kBN;
    bulk_load(&st.a[h][0][0], m.colA + col_off, sizeof(st.a[h]), bar);
    bulk_load(&st.b[h][0][0], m.colB + col_off, sizeof(st.b[h]), bar);
    if (h < band_halves) bulk_load(&st.n[h][0][0], m.band + band_off, sizeof(st.n[h]), bar);
  }
}

// kExact: each complex product is formed before it is added (one rounding of
// the running sum per component and term instead of two, 50 % more FP32
// operations), which brings the error to the per-band kernel's.
template <bool kExact>
__device__ __forceinline__ bool sch_mixedy_item(const GppDev& p, const GppWork& w, const MixedPrep& m,
                                                int item, SchSmemY& sm, int tid, uint32_t& phase0,
                                                uint32_t& phase1) {
  constexpr int TB = 4, TC = 2;
  const int tx = tid & 15, ty = tid >> 4;
  const int band_end = w.band_begin + w.band_count;
  const ItemCoord ic = decode_item(w, item);
  const int n1_0 = w.band_begin + ic.bb * kYBN;
  const int p0 = ic.cb * kYBP;
  const int ig_begin = ic.s * w.split_len;
  const int ig_end = min(ig_begin + w.split_len, p.nc);
  const int n_chunks = (ig_end - ig_begin + kCK - 1) / kCK;
  float wxh[kNW], wxl[kNW];
#pragma unroll
  for (int iw = 0; iw < kNW; ++iw) split_f(p.wx[iw], wxh[iw], wxl[iw]);

  float2 acc[TB][TC][kNW], hi[TB][TC][kNW], lo[TB][TC][kNW];
#pragma unroll
  for (int i = 0; i < TB; ++i)
#pragma unroll
    for (int j = 0; j < TC; ++j)
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) {
        acc[i][j][iw] = make_float2(0.f, 0.f);
        hi[i][j][iw] = make_float2(0.f, 0.f);
        lo[i][j][iw] = make_float2(0.f, 0.f);
      }
  // this thread's bands: 4 consecutive of one pre-pass band block
  const int nb_blk = ty >> 3, nb_off = (ty & 7) * TB;
  // a last band block of at most kBN bands sums one pre-pass block: warps
  // 4-7 (nb_blk 1) form factors but skip the products, their sums stay 0
  const int band_halves = band_end - n1_0 > kBN ? 2 : 1;
  const bool sums = nb_blk < band_halves;

  if (tid == 0) issue_chunk_y(m, ic.cb, ic.bb, ig_begin, band_halves, sm.st[0], &sm.bar[0]);
  for (int c = 0; c < n_chunks; ++c) {
    const int buf = c & 1;
    const int ig0 = ig_begin + c * kCK;
    if (tid == 0 && c + 1 < n_chunks)
      issue_chunk_y(m, ic.cb, ic.bb, ig0 + kCK, band_halves, sm.st[buf ^ 1], &sm.bar[buf ^ 1]);
    const uint32_t pc = buf ? phase1 : phase0, pn = buf ? phase0 : phase1;
    const bool ok = mbar_wait(&sm.bar[buf], pc, m.status);
    if (buf == 0) phase0 ^= 1; else phase1 ^= 1;
    const StageY& st = sm.st[buf];
    // frequency factors of the chunk; g-vectors past the split's end and
    // padding columns carry a zero mask
    for (int e = tid; e < kCK * kYBP; e += kThreads) {
      const int k = e / kYBP, col = e % kYBP;
      const int h = col / kBPM, pl = col % kBPM;
      const float4 a = st.a[h][k][pl];
      const float2 g = st.b[h][k][pl];
      const unsigned mask = (ig0 + k < ig_end) ? __float_as_uint(a.w) : 0u;
      const float b2 = a.z * a.z;
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) {
        const float cc = (wxh[iw] - a.x) + (wxl[iw] - a.y);
        const float r = rcp_f32(fmaf(cc, cc, b2));
        const float rm = (mask & (1u << iw)) ? r : 0.f;
        sm.y[k][iw][col] = make_float2(fmaf(g.x, cc, -g.y * a.z) * rm, fmaf(g.x, a.z, g.y * cc) * rm);
      }
    }
    __syncthreads();
#pragma unroll 1
    for (int kr = 0; sums && kr < kCK; kr += kRun) {
#pragma unroll 2
      for (int k = kr; k < kr + kRun; ++k) {
        const float4 n01 = *reinterpret_cast<const float4*>(&st.n[nb_blk][k][nb_off]);
        const float4 n23 = *reinterpret_cast<const float4*>(&st.n[nb_blk][k][nb_off + 2]);
        const float2 nn[TB] = {make_float2(n01.x, n01.y), make_float2(n01.z, n01.w),
                               make_float2(n23.x, n23.y), make_float2(n23.z, n23.w)};
        float2 yv[TC][kNW];
#pragma unroll
        for (int iw = 0; iw < kNW; ++iw) {
          const float4 y2 = *reinterpret_cast<const float4*>(&sm.y[k][iw][2 * tx]);
          yv[0][iw] = make_float2(y2.x, y2.y);
          yv[1][iw] = make_float2(y2.z, y2.w);
        }
#pragma unroll
        for (int i = 0; i < TB; ++i)
#pragma unroll
          for (int j = 0; j < TC; ++j)
#pragma unroll
            for (int iw = 0; iw < kNW; ++iw) {
              float2& a = acc[i][j][iw];
              if constexpr (kExact) {
                a.x += fmaf(nn[i].x, yv[j][iw].x, -nn[i].y * yv[j][iw].y);
                a.y += fmaf(nn[i].x, yv[j][iw].y, nn[i].y * yv[j][iw].x);
              } else {
                a.x = fmaf(nn[i].x, yv[j][iw].x, a.x);
                a.x = fmaf(-nn[i].y, yv[j][iw].y, a.x);
                a.y = fmaf(nn[i].x, yv[j][iw].y, a.y);
                a.y = fmaf(nn[i].y, yv[j][iw].x, a.y);
              }
            }
      }
#pragma unroll
      for (int i = 0; i < TB; ++i)
#pragma unroll
        for (int j = 0; j < TC; ++j)
#pragma unroll
          for (int iw = 0; iw < kNW; ++iw) {
            float sum, err;
            two_sum_f(hi[i][j][iw].x, acc[i][j][iw].x, sum, err);
            hi[i][j][iw].x = sum;
            lo[i][j][iw].x += err;
            two_sum_f(hi[i][j][iw].y, acc[i][j][iw].y, sum, err);
            hi[i][j][iw].y = sum;
            lo[i][j][iw].y += err;
            acc[i][j][iw] = make_float2(0.f, 0.f);
          }
    }
    // stage and factors consumed before they are refilled
    if (__syncthreads_or(!ok)) {
      if (tid == 0) drain_chunks(sm.bar, c, n_chunks, pc, pn);
      return false;
    }
  }

  // epilogue: x conj(aqsm[n1][igp]) * 0.5 * vcoul[igp] in FP64; the 16 lanes
  // of a half-warp hold the item's 32 columns for the same 4 bands and sum
  // them with a fixed butterfly
#pragma unroll
  for (int i = 0; i < TB; ++i) {
    const int bl = nb_blk * kBN + nb_off + i;  // band within the item
    const int n1 = n1_0 + bl;
    double2 part[kNW];
#pragma unroll
    for (int iw = 0; iw < kNW; ++iw) part[iw] = make_double2(0.0, 0.0);
#pragma unroll
    for (int j = 0; j < TC; ++j) {
      const int my_igp = p0 + 2 * tx + j;
      const int igp = my_igp < p.ng ? p.igp_of[my_igp] : -1;
      if (n1 < band_end && igp >= 0) {
        const double2 am = p.aqsm[(size_t)n1 * p.nc + igp];
        const double2 mm = make_double2(am.x, -am.y);
        const double f = 0.5 * p.vcoul[igp];
#pragma unroll
        for (int iw = 0; iw < kNW; ++iw) {
          const double2 sv = make_double2((double)hi[i][j][iw].x + (double)lo[i][j][iw].x,
                                          (double)hi[i][j][iw].y + (double)lo[i][j][iw].y);
          const double2 v = cmul(sv, mm);
          part[iw].x = fma(v.x, f, part[iw].x);
          part[iw].y = fma(v.y, f, part[iw].y);
        }
      }
    }
#pragma unroll
    for (int iw = 0; iw < kNW; ++iw)
#pragma unroll
      for (int o = 8; o > 0; o >>= 1) {
        part[iw].x += __shfl_xor_sync(0xffffffffu, part[iw].x, o);
        part[iw].y += __shfl_xor_sync(0xffffffffu, part[iw].y, o);
      }
    if (tx == 0)
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) w.partial[ic.pidx * kYBN * kNW + bl * kNW + iw] = part[iw];
  }
  return true;
}

__global__ void __launch_bounds__(kThreads, 1) sch_mixedy_kernel(GppDev p, GppWork w, MixedPrep m) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  SchSmemY& sm = *reinterpret_cast<SchSmemY*>(smem_raw);
  __shared__ int s_item;
  const int tid = threadIdx.x;
  if (tid == 0) {
    mbar_init(&sm.bar[0], 1);
    mbar_init(&sm.bar[1], 1);
    mbar_fence_init();
  }
  uint32_t phase0 = 0, phase1 = 0;
  for (;;) {
    __syncthreads();
    // no further items once a wait of this launch gave up
    if (tid == 0) s_item = tma::status_set(m.status) ? w.n_items : atomicAdd(w.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= w.n_items) break;
    if (!sch_mixedy_item<false>(p, w, m, item, sm, tid, phase0, phase1)) break;
  }
}

// Batched form: one queue over every instance (all with one frequency set),
// products formed before they are added.
__global__ void __launch_bounds__(kThreads, 1) sch_mixedy_batch_kernel(GppBatchView b) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  SchSmemY& sm = *reinterpret_cast<SchSmemY*>(smem_raw);
  __shared__ int s_item;
  const int tid = threadIdx.x;
  if (tid == 0) {
    mbar_init(&sm.bar[0], 1);
    mbar_init(&sm.bar[1], 1);
    mbar_fence_init();
  }
  uint32_t phase0 = 0, phase1 = 0;
  for (;;) {
    __syncthreads();
    // no further items once a wait of this launch gave up (one status word per batch)
    if (tid == 0) s_item = tma::status_set(b.prep[0].status) ? b.total : atomicAdd(b.counter, 1);
    __syncthreads();
    const int g = s_item;
    if (g >= b.total) break;
    const int inst = batch_owner(b.item_off, b.n_inst, g);
    if (!sch_mixedy_item<true>(b.dev[inst], b.work[inst], b.prep[inst], g - b.item_off[inst], sm, tid,
                               phase0, phase1))
      break;
  }
}

}  // namespace

int sch_batch_blocks_per_sm_mixedy() {
  int n = 0;
  cudaFuncSetAttribute(sch_mixedy_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       sizeof(SchSmemY));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sch_mixedy_batch_kernel, kThreads, sizeof(SchSmemY));
  return n > 0 ? n : 1;
}

cudaError_t launch_sch_mixedy_batch(const GppBatchView& b, int grid, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(sch_mixedy_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       sizeof(SchSmemY));
  if (e != cudaSuccess) return e;
  sch_mixedy_batch_kernel<<<grid, kThreads, sizeof(SchSmemY), s>>>(b);
  return cudaGetLastError();
}

int sch_blocks_per_sm_mixedy() {
  int n = 0;
  cudaFuncSetAttribute(sch_mixedy_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(SchSmemY));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sch_mixedy_kernel, kThreads, sizeof(SchSmemY));
  return n > 0 ? n : 1;
}

cudaError_t launch_sch_mixedy(const GppDev& p, const GppWork& w, const MixedPrep& m, int grid,
                              cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(sch_mixedy_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       sizeof(SchSmemY));
  if (e != cudaSuccess) return e;
  sch_mixedy_kernel<<<grid, kThreads, sizeof(SchSmemY), s>>>(p, w, m);
  return cudaGetLastError();
}

int sch_blocks_per_sm_mixed() {
  int n = 0;
  cudaFuncSetAttribute(sch_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(SchSmemM));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sch_mixed_kernel, kThreads, sizeof(SchSmemM));
  return n > 0 ? n : 1;
}

cudaError_t launch_tensor_factors(const GppDev& p, const GppWork& w, const MixedPrep* m, cudaStream_t s,
                                  const OzakiPrep* oz) {
  const int sms = 152;
  MixedPrep mm{};
  if (m) {
    mm = *m;
    prep_bands_kernel<<<sms * 4, 256, 0, s>>>(p, mm, w.band_begin, w.band_count, w.n_band_blocks);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  } else {
    mm.nc_pad = (p.nc + 31) / 32 * 32;  // tiles over the factor slabs alone
  }
  const int ncb = m ? w.n_col_blocks : (p.ng + kBPM - 1) / kBPM;
  OzakiPrep o{};
  if (oz) o = *oz;
  tensor_factors_kernel<<<sms * 8, 256, 0, s>>>(p, mm, ncb, o);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || !oz) return e;
  return launch_ozaki_zero_rows(*oz, kNW * p.ng, s);
}

cudaError_t launch_prep_mixed(const GppDev& p, const GppWork& w, const MixedPrep& m, cudaStream_t s) {
  const int sms = 152;
  prep_cols_kernel<<<sms * 8, 256, 0, s>>>(p, m, w.n_col_blocks);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  prep_bands_kernel<<<sms * 4, 256, 0, s>>>(p, m, w.band_begin, w.band_count, w.n_band_blocks);
  return cudaGetLastError();
}

cudaError_t launch_sch_mixed(const GppDev& p, const GppWork& w, const MixedPrep& m, int grid,
                             cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(sch_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       sizeof(SchSmemM));
  if (e != cudaSuccess) return e;
  sch_mixed_kernel<<<grid, kThreads, sizeof(SchSmemM), s>>>(p, w, m);
  return cudaGetLastError();
}

namespace {

// ---------------------------------------------------------------- occupied bands
// FP32 form of ssx_fp64_kernel.  The three branch decisions (keep, the
// |delw|^2 > to1 test, and the exact-pole test |wdiff|^2 > 0) fall back to the
// FP64 expressions whenever FP32 |wdiff|^2 is near the corresponding threshold.
constexpr int kSsxCK = 8;

struct __align__(16) ColS {
  float ahi, alo, b, b2;
  float thr, thr2, gx, gy;
  float ox, oy, pad0, pad1;
};

struct SsxSmemF {
  ColS col[kSsxCK][kSsxBP];
  float2 n[kSsxCK][kSsxBN];
};
static_assert(sizeof(SsxSmemF) <= 200 * 1024, "shared memory budget");

// FP64 branch of one occupied-band term: 0 dropped, 1 kept, 2 second branch.
__device__ __forceinline__ int ssx_branch_exact(const GppDev& p, int my_igp, int ig, double wx) {
  const double2 wt = p.wt[(size_t)my_igp * p.nc + ig];
  const double b2 = guard_b2(wt.y);
  const double wv = guard_w(wx, wt.x, b2);
  if (keep_nonneg(wv, guard_thr(wt.x, b2))) return 1;
  if (gt_nonneg(wv, 0.0) && gt_nonneg(guard_thr2(wt.x, b2), wv)) return 2;
  return 0;
}

struct SsxSharedF {
  double2 red[kSsxBN][kNW][kThreads / 32];
  float wxh[kSsxBN][kNW], wxl[kSsxBN][kNW], iwx2[kSsxBN][kNW];
  double wx[kSsxBN][kNW];
};

__device__ __forceinline__ void ssx_mixed_item(const GppDev& p, const GppWork& w, int item,
                                               unsigned char* smem_raw, SsxSharedF& sh, int tid) {
  SsxSmemF& sm = *reinterpret_cast<SsxSmemF*>(smem_raw);
  const int band_end = w.band_begin + w.band_count;
  const float blo = 1.0f - kGuardBand, bhi = 1.0f + kGuardBand;
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
    sh.wx[i][iw] = wx;
    split_f(wx, sh.wxh[i][iw], sh.wxl[i][iw]);
    sh.iwx2[i][iw] = __double2float_rn(rcp_f64(wx * wx));
  }

  float2 acc[kSsxBN][kNW], accl[kSsxBN][kNW];
#pragma unroll
  for (int i = 0; i < kSsxBN; ++i)
#pragma unroll
    for (int iw = 0; iw < kNW; ++iw) {
      acc[i][iw] = make_float2(0.f, 0.f);
      accl[i][iw] = make_float2(0.f, 0.f);
    }
  double2 accd[kSsxBN][kNW];
#pragma unroll
  for (int i = 0; i < kSsxBN; ++i)
#pragma unroll
    for (int iw = 0; iw < kNW; ++iw) accd[i][iw] = make_double2(0.0, 0.0);

  for (int ig0 = ig_begin; ig0 < ig_end; ig0 += kSsxCK) {
    __syncthreads();
    for (int e = tid; e < kSsxCK * kSsxBP; e += kThreads) {
      const int k = e % kSsxCK, pl = e / kSsxCK;
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
    for (int e = tid; e < kSsxCK * kSsxBN; e += kThreads) {
      const int k = e % kSsxCK, bl = e / kSsxCK;
      const int ig = ig0 + k, n1 = n1_0 + bl;
      float2 v = make_float2(0.f, 0.f);
      if (ig < ig_end && n1 < band_end) {
        const double2 d = p.aqsn[(size_t)n1 * p.nc + ig];
        v = make_float2(__double2float_rn(d.x), __double2float_rn(d.y));
      }
      sm.n[k][bl] = v;
    }
    __syncthreads();

    for (int k = 0; k < kSsxCK; ++k) {
      const ColS col = sm.col[k][tid];
#pragma unroll
      for (int i = 0; i < kSsxBN; ++i) {
        if (i < nbl) {
          const float2 an = sm.n[k][i];
#pragma unroll
          for (int iw = 0; iw < kNW; ++iw) {
            const float c = (sh.wxh[i][iw] - col.ahi) + (sh.wxl[i][iw] - col.alo);
            const float wv = fmaf(c, c, col.b2);
            int br;
            const bool near = (wv > col.thr * blo && wv <= col.thr * bhi) ||
                              (wv >= col.thr2 * blo && wv < col.thr2 * bhi) ||
                              wv < 1e-30f;
            if (near) {
              br = (p0 + tid < p.ng && ig0 + k < ig_end)
                       ? ssx_branch_exact(p, p0 + tid, ig0 + k, sh.wx[i][iw])
                       : 0;
            } else {
              br = wv > col.thr ? 1 : (wv < col.thr2 ? 2 : 0);
            }
            float2 s = make_float2(0.f, 0.f);
            if (br == 1) {
              s = make_float2(col.ox * sh.iwx2[i][iw], col.oy * sh.iwx2[i][iw]);
            } else if (br == 2) {
              const float zr = (sh.wxh[i][iw] + col.ahi) + (sh.wxl[i][iw] + col.alo);
              const float q = -0.5f * rcp_f32(fmaf(zr, zr, col.b2));
              s = make_float2(fmaf(col.gx, zr, col.gy * col.b) * q,
                              fmaf(col.gy, zr, -col.gx * col.b) * q);
            }
            // term in FP32, added to a float-float accumulator (TwoSum)
            const float tx = fmaf(an.x, s.x, -an.y * s.y);
            const float ty = fmaf(an.x, s.y, an.y * s.x);
            float t, e;
            two_sum_f(acc[i][iw].x, tx, t, e);
            acc[i][iw].x = t;
            accl[i][iw].x += e;
            two_sum_f(acc[i][iw].y, ty, t, e);
            acc[i][iw].y = t;
            accl[i][iw].y += e;
          }
        }
      }
    }
    // fold the float-float sums into FP64 every 16 chunks
    const bool last_chunk = ig0 + kSsxCK >= ig_end;
    if (((ig0 - ig_begin) / kSsxCK) % 16 != 15 && !last_chunk) continue;
#pragma unroll
    for (int i = 0; i < kSsxBN; ++i)
      if (i < nbl) {
#pragma unroll
        for (int iw = 0; iw < kNW; ++iw) {
          accd[i][iw].x += (double)acc[i][iw].x + (double)accl[i][iw].x;
          accd[i][iw].y += (double)acc[i][iw].y + (double)accl[i][iw].y;
          acc[i][iw] = make_float2(0.f, 0.f);
          accl[i][iw] = make_float2(0.f, 0.f);
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
      if (lane == 0) sh.red[i][iw][warp] = v;
    }
  __syncthreads();
  if (tid < kSsxBN * kNW) {
    const int i = tid / kNW, iw = tid % kNW;
    Comp sx, sy;
    for (int q = 0; q < kThreads / 32; ++q) {
      sx.add(sh.red[i][iw][q].x);
      sy.add(sh.red[i][iw][q].y);
    }
    w.partial[ic.pidx * kSsxBN * kNW + tid] = make_double2(sx.value(), sy.value());
  }
}

// Occupied-band pass when every band shares one frequency set: the main
// pass's pre-pass already holds what each (column, g-vector) needs in FP32
// (Re wtilde as hi/lo, Im wtilde, G = I_eps wtilde, Omega2 = wtilde^2 I_eps
// and the exact branch of every frequency in the mask bits), so this pass
// reads those instead of staging and converting the FP64 inputs.  The
// branch values are
//   kept:           ssx = Omega2 / wx^2
//   second branch:  ssx = -G / (2 (wtilde + wx))
// (see ssx_fp64_item), computed once per (column, g-vector) and shared by
// the item's bands.  Thread = column; each term goes into a float-float
// (TwoSum) accumulator, which leaves the thread in FP64.
struct SsxMaskShared {
  double2 red[kSsxBN][kNW][kThreads / 32];
};

__device__ __forceinline__ void ssx_masked_item(const GppDev& p, const GppWork& w, const MixedPrep& m,
                                                int item, SsxMaskShared& sh, int tid) {
  const int band_end = w.band_begin + w.band_count;
  const ItemCoord ic = decode_item(w, item);
  const int n1_0 = w.band_begin + ic.bb * kSsxBN;
  const int nbl = min(kSsxBN, band_end - n1_0);
  const int my_igp = ic.cb * kSsxBP + tid;
  const int ig_begin = ic.s * w.split_len;
  const int ig_end = min(ig_begin + w.split_len, p.nc);
  const int n_prep_cols = (p.ng + kBPM - 1) / kBPM * kBPM;  // columns the pre-pass laid out
  const bool col_in = my_igp < n_prep_cols;

  float wxh[kNW], wxl[kNW], iwx2[kNW];
#pragma unroll
  for (int iw = 0; iw < kNW; ++iw) {
    split_f(p.wx[iw], wxh[iw], wxl[iw]);
    iwx2[iw] = __double2float_rn(rcp_f64(p.wx[iw] * p.wx[iw]));
  }
  // per (band, frequency): FP32 sums of 2 terms folded into float-float
  // sums (hi, lo)
  float2 acc[kSsxBN][kNW], hi[kSsxBN][kNW], lo[kSsxBN][kNW];
#pragma unroll
  for (int i = 0; i < kSsxBN; ++i)
#pragma unroll
    for (int iw = 0; iw < kNW; ++iw) acc[i][iw] = hi[i][iw] = lo[i][iw] = make_float2(0.f, 0.f);
  auto fold = [&]() {
#pragma unroll
    for (int i = 0; i < kSsxBN; ++i)
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) {
        ff_add(hi[i][iw].x, lo[i][iw].x, acc[i][iw].x);
        ff_add(hi[i][iw].y, lo[i][iw].y, acc[i][iw].y);
        acc[i][iw] = make_float2(0.f, 0.f);
      }
  };

  if (col_in) {
    const size_t cbase = (size_t)(my_igp / kBPM) * m.nc_pad * kBPM + (my_igp % kBPM);
    const float4* ca = m.colA + cbase;
    const float2* cg = m.colB + cbase;
    const float2* co = m.colC + cbase;
    const float2* bands[kSsxBN];
#pragma unroll
    for (int i = 0; i < kSsxBN; ++i) {
      const int n1 = min(n1_0 + i, band_end - 1);
      bands[i] = m.band + ((size_t)(n1 / kBN) * m.nc_pad) * kBN + (n1 % kBN);
    }
    constexpr int kU = 4;  // g-vectors whose operands are loaded together
    for (int ig0 = ig_begin; ig0 < ig_end; ig0 += kU) {
      float4 a[kU];
      float2 g[kU], om[kU], an[kU][kSsxBN];
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const size_t ig = (size_t)min(ig0 + u, ig_end - 1);
        a[u] = ca[ig * kBPM];
        g[u] = cg[ig * kBPM];
        om[u] = co[ig * kBPM];
#pragma unroll
        for (int i = 0; i < kSsxBN; ++i) an[u][i] = i < nbl ? bands[i][ig * kBN] : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        // mask bits: keep (1 << iw), second branch (8 << iw); a tail g-vector past ig_end adds 0
        const unsigned mask = ig0 + u < ig_end ? __float_as_uint(a[u].w) : 0u;
        const float b = a[u].z;
        float2 sv[kNW];
#pragma unroll
        for (int iw = 0; iw < kNW; ++iw) {
          const float zr = (wxh[iw] + a[u].x) + (wxl[iw] + a[u].y);
          const float q = -0.5f * rcp_f32(fmaf(zr, zr, b * b));
          const float2 s2 = make_float2(fmaf(g[u].x, zr, g[u].y * b) * q, fmaf(g[u].y, zr, -g[u].x * b) * q);
          const float2 s1 = make_float2(om[u].x * iwx2[iw], om[u].y * iwx2[iw]);
          sv[iw] = (mask & (1u << iw)) ? s1 : ((mask & (8u << iw)) ? s2 : make_float2(0.f, 0.f));
        }
        // each product formed before it is added: one rounding of the pair sum
#pragma unroll
        for (int i = 0; i < kSsxBN; ++i)
#pragma unroll
          for (int iw = 0; iw < kNW; ++iw) {
            acc[i][iw].x += fmaf(an[u][i].x, sv[iw].x, -an[u][i].y * sv[iw].y);
            acc[i][iw].y += fmaf(an[u][i].x, sv[iw].y, an[u][i].y * sv[iw].x);
          }
        if (u & 1) fold();  // pair sums
      }
    }
  }

  // epilogue: x conj(aqsm[n1][igp]) occ vcoul[igp] in float-float, warp sums
  // in float-float, block sum in FP64 with compensation
  const int igp = my_igp < p.ng ? p.igp_of[my_igp] : -1;
  const int lane = tid & 31, warp = tid >> 5;
  __syncthreads();  // the previous item's epilogue is done with sh.red
#pragma unroll
  for (int i = 0; i < kSsxBN; ++i) {
    FF fr{0.f, 0.f}, fi{0.f, 0.f};  // conj(aqsm) occ vcoul
    if (i < nbl && igp >= 0) {
      const double2 am = p.aqsm[(size_t)(n1_0 + i) * p.nc + igp];
      const FF f = ff_of(p.occ * p.vcoul[igp]);
      fr = ff_mul(ff_of(am.x), f);
      fi = ff_neg(ff_mul(ff_of(am.y), f));
    }
#pragma unroll
    for (int iw = 0; iw < kNW; ++iw) {
      const FF sx{hi[i][iw].x, lo[i][iw].x}, sy{hi[i][iw].y, lo[i][iw].y};
      FF vx = ff_add(ff_mul(sx, fr), ff_neg(ff_mul(sy, fi)));
      FF vy = ff_add(ff_mul(sx, fi), ff_mul(sy, fr));
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        vx = ff_add(vx, FF{__shfl_xor_sync(0xffffffffu, vx.hi, o), __shfl_xor_sync(0xffffffffu, vx.lo, o)});
        vy = ff_add(vy, FF{__shfl_xor_sync(0xffffffffu, vy.hi, o), __shfl_xor_sync(0xffffffffu, vy.lo, o)});
      }
      if (lane == 0)
        sh.red[i][iw][warp] = make_double2((double)vx.hi + (double)vx.lo, (double)vy.hi + (double)vy.lo);
    }
  }
  __syncthreads();
  if (tid < kSsxBN * kNW) {
    const int i = tid / kNW, iw = tid % kNW;
    Comp sx, sy;
    for (int q = 0; q < kThreads / 32; ++q) {
      sx.add(sh.red[i][iw][q].x);
      sy.add(sh.red[i][iw][q].y);
    }
    w.partial[ic.pidx * kSsxBN * kNW + tid] = make_double2(sx.value(), sy.value());
  }
}

__global__ void __launch_bounds__(kThreads, 2) ssx_masked_kernel(GppDev p, GppWork w, MixedPrep m) {
  __shared__ int s_item;
  __shared__ SsxMaskShared sh;
  const int tid = threadIdx.x;
  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(w.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= w.n_items) break;
    ssx_masked_item(p, w, m, item, sh, tid);
  }
}

__global__ void __launch_bounds__(kThreads, 2) ssx_masked_batch_kernel(GppBatchView b) {
  __shared__ int s_item;
  __shared__ SsxMaskShared sh;
  const int tid = threadIdx.x;
  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(b.counter, 1);
    __syncthreads();
    const int g = s_item;
    if (g >= b.total) break;
    const int inst = batch_owner(b.item_off, b.n_inst, g);
    ssx_masked_item(b.dev[inst], b.work[inst], b.prep[inst], g - b.item_off[inst], sh, tid);
  }
}

__global__ void __launch_bounds__(kThreads) ssx_mixed_kernel(GppDev p, GppWork w) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ int s_item;
  __shared__ SsxSharedF sh;
  const int tid = threadIdx.x;
  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(w.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= w.n_items) break;
    ssx_mixed_item(p, w, item, smem_raw, sh, tid);
  }
}

__global__ void __launch_bounds__(kThreads) ssx_mixed_batch_kernel(GppBatchView b) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ int s_item;
  __shared__ SsxSharedF sh;
  const int tid = threadIdx.x;
  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(b.counter, 1);
    __syncthreads();
    const int g = s_item;
    if (g >= b.total) break;
    const int inst = batch_owner(b.item_off, b.n_inst, g);
    ssx_mixed_item(b.dev[inst], b.work[inst], g - b.item_off[inst], smem_raw, sh, tid);
  }
}

}  // namespace

// Grid of the occupied-band pass: sized for the masked kernel (the common
// case); the staged fallback takes the same items with fewer CTAs resident.
int ssx_blocks_per_sm_mixed() {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ssx_masked_kernel, kThreads, 0);
  return n > 0 ? n : 1;
}

int sch_batch_blocks_per_sm_mixed() {
  int n = 0;
  cudaFuncSetAttribute(sch_mixed_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(SchSmemM));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sch_mixed_batch_kernel, kThreads, sizeof(SchSmemM));
  return n > 0 ? n : 1;
}

int ssx_batch_blocks_per_sm_mixed() {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ssx_masked_batch_kernel, kThreads, 0);
  return n > 0 ? n : 1;
}

cudaError_t launch_sch_mixed_batch(const GppBatchView& b, int grid, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(sch_mixed_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       sizeof(SchSmemM));
  if (e != cudaSuccess) return e;
  sch_mixed_batch_kernel<<<grid, kThreads, sizeof(SchSmemM), s>>>(b);
  return cudaGetLastError();
}

cudaError_t launch_ssx_mixed_batch(const GppBatchView& b, int grid, bool all_shared_wx, cudaStream_t s) {
  if (all_shared_wx) {
    ssx_masked_batch_kernel<<<grid, kThreads, 0, s>>>(b);
    return cudaGetLastError();
  }
  cudaError_t e = cudaFuncSetAttribute(ssx_mixed_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       sizeof(SsxSmemF));
  if (e != cudaSuccess) return e;
  ssx_mixed_batch_kernel<<<grid, kThreads, sizeof(SsxSmemF), s>>>(b);
  return cudaGetLastError();
}

cudaError_t launch_ssx_mixed(const GppDev& p, const GppWork& w, const MixedPrep& m, int grid,
                             cudaStream_t s) {
  if (p.wx_stride == 0) {
    ssx_masked_kernel<<<grid, kThreads, 0, s>>>(p, w, m);
    return cudaGetLastError();
  }
  cudaError_t e = cudaFuncSetAttribute(ssx_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       sizeof(SsxSmemF));
  if (e != cudaSuccess) return e;
  ssx_mixed_kernel<<<grid, kThreads, sizeof(SsxSmemF), s>>>(p, w);
  return cudaGetLastError();
}

}  // namespace sigma
