// Factor pass of the tensor-core GPP form, with the occupied bands' ssx sums
// fused in; one instance or a batch of instances per launch.
//
// With one frequency set for every band the band sum is a contraction of the
// band-independent factors
//   Y[iw][my_igp][ig] = G (c + i b) / (c^2 + b^2)        (0 when the guard drops it)
//                     = (wx G - |wtilde|^2 I_eps) / (c^2 + b^2),
// G = I_eps wtilde, c = wx - Re wtilde, b = Im wtilde (BGW-Kernels/gppKer.cpp
// :394-404 with conj(aqsm) and vcoul moved to the contraction's epilogue).
// This pass forms Y in float-float arithmetic (FP32 pairs, ~2^-44 relative)
// from exact splits of the FP64 inputs, rounds it once to FP32 and writes it
// straight into the contraction's A operand as split-BF16 slices.  Keep and
// second-branch decisions are re-taken with the FP64 path's expressions
// within 2^-30 of a threshold.
//
// The occupied bands (n1 < nvband, flagOCC_solver :130-159 with
// ssxt_scht_solver :19-65) need, for the same (column, g-vector), the ssx
// factor of each frequency,
//   kept:          ssx = Omega2 / wx^2,          Omega2 = wtilde G
//   second branch: ssx = -G / (2 (wtilde + wx))  (0 < |wdiff|^2 < |wtilde|^2 / to1)
//   otherwise      0,
// summed over g-vectors with aqsn[n1][ig].  The pass forms them from the
// values it already holds and stages them in shared memory; four lanes per
// (band, frequency, column) then take 8 g-vectors of a tile each and fold
// each 4-term FP32 tree sum into the lane's own float-float accumulator;
// the four accumulators are added at the end of the item.  At the end of an item each
// column's sums are multiplied by conj(aqsm[n1][igp]) occ vcoul[igp] in FP64
// and summed over the item's columns in a fixed order.  The inputs are read
// once for both, and no intermediate operand is written.
//
// Items are (g-vector segment, column block of 16 columns), plus, per
// instance, a few items that zero the A slices' padding rows; a batch
// concatenates the items of every instance (one static schedule).
#include <algorithm>

#include "gpp_tensor.cuh"
#include "floatfloat.cuh"

namespace sigma {
namespace {

constexpr int kFacThreads = 256;
constexpr int kZeroTiles = 64;  // K tiles per padding-row item

// Slot of g-vector k in the ssx planes: the middle two of every four are
// swapped, so that a 16-byte read of g-vectors 4m .. 4m+3 holds the pairs
// (4m, 4m+2) and (4m+1, 4m+3); their paired sum is then (t0 + t1, t2 + t3)
// and the 4-term tree (t0 + t1) + (t2 + t3).
__device__ __forceinline__ int ssx_slot(int k) { return (k & ~3) | ((k & 1) << 1) | ((k >> 1) & 1); }

// Row stride of the ssx factor planes (floats): 16-byte rows, and the eight
// columns x four g-vector quarters of a warp's 16-byte reads fall in distinct
// bank groups (3 x 36 = 12 mod 32 banks per column).
constexpr int kXS = kFacK + 4;

struct FactorSmem {
  float2 y[kNW][kFacCols][kFacK + 1];          // the tile's factors for the slice writes
  union {
    struct {
      float r[kFacCols][kNW][kXS];             // the tile's ssx factors, real parts
      float i[kFacCols][kNW][kXS];             // and imaginary parts
    } x;
    double2 red[kFusedBands][kNW][kFacCols];   // item epilogue: per-column ssx sums
  };
  // occupied bands' aqsn over the tile's g-vectors: real parts, imaginary
  // parts and their negatives (operands of paired FP32 products)
  float anr[kFusedBands][kFacK], ani[kFusedBands][kFacK], anm[kFusedBands][kFacK];
  // the current job's frequency constants, formed once per CTA and job:
  // wx as float-float (hi, lo), its FP32 rounding and remainder, 1 / wx^2
  float wxc[kNW][5];
};
// Dynamic shared memory: ssx float-float accumulators (hi.x, hi.y, lo.x,
// lo.y) per (output, lane quarter), each read and written by its own lane
// only; sized for the launch's largest occupied-band count.
__host__ __device__ constexpr size_t factor_acc_bytes(int nvband) {
  return sizeof(float4) * (size_t)(nvband < kFusedBands ? nvband : kFusedBands) * kNW * kFacCols * 4;
}
// ssx sums: output o = r * 64 + 8 * warp + lane / 4 is computed by the four
// lanes 4 (lane / 4) + q (q = 0..3, 8 g-vectors each) in round r, so every
// warp takes part; each lane owns the accumulator acc[4 o + q]
constexpr int kSsxRounds = (kFusedBands * kNW * kFacCols * 4 + 255) / 256;

__device__ __forceinline__ int find_job(const FactorJob* jobs, int n, int item) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].item_off <= item) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int padding_rows(const FactorJob& j) {
  const int rows = kNW * j.p.ng;
  return (rows + kOzRows - 1) / kOzRows * kOzRows - rows;
}

// Slices of A row R, K values [k0, k0 + 8): real parts in the first half of
// the K' tiles, imaginary parts in the second (the OzakiPrep layout).
__device__ __forceinline__ void put_a(unsigned char* a_tiles, int kt, int R, int k0, const float (&re)[8],
                                      const float (&im)[8]) {
  const int rb = R / kOzRows, r = R % kOzRows, t = k0 / kOzKTile, ch = (k0 % kOzKTile) / 8;
  unsigned char* base = a_tiles + (size_t)rb * 2 * kt * kOzOperandBytes;
  oz_put_row_chunk(base + (size_t)t * kOzOperandBytes, r, ch, re);
  oz_put_row_chunk(base + (size_t)(kt + t) * kOzOperandBytes, r, ch, im);
}

// (w g - se) r rounded once to FP32, for an FP32-exact w (w.lo == 0): w g
// as an exact product pair, the difference by TwoSum, no normalisation
// before the final rounding (same accuracy as the general form).
__device__ __forceinline__ float ff_factor_round(float w, FF g, FF se, FF r) {
  const float p = w * g.hi;
  const float e = fmaf(w, g.lo, fmaf(w, g.hi, -p));
  float s, t;
  two_sum_f(p, -se.hi, s, t);
  t += e - se.lo;
  return fmaf(s, r.hi, fmaf(s, r.lo, t * r.hi));
}

// a g - b h of float-float values rounded once to FP32: the products' exact
// errors by FMA, the difference of the hi products by TwoSum, so the result
// is within 1/2 ulp plus ~2^-46 of the products' magnitude (lo * lo terms
// dropped).
__device__ __forceinline__ float ff_dot2_round(FF a, FF g, FF b, FF h) {
  const float p1 = a.hi * g.hi, p2 = b.hi * h.hi;
  const float e1 = fmaf(a.hi, g.hi, -p1), e2 = fmaf(b.hi, h.hi, -p2);
  const float t = fmaf(a.hi, g.lo, fmaf(a.lo, g.hi, e1)) - fmaf(b.hi, h.lo, fmaf(b.lo, h.hi, e2));
  float s, es;
  two_sum_f(p1, -p2, s, es);  // the difference exact: one rounding at the end
  return s + (es + t);
}

// Decisions of one element that the fast path leaves open, out of line so
// that the common path carries no branch for them: the keep decisions of
// the frequencies in rare bits 0-2 (within 2^-30 of a threshold, or the
// guard's second condition binding: |wtilde|^2 >= 62000), and the
// second-branch tests of dropped terms in bits 3-5 that are not clearly
// inside it.  Returns the element's mask (keep bits 0-2, second-branch bits
// 3-5) with those decisions taken as the FP64 path takes them.
static __device__ __noinline__ unsigned factor_rare(unsigned mask, unsigned rare, const double* wxp,
                                                    double wtx, double wty, bool thr2_binds, bool big_s) {
  const FF a = ff_of(wtx), b = ff_of(wty);
  const FF b2 = ff_mul(b, b);
  const FF s2 = ff_add(ff_mul(a, a), b2);
  const FF quarter{0.25f, 0.f};
  for (int iw = 0; iw < kNW; ++iw) {
    const FF wv = ff_sq_add(ff_sub_raw(ff_of(wxp[iw]), a), b2);
    bool keep = (mask >> iw) & 1u;
    if ((rare >> iw) & 1u) {
      bool near;
      keep = ff_gt_fast(wv, quarter, near);
      if (thr2_binds) {
        bool n2;
        keep = keep && ff_gt(ff_mul(wv, FF{250000.f, 0.f}), s2, n2);
        near = near || n2;
      }
      if (near) keep = keep_fp64(wxp[iw], wtx, wty);
    }
    const bool plain = big_s && wv.hi >= 1e-30f;
    bool second = !keep && plain;
    if ((rare >> (3 + iw)) & 1u || (!keep && !plain)) {
      bool n3;
      const FF s_big = ff_mul(s2, FF{1e6f, 0.f});  // |wtilde|^2 / to1 (1e6 exact)
      second = !keep && wv.hi > 0.f && ff_gt_fast(s_big, wv, n3);
      if (!keep && (n3 || wv.hi < 1e-30f)) second = second_fp64(wxp[iw], wtx, wty);
    }
    mask = (mask & ~((1u << iw) | (8u << iw))) | (keep ? (1u << iw) : 0u) | (second ? (8u << iw) : 0u);
  }
  return mask;
}

// kGroup: the jobs of a batch from a device array; else the one job `single`
// (a kernel parameter, so that an execution can be captured in a graph).
template <bool kGroup>
__global__ void __launch_bounds__(kFacThreads, 4) factor_kernel(const FactorJob single,
                                                                 const FactorJob* __restrict__ jobs, int n_jobs,
                                                                 int total) {
  __shared__ FactorSmem sm;
  extern __shared__ float4 acc_dyn[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int cached = -1;  // job whose frequency constants sm.wxc holds
  for (int item = blockIdx.x; item < total; item += gridDim.x) {
    const int ji = kGroup ? find_job(jobs, n_jobs, item) : 0;
    const FactorJob& J = kGroup ? jobs[ji] : single;
    const GppDev& p = J.p;
    const int local = item - J.item_off;
    const int main_items = J.ncb * J.n_seg;
    __syncthreads();  // the previous item is done with shared memory
    if (local >= main_items) {
      // zero the A slices of the padding rows for kZeroTiles K tiles
      const int rows = kNW * p.ng, pad = padding_rows(J);
      const int t0 = (local - main_items) * kZeroTiles, t1 = min(J.kt, t0 + kZeroTiles);
      const float z[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      for (int e = tid; e < (t1 - t0) * pad * 4; e += kFacThreads) {
        const int ch = e % 4, r = (e / 4) % pad, t = t0 + e / (4 * pad);
        put_a(J.a_tiles, J.kt, rows + r, t * kOzKTile + ch * 8, z, z);
      }
      continue;
    }
    {  // this item's share of the B slices and epilogue factors
      const long long b0 = (long long)local * J.b_per_item, w0 = (long long)local * J.w_per_item;
      const long long b1 = min(b0 + J.b_per_item, oz_prep_b_count(J.oz));
      const long long w1 = min(w0 + J.w_per_item, oz_weights_count(J.oz));
      for (long long e = b0 + tid; e < b1; e += kFacThreads) oz_prep_b_elem(J.d, J.oz, e);
      for (long long e = w0 + tid; e < w1; e += kFacThreads) oz_weights_elem(J.d, J.oz, e);
    }
    const int s = local / J.ncb, cb = local % J.ncb;
    const int t_begin = s * J.seg_tiles, t_end = min(J.kt, t_begin + J.seg_tiles);
    const int nvb = p.nvband <= kFusedBands ? p.nvband : 0;
    const int outputs = nvb * kNW * kFacCols;  // ssx sums: (band, frequency, column)
    if (ji != cached) {  // the same for the whole CTA
      if (tid < kNW) {
        const double w = p.wx[tid];
        const FF f = ff_of(w);
        const float h = __double2float_rn(w);
        sm.wxc[tid][0] = f.hi;
        sm.wxc[tid][1] = f.lo;
        sm.wxc[tid][2] = h;
        sm.wxc[tid][3] = __double2float_rn(w - (double)h);
        sm.wxc[tid][4] = __double2float_rn(rcp_f64(w * w));
      }
      __syncthreads();
      cached = ji;
    }
    FF wx[kNW];
    float wxh[kNW], wxl[kNW], iwx2[kNW];
    bool wx32 = true;  // every frequency exact in FP32 (the mini-app's 3, 4, 5)
#pragma unroll
    for (int iw = 0; iw < kNW; ++iw) {
      wx[iw] = FF{sm.wxc[iw][0], sm.wxc[iw][1]};
      wx32 = wx32 && wx[iw].lo == 0.f;
      wxh[iw] = sm.wxc[iw][2];
      wxl[iw] = sm.wxc[iw][3];
      iwx2[iw] = sm.wxc[iw][4];
    }
    // float-float accumulators of the ssx sums this thread owns
    for (int r = 0; r < kSsxRounds; ++r) {
      const int o = r * (kFacThreads / 4) + warp * 8 + (lane >> 2);
      if (o < outputs) acc_dyn[4 * o + (lane & 3)] = make_float4(0.f, 0.f, 0.f, 0.f);
    }

    for (int t = t_begin; t < t_end; ++t) {
      const int ig0 = t * kFacK;
      for (int e = tid; e < nvb * kFacK; e += kFacThreads) {
        const int n1 = e / kFacK, k = e % kFacK, ig = ig0 + k;
        float2 v = make_float2(0.f, 0.f);
        if (ig < p.nc) {
          const double2 d = p.aqsn[(size_t)n1 * p.nc + ig];
          v = make_float2(__double2float_rn(d.x), __double2float_rn(d.y));
        }
        const int ks = ssx_slot(k);
        sm.anr[n1][ks] = v.x;
        sm.ani[n1][ks] = v.y;
        sm.anm[n1][ks] = -v.y;
      }
#pragma unroll 1
      for (int j = 0; j < 2; ++j) {
        const int pl = warp + 8 * j, my_igp = cb * kFacCols + pl, ig = ig0 + lane;
        float2 yt[kNW] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
        float2 sv[kNW] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
        if (my_igp < p.ng && ig < p.nc) {
          const size_t off = (size_t)my_igp * p.nc + ig;
          const double2 wt = p.wt[off];
          const double2 ie = p.ieps[off];
          const FF a = ff_of(wt.x), b = ff_of(wt.y), er = ff_of(ie.x), ei = ff_of(ie.y);
          const FF gx = ff_dot2_raw(er, a, ei, b);           // G = I_eps wtilde
          const FF gy = ff_dot2_raw(er, b, ff_neg(ei), a);
          const FF b2 = ff_mul_raw(b, b);
          const FF s2 = ff_dot2_raw(a, a, b, ff_neg(b));     // |wtilde|^2
          // G (c + i b) = wx G - G conj(wtilde) = wx G - |wtilde|^2 I_eps
          const FF sex = ff_mul_raw(s2, er), sey = ff_mul_raw(s2, ei);
          // |wtilde|^2 * 4e-6 >= 0.25 only for |wtilde|^2 >= 62500; below,
          // |wdiff|^2 > 0.25 implies the guard's second condition
          const bool thr2_binds = s2.hi >= 62000.f;
          // |wtilde|^2 / to1 > 1 >= |wdiff|^2 of a dropped term: its second
          // occupied-band branch is then the exact-pole test alone
          const bool big_s = s2.hi > 1.01e-6f;
          unsigned mask = 0u, rare = thr2_binds ? 7u : 0u;
          float2 yv[kNW];
#pragma unroll
          for (int iw = 0; iw < kNW; ++iw) {
            const FF wv = ff_sq_add(ff_sub_raw(wx[iw], a), b2);  // |wdiff|^2
            // keep: |wdiff|^2 > max(0.25, |wtilde|^2 * 4e-6), i.e. both
            // wv > 0.25 and wv * 250000 > |wtilde|^2 (250000 exact in FP32);
            // the second condition only binds for thr2_binds (rare path)
            bool near;
            const bool keep = ff_gt_quarter(wv, near);
            // the factor of every term (the warp's lanes almost always
            // disagree on keep), selected by the final keep bit below
            const FF r = ff_rcp_raw(wv);
            if (wx32) {
              yv[iw] = make_float2(ff_factor_round(wx[iw].hi, gx, sex, r), ff_factor_round(wx[iw].hi, gy, sey, r));
            } else {
              yv[iw] = make_float2(ff_mul_round(ff_add(ff_mul(wx[iw], gx), ff_neg(sex)), r),
                                   ff_mul_round(ff_add(ff_mul(wx[iw], gy), ff_neg(sey)), r));
            }
            // second occupied-band branch: 0 < |wdiff|^2 < |wtilde|^2 / to1,
            // which for |wtilde|^2 > 1e-6 and a dropped term is |wdiff|^2 > 0
            const bool plain = big_s && wv.hi >= 1e-30f;
            mask |= (keep ? (1u << iw) : 0u) | ((!keep && plain) ? (8u << iw) : 0u);
            rare |= (near ? (1u << iw) : 0u) | ((nvb > 0 && !keep && !plain) ? (8u << iw) : 0u);
          }
          if (rare) mask = factor_rare(mask, rare, p.wx, wt.x, wt.y, thr2_binds, big_s);
          if (nvb == 0) mask &= 7u;
#pragma unroll
          for (int iw = 0; iw < kNW; ++iw) yt[iw] = (mask & (1u << iw)) ? yv[iw] : make_float2(0.f, 0.f);
          if (nvb > 0) {
            const float2 g32 = make_float2(ff_round(gx), ff_round(gy));
            const float bb = ff_round(b);
            // Omega2 = wtilde G
            const float2 om = make_float2(ff_dot2_round(a, gx, b, gy), ff_dot2_round(a, gy, ff_neg(b), gx));
#pragma unroll
            for (int iw = 0; iw < kNW; ++iw) {
              const float zr = (wxh[iw] + a.hi) + (wxl[iw] + a.lo);
              const float q = -0.5f * rcp_f32(fmaf(zr, zr, bb * bb));
              const float2 s1 = make_float2(om.x * iwx2[iw], om.y * iwx2[iw]);
              const float2 s2v = make_float2(fmaf(g32.x, zr, g32.y * bb) * q, fmaf(g32.y, zr, -g32.x * bb) * q);
              sv[iw] = (mask & (1u << iw)) ? s1 : ((mask & (8u << iw)) ? s2v : make_float2(0.f, 0.f));
            }
          }
        }
#pragma unroll
        for (int iw = 0; iw < kNW; ++iw) {
          sm.y[iw][pl][lane] = yt[iw];
          sm.x.r[pl][iw][ssx_slot(lane)] = sv[iw].x;
          sm.x.i[pl][iw][ssx_slot(lane)] = sv[iw].y;
        }
      }
      __syncthreads();
      // split-BF16 slices of the A rows (iw, column): 8 g-vectors per chunk,
      // consecutive threads fill one 8-row group
      for (int c = tid; c < kNW * kFacCols * 4; c += kFacThreads) {
        const int ch = c % 4, pl = (c / 4) % kFacCols, iw = c / (4 * kFacCols);
        const int col = cb * kFacCols + pl;
        if (col >= p.ng) continue;
        float re[8], im[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const float2 v = sm.y[iw][pl][ch * 8 + q];
          re[q] = v.x;
          im[q] = v.y;
        }
        put_a(J.a_tiles, J.kt, iw * p.ng + col, ig0 + ch * 8, re, im);
      }
      // the tile's ssx products: output o = (band n1, frequency iw, column
      // pl); lane quarter q takes g-vectors 8q .. 8q+7 and folds two 4-term
      // FP32 tree sums into its float-float accumulator.  Paired FP32
      // instructions: the products of g-vector pairs (4m, 4m + 2) and
      // (4m + 1, 4m + 3) (the planes' slot order), then the x and y
      // components' float-float additions as one pair.
      const float2 m1 = make_float2(-1.f, -1.f);
#pragma unroll 1
      for (int r = 0; r < kSsxRounds; ++r) {
        const int o = r * (kFacThreads / 4) + warp * 8 + (lane >> 2), q = lane & 3;
        if (o < outputs) {
          const int n1 = o / (kNW * kFacCols), iw = (o / kFacCols) % kNW, pl = o % kFacCols;
          const float4 a = acc_dyn[4 * o + q];
          float2 hi = make_float2(a.x, a.y), lo = make_float2(a.z, a.w);
#pragma unroll
          for (int half = 0; half < 2; ++half) {
            const int kk = 8 * q + 4 * half;
            const float4 ar = *reinterpret_cast<const float4*>(&sm.anr[n1][kk]);
            const float4 ai = *reinterpret_cast<const float4*>(&sm.ani[n1][kk]);
            const float4 am = *reinterpret_cast<const float4*>(&sm.anm[n1][kk]);
            const float4 xr = *reinterpret_cast<const float4*>(&sm.x.r[pl][iw][kk]);
            const float4 xi = *reinterpret_cast<const float4*>(&sm.x.i[pl][iw][kk]);
            // t = an x: t.x = an.x x.x - an.y x.y, t.y = an.x x.y + an.y x.x
            const float2 px0 = __ffma2_rn(f4_lo(ar), f4_lo(xr), __fmul2_rn(f4_lo(am), f4_lo(xi)));
            const float2 px1 = __ffma2_rn(f4_hi(ar), f4_hi(xr), __fmul2_rn(f4_hi(am), f4_hi(xi)));
            const float2 py0 = __ffma2_rn(f4_lo(ar), f4_lo(xi), __fmul2_rn(f4_lo(ai), f4_lo(xr)));
            const float2 py1 = __ffma2_rn(f4_hi(ar), f4_hi(xi), __fmul2_rn(f4_hi(ai), f4_hi(xr)));
            const float2 tx = __fadd2_rn(px0, px1), ty = __fadd2_rn(py0, py1);
            ff_add2(hi, lo, make_float2(tx.x + tx.y, ty.x + ty.y), m1);
          }
          acc_dyn[4 * o + q] = make_float4(hi.x, hi.y, lo.x, lo.y);
        }
      }
      __syncthreads();  // the aqsn planes, sm.x and sm.y are refilled by the next tile
    }

    if (nvb > 0) {
      // each column's sums x conj(aqsm[n1][igp]) occ vcoul[igp] in FP64
      // (sm.red aliases sm.x, whose last reads precede the tile loop's
      // final barrier)
      for (int r = 0; r < kSsxRounds; ++r) {
        const int o = r * (kFacThreads / 4) + warp * 8 + (lane >> 2);
        if ((lane & 3) == 0 && o < outputs) {
          const int n1 = o / (kNW * kFacCols), iw = (o / kFacCols) % kNW, pl = o % kFacCols;
          const int my_igp = cb * kFacCols + pl;
          const int igp = my_igp < p.ng ? p.igp_of[my_igp] : -1;
          double2 v = make_double2(0.0, 0.0);
          if (igp >= 0) {
            const double2 am = p.aqsm[(size_t)n1 * p.nc + igp];
            const double f = p.occ * p.vcoul[igp];
            // the four quarters' float-float sums added in float-float,
            // then widened once
            float4 a = acc_dyn[4 * o];
            FF fx{a.x, a.z}, fy{a.y, a.w};
#pragma unroll
            for (int q = 1; q < 4; ++q) {
              a = acc_dyn[4 * o + q];
              fx = ff_add(fx, FF{a.x, a.z});
              fy = ff_add(fy, FF{a.y, a.w});
            }
            const double sx = (double)fx.hi + (double)fx.lo, sy = (double)fy.hi + (double)fy.lo;
            // (sx + i sy) conj(am) f
            v = make_double2(fma(sx, am.x, sy * am.y) * f, fma(sy, am.x, -sx * am.y) * f);
          }
          sm.red[n1][iw][pl] = v;
        }
      }
      __syncthreads();
      if (tid < nvb * kNW) {
        const int n1 = tid / kNW, iw = tid % kNW;
        Comp sx, sy;
        for (int q = 0; q < kFacCols; ++q) {
          sx.add(sm.red[n1][iw][q].x);
          sy.add(sm.red[n1][iw][q].y);
        }
        const GppWork& w = J.ssx;
        const size_t pidx = ((size_t)(n1 / kSsxBN) * w.n_col_blocks + cb) * w.n_splits + s;
        w.partial[pidx * kSsxBN * kNW + (n1 % kSsxBN) * kNW + iw] = make_double2(sx.value(), sy.value());
      }
    }
  }
}

}  // namespace

void factor_job_size(FactorJob& j, const GppDev& p, int kt, int grid, double share) {
  j.p = p;
  j.kt = kt;
  j.ncb = (p.ng + kFacCols - 1) / kFacCols;
  // about 12 items per CTA over this instance's share of the launch
  const double want = std::max(1.0, 12.0 * grid * share);
  int seg = (int)std::max(1.0, std::min((double)kt, want / j.ncb + 0.5));
  j.seg_tiles = (kt + seg - 1) / seg;
  j.n_seg = (kt + j.seg_tiles - 1) / j.seg_tiles;
  GppWork& w = j.ssx;
  w = GppWork{};
  w.band_begin = 0;
  w.band_count = factor_fuses_ssx(p.nvband) ? p.nvband : 0;
  w.bn = kSsxBN;
  w.n_band_blocks = (w.band_count + kSsxBN - 1) / kSsxBN;
  w.n_col_blocks = j.ncb;
  w.n_splits = j.n_seg;
  w.split_len = j.seg_tiles * kFacK;
  w.n_items = w.n_band_blocks * j.ncb * j.n_seg;
}

void factor_job_operands(FactorJob& j, const FfDev& d, const OzakiPrep& oz) {
  j.d = d;
  j.oz = oz;
  j.oz.stab = nullptr;
  const long long main_items = std::max(1LL, (long long)j.ncb * j.n_seg);
  const long long b = (long long)oz.n_col_blocks * oz.kt * 64 * (kOzKTile / 8);
  const long long w = (long long)oz.ng * oz.nb_pad;
  j.b_per_item = (b + main_items - 1) / main_items;
  j.w_per_item = (w + main_items - 1) / main_items;
}

size_t factor_ssx_partial_bytes(const FactorJob& j) {
  return sizeof(double2) * (size_t)j.ssx.n_band_blocks * j.ncb * j.n_seg * kSsxBN * kNW;
}

int factor_job_items(const FactorJob& j) {
  const int rows = kNW * j.p.ng;
  const int pad = (rows + kOzRows - 1) / kOzRows * kOzRows - rows;
  return j.ncb * j.n_seg + (pad > 0 ? (j.kt + kZeroTiles - 1) / kZeroTiles : 0);
}

// Dynamic shared memory above the default 48 KB per block needs the opt-in.
template <bool kGroup>
cudaError_t factor_smem_attr() {
  return cudaFuncSetAttribute(factor_kernel<kGroup>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)factor_acc_bytes(kFusedBands));
}

int factor_blocks_per_sm(int max_nvband) {
  factor_smem_attr<true>();
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, factor_kernel<true>, kFacThreads,
                                                factor_acc_bytes(max_nvband));
  return n > 0 ? n : 1;
}

cudaError_t launch_factor_pass(const FactorJob* jobs, int n_jobs, int total, int grid, int max_nvband,
                               cudaStream_t s) {
  if (total <= 0) return cudaSuccess;
  cudaError_t e = factor_smem_attr<true>();
  if (e != cudaSuccess) return e;
  factor_kernel<true><<<std::min(grid, total), kFacThreads, factor_acc_bytes(max_nvband), s>>>(
      FactorJob{}, jobs, n_jobs, total);
  return cudaGetLastError();
}

cudaError_t launch_factor_pass(const FactorJob& job, int grid, cudaStream_t s) {
  const int total = factor_job_items(job);
  if (total <= 0) return cudaSuccess;
  cudaError_t e = factor_smem_attr<false>();
  if (e != cudaSuccess) return e;
  factor_kernel<false><<<std::min(grid, total), kFacThreads, factor_acc_bytes(job.p.nvband), s>>>(
      job, nullptr, 1, total);
  return cudaGetLastError();
}

}  // namespace sigma
