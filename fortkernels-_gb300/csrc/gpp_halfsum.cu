// gppsum = 1 ("half sum") GPP variant of gppKerSeq.cpp, FP64.
//
// For column my_igp (igp = its mapped g-vector) and band n1 the reference
// sums over g-vectors ig < igp only, pairing each term with its Hermitian
// partner:
//   term = conj(aqsm[n1][igp]) aqsn[n1][ig] Z + v_p conj(aqsm[n1][ig]) conj(Z)
// so with T = sum aqsn[n1][ig] Z and U = sum aqsm[n1][ig] Z over the column's
// g-vector set,  scht = conj(aqsm[n1][igp]) T + v_p conj(U).
//
//   non-occupied bands (noflagOCC_solver, gppKerSeq.cpp:206-242, driven in
//     512-wide blocks at :457-470): Z = delw I_eps with delw = wtilde / wdiff,
//     kept where |wdiff|^2 < 0.25 or |delw|^2 > limitone (the complement of
//     the gppsum = 0 guard), v_p = aqsm[n1][igp].  The block loop visits
//     g-vectors ig < igp - 1 with ig mod 512 != 511, plus ig = igp alone
//     (no partner term) when igp is a positive multiple of 512.
//   static remainder (reduce_achstemp, gppKerSeq.cpp:13-72): Z = -I_eps over
//     ig < igp, v_p = aqsn[n1][igp], plus ig = igp alone when |I_eps| > to1.
//   occupied bands (flagOCC_solver, gppKerSeq.cpp:90-139): per g-vector
//     sch = G / (wx - wtilde) unless |wx - wtilde| < 0.5 or |delw|^2 < to1
//     (delw = (wx - wtilde) / (2 wtilde)), ssx = Omega2 / (wx^2 - wtilde^2) or
//     -G / (2 (wx + wtilde)) (= -Omega2 / (4 wtilde^2 (1 + delw))); the loop
//     stops at the first g-vector with |Omega2| < to1; the term at
//     ig = igp - 1 has no partner.
//
// Z does not depend on the band (one frequency set for every band), so the
// non-occupied pass and the static remainder are two complex FP64 GEMMs over
// a triangular g-vector range: items of 32 bands x 32 columns x a g-vector
// split stage Z once per 16-g-vector chunk for all 32 bands; each thread
// keeps 2 bands x 2 columns x NF frequencies of T and U, each complex
// multiply-add as three real products (the chunk's sums x.x + x.y staged
// beside the operands: P1 = sum x.x z.x, P2 = sum x.y z.y, P3 = sum
// (x.x + x.y)(z.x + z.y), sum x z = (P1 - P2) + i (P3 - P1 - P2)), 6 DFMA per
// term.
// Items past a column block's range write zero partials.  Occupied bands run
// one CTA per (column, frequency).  All partials have fixed slots and are
// summed in a fixed order with compensation: results are identical run to
// run.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "sigma_gpp.h"
#include "sigma_internal.cuh"
#include "floatfloat.cuh"
#include "ff_plan.h"
#include "ff_ozaki.cuh"
#include "runtime.h"

namespace sigma {
namespace {

constexpr int kHBN = 64, kHBP = 16;  // bands x columns per item
static_assert(kHBP <= 32, "one warp finds the item's g-vector limit");
constexpr int kHCK = 16;             // g-vectors per staged chunk
constexpr int kHTB = kHBN / 16, kHTC = kHBP / 16;
constexpr int kOccBands = 4;         // occupied bands per accumulation pass (FP64)
constexpr int kOccBandsF = 2;        // the same for the float-float form
constexpr int kIgBlk = 512;          // g-vector block of the reference's loop

struct HalfDev {
  int nb, nvband, nc, ng;
  double occ;
  const double2 *aqsm, *aqsn, *ieps, *wt;  // [nb][nc], [nb][nc], [ng][nc], [ng][nc]
  const double* vcoul;                     // [nc]
  const double* wx;                        // [3]
  const int* igp_of;                       // [ng], -1 = skipped column
  const int* brk;                          // [ng] occupied-band cut
};

// Rows padded by one element: the staging writes run along g-vectors (the
// coalesced direction of the global reads), so unpadded rows, whose strides
// are multiples of 128 bytes, put a warp's writes in one bank group.
template <int NF>
struct HalfSmem {
  // each thread's FP64 sums T and U (4 bands x 1 column x NF frequencies),
  // one slot row per output
  double2 acc[2 * kHTB * kHTC * NF][kThreads];
  // Z as float-float operands of paired instructions (lanes: real and
  // imaginary parts): [k][f * kHBP + column] (Re.hi, Im.hi, -Re.lo, -Im.lo)
  // of Z, [k][NF * kHBP + f * kHBP + column] those of i Z
  float4 z[kHCK][2 * NF * kHBP + 1];
  // aqsn and aqsm as broadcast pairs: [k][band] (Re.hi, Re.hi, Re.lo, Re.lo),
  // [k][kHBN + band] the same of Im
  float4 n[kHCK][2 * kHBN + 1];
  float4 m[kHCK][2 * kHBN + 1];
};

// n Z + (float-float sum h, l): the paired float-float product of a
// broadcast pair n (high rh, ih; low rl, il) and a staged factor (a: high
// pair, its negation, negated low pair; the same three of i Z), its high
// pair added exactly to h (TwoSum), the errors and low halves to l.
__device__ __forceinline__ void half_ff_mac(float2& h, float2& l, float2 rh, float2 rl, float2 ih, float2 il,
                                            float2 ah, float2 anh, float2 anl, float2 bh, float2 bnh,
                                            float2 bnl) {
  const float2 m1 = make_float2(-1.f, -1.f);
  const float2 p1 = __fmul2_rn(rh, ah), p2 = __fmul2_rn(ih, bh);
  const float2 g1 = __ffma2_rn(rh, anl, __ffma2_rn(rl, anh, __ffma2_rn(rh, anh, p1)));
  const float2 g2 = __ffma2_rn(ih, bnl, __ffma2_rn(il, bnh, __ffma2_rn(ih, bnh, p2)));
  const float2 s = __fadd2_rn(p1, p2);
  const float2 bv = __ffma2_rn(p1, m1, s);
  const float2 av = __ffma2_rn(bv, m1, s);
  const float2 es = __fadd2_rn(__ffma2_rn(av, m1, p1), __ffma2_rn(bv, m1, p2));
  const float2 lo = __ffma2_rn(__fadd2_rn(g1, g2), m1, es);
  const float2 hs = __fadd2_rn(h, s);
  const float2 hb = __ffma2_rn(h, m1, hs);
  const float2 ha = __ffma2_rn(hb, m1, hs);
  const float2 he = __fadd2_rn(__ffma2_rn(ha, m1, h), __ffma2_rn(hb, m1, s));
  h = hs;
  l = __fadd2_rn(l, __fadd2_rn(he, lo));
}

__device__ __forceinline__ void cfma(double2& acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, fma(-a.y, b.y, acc.x));
  acc.y = fma(a.x, b.y, fma(a.y, b.x, acc.y));
}
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }

// End of the (non-diagonal) g-vector range of a column: [0, lim).
template <int NF>
__device__ __forceinline__ int column_limit(int igp) {
  if (igp < 0) return 0;
  return NF == 1 ? igp : max(igp - 1, 0);
}

// Z of the non-occupied half sum at one (column, g-vector) for the three
// frequencies: G (c + i b) / (c^2 + b^2), G = I_eps wtilde, c = wx - Re wtilde,
// b = Im wtilde (= delw I_eps), kept where |wdiff|^2 is below the threshold.
__device__ __forceinline__ void half_factor(double2 wt, double2 ie, const double* wx,
                                            double2 (&z)[3]) {
  const double a = wt.x, b = wt.y;
  const double b2 = guard_b2(b);
  const double thr = guard_thr(a, b2);
  const double2 g = cmul(ie, wt);
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    const double c = __dsub_rn(wx[f], a);
    const double wv = fma(c, c, b2);
    const double r = rcp_f64_seed32(wv);
    const double2 y = make_double2(fma(g.x, c, -g.y * b) * r, fma(g.x, b, g.y * c) * r);
    z[f] = gt_nonneg(thr, wv) ? y : make_double2(0.0, 0.0);
  }
}

// A chunk holding a value outside the float-float range: FP64 complex
// multiply-adds of the thread's tile, Z formed again from the inputs and
// aqsn / aqsm read again, added to the FP64 sums.  Out of line.
template <int NF>
static __device__ __noinline__ void half_wide_chunk(const HalfDev& p, double2 (*acc)[kThreads], int tid, int ig0,
                                                    int ig_end, int n1_0, int p0, const double* wx) {
  constexpr int NO = kHTB * kHTC * NF;
  const int tx = tid & 15, ty = tid >> 4;
  double2 ta[NO], ua[NO];
  for (int o = 0; o < NO; ++o) ta[o] = ua[o] = make_double2(0.0, 0.0);
  for (int k = 0; k < kHCK; ++k) {
    const int ig = ig0 + k;
    double2 z[kHTC][3];
    for (int j = 0; j < kHTC; ++j) {
      const int col = p0 + tx + 16 * j;
      const int lim = column_limit<NF>(col < p.ng ? p.igp_of[col] : -1);
      bool in = ig < ig_end && ig < lim;
      if (NF == 3) in = in && (ig % kIgBlk) != kIgBlk - 1;
      for (int f = 0; f < 3; ++f) z[j][f] = make_double2(0.0, 0.0);
      if (in) {
        const size_t off = (size_t)col * p.nc + ig;
        const double2 ie = p.ieps[off];
        if (NF == 1)
          z[j][0] = make_double2(-ie.x, -ie.y);
        else
          half_factor(p.wt[off], ie, wx, z[j]);
      }
    }
    for (int i = 0; i < kHTB; ++i) {
      const int n1 = n1_0 + ty + 16 * i;
      const bool in = ig < ig_end && n1 < p.nb;
      const size_t off = (size_t)n1 * p.nc + ig;
      const double2 nv = in ? p.aqsn[off] : make_double2(0.0, 0.0);
      const double2 mv = in ? p.aqsm[off] : make_double2(0.0, 0.0);
      for (int j = 0; j < kHTC; ++j)
        for (int f = 0; f < NF; ++f) {
          const int o = (i * kHTC + j) * NF + f;
          cfma(ta[o], nv, z[j][f]);
          cfma(ua[o], mv, z[j][f]);
        }
    }
  }
  for (int o = 0; o < NO; ++o) {
    acc[o][tid].x += ta[o].x;
    acc[o][tid].y += ta[o].y;
    acc[NO + o][tid].x += ua[o].x;
    acc[NO + o][tid].y += ua[o].y;
  }
}

template <int NF>
__global__ void __launch_bounds__(kThreads, 1) half_main_kernel(HalfDev p, GppWork w) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  HalfSmem<NF>& sm = *reinterpret_cast<HalfSmem<NF>*>(smem_raw);
  __shared__ int s_item, s_kmax;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const double wx[3] = {p.wx[0], p.wx[1], p.wx[2]};
  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(w.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= w.n_items) break;
    const ItemCoord ic = decode_item(w, item);
    const int n1_0 = w.band_begin + ic.bb * kHBN, p0 = ic.cb * kHBP;
    if (tid < 32) {
      const int col = p0 + tid;
      const int lim = column_limit<NF>(tid < kHBP && col < p.ng ? p.igp_of[col] : -1);
      const int mx = __reduce_max_sync(0xffffffffu, lim);
      if (tid == 0) s_kmax = mx;
    }
    __syncthreads();
    const int ig_begin = ic.s * w.split_len;
    const int ig_end = min(min(ig_begin + w.split_len, p.nc), s_kmax);

    // T = sum aqsn Z, U = sum aqsm Z: every term a float-float product in
    // paired instructions (real and imaginary parts as the lanes) added to a
    // per-chunk float-float sum; after each chunk the sum is renormalised,
    // its high pair added to the FP64 sums in shared memory and its low pair
    // carried on.  A chunk with a value outside the float-float range runs
    // FP64 multiply-adds on factors formed again from the inputs.
    constexpr int NO = kHTB * kHTC * NF;  // outputs of each of T and U
    const float2 m1 = make_float2(-1.f, -1.f);
    float2 th[NO], tl[NO], uh[NO], ul[NO];
#pragma unroll
    for (int o = 0; o < NO; ++o) {
      sm.acc[o][tid] = make_double2(0.0, 0.0);
      sm.acc[NO + o][tid] = make_double2(0.0, 0.0);
      th[o] = tl[o] = uh[o] = ul[o] = make_float2(0.f, 0.f);
    }

    for (int ig0 = ig_begin; ig0 < ig_end; ig0 += kHCK) {
      __syncthreads();
      bool chunk_wide = false;
      for (int e = tid; e < kHCK * kHBP; e += kThreads) {
        const int k = e % kHCK, pl = e / kHCK;
        const int ig = ig0 + k, col = p0 + pl;
        const int lim = column_limit<NF>(col < p.ng ? p.igp_of[col] : -1);
        bool in = ig < ig_end && ig < lim;
        if (NF == 3) in = in && (ig % kIgBlk) != kIgBlk - 1;
        double2 z[3] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
        if (in) {
          const size_t off = (size_t)col * p.nc + ig;
          const double2 ie = p.ieps[off];
          if (NF == 1)
            z[0] = make_double2(-ie.x, -ie.y);
          else
            half_factor(p.wt[off], ie, wx, z);
        }
#pragma unroll
        for (int f = 0; f < NF; ++f) {
          const FF vx = ff_of_rn(z[f].x), vy = ff_of_rn(z[f].y);
          sm.z[k][f * kHBP + pl] = make_float4(vx.hi, vy.hi, -vx.lo, -vy.lo);
          sm.z[k][NF * kHBP + f * kHBP + pl] = make_float4(-vy.hi, vx.hi, vy.lo, -vx.lo);
          chunk_wide = chunk_wide || !ff_range(z[f].x, z[f].y);
        }
      }
      for (int e = tid; e < kHCK * kHBN; e += kThreads) {
        const int k = e % kHCK, bl = e / kHCK;
        const int ig = ig0 + k, n1 = n1_0 + bl;
        const bool in = ig < ig_end && n1 < p.nb;
        const size_t off = (size_t)n1 * p.nc + ig;
        const double2 nv = in ? p.aqsn[off] : make_double2(0.0, 0.0);
        const double2 mv = in ? p.aqsm[off] : make_double2(0.0, 0.0);
        const FF nx = ff_of_rn(nv.x), ny = ff_of_rn(nv.y), mx = ff_of_rn(mv.x), my = ff_of_rn(mv.y);
        sm.n[k][bl] = make_float4(nx.hi, nx.hi, nx.lo, nx.lo);
        sm.n[k][kHBN + bl] = make_float4(ny.hi, ny.hi, ny.lo, ny.lo);
        sm.m[k][bl] = make_float4(mx.hi, mx.hi, mx.lo, mx.lo);
        sm.m[k][kHBN + bl] = make_float4(my.hi, my.hi, my.lo, my.lo);
        chunk_wide = chunk_wide || !ff_range(nv.x, nv.y) || !ff_range(mv.x, mv.y);
      }
      chunk_wide = __syncthreads_or(chunk_wide);
      if (!chunk_wide) {
#pragma unroll 1
        for (int k = 0; k < kHCK; ++k) {
          float2 ah[kHTC][NF], anh[kHTC][NF], anl[kHTC][NF], bh[kHTC][NF], bnh[kHTC][NF], bnl[kHTC][NF];
#pragma unroll
          for (int j = 0; j < kHTC; ++j)
#pragma unroll
            for (int f = 0; f < NF; ++f) {
              const float4 a = sm.z[k][f * kHBP + tx + 16 * j];
              const float4 b = sm.z[k][NF * kHBP + f * kHBP + tx + 16 * j];
              ah[j][f] = f4_lo(a);
              anl[j][f] = f4_hi(a);
              anh[j][f] = __fmul2_rn(ah[j][f], m1);
              bh[j][f] = f4_lo(b);
              bnl[j][f] = f4_hi(b);
              bnh[j][f] = __fmul2_rn(bh[j][f], m1);
            }
#pragma unroll
          for (int i = 0; i < kHTB; ++i) {
            const float4 nr = sm.n[k][ty + 16 * i], ni = sm.n[k][kHBN + ty + 16 * i];
            const float4 mr = sm.m[k][ty + 16 * i], mi = sm.m[k][kHBN + ty + 16 * i];
#pragma unroll
            for (int j = 0; j < kHTC; ++j)
#pragma unroll
              for (int f = 0; f < NF; ++f) {
                const int o = (i * kHTC + j) * NF + f;
                half_ff_mac(th[o], tl[o], f4_lo(nr), f4_hi(nr), f4_lo(ni), f4_hi(ni), ah[j][f], anh[j][f],
                            anl[j][f], bh[j][f], bnh[j][f], bnl[j][f]);
                half_ff_mac(uh[o], ul[o], f4_lo(mr), f4_hi(mr), f4_lo(mi), f4_hi(mi), ah[j][f], anh[j][f],
                            anl[j][f], bh[j][f], bnh[j][f], bnl[j][f]);
              }
          }
        }
#pragma unroll
        for (int o = 0; o < NO; ++o) {
          const float2 s = __fadd2_rn(th[o], tl[o]);
          tl[o] = __ffma2_rn(__ffma2_rn(th[o], m1, s), m1, tl[o]);
          th[o] = make_float2(0.f, 0.f);
          double2& a = sm.acc[o][tid];
          a.x += f32_widen(s.x);
          a.y += f32_widen(s.y);
          const float2 su = __fadd2_rn(uh[o], ul[o]);
          ul[o] = __ffma2_rn(__ffma2_rn(uh[o], m1, su), m1, ul[o]);
          uh[o] = make_float2(0.f, 0.f);
          double2& b = sm.acc[NO + o][tid];
          b.x += f32_widen(su.x);
          b.y += f32_widen(su.y);
        }
      } else {
        half_wide_chunk<NF>(p, sm.acc, tid, ig0, ig_end, n1_0, p0, wx);
      }
    }
    double2 tsum[NO], usum[NO];
#pragma unroll
    for (int o = 0; o < NO; ++o) {
      const double2 a = sm.acc[o][tid], b = sm.acc[NO + o][tid];
      tsum[o] = make_double2(a.x + f32_widen(tl[o].x), a.y + f32_widen(tl[o].y));
      usum[o] = make_double2(b.x + f32_widen(ul[o].x), b.y + f32_widen(ul[o].y));
    }
    // epilogue: 0.5 vcoul (conj(aqsm_p) T + v_p conj(U)) [+ the diagonal term
    // in the first split], half-warp butterfly over the columns
#pragma unroll
    for (int i = 0; i < kHTB; ++i) {
      const int bl = ty + 16 * i, n1 = n1_0 + bl;
      double2 part[NF];
#pragma unroll
      for (int f = 0; f < NF; ++f) part[f] = make_double2(0.0, 0.0);
#pragma unroll
      for (int j = 0; j < kHTC; ++j) {
        const int col = p0 + tx + 16 * j;
        const int igp = col < p.ng ? p.igp_of[col] : -1;
        if (n1 < p.nb && igp >= 0) {
          const double2 am = p.aqsm[(size_t)n1 * p.nc + igp];
          const double2 an = p.aqsn[(size_t)n1 * p.nc + igp];
          const double2 vp = NF == 1 ? an : am;
          const double wgt = 0.5 * p.vcoul[igp];
          double2 val[NF];
#pragma unroll
          for (int f = 0; f < NF; ++f) {
            const double2 T = tsum[(i * kHTC + j) * NF + f];
            const double2 U = usum[(i * kHTC + j) * NF + f];
            val[f] = cmul(cconj(am), T);
            cfma(val[f], vp, cconj(U));
          }
          if (ic.s == 0) {
            const size_t off = (size_t)col * p.nc + igp;
            const double2 d = cmul(cconj(am), an);
            if (NF == 1) {
              const double2 ie = p.ieps[off];
              if (fma(ie.x, ie.x, ie.y * ie.y) > kTo1 * kTo1)
                cfma(val[0], d, make_double2(-ie.x, -ie.y));
            } else if (igp > 0 && igp % kIgBlk == 0) {
              double2 z[3];
              half_factor(p.wt[off], p.ieps[off], wx, z);
#pragma unroll
              for (int f = 0; f < NF; ++f) cfma(val[f], d, z[f]);
            }
          }
#pragma unroll
          for (int f = 0; f < NF; ++f) {
            part[f].x = fma(wgt, val[f].x, part[f].x);
            part[f].y = fma(wgt, val[f].y, part[f].y);
          }
        }
      }
#pragma unroll
      for (int f = 0; f < NF; ++f)
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) {
          part[f].x += __shfl_xor_sync(0xffffffffu, part[f].x, o);
          part[f].y += __shfl_xor_sync(0xffffffffu, part[f].y, o);
        }
      if (tx == 0)
#pragma unroll
        for (int f = 0; f < NF; ++f) w.partial[ic.pidx * kHBN * NF + bl * NF + f] = part[f];
    }
  }
}

// First g-vector below igp of each column with |Omega2| < to1 (ncouls if
// none): the occupied-band loop of the reference stops there
// (gppKerSeq.cpp:96) and never passes igp.  |Omega2|^2 = |wtilde|^4 |I_eps|^2
// is screened in FP32 (relative error below 2^-20); values not clearly above
// to1^2 take the FP64 expression, so the cut is the FP64 one.
__global__ void __launch_bounds__(kThreads) half_brk_kernel(HalfDev p, int* brk) {
  __shared__ int s_min;
  const int col = blockIdx.x;
  if (threadIdx.x == 0) s_min = p.nc;
  __syncthreads();
  int first = p.nc;
  const int igp = p.igp_of[col];
  const int lim = igp >= 0 ? igp : 0;
  constexpr float kAbove = 1.0000153e-12f;  // to1^2 (1 + 2^-16)
  for (int ig = threadIdx.x; ig < lim; ig += kThreads) {
    const size_t off = (size_t)col * p.nc + ig;
    const double2 wt = p.wt[off], ie = p.ieps[off];
    const float a = __double2float_rn(wt.x), b = __double2float_rn(wt.y);
    const float ex = __double2float_rn(ie.x), ey = __double2float_rn(ie.y);
    const float s2 = fmaf(a, a, b * b);
    if (s2 * s2 * fmaf(ex, ex, ey * ey) > kAbove) continue;
    const double2 w2 = make_double2(fma(wt.x, wt.x, -wt.y * wt.y), 2.0 * wt.x * wt.y);
    const double2 om = cmul(w2, ie);
    if (fma(om.x, om.x, om.y * om.y) < kTo1 * kTo1) {
      first = ig;
      break;
    }
  }
  if (first < p.nc) atomicMin(&s_min, first);
  __syncthreads();
  if (threadIdx.x == 0) brk[col] = s_min;
}

// Fixed-order block reduction of the occupied-band sums of kVals / 8 bands
// (per band T_sch, U_sch, T_ssx, U_ssx, complex), then the column's
// contributions 0.5 vcoul scht (achtemp) and occ vcoul ssxt (asxtemp) per band:
// scht = conj(aqsm_p) T_sch + aqsm_p conj(U_sch), likewise ssxt.
template <int kVals>
__device__ __forceinline__ void occ_finish(const HalfDev& p, const double (&acc)[kVals],
                                           double (*red)[kVals], double* tot, int g0, int nbl,
                                           int col, int igp, int iw, double2* occ_ach,
                                           double2* occ_asx) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
#pragma unroll
  for (int v = 0; v < kVals; ++v) {
    double x = acc[v];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][v] = x;
  }
  __syncthreads();
  if (tid < kVals) {
    double s = 0.0;
    for (int q = 0; q < kThreads / 32; ++q) s += red[q][tid];
    tot[tid] = s;
  }
  __syncthreads();
  if (tid < nbl) {
    const int n1 = g0 + tid;
    double2 ach = make_double2(0.0, 0.0), asx = make_double2(0.0, 0.0);
    if (igp >= 0) {
      const double2 am = p.aqsm[(size_t)n1 * p.nc + igp];
      const double* t = tot + 8 * tid;
      double2 scht = cmul(cconj(am), make_double2(t[0], t[1]));
      cfma(scht, am, make_double2(t[2], -t[3]));
      double2 ssxt = cmul(cconj(am), make_double2(t[4], t[5]));
      cfma(ssxt, am, make_double2(t[6], -t[7]));
      const double v = p.vcoul[igp];
      ach = make_double2(0.5 * scht.x * v, 0.5 * scht.y * v);
      asx = make_double2(ssxt.x * p.occ * v, ssxt.y * p.occ * v);
    }
    const size_t o = ((size_t)n1 * p.ng + col) * kNW + iw;
    occ_ach[o] = ach;
    occ_asx[o] = asx;
  }
  __syncthreads();
}

// Occupied bands: one CTA per (column, frequency), threads over g-vectors,
// kOccBands bands per pass.
__global__ void __launch_bounds__(kThreads) half_occ_kernel(HalfDev p, double2* occ_ach,
                                                            double2* occ_asx) {
  constexpr int kVals = kOccBands * 8;  // per band: T_sch, U_sch, T_ssx, U_ssx (complex)
  __shared__ double red[kThreads / 32][kVals];
  __shared__ double tot[kVals];
  const int col = blockIdx.x, iw = blockIdx.y;
  const int tid = threadIdx.x;
  const int igp = p.igp_of[col];
  const double wx = p.wx[iw];
  const int kend = igp >= 0 ? min(igp, p.brk[col]) : 0;
  for (int g0 = 0; g0 < p.nvband; g0 += kOccBands) {
    const int nbl = min(kOccBands, p.nvband - g0);
    double acc[kVals];
#pragma unroll
    for (int v = 0; v < kVals; ++v) acc[v] = 0.0;
    for (int ig = tid; ig < kend; ig += kThreads) {
      const size_t off = (size_t)col * p.nc + ig;
      const double2 wt = p.wt[off], ie = p.ieps[off];
      const double a = wt.x, b = wt.y;
      const double b2 = guard_b2(b);
      const double2 g = cmul(ie, wt);
      const double c = __dsub_rn(wx, a);
      const double wv = fma(c, c, b2);
      double2 sch = make_double2(0.0, 0.0), ssx = make_double2(0.0, 0.0);
      if (gt_nonneg(guard_thr(a, b2), wv)) {
        // |wx - wtilde| < gamma or |delw|^2 < to1: sch = 0
        if (fma(a, a, b2) > kTo1 * kTo1) {
          const double dr = wx + a;
          const double r = rcp_f64(fma(dr, dr, b2));
          // -G / (2 (wx + wtilde)) = -0.5 G conj(d) / |d|^2, d = (wx + a, b)
          ssx = make_double2(-0.5 * r * fma(g.x, dr, g.y * b), -0.5 * r * fma(g.y, dr, -g.x * b));
        }
      } else {
        const double r = rcp_f64(wv);
        sch = make_double2(fma(g.x, c, -g.y * b) * r, fma(g.x, b, g.y * c) * r);
        // Omega2 / (wx^2 - wtilde^2), Omega2 = wtilde^2 I_eps
        const double2 w2 = make_double2(fma(a, a, -b2), 2.0 * a * b);
        const double2 om = cmul(w2, ie);
        const double2 d = make_double2(fma(wx, wx, -w2.x), -w2.y);
        const double rd = rcp_f64(fma(d.x, d.x, d.y * d.y));
        ssx = make_double2(fma(om.x, d.x, om.y * d.y) * rd, fma(om.y, d.x, -om.x * d.y) * rd);
      }
      const bool pair = ig != igp - 1;
#pragma unroll
      for (int q = 0; q < kOccBands; ++q)
        if (q < nbl) {
          const size_t bo = (size_t)(g0 + q) * p.nc + ig;
          const double2 an = p.aqsn[bo];
          double2 ts = make_double2(acc[8 * q + 0], acc[8 * q + 1]);
          double2 tx2 = make_double2(acc[8 * q + 4], acc[8 * q + 5]);
          cfma(ts, an, sch);
          cfma(tx2, an, ssx);
          acc[8 * q + 0] = ts.x;
          acc[8 * q + 1] = ts.y;
          acc[8 * q + 4] = tx2.x;
          acc[8 * q + 5] = tx2.y;
          if (pair) {
            const double2 am = p.aqsm[bo];
            double2 us = make_double2(acc[8 * q + 2], acc[8 * q + 3]);
            double2 ux = make_double2(acc[8 * q + 6], acc[8 * q + 7]);
            cfma(us, am, sch);
            cfma(ux, am, ssx);
            acc[8 * q + 2] = us.x;
            acc[8 * q + 3] = us.y;
            acc[8 * q + 6] = ux.x;
            acc[8 * q + 7] = ux.y;
          }
        }
    }
    occ_finish<kVals>(p, acc, red, tot, g0, nbl, col, igp, iw, occ_ach, occ_asx);
  }
}

// Occupied bands of the tensor-core form.  The factors sch and ssx of
// half_occ_kernel in float-float arithmetic on the FP32 pipe (~2^-44 before
// the one rounding to FP32); decisions within 2^-30 of a threshold take the
// FP64 expressions of half_occ_kernel.  The band sums are FP32 products over
// FP32 copies of the occupied bands' aqsm / aqsn rows (m32, n32: [nvband][nc]),
// folded into float-float accumulators every 8 g-vectors.  The three
// frequency CTAs of a column are adjacent in the grid, so the column's
// wtilde and I_eps rows are read from DRAM once.
__global__ void __launch_bounds__(kThreads) half_occ_ff_kernel(HalfDev p, const float2* m32,
                                                               const float2* n32, double2* occ_ach,
                                                               double2* occ_asx) {
  constexpr int kVals = kOccBandsF * 8;
  __shared__ double red[kThreads / 32][kVals];
  __shared__ double tot[kVals];
  const int iw = blockIdx.x, col = blockIdx.y;
  const int tid = threadIdx.x;
  const int igp = p.igp_of[col];
  const double wxd = p.wx[iw];
  const FF wx = ff_of(wxd);
  const double to2 = kTo1 * kTo1;
  const FF to2f = ff_of(to2);
  const int kend = igp >= 0 ? min(igp, p.brk[col]) : 0;
  for (int g0 = 0; g0 < p.nvband; g0 += kOccBandsF) {
    const int nbl = min(kOccBandsF, p.nvband - g0);
    float acc[kVals], hi[kVals], lo[kVals];
#pragma unroll
    for (int v = 0; v < kVals; ++v) acc[v] = hi[v] = lo[v] = 0.f;
    int run = 0;
    // operands of the next g-vector are loaded one iteration ahead
    const double2* wt_row = p.wt + (size_t)col * p.nc;
    const double2* ie_row = p.ieps + (size_t)col * p.nc;
    double2 wt_n = make_double2(0.0, 0.0), ie_n = make_double2(0.0, 0.0);
    float2 an_n[kOccBandsF], am_n[kOccBandsF];
    auto fetch = [&](int ig) {
      wt_n = wt_row[ig];
      ie_n = ie_row[ig];
#pragma unroll
      for (int q = 0; q < kOccBandsF; ++q) {
        const size_t bo = (size_t)(g0 + min(q, nbl - 1)) * p.nc + ig;
        an_n[q] = n32[bo];
        am_n[q] = m32[bo];
      }
    };
    if (tid < kend) fetch(tid);
    for (int ig = tid; ig < kend; ig += kThreads) {
      const double2 wt = wt_n, ie = ie_n;
      float2 an_c[kOccBandsF], am_c[kOccBandsF];
#pragma unroll
      for (int q = 0; q < kOccBandsF; ++q) {
        an_c[q] = an_n[q];
        am_c[q] = am_n[q];
      }
      if (ig + kThreads < kend) fetch(ig + kThreads);
      const FF a = ff_of(wt.x), b = ff_of(wt.y), er = ff_of(ie.x), ei = ff_of(ie.y);
      const FF b2 = ff_mul(b, b);
      const FF s2 = ff_add(ff_mul(a, a), b2);  // |wtilde|^2
      const FF c = ff_add(wx, ff_neg(a));
      const FF wv = ff_add(ff_mul(c, c), b2);  // |wdiff|^2
      const FF gx = ff_add(ff_mul(er, a), ff_neg(ff_mul(ei, b)));  // G = I_eps wtilde
      const FF gy = ff_add(ff_mul(er, b), ff_mul(ei, a));
      // sch = 0 where |wdiff|^2 < max(0.25, 4e-6 |wtilde|^2): wv < 0.25 or
      // 250000 wv < |wtilde|^2 (250000 exact in FP32)
      bool n1, n2;
      const bool z1 = ff_gt(FF{0.25f, 0.f}, wv, n1);
      const bool z2 = ff_gt(s2, ff_mul(wv, FF{250000.f, 0.f}), n2);
      bool zero = z1 || z2;
      if (n1 || n2) {
        const double b2d = guard_b2(wt.y);
        zero = gt_nonneg(guard_thr(wt.x, b2d), guard_w(wxd, wt.x, b2d));
      }
      // d = wx + wtilde = (wx + a, b), in both branches
      const FF dr = ff_add(wx, a);
      const FF rd = ff_rcp(ff_add(ff_mul(dr, dr), b2));  // 1 / |d|^2
      float2 sch = make_float2(0.f, 0.f), ssx = make_float2(0.f, 0.f);
      if (!zero) {
        // sch = G (c + i b) / wv = G / (wx - wtilde)
        const FF r = ff_rcp(wv);
        const FF zr = ff_mul(c, r), zi = ff_mul(b, r);
        const FF sx = ff_add(ff_mul(gx, zr), ff_neg(ff_mul(gy, zi)));
        const FF sy = ff_add(ff_mul(gx, zi), ff_mul(gy, zr));
        sch = make_float2(ff_round(sx), ff_round(sy));
        // ssx = Omega2 / (wx^2 - wtilde^2) = sch wtilde / (wx + wtilde),
        // wtilde conj(d) = (a (wx + a) + b^2, b wx)
        const FF qr = ff_mul(ff_add(ff_mul(a, dr), b2), rd), qi = ff_mul(ff_mul(b, wx), rd);
        ssx = make_float2(ff_round(ff_add(ff_mul(sx, qr), ff_neg(ff_mul(sy, qi)))),
                          ff_round(ff_add(ff_mul(sx, qi), ff_mul(sy, qr))));
      } else {
        bool n3;
        bool big = ff_gt(s2, to2f, n3);  // |wtilde|^2 > to1^2
        if (n3) big = fma(wt.x, wt.x, guard_b2(wt.y)) > to2;
        if (big) {
          // -G / (2 (wx + wtilde)) = -0.5 G conj(d) / |d|^2
          const FF hr{-0.5f * rd.hi, -0.5f * rd.lo};
          ssx = make_float2(ff_round(ff_mul(ff_add(ff_mul(gx, dr), ff_mul(gy, b)), hr)),
                            ff_round(ff_mul(ff_add(ff_mul(gy, dr), ff_neg(ff_mul(gx, b))), hr)));
        }
      }
      const bool pair = ig != igp - 1;
#pragma unroll
      for (int q = 0; q < kOccBandsF; ++q)
        if (q < nbl) {
          const float2 an = an_c[q];
          float* t = acc + 8 * q;
          t[0] = fmaf(an.x, sch.x, fmaf(-an.y, sch.y, t[0]));
          t[1] = fmaf(an.x, sch.y, fmaf(an.y, sch.x, t[1]));
          t[4] = fmaf(an.x, ssx.x, fmaf(-an.y, ssx.y, t[4]));
          t[5] = fmaf(an.x, ssx.y, fmaf(an.y, ssx.x, t[5]));
          if (pair) {
            const float2 am = am_c[q];
            t[2] = fmaf(am.x, sch.x, fmaf(-am.y, sch.y, t[2]));
            t[3] = fmaf(am.x, sch.y, fmaf(am.y, sch.x, t[3]));
            t[6] = fmaf(am.x, ssx.x, fmaf(-am.y, ssx.y, t[6]));
            t[7] = fmaf(am.x, ssx.y, fmaf(am.y, ssx.x, t[7]));
          }
        }
      if (++run == 8) {
#pragma unroll
        for (int v = 0; v < kVals; ++v) {
          ff_add(hi[v], lo[v], acc[v]);
          acc[v] = 0.f;
        }
        run = 0;
      }
    }
    double sum[kVals];
#pragma unroll
    for (int v = 0; v < kVals; ++v) {
      ff_add(hi[v], lo[v], acc[v]);
      sum[v] = (double)hi[v] + (double)lo[v];
    }
    occ_finish<kVals>(p, sum, red, tot, g0, nbl, col, igp, iw, occ_ach, occ_asx);
  }
}

// FP32 copies of the occupied bands' aqsm and aqsn rows.
__global__ void __launch_bounds__(256) half_occ_rows32_kernel(HalfDev p, float2* m32, float2* n32) {
  const long long total = (long long)p.nvband * p.nc;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const double2 m = p.aqsm[t], n = p.aqsn[t];
    m32[t] = make_float2(__double2float_rn(m.x), __double2float_rn(m.y));
    n32[t] = make_float2(__double2float_rn(n.x), __double2float_rn(n.y));
  }
}

struct HalfReduceArgs {
  int nb, nvband, ng;
  const double2* main_part;  // non-occupied bands [nvband, nb), kNW per row
  int main_count;            // column blocks x splits
  const double2* stat_part;  // all bands, 1 per row (null without the static remainder)
  int stat_count;
  const double2* occ_ach;    // [nvband][ng][3]
  const double2* occ_asx;
  double2* acht_n1;  // [nb][3]
  double2* asx_n1;   // [nvband][3]
  double2* stat_n1;  // [nb]
};

// One warp per output row, fixed order, compensated.
__global__ void half_reduce_bands_kernel(HalfReduceArgs a) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int n_ach = a.nb * kNW, n_asx = a.nvband * kNW, n_stat = a.stat_part ? a.nb : 0;
  if (warp >= n_ach + n_asx + n_stat) return;
  Comp sx, sy;
  double2* dst;
  if (warp < n_ach) {
    const int n1 = warp / kNW, iw = warp % kNW;
    if (n1 >= a.nvband) {
      const int r = n1 - a.nvband, bb = r / kHBN, bl = r % kHBN;
      for (int q = lane; q < a.main_count; q += 32) {
        const double2 v = a.main_part[((size_t)bb * a.main_count + q) * kHBN * kNW + bl * kNW + iw];
        sx.add(v.x);
        sy.add(v.y);
      }
    } else {
      for (int c = lane; c < a.ng; c += 32) {
        const double2 v = a.occ_ach[((size_t)n1 * a.ng + c) * kNW + iw];
        sx.add(v.x);
        sy.add(v.y);
      }
    }
    dst = a.acht_n1 + warp;
  } else if (warp < n_ach + n_asx) {
    const int e = warp - n_ach, n1 = e / kNW, iw = e % kNW;
    for (int c = lane; c < a.ng; c += 32) {
      const double2 v = a.occ_asx[((size_t)n1 * a.ng + c) * kNW + iw];
      sx.add(v.x);
      sy.add(v.y);
    }
    dst = a.asx_n1 + e;
  } else {
    const int n1 = warp - n_ach - n_asx, bb = n1 / kHBN, bl = n1 % kHBN;
    for (int q = lane; q < a.stat_count; q += 32) {
      const double2 v = a.stat_part[((size_t)bb * a.stat_count + q) * kHBN + bl];
      sx.add(v.x);
      sy.add(v.y);
    }
    dst = a.stat_n1 + n1;
  }
  const double rx = warp_sum_comp(sx), ry = warp_sum_comp(sy);
  if (lane == 0) *dst = make_double2(rx, ry);
}

__global__ void half_reduce_total_kernel(const double2* acht_n1, const double2* asx_n1,
                                         const double2* stat_n1, int nb, int nvband,
                                         double2* achtemp, double2* asxtemp, double2* achstemp,
                                         double2* acht_n1_loc) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp < 2 * kNW + 1) {
    Comp sx, sy;
    if (warp < 2 * kNW) {
      const bool ach = warp < kNW;
      const int iw = ach ? warp : warp - kNW;
      const double2* src = ach ? acht_n1 : asx_n1;
      const int n = ach ? nb : nvband;
      for (int n1 = lane; n1 < n; n1 += 32) {
        sx.add(src[n1 * kNW + iw].x);
        sy.add(src[n1 * kNW + iw].y);
      }
    } else if (achstemp) {
      for (int n1 = lane; n1 < nb; n1 += 32) {
        sx.add(stat_n1[n1].x);
        sy.add(stat_n1[n1].y);
      }
    }
    const double rx = warp_sum_comp(sx), ry = warp_sum_comp(sy);
    if (lane == 0) {
      if (warp < kNW)
        achtemp[warp] = make_double2(rx, ry);
      else if (warp < 2 * kNW)
        asxtemp[warp - kNW] = make_double2(rx, ry);
      else if (achstemp)
        achstemp[0] = make_double2(rx, ry);
    }
  }
  if (acht_n1_loc)
    for (int n1 = threadIdx.x; n1 < nb; n1 += blockDim.x) acht_n1_loc[n1] = acht_n1[n1 * kNW + 2];
}

// [rows][cols] complex -> [cols][rows], 32 x 32 tiles through shared memory.
__global__ void transpose_c128_kernel(const double2* __restrict__ src, double2* __restrict__ dst,
                                      int rows, int cols) {
  __shared__ double2 tile[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 256 threads: 8 rows per pass
  for (int r = ty; r < 32; r += 8) {
    const int rr = r0 + r, cc = c0 + tx;
    if (rr < rows && cc < cols) tile[r][tx] = src[(size_t)rr * cols + cc];
  }
  __syncthreads();
  for (int c = ty; c < 32; c += 8) {
    const int cc = c0 + c, rr = r0 + tx;
    if (rr < rows && cc < cols) dst[(size_t)cc * rows + rr] = tile[tx][c];
  }
}

cudaError_t launch_transpose(const double2* src, double2* dst, int rows, int cols, cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  const dim3 grid((cols + 31) / 32, (rows + 31) / 32);
  transpose_c128_kernel<<<grid, kThreads, 0, s>>>(src, dst, rows, cols);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- tensor-core form
// The non-occupied sums T and U and the static remainder's are weighted FF
// contractions (ff_ozaki.cu) of band-independent factor slabs:
//   sum_col 0.5 vcoul conj(aqsm_p) T = FF(Z, B = aqsn, M = aqsm)
//   sum_col 0.5 vcoul aqsm_p conj(U) = conj(FF(Z, B = aqsm, M = aqsm))
// and for the static remainder (v_p = aqsn_p) FF(Zs, aqsn, aqsm) +
// conj(FF(Zs, B = aqsm, M = aqsn)).  Z[iw][col][ig] is the masked factor over
// the reference's g-vector set, Zs = -I_eps below igp; the unpaired igp terms
// and the occupied bands run in FP64.

// Tiles of 32 g-vectors x kZCols columns: the factors are formed into shared
// memory, then written as the split-BF16 contraction's A slices (rows
// f * ngpown + column, 8 g-vectors per 16-byte chunk; consecutive threads fill
// one 8-row group), skipping the K tiles past a row block's limit.
constexpr int kZCols = 16;

template <int NF>
__device__ __forceinline__ void put_z_tile(const HalfDev& p, const OzakiPrep& oz, int c0, int ig0,
                                           float2 (*tz)[kZCols][33]) {
  for (int c = threadIdx.x; c < NF * kZCols * 4; c += blockDim.x) {
    const int ch = c % 4, pl = (c / 4) % kZCols, f = c / (4 * kZCols);
    const int col = c0 + pl;
    if (col >= p.ng) continue;
    const int R = f * p.ng + col;
    if (ig0 / kOzKTile >= oz.kt_lim[R / kOzRows]) continue;
    float re[8], im[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const float2 v = tz[f][pl][ch * 8 + j];
      re[j] = v.x;
      im[j] = v.y;
    }
    oz_put_a(oz, R, ig0 + ch * 8, re, im);
  }
}

// Z slabs of the non-occupied half sum, [3][ng][nc] as contraction rows: the
// factor of half_factor in float-float arithmetic on the FP32 pipe (~2^-44
// before the one rounding to FP32, the contraction's input precision), with
// the threshold decision of half_factor taken in FP64 within 2^-30 of the
// threshold.
__global__ void __launch_bounds__(256) half_z_slices_kernel(HalfDev p, OzakiPrep oz) {
  __shared__ float2 tz[3][kZCols][33];
  FF wx[3];
#pragma unroll
  for (int f = 0; f < 3; ++f) wx[f] = ff_of(p.wx[f]);
  const int kt_all = (p.nc + kOzKTile - 1) / kOzKTile;
  const long long tiles = (long long)((p.ng + kZCols - 1) / kZCols) * kt_all;
  for (long long t = blockIdx.x; t < tiles; t += gridDim.x) {
    const int c0 = (int)(t / kt_all) * kZCols, ig0 = (int)(t % kt_all) * kOzKTile;
    __syncthreads();
    for (int e = threadIdx.x; e < 32 * kZCols; e += blockDim.x) {
      const int pl = e / 32, k = e % 32;  // reads run along g-vectors
      const int col = c0 + pl, ig = ig0 + k;
      float2 v[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
      const int lim = col < p.ng ? column_limit<3>(p.igp_of[col]) : 0;
      if (ig < lim && (ig % kIgBlk) != kIgBlk - 1) {
        const size_t off = (size_t)col * p.nc + ig;
        const double2 wt = p.wt[off], ie = p.ieps[off];
        const FF a = ff_of(wt.x), b = ff_of(wt.y), er = ff_of(ie.x), ei = ff_of(ie.y);
        const FF b2 = ff_mul(b, b);
        const FF s2 = ff_add(ff_mul(a, a), b2);
        const FF gx = ff_add(ff_mul(er, a), ff_neg(ff_mul(ei, b)));
        const FF gy = ff_add(ff_mul(er, b), ff_mul(ei, a));
        // G (c + i b) = wx G - G conj(wtilde) = wx G - |wtilde|^2 I_eps
        const FF sex = ff_mul(s2, er), sey = ff_mul(s2, ei);
#pragma unroll
        for (int f = 0; f < 3; ++f) {
          const FF c = ff_add(wx[f], ff_neg(a));
          const FF wv = ff_add(ff_mul(c, c), b2);
          // kept where wv < max(0.25, 4e-6 |wtilde|^2)
          bool n1, n2;
          const bool k1 = ff_gt(FF{0.25f, 0.f}, wv, n1);
          const bool k2 = ff_gt(s2, ff_mul(wv, FF{250000.f, 0.f}), n2);
          bool keep = k1 || k2;
          if (n1 || n2) {
            const double b2d = guard_b2(wt.y);
            keep = gt_nonneg(guard_thr(wt.x, b2d), guard_w(p.wx[f], wt.x, b2d));
          }
          if (keep) {
            const FF r = ff_rcp(wv);
            v[f] = make_float2(ff_mul_round(ff_add(ff_mul(wx[f], gx), ff_neg(sex)), r),
                               ff_mul_round(ff_add(ff_mul(wx[f], gy), ff_neg(sey)), r));
          }
        }
      }
#pragma unroll
      for (int f = 0; f < 3; ++f) tz[f][pl][k] = v[f];
    }
    __syncthreads();
    put_z_tile<3>(p, oz, c0, ig0, tz);
  }
}

// Zs of the static remainder as contraction rows: -I_eps below igp, in FP32.
__global__ void __launch_bounds__(256) half_zs_slices_kernel(HalfDev p, OzakiPrep oz) {
  __shared__ float2 tz[1][kZCols][33];
  const int kt_all = (p.nc + kOzKTile - 1) / kOzKTile;
  const long long tiles = (long long)((p.ng + kZCols - 1) / kZCols) * kt_all;
  for (long long t = blockIdx.x; t < tiles; t += gridDim.x) {
    const int c0 = (int)(t / kt_all) * kZCols, ig0 = (int)(t % kt_all) * kOzKTile;
    __syncthreads();
    for (int e = threadIdx.x; e < 32 * kZCols; e += blockDim.x) {
      const int pl = e / 32, k = e % 32;
      const int col = c0 + pl, ig = ig0 + k;
      const int lim = col < p.ng ? column_limit<1>(p.igp_of[col]) : 0;
      float2 v = make_float2(0.f, 0.f);
      if (ig < lim) {
        const double2 e2 = p.ieps[(size_t)col * p.nc + ig];
        v = make_float2(-__double2float_rn(e2.x), -__double2float_rn(e2.y));
      }
      tz[0][pl][k] = v;
    }
    __syncthreads();
    put_z_tile<1>(p, oz, c0, ig0, tz);
  }
}

// Band rows of the tensor form: one CTA per band, its 8 warps over the
// columns, compensated sums of the unpaired igp terms (and of the
// occupied-band partials) combined in a fixed order, then
//   acht_n1[n1][iw] = T + conj(U) + unpaired       (n1 >= nvband)
//                   = sum_col occ_ach                (n1 <  nvband)
//   asx_n1[n1][iw]  = sum_col occ_asx                (n1 <  nvband)
//   stat_n1[n1]     = Ts + conj(Us) + unpaired       (static remainder)
constexpr int kRowWarps = 8;
__global__ void __launch_bounds__(kRowWarps * 32) half_tensor_rows_kernel(
    HalfDev p, const double2* t3, const double2* u3, const double2* ts, const double2* us,
    const double2* occ_ach, const double2* occ_asx, double2* acht_n1, double2* asx_n1, double2* stat_n1) {
  constexpr int kVals = 4 * kNW + 2;  // ax, ay, sx, sy per frequency; qx, qy
  __shared__ double part[kRowWarps][kVals];
  const int n1 = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool occ = n1 < p.nvband;
  const double wx[3] = {p.wx[0], p.wx[1], p.wx[2]};
  Comp ax[3], ay[3], sx[3], sy[3], qx, qy;
  for (int col = warp * 32 + lane; col < p.ng; col += kRowWarps * 32) {
    const int igp = p.igp_of[col];
    if (igp < 0) continue;
    const size_t off = (size_t)col * p.nc + igp;
    const double2 am = p.aqsm[(size_t)n1 * p.nc + igp];
    const double2 an = p.aqsn[(size_t)n1 * p.nc + igp];
    const double w = 0.5 * p.vcoul[igp];
    const double2 d = cmul(cconj(am), an);
    if (ts) {  // static remainder's unpaired igp term
      const double2 e = p.ieps[off];
      if (fma(e.x, e.x, e.y * e.y) > kTo1 * kTo1) {
        const double2 v = cmul(d, make_double2(-e.x, -e.y));
        qx.add(w * v.x);
        qy.add(w * v.y);
      }
    }
    if (occ) {
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) {
        const double2 a = occ_ach[((size_t)n1 * p.ng + col) * kNW + iw];
        const double2 x = occ_asx[((size_t)n1 * p.ng + col) * kNW + iw];
        ax[iw].add(a.x);
        ay[iw].add(a.y);
        sx[iw].add(x.x);
        sy[iw].add(x.y);
      }
    } else if (igp > 0 && igp % kIgBlk == 0) {
      double2 z[3];
      half_factor(p.wt[off], p.ieps[off], wx, z);
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) {
        const double2 v = cmul(d, z[iw]);
        ax[iw].add(w * v.x);
        ay[iw].add(w * v.y);
      }
    }
  }
#pragma unroll
  for (int iw = 0; iw < kNW; ++iw) {
    const double v0 = warp_sum_comp(ax[iw]), v1 = warp_sum_comp(ay[iw]);
    const double v2 = warp_sum_comp(sx[iw]), v3 = warp_sum_comp(sy[iw]);
    if (lane == 0) {
      part[warp][4 * iw + 0] = v0;
      part[warp][4 * iw + 1] = v1;
      part[warp][4 * iw + 2] = v2;
      part[warp][4 * iw + 3] = v3;
    }
  }
  const double q0 = warp_sum_comp(qx), q1 = warp_sum_comp(qy);
  if (lane == 0) {
    part[warp][4 * kNW] = q0;
    part[warp][4 * kNW + 1] = q1;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  double tot[kVals];
  for (int v = 0; v < kVals; ++v) {
    Comp c;
    for (int q = 0; q < kRowWarps; ++q) c.add(part[q][v]);
    tot[v] = c.value();
  }
#pragma unroll
  for (int iw = 0; iw < kNW; ++iw) {
    const double rx = tot[4 * iw], ry = tot[4 * iw + 1], ux = tot[4 * iw + 2], uy = tot[4 * iw + 3];
    if (occ) {
      acht_n1[n1 * kNW + iw] = make_double2(rx, ry);
      asx_n1[n1 * kNW + iw] = make_double2(ux, uy);
    } else {
      const double2 a = t3[(size_t)n1 * kNW + iw], b = u3[(size_t)n1 * kNW + iw];
      acht_n1[n1 * kNW + iw] = make_double2(rx + a.x + b.x, ry + a.y - b.y);
    }
  }
  if (ts) stat_n1[n1] = make_double2(tot[4 * kNW] + ts[n1].x + us[n1].x, tot[4 * kNW + 1] + ts[n1].y - us[n1].y);
}

size_t up256(size_t v) { return (v + 255) / 256 * 256; }

template <int NF>
cudaError_t launch_half_main(const HalfDev& p, const GppWork& w, int grid, cudaStream_t s) {
  constexpr int smem = (int)sizeof(HalfSmem<NF>);
  cudaError_t e = cudaFuncSetAttribute(half_main_kernel<NF>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  half_main_kernel<NF><<<grid, kThreads, smem, s>>>(p, w);
  return cudaGetLastError();
}

}  // namespace
}  // namespace sigma

struct sigma_gpp_halfsum_plan_s {
  int device = 0, nb = 0, nvband = 0, nc = 0, ng = 0, flags = 0;
  int main_grid = 0, stat_grid = 0;
  sigma::GppWork wm{}, ws{};
  void* block = nullptr;
  int* igp_of = nullptr;
  int* brk = nullptr;
  int* counters = nullptr;
  double2 *occ_ach = nullptr, *occ_asx = nullptr;
  double2 *acht_n1 = nullptr, *asx_n1 = nullptr, *stat_n1 = nullptr;
  double2 *t_aqsm = nullptr, *t_aqsn = nullptr, *t_ieps = nullptr, *t_wt = nullptr;
  // tensor-core form: contraction plans over a shared slice workspace, the
  // factor slabs and the four contraction results
  sigma_ff_plan ff3 = nullptr, ff1 = nullptr;
  void* tblock = nullptr;
  float2 *m32 = nullptr, *n32 = nullptr;  // occupied bands' aqsm / aqsn rows in FP32
  double2 *t3 = nullptr, *u3 = nullptr, *ts = nullptr, *us = nullptr;  // [nb][3], [nb][1]
};

extern "C" int sigma_gpp_halfsum_plan_create(sigma_gpp_halfsum_plan* out, int number_bands,
                                             int nvband, int ncouls, int ngpown, int nstart,
                                             int nend, const int* inv_igp_index,
                                             const int* indinv, int indinv_len, int flags) {
  using namespace sigma;
  if (!out || !inv_igp_index || !indinv) return SIGMA_ERR_NULL;
  *out = nullptr;
  if (flags & ~(SIGMA_HALFSUM_STATIC | SIGMA_HALFSUM_GVEC_MAJOR | SIGMA_HALFSUM_TENSOR))
    return SIGMA_ERR_UNSUPPORTED;
  const bool tensor = (flags & SIGMA_HALFSUM_TENSOR) != 0;
  int st = gpp_check_shape(number_bands, nvband, ncouls, ngpown, nstart, nend);
  if (st != SIGMA_OK) return st;
  if (indinv_len < ncouls) return SIGMA_ERR_INVALID_SHAPE;
  std::vector<int> igp_of;
  int valid = 0;
  st = gpp_map_columns(ncouls, ngpown, inv_igp_index, indinv, indinv_len, igp_of, valid);
  if (st != SIGMA_OK) return st;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return SIGMA_ERR_NO_DEVICE;
  }
  const int sms = device_sm_count();
  if (sms <= 0) return SIGMA_ERR_NO_DEVICE;
  auto* p = new sigma_gpp_halfsum_plan_s();
  p->device = dev;
  p->nb = number_bands;
  p->nvband = nvband;
  p->nc = ncouls;
  p->ng = ngpown;
  p->flags = flags;
  p->main_grid = p->stat_grid = sms;
  // about half of the items fall past their column block's range (triangle)
  if (!tensor) {
    gpp_size_work(p->wm, nvband, number_bands - nvband, kHBN, kHBP, ncouls, ngpown, p->main_grid, 48);
    if (flags & SIGMA_HALFSUM_STATIC)
      gpp_size_work(p->ws, 0, number_bands, kHBN, kHBP, ncouls, ngpown, p->stat_grid, 48);
  }
  if (p->wm.n_items < p->main_grid) p->main_grid = std::max(1, p->wm.n_items);
  if (p->ws.n_items < p->stat_grid) p->stat_grid = std::max(1, p->ws.n_items);
  const size_t nbc = (size_t)number_bands * ncouls, ngc = (size_t)ngpown * ncouls;
  const size_t b_igp = up256(sizeof(int) * ngpown), b_brk = b_igp, b_cnt = 256;
  const size_t b_occ = up256(sizeof(double2) * (size_t)nvband * ngpown * kNW);
  const size_t b_n1 = up256(sizeof(double2) * (size_t)number_bands * kNW);
  const size_t b_asx = up256(sizeof(double2) * (size_t)std::max(nvband, 1) * kNW);
  const size_t b_st = up256(sizeof(double2) * (size_t)number_bands);
  const size_t b_pm = up256(sizeof(double2) * (size_t)p->wm.n_items * kHBN * kNW);
  const size_t b_ps = up256(sizeof(double2) * (size_t)p->ws.n_items * kHBN);
  const size_t b_tr = (flags & SIGMA_HALFSUM_GVEC_MAJOR) ? up256(sizeof(double2) * nbc) * 2 +
                                                               up256(sizeof(double2) * ngc) * 2
                                                         : 0;
  const size_t total = b_igp + b_brk + b_cnt + 2 * b_occ + b_n1 + b_asx + b_st + b_pm + b_ps + b_tr;
  cudaError_t e = cudaMalloc(&p->block, total);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_last_cuda_error(e, "cudaMalloc(halfsum plan)", __LINE__);
    delete p;
    return SIGMA_ERR_ALLOC;
  }
  char* b = static_cast<char*>(p->block);
  size_t off = 0;
  auto take = [&](size_t n) {
    char* r = b + off;
    off += n;
    return r;
  };
  p->igp_of = reinterpret_cast<int*>(take(b_igp));
  p->brk = reinterpret_cast<int*>(take(b_brk));
  p->counters = reinterpret_cast<int*>(take(b_cnt));
  p->occ_ach = reinterpret_cast<double2*>(take(b_occ));
  p->occ_asx = reinterpret_cast<double2*>(take(b_occ));
  p->acht_n1 = reinterpret_cast<double2*>(take(b_n1));
  p->asx_n1 = reinterpret_cast<double2*>(take(b_asx));
  p->stat_n1 = reinterpret_cast<double2*>(take(b_st));
  p->wm.partial = reinterpret_cast<double2*>(take(b_pm));
  p->ws.partial = (flags & SIGMA_HALFSUM_STATIC) && !tensor ? reinterpret_cast<double2*>(take(b_ps))
                                                            : nullptr;
  if (flags & SIGMA_HALFSUM_GVEC_MAJOR) {
    p->t_aqsm = reinterpret_cast<double2*>(take(up256(sizeof(double2) * nbc)));
    p->t_aqsn = reinterpret_cast<double2*>(take(up256(sizeof(double2) * nbc)));
    p->t_ieps = reinterpret_cast<double2*>(take(up256(sizeof(double2) * ngc)));
    p->t_wt = reinterpret_cast<double2*>(take(up256(sizeof(double2) * ngc)));
  }
  p->wm.counter = p->counters;
  p->ws.counter = p->counters + 1;
  e = cudaMemcpy(p->igp_of, igp_of.data(), sizeof(int) * ngpown, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    set_last_cuda_error(e, "cudaMemcpy(halfsum igp_of)", __LINE__);
    cudaFree(p->block);
    delete p;
    return SIGMA_ERR_CUDA;
  }
  if (tensor) {
    size_t b3 = 0, b1 = 0;
    st = ff_plan_tile_bytes(number_bands, ncouls, ngpown, 3, &b3);
    if (st == SIGMA_OK && (flags & SIGMA_HALFSUM_STATIC))
      st = ff_plan_tile_bytes(number_bands, ncouls, ngpown, 1, &b1);
    const size_t b_tiles = up256(std::max(b3, b1));
    const size_t b_r3 = up256(sizeof(double2) * (size_t)number_bands * kNW);
    const size_t b_r1 = up256(sizeof(double2) * (size_t)number_bands);
    const size_t b_o = up256(sizeof(float2) * (size_t)std::max(nvband, 1) * ncouls);
    if (st == SIGMA_OK) {
      e = cudaMalloc(&p->tblock, b_tiles + 2 * b_r3 + 2 * b_r1 + 2 * b_o);
      if (e != cudaSuccess) {
        cudaGetLastError();
        set_last_cuda_error(e, "cudaMalloc(halfsum tensor)", __LINE__);
        st = SIGMA_ERR_ALLOC;
      }
    }
    if (st == SIGMA_OK) {
      char* t = static_cast<char*>(p->tblock);
      p->t3 = reinterpret_cast<double2*>(t + b_tiles);
      p->u3 = reinterpret_cast<double2*>(t + b_tiles + b_r3);
      p->ts = reinterpret_cast<double2*>(t + b_tiles + 2 * b_r3);
      p->us = reinterpret_cast<double2*>(t + b_tiles + 2 * b_r3 + b_r1);
      p->m32 = reinterpret_cast<float2*>(t + b_tiles + 2 * b_r3 + 2 * b_r1);
      p->n32 = reinterpret_cast<float2*>(t + b_tiles + 2 * b_r3 + 2 * b_r1 + b_o);
      // Z rows (iw, col) are zero from the column's g-vector limit on
      std::vector<int> kend3((size_t)kNW * ngpown), kend1(ngpown);
      for (int g = 0; g < ngpown; ++g) {
        const int igp = igp_of[g];
        kend1[g] = igp < 0 ? 0 : igp;
        for (int f = 0; f < kNW; ++f) kend3[(size_t)f * ngpown + g] = igp < 0 ? 0 : std::max(igp - 1, 0);
      }
      st = ff_plan_build(&p->ff3, number_bands, ncouls, ngpown, kNW, igp_of, SIGMA_FF_OZAKI_BF16,
                         p->tblock, kend3.data());
      if (st == SIGMA_OK && (flags & SIGMA_HALFSUM_STATIC))
        st = ff_plan_build(&p->ff1, number_bands, ncouls, ngpown, 1, igp_of, SIGMA_FF_OZAKI_BF16,
                           p->tblock, kend1.data());
    }
    if (st != SIGMA_OK) {
      sigma_gpp_halfsum_plan_destroy(p);
      return st;
    }
  }
  *out = p;
  return SIGMA_OK;
}

extern "C" int sigma_gpp_halfsum_plan_destroy(sigma_gpp_halfsum_plan p) {
  if (!p) return SIGMA_OK;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(p->device);
  if (p->block) cudaFree(p->block);
  if (p->ff3) sigma_ff_plan_destroy(p->ff3);
  if (p->ff1) sigma_ff_plan_destroy(p->ff1);
  if (p->tblock) cudaFree(p->tblock);
  cudaSetDevice(cur);
  delete p;
  return SIGMA_OK;
}

extern "C" int sigma_gpp_halfsum_execute(sigma_gpp_halfsum_plan plan, const double* wx_array,
                                         double occ, const sigma_complex128* aqsmtemp,
                                         const sigma_complex128* aqsntemp,
                                         const sigma_complex128* I_eps_array,
                                         const sigma_complex128* wtilde_array,
                                         const double* vcoul, sigma_complex128* achtemp,
                                         sigma_complex128* asxtemp, sigma_complex128* acht_n1_loc,
                                         sigma_complex128* achstemp, void* stream) {
  using namespace sigma;
  if (!plan) return SIGMA_ERR_NULL;
  if (!wx_array || !aqsmtemp || !aqsntemp || !I_eps_array || !wtilde_array || !vcoul || !achtemp ||
      !asxtemp)
    return SIGMA_ERR_NULL;
  if (achstemp && !(plan->flags & SIGMA_HALFSUM_STATIC)) return SIGMA_ERR_UNSUPPORTED;
  int dev = 0;
  SIGMA_CUDA_TRY(cudaGetDevice(&dev));
  if (dev != plan->device) return SIGMA_ERR_UNSUPPORTED;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const double2* aqsm = reinterpret_cast<const double2*>(aqsmtemp);
  const double2* aqsn = reinterpret_cast<const double2*>(aqsntemp);
  const double2* ieps = reinterpret_cast<const double2*>(I_eps_array);
  const double2* wt = reinterpret_cast<const double2*>(wtilde_array);
  if (plan->flags & SIGMA_HALFSUM_GVEC_MAJOR) {
    // gppKerSeq.cpp's layout: aqsmtemp[ncouls][number_bands], I_eps_array[ncouls][ngpown]
    SIGMA_CUDA_TRY(launch_transpose(aqsm, plan->t_aqsm, plan->nc, plan->nb, s));
    SIGMA_CUDA_TRY(launch_transpose(aqsn, plan->t_aqsn, plan->nc, plan->nb, s));
    SIGMA_CUDA_TRY(launch_transpose(ieps, plan->t_ieps, plan->nc, plan->ng, s));
    SIGMA_CUDA_TRY(launch_transpose(wt, plan->t_wt, plan->nc, plan->ng, s));
    aqsm = plan->t_aqsm;
    aqsn = plan->t_aqsn;
    ieps = plan->t_ieps;
    wt = plan->t_wt;
  }
  HalfDev p{plan->nb, plan->nvband, plan->nc, plan->ng, occ, aqsm, aqsn, ieps, wt,
            vcoul, wx_array, plan->igp_of, plan->brk};
  SIGMA_CUDA_TRY(cudaMemsetAsync(plan->counters, 0, 2 * sizeof(int), s));
  if (plan->nvband > 0) {
    half_brk_kernel<<<plan->ng, kThreads, 0, s>>>(p, plan->brk);
    SIGMA_CUDA_TRY(cudaGetLastError());
    if (plan->ff3) {
      half_occ_rows32_kernel<<<152, 256, 0, s>>>(p, plan->m32, plan->n32);
      SIGMA_CUDA_TRY(cudaGetLastError());
      half_occ_ff_kernel<<<dim3(kNW, plan->ng), kThreads, 0, s>>>(p, plan->m32, plan->n32,
                                                                  plan->occ_ach, plan->occ_asx);
    } else {
      half_occ_kernel<<<dim3(plan->ng, kNW), kThreads, 0, s>>>(p, plan->occ_ach, plan->occ_asx);
    }
    SIGMA_CUDA_TRY(cudaGetLastError());
  }
  if (plan->ff3) {
    const bool stat = plan->ff1 && achstemp;
    auto C = [](const double2* x) { return reinterpret_cast<const sigma_complex128*>(x); };
    auto M = [](double2* x) { return reinterpret_cast<sigma_complex128*>(x); };
    // the slabs are written directly as the contractions' A slices; T and U
    // (and the static pair) contract the same slices
    const OzakiPrep& oz3 = *ff_plan_ozaki(plan->ff3);
    half_z_slices_kernel<<<152 * 8, 256, 0, s>>>(p, oz3);
    SIGMA_CUDA_TRY(cudaGetLastError());
    SIGMA_CUDA_TRY(launch_ozaki_zero_rows(oz3, kNW * plan->ng, s));
    int st = ff_execute_weighted(plan->ff3, nullptr, C(aqsn), C(aqsm), vcoul, 0.5, M(plan->t3), stream,
                                 nullptr, true);
    if (st == SIGMA_OK)
      st = ff_execute_weighted(plan->ff3, nullptr, C(aqsm), C(aqsm), vcoul, 0.5, M(plan->u3), stream,
                               nullptr, true);
    if (st == SIGMA_OK && stat) {
      const OzakiPrep& oz1 = *ff_plan_ozaki(plan->ff1);
      half_zs_slices_kernel<<<152 * 8, 256, 0, s>>>(p, oz1);
      SIGMA_CUDA_TRY(cudaGetLastError());
      SIGMA_CUDA_TRY(launch_ozaki_zero_rows(oz1, plan->ng, s));
      st = ff_execute_weighted(plan->ff1, nullptr, C(aqsn), C(aqsm), vcoul, 0.5, M(plan->ts), stream,
                               nullptr, true);
      if (st == SIGMA_OK)
        st = ff_execute_weighted(plan->ff1, nullptr, C(aqsm), C(aqsn), vcoul, 0.5, M(plan->us), stream,
                                 nullptr, true);
    }
    if (st != SIGMA_OK) return st;
    half_tensor_rows_kernel<<<plan->nb, kRowWarps * 32, 0, s>>>(
        p, plan->t3, plan->u3, stat ? plan->ts : nullptr, plan->us, plan->occ_ach, plan->occ_asx,
        plan->acht_n1, plan->asx_n1, plan->stat_n1);
    SIGMA_CUDA_TRY(cudaGetLastError());
    half_reduce_total_kernel<<<1, 256, 0, s>>>(plan->acht_n1, plan->asx_n1, plan->stat_n1, plan->nb,
                                               plan->nvband, reinterpret_cast<double2*>(achtemp),
                                               reinterpret_cast<double2*>(asxtemp),
                                               stat ? reinterpret_cast<double2*>(achstemp) : nullptr,
                                               reinterpret_cast<double2*>(acht_n1_loc));
    SIGMA_CUDA_TRY(cudaGetLastError());
    return SIGMA_OK;
  }
  if (plan->wm.n_items > 0) SIGMA_CUDA_TRY(launch_half_main<3>(p, plan->wm, plan->main_grid, s));
  const bool stat = plan->ws.partial && achstemp;
  if (stat && plan->ws.n_items > 0) SIGMA_CUDA_TRY(launch_half_main<1>(p, plan->ws, plan->stat_grid, s));
  HalfReduceArgs a;
  a.nb = plan->nb;
  a.nvband = plan->nvband;
  a.ng = plan->ng;
  a.main_part = plan->wm.partial;
  a.main_count = plan->wm.n_col_blocks * plan->wm.n_splits;
  a.stat_part = stat ? plan->ws.partial : nullptr;
  a.stat_count = plan->ws.n_col_blocks * plan->ws.n_splits;
  a.occ_ach = plan->occ_ach;
  a.occ_asx = plan->occ_asx;
  a.acht_n1 = plan->acht_n1;
  a.asx_n1 = plan->asx_n1;
  a.stat_n1 = plan->stat_n1;
  const int warps = plan->nb * kNW + plan->nvband * kNW + (stat ? plan->nb : 0);
  half_reduce_bands_kernel<<<(warps * 32 + 255) / 256, 256, 0, s>>>(a);
  SIGMA_CUDA_TRY(cudaGetLastError());
  half_reduce_total_kernel<<<1, 256, 0, s>>>(plan->acht_n1, plan->asx_n1, plan->stat_n1, plan->nb,
                                             plan->nvband, reinterpret_cast<double2*>(achtemp),
                                             reinterpret_cast<double2*>(asxtemp),
                                             stat ? reinterpret_cast<double2*>(achstemp) : nullptr,
                                             reinterpret_cast<double2*>(acht_n1_loc));
  SIGMA_CUDA_TRY(cudaGetLastError());
  return SIGMA_OK;
}

namespace {

int halfsum_host(bool tensor, int number_bands, int nvband, int ncouls, int ngpown, int nstart,
                 int nend, const int* inv_igp_index, const int* indinv, const double* wx_array,
                 double occ, const sigma_complex128* aqsmtemp, const sigma_complex128* aqsntemp,
                 const sigma_complex128* I_eps_array, const sigma_complex128* wtilde_array,
                 const double* vcoul, sigma_complex128* achtemp, sigma_complex128* asxtemp,
                 sigma_complex128* acht_n1_loc, sigma_complex128* achstemp, void* stream) {
  using namespace sigma;
  if (!inv_igp_index || !indinv || !wx_array || !aqsmtemp || !aqsntemp || !I_eps_array ||
      !wtilde_array || !vcoul || !achtemp || !asxtemp)
    return SIGMA_ERR_NULL;
  int st = gpp_check_shape(number_bands, nvband, ncouls, ngpown, nstart, nend);
  if (st != SIGMA_OK) return st;
  std::lock_guard<std::mutex> lk(api_mutex());
  sigma_gpp_halfsum_plan plan = nullptr;
  const int flags = SIGMA_HALFSUM_GVEC_MAJOR | (achstemp ? SIGMA_HALFSUM_STATIC : 0) |
                    (tensor ? SIGMA_HALFSUM_TENSOR : 0);
  st = sigma_gpp_halfsum_plan_create(&plan, number_bands, nvband, ncouls, ngpown, nstart, nend,
                                     inv_igp_index, indinv, ncouls, flags);
  if (st != SIGMA_OK) return st;
  const size_t bb = sizeof(sigma_complex128) * (size_t)number_bands * ncouls;
  const size_t cb = sizeof(sigma_complex128) * (size_t)ngpown * ncouls;
  size_t off = 0;
  auto take = [&](size_t n) {
    const size_t o = off;
    off += up256(n);
    return o;
  };
  const size_t o_m = take(bb), o_n = take(bb), o_e = take(cb), o_w = take(cb),
               o_v = take(sizeof(double) * ncouls), o_x = take(sizeof(double) * kNW),
               o_out = take(sizeof(sigma_complex128) * (2 * kNW + 1 + (size_t)number_bands));
  void* arena = nullptr;
  st = arena_get(kArenaMisc, off, &arena);
  if (st != SIGMA_OK) {
    sigma_gpp_halfsum_plan_destroy(plan);
    return st;
  }
  char* a = static_cast<char*>(arena);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  auto C = [&](size_t o) { return reinterpret_cast<sigma_complex128*>(a + o); };
  sigma_complex128* out = C(o_out);  // achtemp[3], asxtemp[3], achstemp[1], acht_n1_loc[nb]
  auto run = [&]() -> int {
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_m, aqsmtemp, bb, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_n, aqsntemp, bb, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_e, I_eps_array, cb, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_w, wtilde_array, cb, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_v, vcoul, sizeof(double) * ncouls, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_x, wx_array, sizeof(double) * kNW, cudaMemcpyHostToDevice, s));
    int r = sigma_gpp_halfsum_execute(plan, reinterpret_cast<const double*>(a + o_x), occ, C(o_m),
                                      C(o_n), C(o_e), C(o_w), reinterpret_cast<const double*>(a + o_v),
                                      out, out + kNW, acht_n1_loc ? out + 2 * kNW + 1 : nullptr,
                                      achstemp ? out + 2 * kNW : nullptr, stream);
    if (r != SIGMA_OK) return r;
    SIGMA_CUDA_TRY(cudaMemcpyAsync(achtemp, out, sizeof(sigma_complex128) * kNW, cudaMemcpyDeviceToHost, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(asxtemp, out + kNW, sizeof(sigma_complex128) * kNW,
                                   cudaMemcpyDeviceToHost, s));
    if (achstemp)
      SIGMA_CUDA_TRY(cudaMemcpyAsync(achstemp, out + 2 * kNW, sizeof(sigma_complex128),
                                     cudaMemcpyDeviceToHost, s));
    if (acht_n1_loc)
      SIGMA_CUDA_TRY(cudaMemcpyAsync(acht_n1_loc, out + 2 * kNW + 1,
                                     sizeof(sigma_complex128) * number_bands, cudaMemcpyDeviceToHost, s));
    SIGMA_CUDA_TRY(cudaStreamSynchronize(s));
    return SIGMA_OK;
  };
  const int rc = run();
  sigma_gpp_halfsum_plan_destroy(plan);
  return rc;
}

}  // namespace

extern "C" int sigma_gpp_halfsum_fp64(int number_bands, int nvband, int ncouls, int ngpown,
                                      int nstart, int nend, const int* inv_igp_index,
                                      const int* indinv, const double* wx_array, double occ,
                                      const sigma_complex128* aqsmtemp,
                                      const sigma_complex128* aqsntemp,
                                      const sigma_complex128* I_eps_array,
                                      const sigma_complex128* wtilde_array, const double* vcoul,
                                      sigma_complex128* achtemp, sigma_complex128* asxtemp,
                                      sigma_complex128* acht_n1_loc, sigma_complex128* achstemp,
                                      void* stream) {
  return halfsum_host(false, number_bands, nvband, ncouls, ngpown, nstart, nend, inv_igp_index,
                      indinv, wx_array, occ, aqsmtemp, aqsntemp, I_eps_array, wtilde_array, vcoul,
                      achtemp, asxtemp, acht_n1_loc, achstemp, stream);
}

extern "C" int sigma_gpp_halfsum_tensor(int number_bands, int nvband, int ncouls, int ngpown,
                                        int nstart, int nend, const int* inv_igp_index,
                                        const int* indinv, const double* wx_array, double occ,
                                        const sigma_complex128* aqsmtemp,
                                        const sigma_complex128* aqsntemp,
                                        const sigma_complex128* I_eps_array,
                                        const sigma_complex128* wtilde_array, const double* vcoul,
                                        sigma_complex128* achtemp, sigma_complex128* asxtemp,
                                        sigma_complex128* acht_n1_loc, sigma_complex128* achstemp,
                                        void* stream) {
  return halfsum_host(true, number_bands, nvband, ncouls, ngpown, nstart, nend, inv_igp_index,
                      indinv, wx_array, occ, aqsmtemp, aqsntemp, I_eps_array, wtilde_array, vcoul,
                      achtemp, asxtemp, acht_n1_loc, achstemp, stream);
}
