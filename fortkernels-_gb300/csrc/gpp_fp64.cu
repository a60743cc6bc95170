// GPP sigma sum, plain FP64 path (sm_103a).
//
// Replaces the band / column / g-vector / frequency loop nest of
// BGW-Kernels/gppKer.cpp:303-439.  Work is cut into items (BN bands x BP
// columns x one g-vector split); a persistent grid takes items from a device
// counter, stages the columns' wtilde / I_eps and the bands' aqsn through
// shared memory with coalesced 16-byte loads, and every thread evaluates a
// 2 x 2 (band x column) register tile over the three frequencies.  Three tile
// shapes (32x32, 16x64, 64x16) exist so that ragged band / column counts can
// pick the one that pads least; the batched kernel takes a shape per instance.
//
// GB300 runs FP64 at 1/64 of its FP32 rate, so the term is rewritten to
// spend as few FP64 pipe instructions as possible:
//   scha / conj(aqsm[n1][igp]) = aqsn * I_eps * wtilde * conj(wdiff) / |wdiff|^2
//                              = R * (c + i b) * r,   R = aqsn * (I_eps * wtilde),
//   c = wx - Re wtilde, b = Im wtilde, r = 1 / (c^2 + b^2).
// With per-band frequencies (this first pass) every term is formed in
// float-float arithmetic (FP32 pairs on the FP32 pipe: G in FP64 per column
// and g-vector, c = wx - Re wtilde in FP64 per term, the rest from exact
// splits), its FP32 high half widened and added to an FP64 sum and its low
// half to an FP32 sum of one staged chunk, added to the FP64 sum at the
// chunk's end: ~3 FP64 operations per term instead of 10 (the FP64
// form had 8 per term plus 6 per band, column and g-vector).  A term's error
// is about twice the FP64 form's, whose reciprocal is itself an FP32 seed
// refined once (rcp_f64_seed32, within 2^-44.8).  conj(aqsm[n1][igp]), 0.5
// and vcoul[igp] are applied once per column after the g-vector sum.  The
// pole guard's decisions are taken in float-float and re-taken with the FP64
// expressions near a threshold; exact poles are dropped by a select, never
// multiplied.
#include "sigma_internal.cuh"
#include "floatfloat.cuh"
#include "gpp_batch.cuh"

namespace sigma {
namespace {

constexpr int kPad = 1;

// Staging of the per-band-frequency pass: per (g-vector, column) wtilde's
// parts in FP64 (c = wx - Re wtilde is formed in FP64, and the rare FP64
// decisions read them), Im wtilde and its square and G = I_eps wtilde as
// float-float values, and flags (bit 0: the guard's second condition can
// bind, bit 1: outside the float-float range, bit 2: no term); per
// (g-vector, band) aqsn as a float-float pair and its range flag.
// Each thread's FP64 sums (its 2 x 2 tile x 3 frequencies) live in shared
// memory, one slot row per output; 16-g-vector chunks keep two CTAs' staging
// and sums within an SM.
constexpr int kCKB = 16;
static_assert(kCK % kCKB == 0, "split lengths are multiples of the chunk");
template <int BN, int BP>
struct SchSmem {
  double2 acc[2 * 2 * kNW][kThreads];
  double a[kCKB][BP + kPad];
  double b[kCKB][BP + kPad];
  float4 fb[kCKB][BP + kPad];  // (b.hi, b.lo, b^2.hi, b^2.lo)
  float4 fg[kCKB][BP + kPad];  // (G.x hi, lo, G.y hi, lo)
  unsigned flag[kCKB][BP + kPad];
  float4 fn[kCKB][BN + kPad];  // (aqsn.x hi, lo, aqsn.y hi, lo)
  unsigned nflag[kCKB][BN + kPad];
};
constexpr unsigned kFlagBinds = 1u, kFlagWide = 2u, kFlagDead = 4u;

__device__ __forceinline__ double2 cmul(double2 x, double2 y) {
  return make_double2(fma(x.x, y.x, -__dmul_rn(x.y, y.y)), fma(x.x, y.y, __dmul_rn(x.y, y.x)));
}

// One term of the per-band-frequency pass in FP64, for terms whose inputs
// leave the float-float range; out of line, reading its inputs from global
// memory (noff: aqsn's offset, ~0 for a padding band).
static __device__ __noinline__ double2 sch_term_fp64(const double2* aqsn, const double2* wtp,
                                                     const double2* ieps, size_t noff, size_t off, double wx) {
  const double2 n = noff != ~size_t(0) ? aqsn[noff] : make_double2(0.0, 0.0);
  const double2 wt = wtp[off], ie = ieps[off];
  const double2 R = cmul(n, cmul(ie, wt));
  const double b = wt.y, b2 = guard_b2(b);
  const double c = __dsub_rn(wx, wt.x), wv = fma(c, c, b2);
  const double r = keep_nonneg(wv, guard_thr(wt.x, b2)) ? rcp_f64_seed32(wv) : 0.0;
  return make_double2(fma(R.x, c, -__dmul_rn(b, R.y)) * r, fma(R.y, c, __dmul_rn(b, R.x)) * r);
}

// One work item of the main pass.  Leaves the item's partial sums in
// w.partial[pidx * BN * 3 + bl * 3 + iw].
template <int BN, int BP>
__device__ __forceinline__ void sch_fp64_item(const GppDev& p, const GppWork& w, int item,
                                              unsigned char* smem_raw, int tid) {
  constexpr int TXN = BP / 2, TYN = BN / 2;  // threads across columns / bands
  static_assert(TXN * TYN == kThreads, "2 x 2 register tiles over 256 threads");
  static_assert(sizeof(double2) * BN * kNW * BP <= sizeof(SchSmem<BN, BP>), "epilogue reuses staging");
  SchSmem<BN, BP>& sm = *reinterpret_cast<SchSmem<BN, BP>*>(smem_raw);
  const int tx = tid % TXN, ty = tid / TXN;
  const int band_end = w.band_begin + w.band_count;
  const ItemCoord ic = decode_item(w, item);
  const int n1_0 = w.band_begin + ic.bb * BN;
  const int p0 = ic.cb * BP;
  const int ig_begin = ic.s * w.split_len;
  const int ig_end = min(ig_begin + w.split_len, p.nc);

  double wxr[2][kNW];
  bool wx_wide[2];
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int n1 = n1_0 + ty + TYN * i;
    wx_wide[i] = false;
#pragma unroll
    for (int iw = 0; iw < kNW; ++iw) {
      wxr[i][iw] = n1 < band_end ? p.wx[(size_t)n1 * p.wx_stride + iw] : 1.0;
      wx_wide[i] = wx_wide[i] || !ff_freq_range(wxr[i][iw]);
    }
  }
  // float-float sums in registers (lanes: real and imaginary parts): each
  // term's high pair added exactly (TwoSum) to the high pair, the errors and
  // low halves to the low pair; after each chunk the pair renormalised
  // (Fast2Sum), its high pair added to the FP64 sums in shared memory and
  // its low pair carried on (an FP32 sum over a whole item's thousands of
  // terms would lose ~n 2^-47 of the output)
  const float2 m1 = make_float2(-1.f, -1.f);
  float2 ach[2][2][kNW], acl[2][2][kNW];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) {
        sm.acc[(i * 2 + j) * kNW + iw][tid] = make_double2(0.0, 0.0);
        ach[i][j][iw] = make_float2(0.f, 0.f);
        acl[i][j][iw] = make_float2(0.f, 0.f);
      }

  for (int ig0 = ig_begin; ig0 < ig_end; ig0 += kCKB) {
    __syncthreads();
    for (int e = tid; e < kCKB * BP; e += kThreads) {
      const int k = e % kCKB, pl = e / kCKB;
      const int ig = ig0 + k, my_igp = p0 + pl;
      double a = 0.0, b = 0.0;
      float4 fb = make_float4(0.f, 0.f, 0.f, 0.f), fg = fb;
      unsigned flag = kFlagDead;
      if (ig < ig_end && my_igp < p.ng) {
        const size_t off = (size_t)my_igp * p.nc + ig;
        const double2 wt = p.wt[off];
        const double2 ie = p.ieps[off];
        const double2 g = cmul(ie, wt);
        a = wt.x;
        b = wt.y;
        const FF f = ff_of_rn(b), f2 = ff_mul_raw(f, f), gx = ff_of_rn(g.x), gy = ff_of_rn(g.y);
        fb = make_float4(f.hi, f.lo, f2.hi, f2.lo);
        fg = make_float4(gx.hi, gx.lo, gy.hi, gy.lo);
        const float ah = ff_of_rn(a).hi;
        // |wtilde|^2 * 4e-6 > 0.25 needs |wtilde|^2 > 62500
        flag = (fmaf(ah, ah, f.hi * f.hi) >= 62000.f ? kFlagBinds : 0u) |
               (ff_range(wt.x, wt.y) && ff_range(ie.x, ie.y) ? 0u : kFlagWide);
      }
      sm.a[k][pl] = a;
      sm.b[k][pl] = b;
      sm.fb[k][pl] = fb;
      sm.fg[k][pl] = fg;
      sm.flag[k][pl] = flag;
    }
    for (int e = tid; e < kCKB * BN; e += kThreads) {
      const int k = e % kCKB, bl = e / kCKB;
      const int ig = ig0 + k, n1 = n1_0 + bl;
      double2 v = make_double2(0.0, 0.0);
      if (ig < ig_end && n1 < band_end) v = p.aqsn[(size_t)n1 * p.nc + ig];
      const FF nx = ff_of_rn(v.x), ny = ff_of_rn(v.y);
      sm.fn[k][bl] = make_float4(nx.hi, nx.lo, ny.hi, ny.lo);
      sm.nflag[k][bl] = ff_range(v.x, v.y) ? 0u : kFlagWide;
    }
    __syncthreads();

#pragma unroll 1
    for (int k = 0; k < kCKB; ++k) {
      double a[2], b[2];
      FF fb[2], fb2[2], gx[2], gy[2], nx[2], ny[2];
      unsigned flag[2], nflag[2];
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int pl = tx + TXN * j;
        a[j] = sm.a[k][pl];
        b[j] = sm.b[k][pl];
        const float4 v = sm.fb[k][pl], g = sm.fg[k][pl];
        fb[j] = FF{v.x, v.y};
        fb2[j] = FF{v.z, v.w};
        gx[j] = FF{g.x, g.y};
        gy[j] = FF{g.z, g.w};
        flag[j] = sm.flag[k][pl];
      }
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const float4 v = sm.fn[k][ty + TYN * i];
        nx[i] = FF{v.x, v.y};
        ny[i] = FF{v.z, v.w};
        nflag[i] = sm.nflag[k][ty + TYN * i];
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          // R = aqsn G, then per frequency (R (c + i b)) / |wdiff|^2
          const FF rx = ff_dot2_raw(nx[i], gx[j], ny[i], gy[j]);
          const FF ry = ff_dot2_raw(nx[i], gy[j], ff_neg(ny[i]), gx[j]);
          const bool wide = (flag[j] & kFlagWide) || nflag[i] || wx_wide[i];
          const bool any_wide = __any_sync(0xffffffffu, wide);
#pragma unroll
          for (int iw = 0; iw < kNW; ++iw) {
            const FF c = ff_of_rn(__dsub_rn(wxr[i][iw], a[j]));  // wx - Re wtilde in FP64
            const FF wv = ff_sq_add(c, fb2[j]);               // |wdiff|^2
            bool near;
            bool keep = ff_gt_quarter(wv, near);
            if (near || (flag[j] & kFlagBinds)) keep = keep_fp64(wxr[i][iw], a[j], b[j]);
            keep = keep && !(flag[j] & kFlagDead);
            const FF r = ff_rcp_raw(wv);
            const FF ux = ff_dot2_raw(rx, c, ry, fb[j]), uy = ff_dot2_raw(rx, fb[j], ff_neg(ry), c);
            const FF sx = ff_mul_raw(ux, r), sy = ff_mul_raw(uy, r);
            if (any_wide && wide) {
              if (!(flag[j] & kFlagDead)) {
                const int n1 = n1_0 + ty + TYN * i, ig = ig0 + k, my_igp = p0 + tx + TXN * j;
                const double2 s = sch_term_fp64(p.aqsn, p.wt, p.ieps,
                                                n1 < band_end ? (size_t)n1 * p.nc + ig : ~size_t(0),
                                                (size_t)my_igp * p.nc + ig, wxr[i][iw]);
                double2& a = sm.acc[(i * 2 + j) * kNW + iw][tid];
                a.x += s.x;
                a.y += s.y;
              }
            } else {
              const float2 hv = keep ? make_float2(sx.hi, sy.hi) : make_float2(0.f, 0.f);
              const float2 lv = keep ? make_float2(sx.lo, sy.lo) : make_float2(0.f, 0.f);
              float2& h = ach[i][j][iw];
              const float2 hs = __fadd2_rn(h, hv);
              const float2 hb = __ffma2_rn(h, m1, hs);
              const float2 ha = __ffma2_rn(hb, m1, hs);
              const float2 he = __fadd2_rn(__ffma2_rn(ha, m1, h), __ffma2_rn(hb, m1, hv));
              h = hs;
              acl[i][j][iw] = __fadd2_rn(acl[i][j][iw], __fadd2_rn(he, lv));
            }
          }
        }
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int iw = 0; iw < kNW; ++iw) {
          const float2 s = __fadd2_rn(ach[i][j][iw], acl[i][j][iw]);
          acl[i][j][iw] = __ffma2_rn(__ffma2_rn(ach[i][j][iw], m1, s), m1, acl[i][j][iw]);
          ach[i][j][iw] = make_float2(0.f, 0.f);
          double2& a = sm.acc[(i * 2 + j) * kNW + iw][tid];
          a.x += f32_widen(s.x);
          a.y += f32_widen(s.y);
        }
  }
  double2 acc[2][2][kNW];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) {
        const double2 a = sm.acc[(i * 2 + j) * kNW + iw][tid];
        acc[i][j][iw] = make_double2(a.x + f32_widen(acl[i][j][iw].x), a.y + f32_widen(acl[i][j][iw].y));
      }

  // epilogue: x conj(aqsm[n1][igp]) * 0.5 * vcoul[igp], then a fixed-order
  // sum over the tile's columns
  __syncthreads();
  double2(*red)[kNW][BP] = reinterpret_cast<double2(*)[kNW][BP]>(smem_raw);
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int bl = ty + TYN * i, pl = tx + TXN * j;
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
  if (tid < BN * kNW) {
    const int bl = tid / kNW, iw = tid % kNW;
    double sx = 0.0, sy = 0.0;
    for (int pl = 0; pl < BP; ++pl) {
      sx += red[bl][iw][pl].x;
      sy += red[bl][iw][pl].y;
    }
    w.partial[ic.pidx * BN * kNW + tid] = make_double2(sx, sy);
  }
}

template <int BN, int BP>
__global__ void __launch_bounds__(kThreads, 2) sch_fp64_kernel(GppDev p, GppWork w) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  const int tid = threadIdx.x;
  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(w.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= w.n_items) break;
    sch_fp64_item<BN, BP>(p, w, item, smem_raw, tid);
  }
}

// ---------------------------------------------------------------- shared frequencies
// When every band uses the same three frequencies (the mini-app's case,
// BGW-Kernels/gppKer.cpp:310-314: e_n1kq is the same for every band), the
// frequency factor of a term,
//   Y_iw = G (c + i b) r   (0 when the pole guard drops the term),
// depends on the column and the g-vector only.  Each staged chunk forms Y
// once for its columns, shared by the item's BN bands, and every term is
// then one complex multiply-add acc += aqsn * Y: 4 DFMA, against 10 FP64
// operations per term when the factor is rebuilt for every band.
//
// Y is formed in float-float arithmetic (FP32 pairs) from G = I_eps wtilde
// and c = wx - Re wtilde taken in FP64 and split, and widened to FP64 once:
// 3 FP64 operations per frequency instead of ~12 (the chunk's factor phase
// is time in which the FP64 pipe does no band work).  Its error is about
// twice the FP64 form's, whose reciprocal is itself an FP32 seed refined
// once (within 2^-44.8).  The keep decisions are taken in float-float and re-taken with the
// FP64 expressions, out of line, within 2^-30 of the threshold or where the
// guard's second condition can bind (|wtilde|^2 >= 62000); elements outside
// the float-float range take the FP64 factor.  The sum over
// g-vectors is then a complex GEMM (bands x g-vectors times g-vectors x
// (column, frequency)) on the FP64 pipe, 16 x 16 threads with a
// (BN/16 bands x BP/16 columns x 3 frequencies) register tile each.
//
// The complex multiply-accumulate runs with three real products per term
// instead of four: with the chunk's sums n.x + n.y (per band) and
// Y.x + Y.y (per column and frequency) staged beside the operands,
//   P1 = sum n.x Y.x,  P2 = sum n.y Y.y,  P3 = sum (n.x + n.y)(Y.x + Y.y),
//   sum n Y = (P1 - P2) + i (P3 - P1 - P2),
// 3 DFMA per term.  In FP64 the extra roundings (the two sums and the final
// subtractions) stay near 1e-16 of the partial sums.
constexpr int kCKY = 16;  // g-vectors per staged chunk

// Rows padded by one element: the staging writes run along g-vectors (the
// coalesced direction of the global reads), so unpadded rows, whose strides
// are multiples of 128 bytes, put a warp's writes in one bank group.
template <int BN, int BP>
struct SchYSmem {
  // each thread's FP64 sums (its 16-column x 16-band register tile's outputs
  // x 3 frequencies), one slot row per output: a warp's accesses are 512
  // contiguous bytes
  double2 acc[(BN / 16) * (BP / 16) * kNW][kThreads];
  // Y as float-float operands of paired (f32x2) instructions whose lanes are
  // a term's real and imaginary parts: [k][iw * BP + column] holds (Re.hi,
  // Im.hi, -Re.lo, -Im.lo) of Y and [k][kNW * BP + iw * BP + column] those of
  // i Y, (-Im.hi, Re.hi, Im.lo, -Re.lo); one padding element per row
  float4 y[kCKY][2 * kNW * BP + 1];
  // aqsn: [k][band] (Re.hi, Re.hi, Re.lo, Re.lo), [k][BN + band] the same of Im
  float4 n[kCKY][2 * BN + 1];
};

// Y = G (c + i b) / |wdiff|^2 of one (column, g-vector) element at frequency
// wx in FP64 (G = I_eps wtilde, a + i b = wtilde, c = wx - a, b2 = b^2, gb =
// G b, thr the pole guard's threshold; 0 where the guard drops the term, and
// for padding elements, whose thr is infinite): ~9 FP64 operations and a
// reciprocal to the FP64 rounding unit, shared by every band of the item.
// (A float-float quotient, or the reciprocal's two-DFMA form from an FP32
// seed, measured 1.8 and 1.4 times the error in the most cancelling band
// sums.)
__device__ __forceinline__ double2 sch_y_fp64(double2 g, double2 gb, double a, double b2, double thr, double wx) {
  const double c = __dsub_rn(wx, a);
  const double wv = fma(c, c, b2);
  if (!keep_nonneg(wv, thr)) return make_double2(0.0, 0.0);
  const double r = rcp_f64(wv);
  return make_double2(__dmul_rn(fma(g.x, c, -gb.y), r), __dmul_rn(fma(g.y, c, gb.x), r));
}

// A chunk holding a factor or an aqsn element outside the float-float range:
// FP64 complex multiply-adds of the thread's register tile, its factors
// formed again from the inputs (as the staging formed them) and aqsn read
// again, the chunk's sums added to the thread's FP64 sums.  Out of line: the
// common path carries none of its registers.
template <int BN, int BP>
static __device__ __noinline__ void sch_fp64y_wide_chunk(const GppDev& p, double2 (*acc)[kThreads], int tid,
                                                         int ig0, int ig_end, int n1_0, int band_end, int p0,
                                                         double wx0, double wx1, double wx2) {
  constexpr int TB = BN / 16, TC = BP / 16;
  const int tx = tid & 15, ty = tid >> 4;
  double2 aw[TB][TC][kNW];
  for (int i = 0; i < TB; ++i)
    for (int j = 0; j < TC; ++j)
      for (int iw = 0; iw < kNW; ++iw) aw[i][j][iw] = make_double2(0.0, 0.0);
  for (int k = 0; k < kCKY; ++k) {
    const int ig = ig0 + k;
    double2 y[TC][kNW];
    for (int j = 0; j < TC; ++j) {
      const int my_igp = p0 + tx + 16 * j;
      const bool valid = ig < ig_end && my_igp < p.ng;
      double2 wt = make_double2(0.0, 0.0), ie = wt;
      if (valid) {
        const size_t off = (size_t)my_igp * p.nc + ig;
        wt = p.wt[off];
        ie = p.ieps[off];
      }
      const double2 g = cmul(ie, wt);
      const double2 gb = make_double2(__dmul_rn(g.x, wt.y), __dmul_rn(g.y, wt.y));
      const double b2 = guard_b2(wt.y);
      const double thr = valid ? guard_thr(wt.x, b2) : __longlong_as_double(0x7ff0000000000000LL);
      for (int iw = 0; iw < kNW; ++iw)
        y[j][iw] = sch_y_fp64(g, gb, wt.x, b2, thr, iw == 0 ? wx0 : (iw == 1 ? wx1 : wx2));
    }
    for (int i = 0; i < TB; ++i) {
      const int n1 = n1_0 + ty + 16 * i;
      const double2 nn = (ig < ig_end && n1 < band_end) ? p.aqsn[(size_t)n1 * p.nc + ig] : make_double2(0.0, 0.0);
      for (int j = 0; j < TC; ++j)
        for (int iw = 0; iw < kNW; ++iw) {
          const double2 yv = y[j][iw];
          aw[i][j][iw].x = fma(nn.x, yv.x, fma(-nn.y, yv.y, aw[i][j][iw].x));
          aw[i][j][iw].y = fma(nn.x, yv.y, fma(nn.y, yv.x, aw[i][j][iw].y));
        }
    }
  }
  for (int i = 0; i < TB; ++i)
    for (int j = 0; j < TC; ++j)
      for (int iw = 0; iw < kNW; ++iw) {
        double2& a = acc[(i * TC + j) * kNW + iw][tid];
        a.x += aw[i][j][iw].x;
        a.y += aw[i][j][iw].y;
      }
}

// Bounded wait for a gate word written by a host-to-device copy (`polls`
// polls 256 ns apart: about 1 s with the default bound).  False when it gave
// up (SIGMA_ERR_TIMEOUT recorded) or an earlier wait of the launch had; the
// item is then dropped and the CTA takes no further item.
__device__ __forceinline__ bool wait_ready(const unsigned* flag, unsigned epoch, int* status, int polls) {
  if (*reinterpret_cast<volatile int*>(status) != 0) return false;  // an earlier wait gave up
  for (int i = 0; i < polls; ++i) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(flag) : "memory");
    if (v == epoch) return true;
    __nanosleep(256);
  }
  atomicCAS(status, 0, (int)SIGMA_ERR_TIMEOUT);
  return false;
}

template <int BN, int BP>
__device__ __forceinline__ void sch_fp64y_item(const GppDev& p, const GppWork& w, int item,
                                               unsigned char* smem_raw, int tid) {
  if (w.ready) {  // inputs of this item copied yet?
    const ItemCoord g = decode_item(w, item);
    if (!__syncthreads_and(tid != 0 ||
                           wait_ready(w.ready + gate_word(w, g.cb, g.s), w.epoch, w.ready_status, w.ready_polls)))
      return;
  }
  constexpr int TB = BN / 16, TC = BP / 16;
  SchYSmem<BN, BP>& sm = *reinterpret_cast<SchYSmem<BN, BP>*>(smem_raw);
  const int tx = tid & 15, ty = tid >> 4;
  const int band_end = w.band_begin + w.band_count;
  const ItemCoord ic = decode_item(w, item);
  // block origin and partial-slot stride from the pass's layout (w.bn): a
  // ragged last band block may run a shorter item (BN < w.bn)
  const int n1_0 = w.band_begin + ic.bb * w.bn;
  const int p0 = ic.cb * BP;
  const int ig_begin = ic.s * w.split_len;
  const int ig_end = min(ig_begin + w.split_len, p.nc);
  const double wx0 = p.wx[0], wx1 = p.wx[1], wx2 = p.wx[2];

  // the item's FP64 sums live in shared memory, each thread touching only
  // its own slots; registers hold float-float sums (lanes: real and
  // imaginary parts): the high pair is added to the FP64 sums after each
  // float-float chunk, the low pair carries the remainder on
#pragma unroll
  for (int o = 0; o < TB * TC * kNW; ++o) sm.acc[o][tid] = make_double2(0.0, 0.0);
  float2 ach[TB][TC][kNW], acl[TB][TC][kNW];
#pragma unroll
  for (int i = 0; i < TB; ++i)
#pragma unroll
    for (int j = 0; j < TC; ++j)
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) {
        ach[i][j][iw] = make_float2(0.f, 0.f);
        acl[i][j][iw] = make_float2(0.f, 0.f);
      }

  for (int ig0 = ig_begin; ig0 < ig_end; ig0 += kCKY) {
    __syncthreads();
    bool chunk_wide = false;  // an input of the chunk outside the float-float range
    // frequency factors of the chunk's (g-vector, column) pairs; reads run
    // along g-vectors
    for (int e = tid; e < kCKY * BP; e += kThreads) {
      const int k = e % kCKY, pl = e / kCKY;
      const int ig = ig0 + k, my_igp = p0 + pl;
      const bool valid = ig < ig_end && my_igp < p.ng;
      double2 wt = make_double2(0.0, 0.0), ie = wt;
      if (valid) {
        const size_t off = (size_t)my_igp * p.nc + ig;
        wt = p.wt[off];
        ie = p.ieps[off];
      }
      // Y in FP64 (~37 FP64 operations per column and g-vector, shared by
      // the item's 64 bands x 3 frequencies; the pole guard the int64
      // compare against the per-element threshold), split as float-float
      // pairs for the terms; a factor outside the float-float range sends
      // the chunk to the FP64 path
      const double2 g = cmul(ie, wt);
      const double2 gb = make_double2(__dmul_rn(g.x, wt.y), __dmul_rn(g.y, wt.y));
      const double b2 = guard_b2(wt.y);
      const double thr = valid ? guard_thr(wt.x, b2) : __longlong_as_double(0x7ff0000000000000LL);
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) {
        const double2 v = sch_y_fp64(g, gb, wt.x, b2, thr, iw == 0 ? wx0 : (iw == 1 ? wx1 : wx2));
        const FF vx = ff_of_rn(v.x), vy = ff_of_rn(v.y);
        sm.y[k][iw * BP + pl] = make_float4(vx.hi, vy.hi, -vx.lo, -vy.lo);
        sm.y[k][kNW * BP + iw * BP + pl] = make_float4(-vy.hi, vx.hi, vy.lo, -vx.lo);
        chunk_wide = chunk_wide || !ff_range(v.x, v.y);
      }
    }
    for (int e = tid; e < kCKY * BN; e += kThreads) {
      const int k = e % kCKY, bl = e / kCKY;
      const int ig = ig0 + k, n1 = n1_0 + bl;
      double2 v = make_double2(0.0, 0.0);
      if (ig < ig_end && n1 < band_end) v = p.aqsn[(size_t)n1 * p.nc + ig];
      const FF nx = ff_of_rn(v.x), ny = ff_of_rn(v.y);
      sm.n[k][bl] = make_float4(nx.hi, nx.hi, nx.lo, nx.lo);
      sm.n[k][BN + bl] = make_float4(ny.hi, ny.hi, ny.lo, ny.lo);
      chunk_wide = chunk_wide || !ff_range(v.x, v.y);
    }
    chunk_wide = __syncthreads_or(chunk_wide);

    if (!chunk_wide) {
      // every term n Y as a float-float product on the FP32 pipe, in paired
      // (f32x2) instructions whose two lanes are the term's real and
      // imaginary parts: n Y = nr Y + ni (i Y), two products of a broadcast
      // pair and a lane pair; the products' exact errors and cross terms
      // formed negated (negated multiplicands: no instruction negates an
      // addend); the term's high half added exactly (TwoSum) to the chunk's
      // FP32 sum, the rounding errors and low halves summed in FP32; at the
      // chunk's end the pair renormalised (Fast2Sum: |high| >= |low| up to
      // cancellation, where the low pair's bits are few), the new high half
      // widened on the integer pipe and added to the FP64 sums and the low
      // half kept (2 FP64 operations per output and chunk: 1/8 per term;
      // a flush every second chunk measured 3 % slower, its registers
      // spilling).  Differences as fma(x, -1, y), exact up to their one
      // rounding.
      const float2 m1 = make_float2(-1.f, -1.f);
#pragma unroll 1
      for (int k = 0; k < kCKY; ++k) {
        // per (column, frequency): Y's high pair and its negation, the
        // negated low pair, and the same three of i Y
        float2 ah[TC][kNW], anh[TC][kNW], anl[TC][kNW], bh[TC][kNW], bnh[TC][kNW], bnl[TC][kNW];
#pragma unroll
        for (int j = 0; j < TC; ++j)
#pragma unroll
          for (int iw = 0; iw < kNW; ++iw) {
            const float4 a = sm.y[k][iw * BP + tx + 16 * j];
            const float4 b = sm.y[k][kNW * BP + iw * BP + tx + 16 * j];
            ah[j][iw] = f4_lo(a);
            anl[j][iw] = f4_hi(a);
            anh[j][iw] = __fmul2_rn(ah[j][iw], m1);
            bh[j][iw] = f4_lo(b);
            bnl[j][iw] = f4_hi(b);
            bnh[j][iw] = __fmul2_rn(bh[j][iw], m1);
          }
#pragma unroll
        for (int i = 0; i < TB; ++i) {
          const float4 vr = sm.n[k][ty + 16 * i], vi = sm.n[k][BN + ty + 16 * i];
          const float2 rh = f4_lo(vr), rl = f4_hi(vr), ih = f4_lo(vi), il = f4_hi(vi);
#pragma unroll
          for (int j = 0; j < TC; ++j)
#pragma unroll
            for (int iw = 0; iw < kNW; ++iw) {
              const float2 p1 = __fmul2_rn(rh, ah[j][iw]);
              const float2 p2 = __fmul2_rn(ih, bh[j][iw]);
              // -(exact errors of p1, p2 + cross terms)
              const float2 g1 = __ffma2_rn(rh, anl[j][iw], __ffma2_rn(rl, anh[j][iw], __ffma2_rn(rh, anh[j][iw], p1)));
              const float2 g2 = __ffma2_rn(ih, bnl[j][iw], __ffma2_rn(il, bnh[j][iw], __ffma2_rn(ih, bnh[j][iw], p2)));
              // s + es = p1 + p2 (TwoSum)
              const float2 s = __fadd2_rn(p1, p2);
              const float2 bv = __ffma2_rn(p1, m1, s);
              const float2 av = __ffma2_rn(bv, m1, s);
              const float2 es = __fadd2_rn(__ffma2_rn(av, m1, p1), __ffma2_rn(bv, m1, p2));
              const float2 lo = __ffma2_rn(__fadd2_rn(g1, g2), m1, es);
              // chunk sum: high pair += s (TwoSum), low pair += its error + lo
              float2& h = ach[i][j][iw];
              const float2 hs = __fadd2_rn(h, s);
              const float2 hb = __ffma2_rn(h, m1, hs);
              const float2 ha = __ffma2_rn(hb, m1, hs);
              const float2 he = __fadd2_rn(__ffma2_rn(ha, m1, h), __ffma2_rn(hb, m1, s));
              h = hs;
              acl[i][j][iw] = __fadd2_rn(acl[i][j][iw], __fadd2_rn(he, lo));
            }
        }
      }
#pragma unroll
      for (int i = 0; i < TB; ++i)
#pragma unroll
        for (int j = 0; j < TC; ++j)
#pragma unroll
          for (int iw = 0; iw < kNW; ++iw) {
            const float2 s = __fadd2_rn(ach[i][j][iw], acl[i][j][iw]);
            acl[i][j][iw] = __ffma2_rn(__ffma2_rn(ach[i][j][iw], m1, s), m1, acl[i][j][iw]);
            ach[i][j][iw] = make_float2(0.f, 0.f);
            double2& a = sm.acc[(i * TC + j) * kNW + iw][tid];
            a.x += f32_widen(s.x);
            a.y += f32_widen(s.y);
          }
    } else {
      sch_fp64y_wide_chunk<BN, BP>(p, sm.acc, tid, ig0, ig_end, n1_0, band_end, p0, wx0, wx1, wx2);
    }
  }
  // what the float-float sums still hold
#pragma unroll
  for (int i = 0; i < TB; ++i)
#pragma unroll
    for (int j = 0; j < TC; ++j)
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) {
        double2& a = sm.acc[(i * TC + j) * kNW + iw][tid];
        a.x = (a.x + f32_widen(ach[i][j][iw].x)) + f32_widen(acl[i][j][iw].x);
        a.y = (a.y + f32_widen(ach[i][j][iw].y)) + f32_widen(acl[i][j][iw].y);
      }

  // epilogue: x conj(aqsm[n1][igp]) * 0.5 * vcoul[igp]; the 16 lanes of a
  // half-warp hold the item's columns for the same bands and sum them with
  // a fixed butterfly
  if (w.ready_m) {  // aqsm copied yet?
    if (!__syncthreads_and(tid != 0 || wait_ready(w.ready_m, w.epoch, w.ready_status, w.ready_polls)))
      return;
  }
#pragma unroll
  for (int i = 0; i < TB; ++i) {
    const int bl = ty + 16 * i, n1 = n1_0 + bl;
    double2 part[kNW];
#pragma unroll
    for (int iw = 0; iw < kNW; ++iw) part[iw] = make_double2(0.0, 0.0);
#pragma unroll
    for (int j = 0; j < TC; ++j) {
      const int my_igp = p0 + tx + 16 * j;
      const int igp = my_igp < p.ng ? p.igp_of[my_igp] : -1;
      if (n1 < band_end && igp >= 0) {
        const double2 am = p.aqsm[(size_t)n1 * p.nc + igp];
        const double2 m = make_double2(am.x, -am.y);
        const double f = 0.5 * p.vcoul[igp];
#pragma unroll
        for (int iw = 0; iw < kNW; ++iw) {
          const double2 v = cmul(sm.acc[(i * TC + j) * kNW + iw][tid], m);
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
    if (tx == 0) {
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) w.partial[ic.pidx * w.bn * kNW + bl * kNW + iw] = part[iw];
    }
  }
}

template <int BN, int BP>
__global__ void __launch_bounds__(kThreads, 2) sch_fp64y_kernel(GppDev p, GppWork w) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  const int tid = threadIdx.x;
  for (;;) {
    __syncthreads();
    // gated launch: no further items once a wait gave up
    if (tid == 0)
      s_item = (w.ready && *reinterpret_cast<volatile int*>(w.ready_status) != 0) ? w.n_items
                                                                                  : atomicAdd(w.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= w.n_items) break;
    sch_fp64y_item<BN, BP>(p, w, item, smem_raw, tid);
  }
}

constexpr size_t smax(size_t a, size_t b) { return a > b ? a : b; }
constexpr size_t kSchYBatchSmem =
    smax(smax(sizeof(SchYSmem<64, 32>), sizeof(SchYSmem<32, 64>)), sizeof(SchYSmem<64, 16>));
// the two-CTA kernel's tiles (32 x 32 and 64 x 16: 12 outputs per thread)
constexpr size_t kSchYBatchSmallSmem = smax(sizeof(SchYSmem<32, 32>), sizeof(SchYSmem<64, 16>));

// Item of an instance's shared-frequency pass with tile t: the last band
// block runs the shortest item (a multiple of 16 bands) that holds its
// remaining bands (less padded work; the slot layout stays the tile's).
// kSmall: only the tiles of 12 outputs per thread (32 x 32, 64 x 16), for
// the kernel that runs two CTAs per SM.
template <bool kSmall>
__device__ __forceinline__ void sch_fp64y_batch_item(const GppDev& p, const GppWork& w, int tile, int local,
                                                     unsigned char* smem_raw, int tid) {
  const ItemCoord ic = decode_item(w, local);
  const int slabs = (min(w.band_count - ic.bb * w.bn, w.bn) + 15) / 16;  // 16-band slabs of this block
  if constexpr (kSmall) {
    if (tile == kTileY32x32) {
      if (slabs == 1) sch_fp64y_item<16, 32>(p, w, local, smem_raw, tid);
      else sch_fp64y_item<32, 32>(p, w, local, smem_raw, tid);
    } else {
      switch (slabs) {
        case 1: sch_fp64y_item<16, 16>(p, w, local, smem_raw, tid); break;
        case 2: sch_fp64y_item<32, 16>(p, w, local, smem_raw, tid); break;
        case 3: sch_fp64y_item<48, 16>(p, w, local, smem_raw, tid); break;
        default: sch_fp64y_item<64, 16>(p, w, local, smem_raw, tid); break;
      }
    }
    return;
  }
  switch (tile) {
    case kTileY32x64:
      if (slabs == 1) sch_fp64y_item<16, 64>(p, w, local, smem_raw, tid);
      else sch_fp64y_item<32, 64>(p, w, local, smem_raw, tid);
      break;
    case kTileY32x32:
      if (slabs == 1) sch_fp64y_item<16, 32>(p, w, local, smem_raw, tid);
      else sch_fp64y_item<32, 32>(p, w, local, smem_raw, tid);
      break;
    case kTileY64x16:
      switch (slabs) {
        case 1: sch_fp64y_item<16, 16>(p, w, local, smem_raw, tid); break;
        case 2: sch_fp64y_item<32, 16>(p, w, local, smem_raw, tid); break;
        case 3: sch_fp64y_item<48, 16>(p, w, local, smem_raw, tid); break;
        default: sch_fp64y_item<64, 16>(p, w, local, smem_raw, tid); break;
      }
      break;
    default:
      switch (slabs) {
        case 1: sch_fp64y_item<16, 32>(p, w, local, smem_raw, tid); break;
        case 2: sch_fp64y_item<32, 32>(p, w, local, smem_raw, tid); break;
        case 3: sch_fp64y_item<48, 32>(p, w, local, smem_raw, tid); break;
        default: sch_fp64y_item<64, 32>(p, w, local, smem_raw, tid); break;
      }
      break;
  }
}

template <bool kSmall>
__global__ void __launch_bounds__(kThreads, kSmall ? 2 : 1) sch_fp64y_batch_kernel(GppBatchView b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  const int tid = threadIdx.x;
  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(b.counter, 1);
    __syncthreads();
    const int g = s_item;
    if (g >= b.total) break;
    const int inst = batch_owner(b.item_off, b.n_inst, g);
    const GppDev p = b.dev[inst];
    const GppWork w = b.work[inst];
    const int local = g - b.item_off[inst];
    sch_fp64y_batch_item<kSmall>(p, w, b.tile[inst], local, smem_raw, tid);
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
// With one frequency set for every band, the factors are formed in
// float-float arithmetic (FP32 pairs, ~2^-44 relative, from exact splits of
// the FP64 inputs) on the FP32 pipe and each term aqsn ssx is a float-float
// product; the high halves of two g-vectors' terms are added exactly
// (TwoSum) and then once in FP64, the rounding errors and low halves summed
// in FP32 and folded into the FP64 sums once per staged chunk.  GB300's FP64
// pipe, at 1/64 of the FP32 rate, keeps the guard decisions (the FP64 path's
// own expressions) and those sums.  Both branches are formed for every term
// (about a fifth of the terms take the second one, so a warp almost always
// needs both).  With per-band frequencies each band forms its own factors
// and each term's high halves are added in FP64 one at a time.  Chunks
// holding a value outside the float-float range take FP64 factors and FP64
// multiply-adds.
constexpr int kSsxCK = 8;      // g-vectors per staged chunk

struct SsxSmem {  // column rows padded by one element (see SchYSmem)
  double a[kSsxCK][kSsxBP + 1];
  double b[kSsxCK][kSsxBP + 1];
  double2 ie[kSsxCK][kSsxBP + 1];
  double2 n[kSsxCK][kSsxBN];
  float4 nf[kSsxCK][kSsxBN];  // aqsn as float-float pairs
};
static_assert(sizeof(SsxSmem) <= 200 * 1024, "shared memory budget");

struct SsxShared {
  double2 red[kSsxBN][kNW][kThreads / 32];
  double wx[kSsxBN][kNW], iwx2[kSsxBN][kNW];
  float wxf[kSsxBN][kNW][2], iwx2f[kSsxBN][kNW][2];  // wx and 1 / wx^2 as float-float
};

// One term's ssx factor from the element's float-float values (a + i b =
// wtilde, G = I_eps wtilde, Omega2 = wtilde G): Omega2 / wx^2 when kept,
// -G conj(z) / (2 |z|^2) with z = wtilde + wx in the second branch, else 0;
// as float-float pairs (x.hi, x.lo, y.hi, y.lo).
__device__ __forceinline__ float4 ssx_factor_ff(FF a, FF b, FF b2, FF gx, FF gy, FF omx, FF omy, FF wx,
                                                FF iwx2, bool keep, bool second) {
  const FF k1x = ff_mul_raw(omx, iwx2), k1y = ff_mul_raw(omy, iwx2);
  const FF zr = ff_add(a, wx);
  const FF r = ff_rcp_raw(ff_sq_add(zr, b2));
  const FF tx = ff_dot2_raw(gx, zr, gy, ff_neg(b)), ty = ff_dot2_raw(gy, zr, gx, b);  // G conj(z)
  const FF k2x = ff_mul_raw(tx, r), k2y = ff_mul_raw(ty, r);
  const FF sx = keep ? k1x : (second ? FF{-0.5f * k2x.hi, -0.5f * k2x.lo} : FF{0.f, 0.f});
  const FF sy = keep ? k1y : (second ? FF{-0.5f * k2y.hi, -0.5f * k2y.lo} : FF{0.f, 0.f});
  return make_float4(sx.hi, sx.lo, sy.hi, sy.lo);
}

// The same factor in FP64, for elements whose inputs leave the float-float
// range: wtilde or I_eps nonzero with its larger component outside
// [2^-20, 2^20), or an item frequency |wx| outside [2^-20, 2^20).  Inside it
// every float-float intermediate (up to wtilde^2 I_eps / wx^2, within
// 2^+-103) keeps both FP32 halves normal; outside it FP32 could overflow or
// lose the low half.  Out of line, taken only by chunks that hold such an
// element.
static __device__ __noinline__ double2 ssx_factor_fp64(double a, double b, double b2, double2 ie, double wx,
                                                       double iwx2, bool keep, bool second) {
  const double2 wt = make_double2(a, b);
  const double2 g = cmul(ie, wt), om = cmul(wt, g);
  if (keep) return make_double2(om.x * iwx2, om.y * iwx2);
  if (!second) return make_double2(0.0, 0.0);
  const double zr = a + wx;
  const double q = -0.5 * rcp_f64(fma(zr, zr, b2));
  return make_double2(fma(g.x, zr, g.y * b) * q, fma(g.y, zr, -g.x * b) * q);
}

__device__ __forceinline__ void ssx_fp64_item(const GppDev& p, const GppWork& w, int item,
                                              unsigned char* smem_raw, SsxShared& sh, int tid) {
  SsxSmem& sm = *reinterpret_cast<SsxSmem*>(smem_raw);
  const int band_end = w.band_begin + w.band_count;
  const ItemCoord ic = decode_item(w, item);
  const int n1_0 = w.band_begin + ic.bb * kSsxBN;
  const int nbl = min(kSsxBN, band_end - n1_0);
  const int p0 = ic.cb * kSsxBP;
  const int ig_begin = ic.s * w.split_len;
  const int ig_end = min(ig_begin + w.split_len, p.nc);
  bool wx_out = false;
  if (tid < kSsxBN * kNW) {
    const int i = tid / kNW, iw = tid % kNW;
    const double wx = i < nbl ? p.wx[(size_t)(n1_0 + i) * p.wx_stride + iw] : 1.0;
    wx_out = !ff_freq_range(wx);
    sh.wx[i][iw] = wx;
    sh.iwx2[i][iw] = rcp_f64(wx * wx);
    const FF f = ff_of_rn(wx), g = ff_of_rn(sh.iwx2[i][iw]);
    sh.wxf[i][iw][0] = f.hi;
    sh.wxf[i][iw][1] = f.lo;
    sh.iwx2f[i][iw][0] = g.hi;
    sh.iwx2f[i][iw][1] = g.lo;
  }
  const bool item_wide = __syncthreads_or(wx_out);

  // FP64 sums of the terms' high halves (of g-vector pairs, added exactly),
  // FP32 sums of the rounding errors and low halves folded in per chunk
  double2 acc[kSsxBN][kNW];
  float2 acl[kSsxBN][kNW];
#pragma unroll
  for (int i = 0; i < kSsxBN; ++i)
#pragma unroll
    for (int iw = 0; iw < kNW; ++iw) {
      acc[i][iw] = make_double2(0.0, 0.0);
      acl[i][iw] = make_float2(0.f, 0.f);
    }

  for (int ig0 = ig_begin; ig0 < ig_end; ig0 += kSsxCK) {
    __syncthreads();
    bool chunk_wide = item_wide;  // FP64 factors and multiply-adds
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
      sm.ie[k][pl] = ie;
      chunk_wide = chunk_wide || !(ff_range(wt.x, wt.y) && ff_range(ie.x, ie.y));
    }
    for (int e = tid; e < kSsxCK * kSsxBN; e += kThreads) {
      const int k = e % kSsxCK, bl = e / kSsxCK;
      const int ig = ig0 + k, n1 = n1_0 + bl;
      double2 v = make_double2(0.0, 0.0);
      if (ig < ig_end && n1 < band_end) v = p.aqsn[(size_t)n1 * p.nc + ig];
      const FF nx = ff_of_rn(v.x), ny = ff_of_rn(v.y);
      sm.n[k][bl] = v;
      sm.nf[k][bl] = make_float4(nx.hi, nx.lo, ny.hi, ny.lo);
      chunk_wide = chunk_wide || !ff_range(v.x, v.y);
    }
    chunk_wide = __syncthreads_or(chunk_wide);

    if (!chunk_wide && p.wx_stride != 0) {
      // per-band frequencies: each band's float-float factor and term; the
      // term's high halves added in FP64
      for (int k = 0; k < kSsxCK; ++k) {
        const double a = sm.a[k][tid], b = sm.b[k][tid];
        const double2 ie = sm.ie[k][tid];
        const double b2 = guard_b2(b);
        const double thr = guard_thr(a, b2), thr2 = guard_thr2(a, b2);
        const FF fa = ff_of_rn(a), fb = ff_of_rn(b), er = ff_of_rn(ie.x), ei = ff_of_rn(ie.y);
        const FF gx = ff_dot2_raw(er, fa, ei, fb), gy = ff_dot2_raw(er, fb, ff_neg(ei), fa);  // G
        const FF omx = ff_dot2_raw(fa, gx, fb, gy), omy = ff_dot2_raw(fa, gy, ff_neg(fb), gx);  // Omega2
        const FF fb2 = ff_mul_raw(fb, fb);
#pragma unroll
        for (int i = 0; i < kSsxBN; ++i)
          if (i < nbl) {
            const float4 n0 = sm.nf[k][i];
#pragma unroll
            for (int iw = 0; iw < kNW; ++iw) {
              const double wv = guard_w(sh.wx[i][iw], a, b2);
              const bool keep = keep_nonneg(wv, thr);
              const bool second = !keep && gt_nonneg(wv, 0.0) && gt_nonneg(thr2, wv);
              const float4 s = ssx_factor_ff(fa, fb, fb2, gx, gy, omx, omy, FF{sh.wxf[i][iw][0], sh.wxf[i][iw][1]},
                                             FF{sh.iwx2f[i][iw][0], sh.iwx2f[i][iw][1]}, keep, second);
              const FF r0 = ff_dot2_raw(FF{n0.x, n0.y}, FF{s.x, s.y}, FF{n0.z, n0.w}, FF{s.z, s.w});
              const FF i0 = ff_dot2_raw(FF{n0.x, n0.y}, FF{s.z, s.w}, FF{-n0.z, -n0.w}, FF{s.x, s.y});
              acc[i][iw].x += f32_widen(r0.hi);
              acc[i][iw].y += f32_widen(i0.hi);
              acl[i][iw].x += r0.lo;
              acl[i][iw].y += i0.lo;
            }
          }
      }
#pragma unroll
      for (int i = 0; i < kSsxBN; ++i)
#pragma unroll
        for (int iw = 0; iw < kNW; ++iw) {
          acc[i][iw].x += f32_widen(acl[i][iw].x);
          acc[i][iw].y += f32_widen(acl[i][iw].y);
          acl[i][iw] = make_float2(0.f, 0.f);
        }
    } else if (!chunk_wide) {
      // one frequency set for every band: the element's factors are shared
      // by the item's bands; each term a float-float product, the high
      // halves of two g-vectors' terms added exactly and then in FP64
      static_assert(kSsxCK % 2 == 0, "g-vector pairs");
      for (int k = 0; k < kSsxCK; k += 2) {
        float4 sv[2][kNW];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const double a = sm.a[k + h][tid], b = sm.b[k + h][tid];
          const double2 ie = sm.ie[k + h][tid];
          const double b2 = guard_b2(b);
          const double thr = guard_thr(a, b2), thr2 = guard_thr2(a, b2);
          const FF fa = ff_of_rn(a), fb = ff_of_rn(b), er = ff_of_rn(ie.x), ei = ff_of_rn(ie.y);
          const FF gx = ff_dot2_raw(er, fa, ei, fb), gy = ff_dot2_raw(er, fb, ff_neg(ei), fa);  // G
          const FF omx = ff_dot2_raw(fa, gx, fb, gy), omy = ff_dot2_raw(fa, gy, ff_neg(fb), gx);  // Omega2
          const FF fb2 = ff_mul_raw(fb, fb);
#pragma unroll
          for (int iw = 0; iw < kNW; ++iw) {
            // decisions from the FP64 expressions
            const double wv = guard_w(sh.wx[0][iw], a, b2);
            const bool keep = keep_nonneg(wv, thr);
            const bool second = !keep && gt_nonneg(wv, 0.0) && gt_nonneg(thr2, wv);
            sv[h][iw] = ssx_factor_ff(fa, fb, fb2, gx, gy, omx, omy, FF{sh.wxf[0][iw][0], sh.wxf[0][iw][1]},
                                      FF{sh.iwx2f[0][iw][0], sh.iwx2f[0][iw][1]}, keep, second);
          }
        }
#pragma unroll
        for (int i = 0; i < kSsxBN; ++i)
          if (i < nbl) {
            const float4 n0 = sm.nf[k][i], n1 = sm.nf[k + 1][i];
#pragma unroll
            for (int iw = 0; iw < kNW; ++iw) {
              const float4 s0 = sv[0][iw], s1 = sv[1][iw];
              const FF r0 = ff_dot2_raw(FF{n0.x, n0.y}, FF{s0.x, s0.y}, FF{n0.z, n0.w}, FF{s0.z, s0.w});
              const FF i0 = ff_dot2_raw(FF{n0.x, n0.y}, FF{s0.z, s0.w}, FF{-n0.z, -n0.w}, FF{s0.x, s0.y});
              const FF r1 = ff_dot2_raw(FF{n1.x, n1.y}, FF{s1.x, s1.y}, FF{n1.z, n1.w}, FF{s1.z, s1.w});
              const FF i1 = ff_dot2_raw(FF{n1.x, n1.y}, FF{s1.z, s1.w}, FF{-n1.z, -n1.w}, FF{s1.x, s1.y});
              float sr, er2, si, ei2;
              two_sum_f(r0.hi, r1.hi, sr, er2);
              two_sum_f(i0.hi, i1.hi, si, ei2);
              acc[i][iw].x += f32_widen(sr);
              acc[i][iw].y += f32_widen(si);
              acl[i][iw].x += (er2 + r0.lo) + r1.lo;
              acl[i][iw].y += (ei2 + i0.lo) + i1.lo;
            }
          }
      }
#pragma unroll
      for (int i = 0; i < kSsxBN; ++i)
#pragma unroll
        for (int iw = 0; iw < kNW; ++iw) {
          acc[i][iw].x += f32_widen(acl[i][iw].x);
          acc[i][iw].y += f32_widen(acl[i][iw].y);
          acl[i][iw] = make_float2(0.f, 0.f);
        }
    } else {
      // a value outside the float-float range: FP64 factors and FP64
      // complex multiply-adds
      for (int k = 0; k < kSsxCK; ++k) {
        const double a = sm.a[k][tid], b = sm.b[k][tid];
        const double2 ie = sm.ie[k][tid];
        const double b2 = guard_b2(b);
        const double thr = guard_thr(a, b2), thr2 = guard_thr2(a, b2);
        for (int i = 0; i < kSsxBN; ++i)
          if (i < nbl) {
            const double2 an = sm.n[k][i];
#pragma unroll
            for (int iw = 0; iw < kNW; ++iw) {
              const int ib = p.wx_stride == 0 ? 0 : i;
              const double wv = guard_w(sh.wx[ib][iw], a, b2);
              const bool keep = keep_nonneg(wv, thr);
              const bool second = !keep && gt_nonneg(wv, 0.0) && gt_nonneg(thr2, wv);
              const double2 s = ssx_factor_fp64(a, b, b2, ie, sh.wx[ib][iw], sh.iwx2[ib][iw], keep, second);
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
      if (lane == 0) sh.red[i][iw][warp] = v;
    }
  __syncthreads();
  if (tid < kSsxBN * kNW) {
    const int i = tid / kNW, iw = tid % kNW;
    double sx = 0.0, sy = 0.0;
    for (int q = 0; q < kThreads / 32; ++q) {
      sx += sh.red[i][iw][q].x;
      sy += sh.red[i][iw][q].y;
    }
    w.partial[ic.pidx * kSsxBN * kNW + tid] = make_double2(sx, sy);
  }
}

__global__ void __launch_bounds__(kThreads) ssx_fp64_kernel(GppDev p, GppWork w) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  __shared__ SsxShared sh;
  const int tid = threadIdx.x;
  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(w.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= w.n_items) break;
    ssx_fp64_item(p, w, item, smem_raw, sh, tid);
  }
}

// ---------------------------------------------------------------- batched
constexpr size_t kSchBatchSmem =
    sizeof(SchSmem<16, 64>) > sizeof(SchSmem<64, 16>) ? sizeof(SchSmem<16, 64>) : sizeof(SchSmem<64, 16>);
static_assert(kSchBatchSmem >= sizeof(SchSmem<32, 32>), "batched smem covers every tile shape");

__global__ void __launch_bounds__(kThreads, 1) sch_fp64_batch_kernel(GppBatchView b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  const int tid = threadIdx.x;
  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(b.counter, 1);
    __syncthreads();
    const int g = s_item;
    if (g >= b.total) break;
    const int inst = batch_owner(b.item_off, b.n_inst, g);
    const GppDev p = b.dev[inst];
    const GppWork w = b.work[inst];
    const int local = g - b.item_off[inst];
    switch (b.tile[inst]) {
      case kTile16x64: sch_fp64_item<16, 64>(p, w, local, smem_raw, tid); break;
      case kTile64x16: sch_fp64_item<64, 16>(p, w, local, smem_raw, tid); break;
      default: sch_fp64_item<32, 32>(p, w, local, smem_raw, tid); break;
    }
  }
}

__global__ void __launch_bounds__(kThreads) ssx_fp64_batch_kernel(GppBatchView b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  __shared__ SsxShared sh;
  const int tid = threadIdx.x;
  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(b.counter, 1);
    __syncthreads();
    const int g = s_item;
    if (g >= b.total) break;
    const int inst = batch_owner(b.item_off, b.n_inst, g);
    ssx_fp64_item(b.dev[inst], b.work[inst], g - b.item_off[inst], smem_raw, sh, tid);
  }
}

// The shared-memory carve-out at its maximum: two CTAs of the main passes
// hold up to ~210 KB between them.
template <typename K>
int blocks_per_sm(K kernel, size_t smem) {
  int n = 0;
  cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, kThreads, smem);
  return n > 0 ? n : 1;
}

}  // namespace

int sch_blocks_per_sm_fp64() { return blocks_per_sm(sch_fp64_kernel<kBN, kBP>, sizeof(SchSmem<kBN, kBP>)); }
int sch_blocks_per_sm_fp64y() {
  return blocks_per_sm(sch_fp64y_kernel<kBNY, kBPY>, sizeof(SchYSmem<kBNY, kBPY>));
}

cudaError_t launch_sch_fp64y(const GppDev& p, const GppWork& w, int grid, cudaStream_t s) {
  constexpr size_t smem = sizeof(SchYSmem<kBNY, kBPY>);
  cudaError_t e = cudaFuncSetAttribute(sch_fp64y_kernel<kBNY, kBPY>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(sch_fp64y_kernel<kBNY, kBPY>, cudaFuncAttributePreferredSharedMemoryCarveout,
                           cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  sch_fp64y_kernel<kBNY, kBPY><<<grid, kThreads, smem, s>>>(p, w);
  return cudaGetLastError();
}
int ssx_blocks_per_sm_fp64() { return blocks_per_sm(ssx_fp64_kernel, sizeof(SsxSmem)); }
int sch_batch_blocks_per_sm_fp64() { return blocks_per_sm(sch_fp64_batch_kernel, kSchBatchSmem); }
int sch_batch_blocks_per_sm_fp64y(bool small) {
  return small ? blocks_per_sm(sch_fp64y_batch_kernel<true>, kSchYBatchSmallSmem)
               : blocks_per_sm(sch_fp64y_batch_kernel<false>, kSchYBatchSmem);
}

cudaError_t launch_sch_fp64y_batch(const GppBatchView& b, int grid, bool small, cudaStream_t s) {
  if (small) {
    cudaError_t e = cudaFuncSetAttribute(sch_fp64y_batch_kernel<true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSchYBatchSmallSmem);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(sch_fp64y_batch_kernel<true>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    sch_fp64y_batch_kernel<true><<<grid, kThreads, kSchYBatchSmallSmem, s>>>(b);
    return cudaGetLastError();
  }
  cudaError_t e = cudaFuncSetAttribute(sch_fp64y_batch_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kSchYBatchSmem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(sch_fp64y_batch_kernel<false>, cudaFuncAttributePreferredSharedMemoryCarveout,
                           cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  sch_fp64y_batch_kernel<false><<<grid, kThreads, kSchYBatchSmem, s>>>(b);
  return cudaGetLastError();
}
int ssx_batch_blocks_per_sm_fp64() { return blocks_per_sm(ssx_fp64_batch_kernel, sizeof(SsxSmem)); }

cudaError_t launch_sch_fp64(const GppDev& p, const GppWork& w, int grid, cudaStream_t s) {
  constexpr size_t smem = sizeof(SchSmem<kBN, kBP>);
  cudaError_t e = cudaFuncSetAttribute(sch_fp64_kernel<kBN, kBP>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(sch_fp64_kernel<kBN, kBP>, cudaFuncAttributePreferredSharedMemoryCarveout,
                           cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  sch_fp64_kernel<kBN, kBP><<<grid, kThreads, smem, s>>>(p, w);
  return cudaGetLastError();
}

cudaError_t launch_ssx_fp64(const GppDev& p, const GppWork& w, int grid, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(ssx_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       sizeof(SsxSmem));
  if (e != cudaSuccess) return e;
  ssx_fp64_kernel<<<grid, kThreads, sizeof(SsxSmem), s>>>(p, w);
  return cudaGetLastError();
}

cudaError_t launch_sch_fp64_batch(const GppBatchView& b, int grid, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(sch_fp64_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kSchBatchSmem);
  if (e != cudaSuccess) return e;
  sch_fp64_batch_kernel<<<grid, kThreads, kSchBatchSmem, s>>>(b);
  return cudaGetLastError();
}

cudaError_t launch_ssx_fp64_batch(const GppBatchView& b, int grid, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(ssx_fp64_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       sizeof(SsxSmem));
  if (e != cudaSuccess) return e;
  ssx_fp64_batch_kernel<<<grid, kThreads, sizeof(SsxSmem), s>>>(b);
  return cudaGetLastError();
}

}  // namespace sigma
