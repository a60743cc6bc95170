// Internal declarations shared by the sigma CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <vector>

#include "sigma_common.h"

#define SIGMA_CUDA_TRY(expr)                                  \
  do {                                                        \
    cudaError_t sigma_err_ = (expr);                          \
    if (sigma_err_ != cudaSuccess) {                          \
      sigma::set_last_cuda_error(sigma_err_, #expr, __LINE__); \
      return SIGMA_ERR_CUDA;                                  \
    }                                                         \
  } while (0)

namespace sigma {

void set_last_cuda_error(cudaError_t err, const char* what, int line);

// ---------------------------------------------------------------- constants
// Physics constants of the mini-app (BGW-Kernels/gppKer.cpp:23-27, 195-199).
constexpr double kTo1 = 1e-6;
constexpr double kLimitTwo = 0.25;          // pow(0.5, 2)
constexpr double kInvLimitOne = 4e-6;       // 1 / limitone, limitone = 1 / (4 * to1)
constexpr double kInvTo1 = 1e6;             // 1 / to1
constexpr int kNW = 3;                      // nend - nstart

// Relative half-width of the band around a pole-guard threshold inside which
// the mixed path re-takes its decision in FP64 (its FP32 |wdiff|^2 is within
// 4e-7 relative of the FP64 value; the band is 2^-19 ~ 1.9e-6).
constexpr float kGuardBand = 1.9073486328125e-06f;

// ---------------------------------------------------------------- problem
// Device view of one GPP instance.  igp_of[my_igp] is the mapped column or -1
// for a column the reference skips (BGW-Kernels/gppKer.cpp:322-328).
struct GppDev {
  int nb, nvband, nc, ng;
  int wx_stride;
  double occ;
  const double2* aqsm;   // [nb][nc]
  const double2* aqsn;   // [nb][nc]
  const double2* ieps;   // [ng][nc]
  const double2* wt;     // [ng][nc]
  const double* vcoul;   // [nc]
  const double* wx;      // [nb * wx_stride + 3]
  const int* igp_of;     // [ng]
};

// Work decomposition of one pass (sch over all bands, or ssx over the
// occupied bands): items are (band block, column block, g-vector split).
struct GppWork {
  int band_begin, band_count;  // bands covered by this pass
  int bn;                      // bands per item (partial-sum rows per item)
  int n_band_blocks, n_col_blocks, n_splits, split_len;
  int n_items;
  int* counter;                // dynamic item counter (zeroed before launch)
  double2* partial;            // [n_band_blocks][n_col_blocks][n_splits][BN][3]
  // Items run band block fastest, then the K split, then the column block;
  // with order_ks set, band block, column block, K split (the split slowest).
  int order_ks = 0;
  // Optional gate of the FP64 shared-frequency pass (with order_ks): an item
  // first waits (bounded) until the word of its inputs' piece equals epoch,
  // a word the host copies to the device after that piece, so host copies
  // overlap the sum; a wait that gives up records SIGMA_ERR_TIMEOUT.  Pieces:
  // K split 0 of the first ready_first column blocks (word 0), split 0 of
  // the others (word 1), then ready_gs splits per word.  An item's epilogue
  // (the aqsm reads) waits for ready_m.
  const unsigned* ready = nullptr;
  unsigned epoch = 0;
  int ready_first = 0, ready_gs = 1;
  const unsigned* ready_m = nullptr;
  int* ready_status = nullptr;
  int ready_polls = 1 << 22;   // polls of a gate word (256 ns apart) before a wait gives up
};

__host__ __device__ __forceinline__ int gate_word(const GppWork& w, int cb, int s) {
  return s == 0 ? (cb < w.ready_first ? 0 : 1) : 2 + (s - 1) / w.ready_gs;
}

// Tile shapes.  Every pass uses kBN-band blocks (partial-sum layout of the
// reduction); the column block width differs per precision.
constexpr int kBN = 32;    // bands per sch tile
constexpr int kBP = 32;    // columns (my_igp) per FP64 sch tile
constexpr int kBPM = 16;   // columns per mixed sch tile
constexpr int kCK = 32;    // g-vectors per staged chunk
constexpr int kThreads = 256;
constexpr int kBNY = 64;   // bands per FP64 item when the frequencies are shared
constexpr int kBPY = 16;   // columns per FP64 item when the frequencies are shared
constexpr int kSsxBN = 4;   // bands per occupied-band item
constexpr int kSsxBP = 256; // columns per occupied-band item, one per thread

// The pre-pass work of the tensor form: only the occupied bands' FP32 rows
// are read (by the occupied-band pass); the band sums run on the tensor cores.
inline GppWork occupied_bands(GppWork w, int nvband) {
  w.band_count = w.band_begin < nvband ? nvband - w.band_begin : 0;
  w.n_band_blocks = (w.band_count + kBN - 1) / kBN;
  return w;
}

// Item -> (band block, column block, g-vector split).  Band blocks vary
// fastest so that CTAs running at the same time share column data in L2.
// pidx is the item's slot in the partial-sum array, ordered
// [band block][column block][split] whatever the schedule.
struct ItemCoord {
  int bb, cb, s;
  size_t pidx;
};
__device__ __forceinline__ ItemCoord decode_item(const GppWork& w, int item) {
  ItemCoord c;
  c.bb = item % w.n_band_blocks;
  const int r = item / w.n_band_blocks;
  if (w.order_ks) {
    c.cb = r % w.n_col_blocks;
    c.s = r / w.n_col_blocks;
  } else {
    c.s = r % w.n_splits;
    c.cb = r / w.n_splits;
  }
  c.pidx = ((size_t)c.bb * w.n_col_blocks + c.cb) * w.n_splits + c.s;
  return c;
}

// FP32 operands of the mixed sch pass, prepared once per execution in
// tile-interleaved layouts so that one staged chunk is one contiguous block:
//   colA[cb][ig][pl] = (Re wtilde hi, Re wtilde lo, Im wtilde, pole-guard threshold)
//   colB[cb][ig][pl] = I_eps * wtilde
//   colC[cb][ig][pl] = Omega2 = wtilde^2 * I_eps (only with occupied bands)
//   band[bb][ig][bl] = aqsn
// with my_igp = cb*kBPM + pl, n1 = bb*kBN + bl, ig < nc_pad (padding: zero
// operands and an infinite threshold, so padded terms are dropped).
struct MixedPrep {
  float4* colA;
  float2* colB;
  float2* colC;
  float2* band;
  int nc_pad;
  int* status;  // device status word (0, or SIGMA_ERR_TIMEOUT after a bounded wait gave up)
};

// ---------------------------------------------------------------- host helpers (gpp_api.cu)
// Sizes a pass: band blocks of bn, column blocks of bp, g-vector splits so
// that the grid gets about items_per_slot items per resident CTA.
void gpp_size_work(GppWork& w, int band_begin, int band_count, int bn, int bp, int nc, int ng,
                   int grid, int items_per_slot);
// Column map of BGW-Kernels/gppKer.cpp:322-328 (-1 marks a skipped column);
// SIGMA_ERR_INDEX_RANGE where the reference would read out of bounds.
int gpp_map_columns(int nc, int ng, const int* inv, const int* indinv, int indinv_len,
                    std::vector<int>& igp_of, int& valid);
int gpp_check_shape(int nb, int nvband, int nc, int ng, int nstart, int nend);

// ---------------------------------------------------------------- launchers
cudaError_t launch_sch_fp64(const GppDev& p, const GppWork& w, int grid, cudaStream_t s);
cudaError_t launch_ssx_fp64(const GppDev& p, const GppWork& w, int grid, cudaStream_t s);
// FP64 main pass for one frequency set shared by every band (wx_stride 0):
// items of kBNY bands x kBPY columns.
cudaError_t launch_sch_fp64y(const GppDev& p, const GppWork& w, int grid, cudaStream_t s);
int sch_blocks_per_sm_fp64y();
cudaError_t launch_sch_mixed(const GppDev& p, const GppWork& w, const MixedPrep& m, int grid,
                             cudaStream_t s);
cudaError_t launch_prep_mixed(const GppDev& p, const GppWork& w, const MixedPrep& m, cudaStream_t s);
// Mixed main pass for one frequency set shared by every band: items of
// 2*kBN bands x 2*kBPM columns; the pre-pass must cover an even number of
// band and column blocks.
cudaError_t launch_sch_mixedy(const GppDev& p, const GppWork& w, const MixedPrep& m, int grid,
                              cudaStream_t s);
int sch_blocks_per_sm_mixedy();
// The pre-pass (launch_prep_mixed) must have run for the same execution.
cudaError_t launch_ssx_mixed(const GppDev& p, const GppWork& w, const MixedPrep& m, int grid,
                             cudaStream_t s);
int sch_blocks_per_sm(int precision);
int ssx_blocks_per_sm(int precision);

// The float-float pass over (column, g-vector) of one shared frequency set:
// the FP32 pre-pass operands of the occupied-band and mixed kernels (m; null:
// none; w: the pre-pass blocks) and, with oz set, the tensor form's
// frequency factors Y[iw][my_igp][ig] rounded to FP32 and written as the
// split-BF16 contraction's A slices (rows iw * ngpown + my_igp, padding rows
// zeroed) for an execution with reuse_a.  With m set and oz null it is the
// mixed form's pre-pass.
struct OzakiPrep;
cudaError_t launch_tensor_factors(const GppDev& p, const GppWork& w, const MixedPrep* m, cudaStream_t s,
                                  const OzakiPrep* oz = nullptr);

// Arguments of the fixed-order reduction of one instance.
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
// One instance of a grouped reduction (many instances per launch).
struct ReduceJob {
  ReduceArgs a;
  double2 *achtemp, *asxtemp, *acht_n1_loc;
  int row_off;  // first row (block) of this instance in the band-sum stage
};
ReduceJob gpp_reduce_job(const GppWork& sch, const GppWork& ssx, int nb, double2* acht_n1, double2* achtemp,
                         double2* asxtemp, double2* acht_n1_loc, int row_off);
int gpp_reduce_job_rows(const ReduceJob& j);
// The reductions of jobs[0 .. n) (device array): two launches for all.
cudaError_t launch_gpp_reduce_group(const ReduceJob* jobs, int n, int total_rows, cudaStream_t s);

// Sums the partials of the sch and ssx passes in a fixed order into
// acht_n1[nb][3] (workspace), achtemp[3], asxtemp[3] and acht_n1_loc[nb].
// With sch.partial null, acht_n1's first nb rows already hold the band sums.
cudaError_t launch_gpp_reduce(const GppWork& sch, const GppWork& ssx, int nb, double2* acht_n1,
                              double2* achtemp, double2* asxtemp, double2* acht_n1_loc,
                              cudaStream_t s);

// ---------------------------------------------------------------- device helpers
__device__ __forceinline__ double rcp_f64(double w) {
  // Hardware approximation of the reciprocal's leading bits, then one cubic
  // Newton-Raphson step r = r0 (1 + e + e^2), e = 1 - w r0: the relative error
  // goes from ~2^-20 to below the FP64 rounding unit.
  double r0;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r0) : "d"(w));
  double e = fma(-w, r0, 1.0);
  double e2 = fma(e, e, e);
  return fma(r0, e2, r0);
}

// 1/w for a positive normal double with two DFMA: an FP32 seed from the
// hardware reciprocal of w's leading 23 mantissa bits (the exponent handled
// on the integer pipe), then one Newton-Raphson step.  The seed is within
// 2^-22.4 (23-bit truncation plus the 2^-23.3 error of rcp.approx.f32), so
// the result is within 2^-44.8 ~ 3.2e-14 relative, from below.  For w that is
// zero, denormal or not finite the result is meaningless; callers drop those
// terms.
__device__ __forceinline__ double rcp_f64_seed32(double w) {
  const int hi = __double2hiint(w);
  const unsigned lo = (unsigned)__double2loint(w);
  const unsigned mant = (((unsigned)hi & 0xFFFFFu) << 3) | (lo >> 29);
  const float m = __uint_as_float(0x3F800000u | mant);  // 1.mant in [1, 2)
  float rm;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rm) : "f"(m));
  const unsigned rb = __float_as_uint(rm);
  const int e = (int)((rb >> 23) & 0xFFu) - 127 - (((hi >> 20) & 0x7FF) - 1023) + 1023;
  const double r0 = __hiloint2double((int)(((unsigned)e << 20) | ((rb & 0x7FFFFFu) >> 3)),
                                     (int)((rb & 0x7u) << 29));
  const double eps = fma(-w, r0, 1.0);
  return fma(r0, eps, r0);
}

__device__ __forceinline__ float rcp_f32(float w) {
  // rcp.approx.f32 plus one Newton-Raphson step r = r0 (2 - w r0).
  float r0;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(w));
  float e = fmaf(-w, r0, 1.0f);
  return fmaf(r0, e, r0);
}

// Pole-guard quantities of one (column, g-vector) in FP64.  Both precisions
// take the keep/drop decision from exactly these expressions:
//   |wdiff|^2 = fma(c, c, b*b),  c = wx - a
//   threshold = max(0.25, (a*a + b*b) * 4e-6)
// |wdiff|^2 > threshold is the reference's (wdiffr > limittwo) &&
// (delwr < limitone), since |delw|^2 = |wtilde|^2 / |wdiff|^2.
__device__ __forceinline__ double guard_b2(double b) { return __dmul_rn(b, b); }
__device__ __forceinline__ double guard_thr(double a, double b2) {
  return fmax(kLimitTwo, __dmul_rn(fma(a, a, b2), kInvLimitOne));
}
__device__ __forceinline__ double guard_w(double wx, double a, double b2) {
  double c = __dsub_rn(wx, a);
  return fma(c, c, b2);
}
// Second occupied-band branch (delwr > to1  <=>  |wdiff|^2 < |wtilde|^2 / to1).
__device__ __forceinline__ double guard_thr2(double a, double b2) {
  return __dmul_rn(fma(a, a, b2), kInvTo1);
}

// Ordered compare of non-negative doubles on the integer pipe (keeps the
// FP64 pipe for arithmetic).
__device__ __forceinline__ bool gt_nonneg(double x, double y) {
  return __double_as_longlong(x) > __double_as_longlong(y);
}

// Keep decision of the pole guard, wv = |wdiff|^2 > thr, on the integer pipe,
// with wv finite: an |wdiff|^2 that overflowed to inf drops the term, as in
// the reference, where rden = 1/inf = 0 makes delw NaN (an overflowing
// product times 0) and the guard's delwr < limitone test fails
// (BGW-Kernels/gppKer.cpp:396-404).
__device__ __forceinline__ bool keep_nonneg(double wv, double thr) {
  const long long w = __double_as_longlong(wv);
  return w > __double_as_longlong(thr) && w < 0x7FF0000000000000LL;
}

// Error-free sum (Knuth TwoSum).
__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  float bv = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bv)), __fsub_rn(b, bv));
}
__device__ __forceinline__ void two_sum_d(double a, double b, double& s, double& e) {
  s = __dadd_rn(a, b);
  double bv = __dsub_rn(s, a);
  e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bv)), __dsub_rn(b, bv));
}

// float-float accumulator: (hi, lo) += x
__device__ __forceinline__ void ff_add(float& hi, float& lo, float x) {
  float s, e;
  two_sum_f(hi, x, s, e);
  e = __fadd_rn(e, lo);
  hi = __fadd_rn(s, e);
  lo = __fsub_rn(e, __fsub_rn(hi, s));
}

// Neumaier-compensated double accumulator
struct Comp {
  double s = 0.0, c = 0.0;
  __device__ __forceinline__ void add(double x) {
    double t, e;
    two_sum_d(s, x, t, e);
    s = t;
    c = __dadd_rn(c, e);
  }
  __device__ __forceinline__ double value() const { return __dadd_rn(s, c); }
};

// Butterfly combine of compensated pairs; every lane ends with the same value
// (TwoSum's error term is exact, so a+b and b+a agree bit for bit).
__device__ __forceinline__ double warp_sum_comp(Comp c) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double s2 = __shfl_xor_sync(0xffffffffu, c.s, o);
    const double c2 = __shfl_xor_sync(0xffffffffu, c.c, o);
    double t, e;
    two_sum_d(c.s, s2, t, e);
    c.s = t;
    c.c = __dadd_rn(__dadd_rn(c.c, c2), e);
  }
  return c.value();
}

}  // namespace sigma
