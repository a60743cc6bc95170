// Batched GPP: many sigma instances through one work queue per pass.
//
// The reference evaluates one instance per run of its driver
// (BGW-Kernels/gppKer.cpp:161-449).  A production sigma calculation has many
// (q-points, band windows) of uneven shape.  Here the main pass and the
// occupied-band pass of all instances each run as ONE persistent kernel over
// the concatenation of every instance's work items; per-instance pre-passes
// (mixed form) and the fixed-order reductions run around them, and the whole
// sequence is captured once in a CUDA graph and replayed.
//
// The tensor form (SIGMA_PREC_TENSOR) runs every stage once for all
// instances: one factor pass (frequency factors written as each instance's
// contraction A slices, occupied bands summed in the same pass), one pass
// for the B slices and one for the epilogue factors, ONE split-BF16 tcgen05
// GEMM whose work table lists the items of every instance's contraction, one
// contraction reduction and the two fixed-order GPP reductions: seven
// launches per execution whatever the number of instances.  Every instance
// keeps its own slice images (about 36 B per column and g-vector plus 24 B
// per band and g-vector).  Instances with more than kFusedBands occupied
// bands take the earlier form instead: per-instance contractions in stream
// order over one shared slice workspace, occupied bands in a separate pass.
//
// The FP64 and mixed forms reduce all instances with the grouped reduction
// (two launches).
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "sigma_gpp.h"
#include "sigma_internal.cuh"
#include "gpp_batch.cuh"
#include "ff_plan.h"
#include "ff_ozaki.cuh"
#include "gpp_tensor.cuh"
#include "runtime.h"

namespace sigma {
int sch_blocks_per_sm_fp64();
}

struct sigma_gpp_batch_s {
  int device = 0, n = 0, precision = 0;
  std::vector<sigma::GppDev> dev;
  std::vector<sigma::GppWork> sch, ssx;
  std::vector<sigma::MixedPrep> prep;
  std::vector<sigma::GppWork> prepw;  // pre-pass block counts per instance
  std::vector<int> tile, sch_off, ssx_off;
  std::vector<double2*> acht_n1;
  std::vector<sigma_gpp_instance> inst;
  long long terms = 0;
  int sch_grid = 0, ssx_grid = 0, launches = 0;
  int tensor_split_tiles = 0;  // K' tiles per contraction item, every instance (0: each sized as its plan)
  bool all_shared_wx = true;  // every instance has one frequency set for all bands
  bool fp64y_small = false;   // the shared-frequency FP64 pass runs its two-CTA kernel
  bool mixedy = false;        // mixed main pass on the shared-factor kernel
  void* block = nullptr;
  sigma::GppBatchView sch_view{}, ssx_view{};
  int* counters = nullptr;  // [0] main pass, [1] occupied-band pass, [2] status
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  // tensor form
  std::vector<sigma_ff_plan> ff;   // per instance (3 slabs, GPP column map)
  void* tensor_ws = nullptr;       // slice images: one region per instance (grouped) or one shared
  void* tiles = nullptr;
  bool grouped = false;            // every stage one launch for all instances
  void* group_block = nullptr;     // descriptors, item table, ssx partials
  const sigma::FactorJob* d_fac = nullptr;
  int fac_total = 0, fac_grid = 0, fac_nvband = 0;
  sigma::OzGroup grp{};
  // grouped reductions (every form)
  const sigma::ReduceJob* d_red = nullptr;
  int red_warps = 0;
  void* red_block = nullptr;
  std::vector<sigma::GppWork> fssx;  // grouped tensor form: the factor pass's ssx partials per instance
};

namespace sigma {
namespace {

constexpr int kBatchItemsPerSlot = 16;
size_t up256(size_t v) { return (v + 255) / 256 * 256; }

// Least padded work among the FP64 tile shapes of one kernel family (columns
// padded up to the tile; bands up to the tile, or to 16 in the
// shared-frequency family, whose last band block runs a shorter item), ties
// to the family's first tile.
int least_padding_tile(int nb, int ng, bool shared) {
  const int t0 = shared ? kTileY64x32 : kTile32x32, t1 = shared ? kTileCount : kTileY64x32;
  int best = t0;
  double best_cost = 1e300;
  for (int t = t0; t < t1; ++t) {
    const int bq = shared ? 16 : tile_bn(t);
    const double cost = (double)((nb + bq - 1) / bq * bq) *
                        (double)((ng + tile_bp(t) - 1) / tile_bp(t) * tile_bp(t));
    if (cost < best_cost - 0.5) {
      best_cost = cost;
      best = t;
    }
  }
  return best;
}

// Splits so that one item of this instance holds about `target` terms.
void size_instance(GppWork& w, int band_count, int bn, int bp, int nc, int ng, double target) {
  gpp_size_work(w, 0, band_count, bn, bp, nc, ng, 1, 1);
  if (w.n_items == 0) return;
  const double per_block = (double)bn * bp * nc * kNW;
  int s = (int)(per_block / target + 0.5);
  if (s < 1) s = 1;
  int len = (nc + s - 1) / s;
  len = (len + kCK - 1) / kCK * kCK;
  w.split_len = len;
  w.n_splits = (nc + len - 1) / len;
  w.n_items = w.n_band_blocks * w.n_col_blocks * w.n_splits;
}

// Order of the grouped contraction's item table.  The kernel's static
// schedule gives CTA c the items c, c + G, c + 2G, ... (G CTAs), and the
// instances' items differ in length (K' tiles), so in table order some CTAs
// would draw several long items.  Items are taken longest first, one round
// of G at a time, each to the CTA with the least work so far (a K' tile plus
// a fixed epilogue share per item); CTAs are then numbered so that those
// holding an item of the last, partial round come first.  The reduction
// sums each row block's pieces from fixed slots, so the order changes no
// result.
void balance_item_rounds(std::vector<int4>& items, int G) {
  const int n = (int)items.size();
  if (G <= 0 || n <= G) return;
  constexpr long long kEpilogueTiles = 2;
  auto cost = [](const int4& it) { return (long long)(it.w & 0xFFFF) + kEpilogueTiles; };
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost(items[a]) > cost(items[b]); });
  const int rounds = (n + G - 1) / G;
  std::vector<long long> load(G, 0);
  std::vector<std::vector<int>> held(G);
  std::vector<int> ctas(G);
  std::iota(ctas.begin(), ctas.end(), 0);
  for (int r = 0; r < rounds; ++r) {
    std::stable_sort(ctas.begin(), ctas.end(), [&](int a, int b) { return load[a] < load[b]; });
    const int lo = r * G, hi = std::min(n, lo + G);
    for (int k = 0; k < hi - lo; ++k) {
      held[ctas[k]].push_back(order[lo + k]);
      load[ctas[k]] += cost(items[order[lo + k]]);
    }
  }
  std::vector<int> label(G);
  int next = 0;
  for (int c = 0; c < G; ++c)
    if ((int)held[c].size() == rounds) label[c] = next++;
  for (int c = 0; c < G; ++c)
    if ((int)held[c].size() != rounds) label[c] = next++;
  std::vector<int4> out(n);
  for (int c = 0; c < G; ++c)
    for (int r = 0; r < (int)held[c].size(); ++r) out[(size_t)r * G + label[c]] = items[held[c][r]];
  items.swap(out);
}

// The grouped tensor form: every instance's contraction plan over its own
// slice images (items of about the same number of K tiles in every plan),
// the factor-pass jobs, the contraction jobs and the GEMM's item table in
// one device block.
int build_tensor_group(sigma_gpp_batch_s* b, const sigma_gpp_instance* inst,
                       const std::vector<std::vector<int>>& igp, int sms) {
  const int n = b->n;
  std::vector<size_t> toff(n);
  size_t tbytes = 0;
  long long tiles = 0;  // K' tiles x band blocks of every contraction
  double elems = 0.0;   // (column, g-vector) pairs of every instance
  for (int i = 0; i < n; ++i) {
    const sigma_gpp_instance& q = inst[i];
    size_t tb = 0;
    const int st = ff_plan_tile_bytes(q.number_bands, q.ncouls, q.ngpown, kNW, &tb);
    if (st != SIGMA_OK) return st;
    toff[i] = tbytes;
    tbytes += (tb + 1023) / 1024 * 1024;
    const long long nrb = (kNW * q.ngpown + kOzRows - 1) / kOzRows, kt = (q.ncouls + kOzKTile - 1) / kOzKTile;
    tiles += nrb * 2 * kt * ((q.number_bands + kOzCols - 1) / kOzCols);
    elems += (double)q.ngpown * q.ncouls;
  }
  cudaError_t e = cudaMalloc(&b->tensor_ws, tbytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_last_cuda_error(e, "cudaMalloc(batch slice images)", __LINE__);
    return SIGMA_ERR_ALLOC;
  }
  // GEMM items of tensor_split_tiles K' tiles in every instance (one static
  // schedule of equal items), or each instance's items sized as its
  // single-instance plan sizes them (about 20 per CTA of its own
  // contraction).  The tensor form's errors depend on where the K splits
  // fall (the drain warps' FP32 sums span an item's accumulator lifetimes):
  // the tuner keeps a split size only if the 48-instance set stays within
  // 1e-6 of FP64.
  (void)tiles;
  const int hint = b->tensor_split_tiles;
  b->ff.assign(n, nullptr);
  b->fac_nvband = 0;
  for (int i = 0; i < n; ++i) b->fac_nvband = std::max(b->fac_nvband, inst[i].nvband);
  b->fac_grid = sms * factor_blocks_per_sm(b->fac_nvband);
  std::vector<FactorJob> fac(n);
  std::vector<OzGroupJob> jobs(n);
  std::vector<int4> items;
  std::vector<size_t> ssx_off(n);
  size_t ssx_bytes = 0;
  int rwarps = 0;
  b->fac_total = 0;
  for (int i = 0; i < n; ++i) {
    const sigma_gpp_instance& q = inst[i];
    int st = ff_plan_build(&b->ff[i], q.number_bands, q.ncouls, q.ngpown, kNW, igp[i], SIGMA_FF_OZAKI_BF16,
                           static_cast<char*>(b->tensor_ws) + toff[i], nullptr, hint);
    if (st != SIGMA_OK) return st;
    const OzakiPrep& oz = *ff_plan_ozaki(b->ff[i]);
    // the plan's work entries, for the group's item table (with a split
    // size given, they depend on the shape and the split size only)
    OzakiTables t;
    OzakiPrep again{};
    ozaki_size(again, *ff_plan_dev(b->ff[i]), sms, nullptr, &t, hint);
    if (again.n_items != oz.n_items || again.n_entries != oz.n_entries) return SIGMA_ERR_UNSUPPORTED;
    ozaki_group_items(i, oz, t, items);

    FactorJob& fj = fac[i];
    factor_job_size(fj, b->dev[i], oz.kt, b->fac_grid, (double)q.ngpown * q.ncouls / elems);
    fj.a_tiles = oz.a_tiles;
    fj.item_off = b->fac_total;
    b->fac_total += factor_job_items(fj);
    ssx_off[i] = ssx_bytes;
    ssx_bytes += up256(factor_ssx_partial_bytes(fj));

    OzGroupJob& J = jobs[i];
    J.d = *ff_plan_dev(b->ff[i]);
    J.d.epsr = nullptr;
    J.d.aqsn = reinterpret_cast<const double2*>(q.aqsntemp);
    J.d.aqsm = reinterpret_cast<const double2*>(q.aqsmtemp);
    J.d.vcoul = q.vcoul;  // column weight 0.5 vcoul[igp]
    J.d.vfac = 0.5;
    J.oz = oz;
    J.oz.stab = nullptr;
    J.out = b->acht_n1[i];
    J.r_warp_off = rwarps;
    rwarps += q.number_bands * kNW;
    factor_job_operands(fj, J.d, J.oz);
  }
  balance_item_rounds(items, sms);  // the contraction runs on `sms` CTAs
  const size_t o_fac = 0;
  const size_t o_jobs = o_fac + up256(sizeof(FactorJob) * n);
  const size_t o_items = o_jobs + up256(sizeof(OzGroupJob) * n);
  const size_t o_ssx = o_items + up256(sizeof(int4) * std::max<size_t>(1, items.size()));
  e = cudaMalloc(&b->group_block, o_ssx + ssx_bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_last_cuda_error(e, "cudaMalloc(batch group)", __LINE__);
    return SIGMA_ERR_ALLOC;
  }
  char* base = static_cast<char*>(b->group_block);
  b->fssx.resize(n);
  for (int i = 0; i < n; ++i) {
    fac[i].ssx.partial = reinterpret_cast<double2*>(base + o_ssx + ssx_off[i]);
    b->fssx[i] = fac[i].ssx;
  }
  e = cudaMemcpy(base + o_fac, fac.data(), sizeof(FactorJob) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(base + o_jobs, jobs.data(), sizeof(OzGroupJob) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !items.empty())
    e = cudaMemcpy(base + o_items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    set_last_cuda_error(e, "cudaMemcpy(batch group)", __LINE__);
    return SIGMA_ERR_CUDA;
  }
  b->d_fac = reinterpret_cast<const FactorJob*>(base + o_fac);
  OzGroup& g = b->grp;
  g.jobs = reinterpret_cast<const OzGroupJob*>(base + o_jobs);
  g.n_jobs = n;
  g.items = reinterpret_cast<const int4*>(base + o_items);
  g.total = (int)items.size();
  g.outs = 1;
  g.segs = 1;
  for (const OzGroupJob& j : jobs) g.segs = std::max(g.segs, j.oz.max_seg);
  g.r_warps = rwarps;
  g.status = b->counters + 2;
  return SIGMA_OK;
}

// The grouped reductions of every form: one job per instance.
int build_reductions(sigma_gpp_batch_s* b) {
  const bool tensor = b->precision == SIGMA_PREC_TENSOR;
  std::vector<ReduceJob> r(b->n);
  int warps = 0;
  for (int i = 0; i < b->n; ++i) {
    GppWork main = b->sch[i];
    if (tensor) main.partial = nullptr;  // band sums already in acht_n1
    const GppWork& ssx = (tensor && b->grouped) ? b->fssx[i] : b->ssx[i];
    r[i] = gpp_reduce_job(main, ssx, b->dev[i].nb, b->acht_n1[i], reinterpret_cast<double2*>(b->inst[i].achtemp),
                          reinterpret_cast<double2*>(b->inst[i].asxtemp),
                          reinterpret_cast<double2*>(b->inst[i].acht_n1_loc), warps);
    warps += gpp_reduce_job_rows(r[i]);
  }
  cudaError_t e = cudaMalloc(&b->red_block, sizeof(ReduceJob) * b->n);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_last_cuda_error(e, "cudaMalloc(batch reductions)", __LINE__);
    return SIGMA_ERR_ALLOC;
  }
  e = cudaMemcpy(b->red_block, r.data(), sizeof(ReduceJob) * b->n, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    set_last_cuda_error(e, "cudaMemcpy(batch reductions)", __LINE__);
    return SIGMA_ERR_CUDA;
  }
  b->d_red = static_cast<const ReduceJob*>(b->red_block);
  b->red_warps = warps;
  return SIGMA_OK;
}

}  // namespace
}  // namespace sigma

extern "C" int sigma_gpp_batch_create(sigma_gpp_batch* out, int n_instances,
                                      const sigma_gpp_instance* inst, int precision,
                                      const int* tile_shape) {
  return sigma_gpp_batch_create_tuned(out, n_instances, inst, precision, tile_shape, 0, 0);
}

extern "C" int sigma_gpp_batch_create_tuned(sigma_gpp_batch* out, int n_instances,
                                            const sigma_gpp_instance* inst, int precision,
                                            const int* tile_shape, int items_per_cta,
                                            int tensor_split_tiles) {
  using namespace sigma;
  if (!out || !inst) return SIGMA_ERR_NULL;
  *out = nullptr;
  if (n_instances <= 0 || items_per_cta < 0 || tensor_split_tiles < 0) return SIGMA_ERR_INVALID_SHAPE;
  if (precision != SIGMA_PREC_FP64 && precision != SIGMA_PREC_MIXED && precision != SIGMA_PREC_TENSOR)
    return SIGMA_ERR_UNSUPPORTED;
  const bool tensor = precision == SIGMA_PREC_TENSOR;
  const bool mixed = precision == SIGMA_PREC_MIXED || tensor;  // the tensor form keeps the mixed pre-pass
  bool all_shared = true;
  for (int i = 0; i < n_instances; ++i) all_shared = all_shared && inst[i].wx_band_stride == 0;
  if (tensor && !all_shared) return SIGMA_ERR_UNSUPPORTED;  // needs one frequency set per instance
  std::vector<std::vector<int>> igp(n_instances);
  long long terms = 0;
  for (int i = 0; i < n_instances; ++i) {
    const sigma_gpp_instance& q = inst[i];
    if (!q.inv_igp_index || !q.indinv || !q.wx_array || !q.aqsmtemp || !q.aqsntemp ||
        !q.I_eps_array || !q.wtilde_array || !q.vcoul || !q.achtemp || !q.asxtemp)
      return SIGMA_ERR_NULL;
    int st = gpp_check_shape(q.number_bands, q.nvband, q.ncouls, q.ngpown, 0, kNW);
    if (st != SIGMA_OK) return st;
    if (q.wx_band_stride != 0 && q.wx_band_stride < kNW) return SIGMA_ERR_INVALID_SHAPE;
    if (tile_shape && tile_shape[i] != -1 &&
        (tile_shape[i] < 0 || tile_shape[i] >= kTileCount || tile_shared(tile_shape[i]) != all_shared))
      return SIGMA_ERR_UNSUPPORTED;
    int valid = 0;
    st = gpp_map_columns(q.ncouls, q.ngpown, q.inv_igp_index, q.indinv, q.ncouls, igp[i], valid);
    if (st != SIGMA_OK) return st;
    terms += (long long)q.number_bands * valid * q.ncouls * kNW;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return SIGMA_ERR_NO_DEVICE;
  }
  const int sms = device_sm_count();
  if (sms <= 0) return SIGMA_ERR_NO_DEVICE;

  // tensor form: every stage grouped when every instance's occupied bands
  // fit the fused factor pass; the mixed form's FP32 operands are then unused
  bool grouped = tensor;
  for (int i = 0; i < n_instances; ++i) grouped = grouped && factor_fuses_ssx(inst[i].nvband);
  const bool mixed_ops = mixed && !grouped;

  auto* b = new sigma_gpp_batch_s();
  b->device = dev;
  b->grouped = grouped;
  b->tensor_split_tiles = tensor_split_tiles;
  b->n = n_instances;
  b->precision = precision;
  b->terms = terms;
  b->inst.assign(inst, inst + n_instances);
  for (int i = 0; i < n_instances; ++i) b->all_shared_wx = b->all_shared_wx && inst[i].wx_band_stride == 0;
  // mixed with one frequency set per instance: the shared-factor kernel
  const bool mixedy = precision == SIGMA_PREC_MIXED && all_shared;
  b->mixedy = mixedy;
  // FP64 tiles first: the shared-frequency pass runs two CTAs per SM when
  // every instance takes a tile of 12 outputs per thread
  b->tile.resize(n_instances);
  for (int i = 0; i < n_instances; ++i)
    b->tile[i] = mixed ? kTile32x32
                       : (tile_shape && tile_shape[i] >= 0
                              ? tile_shape[i]
                              : least_padding_tile(inst[i].number_bands, inst[i].ngpown, all_shared));
  b->fp64y_small = !mixed && all_shared;
  for (int i = 0; i < n_instances && b->fp64y_small; ++i)
    b->fp64y_small = b->tile[i] == kTileY32x32 || b->tile[i] == kTileY64x16;
  b->sch_grid = sms * (mixedy ? sch_batch_blocks_per_sm_mixedy()
                              : mixed ? sch_batch_blocks_per_sm_mixed()
                                      : (all_shared ? sch_batch_blocks_per_sm_fp64y(b->fp64y_small)
                                                    : sch_batch_blocks_per_sm_fp64()));
  b->ssx_grid = sms * (mixed ? ssx_batch_blocks_per_sm_mixed() : ssx_batch_blocks_per_sm_fp64());
  b->dev.resize(n_instances);
  b->sch.resize(n_instances);
  b->ssx.resize(n_instances);
  b->prep.resize(n_instances);
  b->prepw.resize(n_instances);
  b->acht_n1.resize(n_instances);
  b->sch_off.assign(n_instances + 1, 0);
  b->ssx_off.assign(n_instances + 1, 0);

  // item size: the batch's terms spread over ~items_per_cta items per resident CTA
  const int ipc = items_per_cta > 0 ? items_per_cta : kBatchItemsPerSlot;
  const double target = std::max(1.0, (double)terms / ((double)b->sch_grid * ipc));
  long long ssx_terms = 0;
  for (int i = 0; i < n_instances; ++i)
    ssx_terms += (long long)inst[i].nvband * inst[i].ngpown * inst[i].ncouls * kNW;
  const double ssx_target = std::max(1.0, (double)ssx_terms / ((double)b->ssx_grid * 8));

  // device layout: per-instance buffers, then the descriptor arrays
  std::vector<size_t> o_igp(n_instances), o_n1(n_instances), o_sch(n_instances), o_ssx(n_instances),
      o_a(n_instances), o_b(n_instances), o_band(n_instances), o_c(n_instances);
  size_t total = 256;  // counters
  for (int i = 0; i < n_instances; ++i) {
    const sigma_gpp_instance& q = inst[i];
    const int t = b->tile[i];
    const int bn = mixedy ? 2 * kBN : (mixed ? kBN : tile_bn(t));
    const int bp = mixedy ? 2 * kBPM : (mixed ? kBPM : tile_bp(t));
    size_instance(b->sch[i], q.number_bands, bn, bp, q.ncouls, q.ngpown, target);
    size_instance(b->ssx[i], q.nvband, kSsxBN, kSsxBP, q.ncouls, q.ngpown, ssx_target);
    b->sch_off[i + 1] = b->sch_off[i] + b->sch[i].n_items;
    b->ssx_off[i + 1] = b->ssx_off[i] + b->ssx[i].n_items;
    const int nc_pad = (q.ncouls + kCK - 1) / kCK * kCK;
    o_igp[i] = total;
    total += up256(sizeof(int) * q.ngpown);
    o_n1[i] = total;
    total += up256(sizeof(double2) * (size_t)(q.number_bands + q.nvband) * kNW);
    o_sch[i] = total;
    total += up256(sizeof(double2) * (size_t)b->sch[i].n_items * bn * kNW);
    o_ssx[i] = total;
    total += up256(sizeof(double2) * (size_t)b->ssx[i].n_items * kSsxBN * kNW);
    // pre-pass blocks (kBN bands, kBPM columns): twice the items' with the
    // shared-factor kernel, whose items span two of each
    GppWork& pw = b->prepw[i];
    pw = b->sch[i];
    if (mixedy) {
      pw.n_col_blocks = 2 * b->sch[i].n_col_blocks;
      pw.n_band_blocks = 2 * b->sch[i].n_band_blocks;
    }
    if (mixed_ops) {
      const size_t col = (size_t)pw.n_col_blocks * kBPM * nc_pad;
      const size_t band = (size_t)pw.n_band_blocks * kBN * nc_pad;
      o_a[i] = total;
      total += up256(sizeof(float4) * col);
      o_b[i] = total;
      total += up256(sizeof(float2) * col);
      o_band[i] = total;
      total += up256(sizeof(float2) * band);
      o_c[i] = total;
      if (q.nvband > 0) total += up256(sizeof(float2) * col);
    }
  }
  const size_t o_dev = total;
  total += up256(sizeof(GppDev) * n_instances);
  const size_t o_wsch = total;
  total += up256(sizeof(GppWork) * n_instances);
  const size_t o_wssx = total;
  total += up256(sizeof(GppWork) * n_instances);
  const size_t o_prep = total;
  total += up256(sizeof(MixedPrep) * n_instances);
  const size_t o_schoff = total;
  total += up256(sizeof(int) * (n_instances + 1));
  const size_t o_ssxoff = total;
  total += up256(sizeof(int) * (n_instances + 1));
  const size_t o_tile = total;
  total += up256(sizeof(int) * n_instances);

  cudaError_t e = cudaMalloc(&b->block, total);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_last_cuda_error(e, "cudaMalloc(batch)", __LINE__);
    delete b;
    return SIGMA_ERR_ALLOC;
  }
  char* base = static_cast<char*>(b->block);
  b->counters = reinterpret_cast<int*>(base);
  for (int i = 0; i < n_instances; ++i) {
    const sigma_gpp_instance& q = inst[i];
    GppDev& p = b->dev[i];
    p.nb = q.number_bands;
    p.nvband = q.nvband;
    p.nc = q.ncouls;
    p.ng = q.ngpown;
    p.wx_stride = q.wx_band_stride;
    p.occ = q.occ;
    p.aqsm = reinterpret_cast<const double2*>(q.aqsmtemp);
    p.aqsn = reinterpret_cast<const double2*>(q.aqsntemp);
    p.ieps = reinterpret_cast<const double2*>(q.I_eps_array);
    p.wt = reinterpret_cast<const double2*>(q.wtilde_array);
    p.vcoul = q.vcoul;
    p.wx = q.wx_array;
    p.igp_of = reinterpret_cast<const int*>(base + o_igp[i]);
    b->sch[i].counter = b->counters;
    b->ssx[i].counter = b->counters + 1;
    b->sch[i].partial = reinterpret_cast<double2*>(base + o_sch[i]);
    b->ssx[i].partial = reinterpret_cast<double2*>(base + o_ssx[i]);
    b->acht_n1[i] = reinterpret_cast<double2*>(base + o_n1[i]);
    MixedPrep& m = b->prep[i];
    m.nc_pad = (q.ncouls + kCK - 1) / kCK * kCK;
    m.status = b->counters + 2;
    m.colA = mixed_ops ? reinterpret_cast<float4*>(base + o_a[i]) : nullptr;
    m.colB = mixed_ops ? reinterpret_cast<float2*>(base + o_b[i]) : nullptr;
    m.colC = mixed_ops && q.nvband > 0 ? reinterpret_cast<float2*>(base + o_c[i]) : nullptr;
    m.band = mixed_ops ? reinterpret_cast<float2*>(base + o_band[i]) : nullptr;
  }
  int rc = SIGMA_OK;
  auto up = [&](size_t off, const void* src, size_t bytes) {
    if (rc != SIGMA_OK) return;
    cudaError_t ce = cudaMemcpy(base + off, src, bytes, cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) {
      set_last_cuda_error(ce, "cudaMemcpy(batch)", __LINE__);
      rc = SIGMA_ERR_CUDA;
    }
  };
  for (int i = 0; i < n_instances; ++i) up(o_igp[i], igp[i].data(), sizeof(int) * igp[i].size());
  up(o_dev, b->dev.data(), sizeof(GppDev) * n_instances);
  up(o_wsch, b->sch.data(), sizeof(GppWork) * n_instances);
  up(o_wssx, b->ssx.data(), sizeof(GppWork) * n_instances);
  up(o_prep, b->prep.data(), sizeof(MixedPrep) * n_instances);
  up(o_schoff, b->sch_off.data(), sizeof(int) * (n_instances + 1));
  up(o_ssxoff, b->ssx_off.data(), sizeof(int) * (n_instances + 1));
  up(o_tile, b->tile.data(), sizeof(int) * n_instances);
  if (rc != SIGMA_OK) {
    cudaFree(b->block);
    delete b;
    return rc;
  }
  GppBatchView& v = b->sch_view;
  v.dev = reinterpret_cast<const GppDev*>(base + o_dev);
  v.work = reinterpret_cast<const GppWork*>(base + o_wsch);
  v.prep = reinterpret_cast<const MixedPrep*>(base + o_prep);
  v.item_off = reinterpret_cast<const int*>(base + o_schoff);
  v.tile = reinterpret_cast<const int*>(base + o_tile);
  v.n_inst = n_instances;
  v.total = b->sch_off[n_instances];
  v.counter = b->counters;
  b->ssx_view = v;
  b->ssx_view.work = reinterpret_cast<const GppWork*>(base + o_wssx);
  b->ssx_view.item_off = reinterpret_cast<const int*>(base + o_ssxoff);
  b->ssx_view.total = b->ssx_off[n_instances];
  b->ssx_view.counter = b->counters + 1;
  if (b->sch_grid > v.total) b->sch_grid = std::max(1, v.total);
  if (b->ssx_grid > b->ssx_view.total) b->ssx_grid = std::max(1, b->ssx_view.total);
  // every form: the two fixed-order reductions for all instances
  b->launches = (mixed ? 2 * n_instances : 0) + 1 + (b->ssx_view.total > 0 ? 1 : 0) + 2;
  if (tensor && grouped) {
    int st = build_tensor_group(b, inst, igp, sms);
    if (st != SIGMA_OK) {
      sigma_gpp_batch_destroy(b);
      return st;
    }
    b->launches = 5;  // factors (with B slices and epilogue factors), GEMM, its reduction, 2 reductions
  } else if (tensor) {
    // one slice workspace, sized for the largest instance
    size_t tbytes = 0;
    for (int i = 0; i < n_instances; ++i) {
      size_t tb = 0;
      int st = ff_plan_tile_bytes(inst[i].number_bands, inst[i].ncouls, inst[i].ngpown, kNW, &tb);
      if (st != SIGMA_OK) {
        sigma_gpp_batch_destroy(b);
        return st;
      }
      tbytes = std::max(tbytes, tb);
    }
    cudaError_t e2 = cudaMalloc(&b->tensor_ws, tbytes);
    if (e2 != cudaSuccess) {
      cudaGetLastError();
      set_last_cuda_error(e2, "cudaMalloc(batch tensor workspace)", __LINE__);
      sigma_gpp_batch_destroy(b);
      return SIGMA_ERR_ALLOC;
    }
    b->tiles = static_cast<char*>(b->tensor_ws);
    b->ff.assign(n_instances, nullptr);
    for (int i = 0; i < n_instances; ++i) {
      int st = ff_plan_build(&b->ff[i], inst[i].number_bands, inst[i].ncouls, inst[i].ngpown, kNW, igp[i],
                             SIGMA_FF_OZAKI_BF16, b->tiles);
      if (st != SIGMA_OK) {
        sigma_gpp_batch_destroy(b);
        return st;
      }
    }
    // per instance: factors written as A slices (+ band operands with
    // occupied bands), zeroed padding rows, B slices and epilogue factors (2),
    // GEMM, its reduction; then ssx and the reductions
    int per = 0;
    for (int i = 0; i < n_instances; ++i) {
      const OzakiPrep* oz = ff_plan_ozaki(b->ff[i]);
      const int pad = oz->n_row_blocks * kOzRows > kNW * inst[i].ngpown ? 1 : 0;
      per += (b->ssx[i].n_items > 0 ? 2 : 1) + pad + 2 + 2;
    }
    b->launches = per + (b->ssx_view.total > 0 ? 1 : 0) + 2;
  }
  int st = build_reductions(b);
  if (st != SIGMA_OK) {
    sigma_gpp_batch_destroy(b);
    return st;
  }
  *out = b;
  return SIGMA_OK;
}

extern "C" int sigma_gpp_batch_execute(sigma_gpp_batch b, void* stream) {
  using namespace sigma;
  if (!b) return SIGMA_ERR_NULL;
  int dev = 0;
  SIGMA_CUDA_TRY(cudaGetDevice(&dev));
  if (dev != b->device) return SIGMA_ERR_UNSUPPORTED;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const bool tensor = b->precision == SIGMA_PREC_TENSOR;
  const bool mixed = b->precision == SIGMA_PREC_MIXED || tensor;
  SIGMA_CUDA_TRY(cudaMemsetAsync(b->counters, 0, 4 * sizeof(int), s));
  if (tensor && b->grouped) {
    // every instance in each launch: factors (A slices, occupied bands),
    // B slices and epilogue factors, the GEMM over the group's item table,
    // its reduction
    // the factor pass writes every operand of the contractions
    SIGMA_CUDA_TRY(launch_factor_pass(b->d_fac, b->n, b->fac_total, b->fac_grid, b->fac_nvband, s));
    SIGMA_CUDA_TRY(launch_ozaki_group_gemm(b->grp, device_sm_count(), s));
    SIGMA_CUDA_TRY(launch_ozaki_group_reduce(b->grp, s));
    SIGMA_CUDA_TRY(launch_gpp_reduce_group(b->d_red, b->n, b->red_warps, s));
    return SIGMA_OK;
  }
  if (mixed && !tensor)
    for (int i = 0; i < b->n; ++i)
      if (b->sch[i].n_items > 0)
        SIGMA_CUDA_TRY(b->mixedy ? launch_tensor_factors(b->dev[i], b->prepw[i], &b->prep[i], s)
                                 : launch_prep_mixed(b->dev[i], b->prepw[i], b->prep[i], s));
  if (tensor) {
    for (int i = 0; i < b->n; ++i) {
      // factors, and the occupied-band operands from the same pass
      // the factors land directly as the contraction's A slices
      SIGMA_CUDA_TRY(launch_tensor_factors(b->dev[i], occupied_bands(b->prepw[i], b->dev[i].nvband),
                                           b->ssx[i].n_items > 0 ? &b->prep[i] : nullptr, s,
                                           ff_plan_ozaki(b->ff[i])));
      const int st = ff_execute_weighted(b->ff[i], nullptr, b->inst[i].aqsntemp, b->inst[i].aqsmtemp,
                                         b->inst[i].vcoul, 0.5,
                                         reinterpret_cast<sigma_complex128*>(b->acht_n1[i]), stream, nullptr,
                                         true);
      if (st != SIGMA_OK) return st;
    }
  } else if (b->sch_view.total > 0)
    SIGMA_CUDA_TRY(b->mixedy ? launch_sch_mixedy_batch(b->sch_view, b->sch_grid, s)
                   : mixed ? launch_sch_mixed_batch(b->sch_view, b->sch_grid, s)
                         : (b->all_shared_wx ? launch_sch_fp64y_batch(b->sch_view, b->sch_grid, b->fp64y_small, s)
                                             : launch_sch_fp64_batch(b->sch_view, b->sch_grid, s)));
  if (b->ssx_view.total > 0)
    SIGMA_CUDA_TRY(mixed ? launch_ssx_mixed_batch(b->ssx_view, b->ssx_grid, b->all_shared_wx, s)
                         : launch_ssx_fp64_batch(b->ssx_view, b->ssx_grid, s));
  SIGMA_CUDA_TRY(launch_gpp_reduce_group(b->d_red, b->n, b->red_warps, s));
  return SIGMA_OK;
}

extern "C" int sigma_gpp_batch_launch_graph(sigma_gpp_batch b, void* stream) {
  using namespace sigma;
  if (!b) return SIGMA_ERR_NULL;
  if (!stream) return SIGMA_ERR_UNSUPPORTED;  // the legacy NULL stream cannot be captured
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!b->exec) {
    SIGMA_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const int st = sigma_gpp_batch_execute(b, stream);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(s, &g);
    if (st != SIGMA_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    if (ce != cudaSuccess) {
      set_last_cuda_error(ce, "cudaStreamEndCapture", __LINE__);
      return SIGMA_ERR_CUDA;
    }
    b->graph = g;
    SIGMA_CUDA_TRY(cudaGraphInstantiate(&b->exec, b->graph, 0));
  }
  SIGMA_CUDA_TRY(cudaGraphLaunch(b->exec, s));
  return SIGMA_OK;
}

extern "C" int sigma_gpp_batch_info(sigma_gpp_batch b, long long* terms, int* items, int* launches) {
  if (!b) return SIGMA_ERR_NULL;
  if (terms) *terms = b->terms;
  if (items) *items = b->sch_view.total;
  if (launches) *launches = b->launches;
  return SIGMA_OK;
}

extern "C" int sigma_gpp_batch_status(sigma_gpp_batch b, void* stream) {
  if (!b) return SIGMA_ERR_NULL;
  int st = 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  SIGMA_CUDA_TRY(cudaMemcpyAsync(&st, b->counters + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
  SIGMA_CUDA_TRY(cudaStreamSynchronize(s));
  for (sigma_ff_plan f : b->ff)
    if (st == SIGMA_OK) st = sigma_ff_plan_status(f, stream);
  return st;
}

extern "C" int sigma_gpp_batch_destroy(sigma_gpp_batch b) {
  if (!b) return SIGMA_OK;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(b->device);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (sigma_ff_plan f : b->ff)
    if (f) sigma_ff_plan_destroy(f);
  if (b->tensor_ws) cudaFree(b->tensor_ws);
  if (b->group_block) cudaFree(b->group_block);
  if (b->red_block) cudaFree(b->red_block);
  if (b->block) cudaFree(b->block);
  cudaSetDevice(cur);
  delete b;
  return SIGMA_OK;
}

extern "C" int sigma_gpp_batched(int n_instances, const sigma_gpp_instance* inst, int precision,
                                 void* stream) {
  sigma_gpp_batch b = nullptr;
  int st = sigma_gpp_batch_create(&b, n_instances, inst, precision, nullptr);
  if (st != SIGMA_OK) return st;
  st = sigma_gpp_batch_execute(b, stream);
  if (st == SIGMA_OK) st = sigma_gpp_batch_status(b, stream);
  sigma_gpp_batch_destroy(b);
  return st;
}
