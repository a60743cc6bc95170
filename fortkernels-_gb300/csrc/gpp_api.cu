// C ABI of the GPP path: plans, device-resident execution and the
// host-pointer drop-in for BGW-Kernels/gppKer.cpp:303-439.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "sigma_gpp.h"
#include "sigma_internal.cuh"
#include "ff_plan.h"
#include "ff_ozaki.cuh"
#include "gpp_tensor.cuh"
#include "runtime.h"

namespace sigma {
int sch_blocks_per_sm_fp64();
int ssx_blocks_per_sm_fp64();
int sch_blocks_per_sm_mixed();
int ssx_blocks_per_sm_mixed();
}  // namespace sigma

struct sigma_gpp_plan_s {
  int device = 0;
  int nb = 0, nvband = 0, nc = 0, ng = 0, precision = 0;
  int valid_columns = 0;
  int sch_grid = 0, ssx_grid = 0, schy_grid = 0, schmy_grid = 0;
  sigma::GppWork sch{}, ssx{};
  sigma::GppWork schy{};      // FP64 main pass for shared frequencies (shares sch's buffers)
  sigma::GppWork schmy{};     // mixed main pass for shared frequencies (shares sch's buffers)
  sigma::GppWork prepw{};     // pre-pass blocks: sch's, rounded up to even counts
  sigma_ff_plan ff = nullptr; // tensor form: the contraction plan (3 slabs = 3 frequencies)
  // tensor form with nvband <= kFusedBands: the factor pass that also sums
  // the occupied bands (its ssx partials in the plan's block)
  bool fused = false;
  sigma::FactorJob fac{};
  int fac_grid = 0;

  sigma::MixedPrep prep{};    // FP32 operands of the mixed path (unused for FP64)
  void* block = nullptr;      // one device allocation for everything below
  int* igp_of = nullptr;      // [ng]
  int* counters = nullptr;    // [2] item counters, [2] device status word
  double2* acht_n1 = nullptr; // [nb + nvband][3]
  std::vector<int> host_inv, host_indinv;  // kept for the host drop-in's plan cache
  // optional per-launch timing: events around the main pass, the occupied-band
  // pass and the rest (pre-pass and reductions) of each execution
  bool timing = false;
  std::vector<cudaEvent_t> events;  // 4 per recorded execution
  int recorded = 0;
};

namespace {
constexpr int kMaxTimedExecutions = 256;
}

namespace sigma {

void gpp_size_work(GppWork& w, int band_begin, int band_count, int bn, int bp, int nc, int ng,
               int grid, int items_per_slot) {
  w.band_begin = band_begin;
  w.band_count = band_count;
  w.bn = bn;
  w.n_band_blocks = (band_count + bn - 1) / bn;
  w.n_col_blocks = (ng + bp - 1) / bp;
  const long long base = (long long)w.n_band_blocks * w.n_col_blocks;
  if (base == 0) {
    w.n_splits = 1;
    w.split_len = nc;
    w.n_items = 0;
    return;
  }
  const long long want = (long long)items_per_slot * grid;
  long long s = (want + base - 1) / base;
  if (s < 1) s = 1;
  int len = (int)((nc + s - 1) / s);
  len = (len + kCK - 1) / kCK * kCK;
  if (len < kCK) len = kCK;
  w.split_len = len;
  w.n_splits = (nc + len - 1) / len;
  w.n_items = (int)(base * w.n_splits);
}

// Column map of BGW-Kernels/gppKer.cpp:322-328.  Returns SIGMA_OK or
// SIGMA_ERR_INDEX_RANGE where the reference would read out of bounds
// (indinv at indigp > ncouls, aqsmtemp / vcoul at igp == ncouls).
int gpp_map_columns(int nc, int ng, const int* inv, const int* indinv, int indinv_len,
                std::vector<int>& igp_of, int& valid) {
  igp_of.resize(ng);
  valid = 0;
  for (int my_igp = 0; my_igp < ng; ++my_igp) {
    const int indigp = inv[my_igp];
    if (indigp < 0 || indigp > nc) return SIGMA_ERR_INDEX_RANGE;
    int igp;
    if (indigp == nc) {
      igp = nc - 1;
    } else {
      if (indigp >= indinv_len) return SIGMA_ERR_INDEX_RANGE;
      igp = indinv[indigp];
    }
    if (igp > nc || igp < 0) {
      igp_of[my_igp] = -1;
      continue;
    }
    if (igp == nc) return SIGMA_ERR_INDEX_RANGE;
    igp_of[my_igp] = igp;
    ++valid;
  }
  return SIGMA_OK;
}

int gpp_check_shape(int nb, int nvband, int nc, int ng, int nstart, int nend) {
  if (nb <= 0 || nc <= 0 || ng <= 0 || ng > nc || nvband < 0 || nvband > nb) return SIGMA_ERR_INVALID_SHAPE;
  if (nstart != 0 || nend - nstart != kNW) return SIGMA_ERR_INVALID_SHAPE;
  return SIGMA_OK;
}

namespace {

constexpr int kItemsPerSlot = 48;       // work items per resident CTA (load balance of the tail)
constexpr int kItemsPerSlotMixed = 12;  // mixed items are 64x cheaper: fewer, longer items
constexpr int kItemsPerSlotY = 24;      // shared-frequency FP64 items (64 x 16 tiles, 2 CTAs per SM)
constexpr int kItemsPerSlotMY = 12;     // shared-frequency mixed items (64 x 32 tiles, 1 CTA per SM)

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace
}  // namespace sigma

extern "C" int sigma_gpp_plan_create(sigma_gpp_plan* plan_out, int number_bands, int nvband,
                                     int ncouls, int ngpown, int nstart, int nend,
                                     const int* inv_igp_index, const int* indinv,
                                     int indinv_len, int precision) {
  using namespace sigma;
  if (!plan_out || !inv_igp_index || !indinv) return SIGMA_ERR_NULL;
  *plan_out = nullptr;
  int st = gpp_check_shape(number_bands, nvband, ncouls, ngpown, nstart, nend);
  if (st != SIGMA_OK) return st;
  if (precision != SIGMA_PREC_FP64 && precision != SIGMA_PREC_MIXED && precision != SIGMA_PREC_TENSOR)
    return SIGMA_ERR_UNSUPPORTED;
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

  auto* p = new sigma_gpp_plan_s();
  p->device = dev;
  p->nb = number_bands;
  p->nvband = nvband;
  p->nc = ncouls;
  p->ng = ngpown;
  p->precision = precision;
  p->valid_columns = valid;
  const bool tensor = precision == SIGMA_PREC_TENSOR;
  // the tensor form keeps the mixed form's pre-pass for the occupied bands
  const bool mixed = precision == SIGMA_PREC_MIXED || tensor;
  p->sch_grid = sms * (mixed ? sch_blocks_per_sm_mixed() : sch_blocks_per_sm_fp64());
  p->ssx_grid = sms * (mixed ? ssx_blocks_per_sm_mixed() : ssx_blocks_per_sm_fp64());
  gpp_size_work(p->sch, 0, number_bands, kBN, mixed ? kBPM : kBP, ncouls, ngpown, p->sch_grid,
            mixed ? kItemsPerSlotMixed : kItemsPerSlot);
  gpp_size_work(p->ssx, 0, nvband, kSsxBN, kSsxBP, ncouls, ngpown, p->ssx_grid, 2);
  if (p->sch.n_items < p->sch_grid) p->sch_grid = p->sch.n_items;
  if (p->ssx.n_items < p->ssx_grid) p->ssx_grid = p->ssx.n_items;
  if (!mixed) {
    p->schy_grid = sms * sch_blocks_per_sm_fp64y();
    gpp_size_work(p->schy, 0, number_bands, kBNY, kBPY, ncouls, ngpown, p->schy_grid, kItemsPerSlotY);
    if (p->schy.n_items < p->schy_grid) p->schy_grid = p->schy.n_items;
  }
  if (mixed && !tensor) {
    p->schmy_grid = sms * sch_blocks_per_sm_mixedy();
    gpp_size_work(p->schmy, 0, number_bands, 2 * kBN, 2 * kBPM, ncouls, ngpown, p->schmy_grid,
                  kItemsPerSlotMY);
    if (p->schmy.n_items < p->schmy_grid) p->schmy_grid = p->schmy.n_items;
  }
  p->prepw = p->sch;
  p->prepw.n_col_blocks = (p->sch.n_col_blocks + 1) / 2 * 2;
  p->prepw.n_band_blocks = (p->sch.n_band_blocks + 1) / 2 * 2;

  const size_t b_igp = align_up(sizeof(int) * ngpown, 256);
  const size_t b_cnt = 256;
  const size_t b_n1 = align_up(sizeof(double2) * (size_t)(number_bands + nvband) * kNW, 256);
  const size_t b_sch = align_up(sizeof(double2) * std::max({(size_t)p->sch.n_items * kBN,
                                                            (size_t)p->schy.n_items * kBNY,
                                                            (size_t)p->schmy.n_items * 2 * kBN}) * kNW,
                                256);
  const size_t b_ssx = align_up(sizeof(double2) * (size_t)p->ssx.n_items * kSsxBN * kNW, 256);
  const int nc_pad = (ncouls + kCK - 1) / kCK * kCK;
  // the fused tensor factor pass needs none of the mixed form's FP32 operands
  const bool fused = tensor && factor_fuses_ssx(nvband);
  const size_t col_elems = mixed && !fused ? (size_t)p->prepw.n_col_blocks * kBPM * nc_pad : 0;
  const size_t band_elems = mixed && !fused ? (size_t)p->prepw.n_band_blocks * kBN * nc_pad : 0;
  const size_t b_colA = align_up(sizeof(float4) * col_elems, 256);
  const size_t b_colB = align_up(sizeof(float2) * col_elems, 256);
  const size_t b_band = align_up(sizeof(float2) * band_elems, 256);
  const size_t b_colC = nvband > 0 ? b_colB : 0;
  size_t b_fssx = 0;
  if (tensor) {
    int st2 = ff_plan_build(&p->ff, number_bands, ncouls, ngpown, kNW, igp_of, SIGMA_FF_OZAKI_BF16);
    if (st2 != SIGMA_OK) {
      delete p;
      return st2;
    }
    if (fused) {
      const OzakiPrep* oz = ff_plan_ozaki(p->ff);
      GppDev d{};
      d.nb = number_bands;
      d.nvband = nvband;
      d.nc = ncouls;
      d.ng = ngpown;
      p->fused = true;
      p->fac_grid = sms * factor_blocks_per_sm(nvband);
      factor_job_size(p->fac, d, oz->kt, p->fac_grid, 1.0);
      p->fac.a_tiles = oz->a_tiles;
      p->fac.item_off = 0;
      factor_job_operands(p->fac, *ff_plan_dev(p->ff), *oz);
      b_fssx = align_up(factor_ssx_partial_bytes(p->fac), 256);
    }
  }
  cudaError_t e = cudaMalloc(&p->block, b_igp + b_cnt + b_n1 + b_sch + b_ssx + b_colA + b_colB + b_band +
                                            b_colC + b_fssx);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_last_cuda_error(e, "cudaMalloc(plan)", __LINE__);
    if (p->ff) sigma_ff_plan_destroy(p->ff);
    delete p;
    return SIGMA_ERR_ALLOC;
  }
  char* base = static_cast<char*>(p->block);
  p->igp_of = reinterpret_cast<int*>(base);
  p->counters = reinterpret_cast<int*>(base + b_igp);
  p->acht_n1 = reinterpret_cast<double2*>(base + b_igp + b_cnt);
  p->sch.partial = reinterpret_cast<double2*>(base + b_igp + b_cnt + b_n1);
  p->ssx.partial = reinterpret_cast<double2*>(base + b_igp + b_cnt + b_n1 + b_sch);
  p->sch.counter = p->counters;
  p->ssx.counter = p->counters + 1;
  p->schy.partial = p->sch.partial;
  p->schy.counter = p->counters;
  p->schmy.partial = p->sch.partial;
  p->schmy.counter = p->counters;
  {
    char* q = base + b_igp + b_cnt + b_n1 + b_sch + b_ssx;
    p->prep.colA = mixed ? reinterpret_cast<float4*>(q) : nullptr;
    p->prep.colB = mixed ? reinterpret_cast<float2*>(q + b_colA) : nullptr;
    p->prep.band = mixed ? reinterpret_cast<float2*>(q + b_colA + b_colB) : nullptr;
    p->prep.colC = mixed && nvband > 0 ? reinterpret_cast<float2*>(q + b_colA + b_colB + b_band) : nullptr;
    p->prep.nc_pad = nc_pad;
    p->prep.status = p->counters + 2;
    p->fac.ssx.partial = b_fssx ? reinterpret_cast<double2*>(q + b_colA + b_colB + b_band + b_colC) : nullptr;
  }
  e = cudaMemcpy(p->igp_of, igp_of.data(), sizeof(int) * ngpown, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    set_last_cuda_error(e, "cudaMemcpy(igp_of)", __LINE__);
    cudaFree(p->block);
    if (p->ff) sigma_ff_plan_destroy(p->ff);
    delete p;
    return SIGMA_ERR_CUDA;
  }
  p->host_inv.assign(inv_igp_index, inv_igp_index + ngpown);
  p->host_indinv.assign(indinv, indinv + ncouls);
  *plan_out = p;
  return SIGMA_OK;
}

extern "C" int sigma_gpp_plan_destroy(sigma_gpp_plan plan) {
  if (!plan) return SIGMA_OK;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(plan->device);
  for (cudaEvent_t e : plan->events) cudaEventDestroy(e);
  if (plan->block) cudaFree(plan->block);
  if (plan->ff) sigma_ff_plan_destroy(plan->ff);
  cudaSetDevice(cur);
  delete plan;
  return SIGMA_OK;
}

extern "C" int sigma_gpp_plan_info(sigma_gpp_plan plan, int* valid_columns, long long* terms) {
  if (!plan) return SIGMA_ERR_NULL;
  if (valid_columns) *valid_columns = plan->valid_columns;
  if (terms) *terms = (long long)plan->nb * plan->valid_columns * plan->nc * sigma::kNW;
  return SIGMA_OK;
}

extern "C" int sigma_gpp_plan_set_timing(sigma_gpp_plan plan, int enable) {
  if (!plan) return SIGMA_ERR_NULL;
  if (enable && plan->events.empty()) {
    plan->events.resize(4 * kMaxTimedExecutions);
    for (auto& e : plan->events) SIGMA_CUDA_TRY(cudaEventCreate(&e));
  }
  plan->timing = enable != 0;
  plan->recorded = 0;
  return SIGMA_OK;
}

extern "C" int sigma_gpp_plan_timing(sigma_gpp_plan plan, int* executions, double* main_ms,
                                     double* occupied_ms, double* other_ms,
                                     int* launches_per_execution) {
  if (!plan) return SIGMA_ERR_NULL;
  double tm = 0.0, to = 0.0, tr = 0.0;
  const int n = plan->recorded < kMaxTimedExecutions ? plan->recorded : kMaxTimedExecutions;
  for (int i = 0; i < n; ++i) {
    cudaEvent_t* e = &plan->events[4 * i];
    SIGMA_CUDA_TRY(cudaEventSynchronize(e[3]));
    float a = 0.f, b = 0.f, c = 0.f, t = 0.f;
    SIGMA_CUDA_TRY(cudaEventElapsedTime(&a, e[0], e[1]));
    SIGMA_CUDA_TRY(cudaEventElapsedTime(&b, e[1], e[2]));
    SIGMA_CUDA_TRY(cudaEventElapsedTime(&t, e[0], e[3]));
    c = t - a - b;
    tm += a;
    to += b;
    tr += c;
  }
  if (executions) *executions = n;
  if (main_ms) *main_ms = tm;
  if (occupied_ms) *occupied_ms = to;
  if (other_ms) *other_ms = tr;
  if (launches_per_execution) {
    const bool mixed = plan->precision == SIGMA_PREC_MIXED;
    if (plan->precision == SIGMA_PREC_TENSOR) {
      // factors written as A slices (+ band operands with occupied bands),
      // zeroed padding rows, B slices and epilogue factors (2), GEMM, its
      // reduction; the occupied-band pass; 2 reductions
      const bool occ = plan->ssx.n_items > 0;
      const sigma::OzakiPrep* oz = sigma::ff_plan_ozaki(plan->ff);
      const int pad = oz && oz->n_row_blocks * sigma::kOzRows > sigma::kNW * plan->ng ? 1 : 0;
      // fused: the factor pass (padding rows, occupied bands, B slices and
      // epilogue factors included), GEMM, its reduction, 2 reductions
      *launches_per_execution = plan->fused ? 1 + 2 + 2 : (occ ? 2 : 1) + pad + 2 + 2 + (occ ? 1 : 0) + 2;
    } else
      *launches_per_execution = (plan->sch.n_items > 0 ? (mixed ? 3 : 1) : 0) +
                                (plan->ssx.n_items > 0 ? 1 : 0) + 2;
  }
  plan->recorded = 0;
  return SIGMA_OK;
}

extern "C" int sigma_gpp_plan_status(sigma_gpp_plan plan, void* stream) {
  if (!plan) return SIGMA_ERR_NULL;
  int st = 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  SIGMA_CUDA_TRY(cudaMemcpyAsync(&st, plan->prep.status, sizeof(int), cudaMemcpyDeviceToHost, s));
  SIGMA_CUDA_TRY(cudaStreamSynchronize(s));
  if (st == SIGMA_OK && plan->ff) return sigma_ff_plan_status(plan->ff, stream);
  return st;
}

extern "C" int sigma_gpp_execute(sigma_gpp_plan plan, const double* wx_array, int wx_band_stride,
                                 double occ, const sigma_complex128* aqsmtemp,
                                 const sigma_complex128* aqsntemp,
                                 const sigma_complex128* I_eps_array,
                                 const sigma_complex128* wtilde_array, const double* vcoul,
                                 sigma_complex128* achtemp, sigma_complex128* asxtemp,
                                 sigma_complex128* acht_n1_loc, void* stream) {
  using namespace sigma;
  if (!plan) return SIGMA_ERR_NULL;
  if (!wx_array || !aqsmtemp || !aqsntemp || !I_eps_array || !wtilde_array || !vcoul || !achtemp ||
      !asxtemp)
    return SIGMA_ERR_NULL;
  if (wx_band_stride != 0 && wx_band_stride < kNW) return SIGMA_ERR_INVALID_SHAPE;
  int dev = 0;
  SIGMA_CUDA_TRY(cudaGetDevice(&dev));
  if (dev != plan->device) return SIGMA_ERR_UNSUPPORTED;
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  GppDev p;
  p.nb = plan->nb;
  p.nvband = plan->nvband;
  p.nc = plan->nc;
  p.ng = plan->ng;
  p.wx_stride = wx_band_stride;
  p.occ = occ;
  p.aqsm = reinterpret_cast<const double2*>(aqsmtemp);
  p.aqsn = reinterpret_cast<const double2*>(aqsntemp);
  p.ieps = reinterpret_cast<const double2*>(I_eps_array);
  p.wt = reinterpret_cast<const double2*>(wtilde_array);
  p.vcoul = vcoul;
  p.wx = wx_array;
  p.igp_of = plan->igp_of;

  cudaEvent_t* ev = nullptr;
  if (plan->timing && plan->recorded < kMaxTimedExecutions) ev = &plan->events[4 * plan->recorded++];
  const bool tensor = plan->precision == SIGMA_PREC_TENSOR;
  if (tensor && wx_band_stride != 0) return SIGMA_ERR_UNSUPPORTED;  // needs one frequency set
  SIGMA_CUDA_TRY(cudaMemsetAsync(plan->counters, 0, 4 * sizeof(int), s));
  const bool mixed = plan->precision == SIGMA_PREC_MIXED;
  // one frequency set for every band: the shared-factor kernels
  const bool ypath = !mixed && !tensor && wx_band_stride == 0 && plan->schy.n_items > 0;
  const bool mypath = mixed && wx_band_stride == 0 && plan->schmy.n_items > 0;
  if (mypath)  // pre-pass in float-float arithmetic (the tensor form's operand pass)
    SIGMA_CUDA_TRY(launch_tensor_factors(p, plan->prepw, &plan->prep, s));
  else if (mixed && plan->sch.n_items > 0)
    SIGMA_CUDA_TRY(launch_prep_mixed(p, plan->prepw, plan->prep, s));
  GppWork main = ypath ? plan->schy : (mypath ? plan->schmy : plan->sch);
  if (tensor) main.partial = nullptr;  // band sums land in acht_n1 directly
  if (ev) SIGMA_CUDA_TRY(cudaEventRecord(ev[0], s));
  if (tensor && plan->fused) {
    // factors written as the contraction's A slices, occupied bands summed
    // in the same pass, and the B slices and epilogue factors spread through it
    FactorJob j = plan->fac;
    j.p = p;
    j.d.aqsn = p.aqsn;
    j.d.aqsm = p.aqsm;
    j.d.vcoul = vcoul;
    j.d.vfac = 0.5;
    SIGMA_CUDA_TRY(launch_factor_pass(j, plan->fac_grid, s));
    const int st = ff_execute_weighted(plan->ff, nullptr, aqsntemp, aqsmtemp, vcoul, 0.5,
                                       reinterpret_cast<sigma_complex128*>(plan->acht_n1), stream, nullptr,
                                       true, nullptr, 1.0, nullptr, true);
    if (st != SIGMA_OK) return st;
  } else if (tensor) {
    // factors, and the occupied-band operands from the same pass
    // the factors land directly as the contraction's A slices
    SIGMA_CUDA_TRY(launch_tensor_factors(p, occupied_bands(plan->prepw, p.nvband),
                                         plan->ssx.n_items > 0 ? &plan->prep : nullptr, s,
                                         ff_plan_ozaki(plan->ff)));
    const int st = ff_execute_weighted(plan->ff, nullptr, aqsntemp, aqsmtemp, vcoul, 0.5,
                                       reinterpret_cast<sigma_complex128*>(plan->acht_n1), stream, nullptr,
                                       true);
    if (st != SIGMA_OK) return st;
  } else if (ypath)
    SIGMA_CUDA_TRY(launch_sch_fp64y(p, plan->schy, plan->schy_grid, s));
  else if (mypath)
    SIGMA_CUDA_TRY(launch_sch_mixedy(p, plan->schmy, plan->prep, plan->schmy_grid, s));
  else if (plan->sch.n_items > 0)
    SIGMA_CUDA_TRY(mixed ? launch_sch_mixed(p, plan->sch, plan->prep, plan->sch_grid, s)
                         : launch_sch_fp64(p, plan->sch, plan->sch_grid, s));
  if (ev) SIGMA_CUDA_TRY(cudaEventRecord(ev[1], s));
  if (plan->ssx.n_items > 0 && !plan->fused)
    SIGMA_CUDA_TRY((mixed || tensor) ? launch_ssx_mixed(p, plan->ssx, plan->prep, plan->ssx_grid, s)
                                     : launch_ssx_fp64(p, plan->ssx, plan->ssx_grid, s));
  if (ev) SIGMA_CUDA_TRY(cudaEventRecord(ev[2], s));
  SIGMA_CUDA_TRY(launch_gpp_reduce(main, plan->fused ? plan->fac.ssx : plan->ssx, plan->nb, plan->acht_n1,
                                   reinterpret_cast<double2*>(achtemp),
                                   reinterpret_cast<double2*>(asxtemp),
                                   reinterpret_cast<double2*>(acht_n1_loc), s));
  if (ev) SIGMA_CUDA_TRY(cudaEventRecord(ev[3], s));
  return SIGMA_OK;
}

extern "C" int sigma_gpp_selftest_gate_timeout(sigma_gpp_plan plan, const double* wx_array,
                                               const sigma_complex128* aqsmtemp,
                                               const sigma_complex128* aqsntemp,
                                               const sigma_complex128* I_eps_array,
                                               const sigma_complex128* wtilde_array, const double* vcoul,
                                               int wait_polls, void* stream) {
  using namespace sigma;
  if (!plan || !wx_array || !aqsmtemp || !aqsntemp || !I_eps_array || !wtilde_array || !vcoul)
    return SIGMA_ERR_NULL;
  if (plan->precision != SIGMA_PREC_FP64 || plan->schy.n_items == 0) return SIGMA_ERR_UNSUPPORTED;
  if (wait_polls < 1) return SIGMA_ERR_INVALID_SHAPE;
  int dev = 0;
  SIGMA_CUDA_TRY(cudaGetDevice(&dev));
  if (dev != plan->device) return SIGMA_ERR_UNSUPPORTED;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  GppDev p;
  p.nb = plan->nb;
  p.nvband = plan->nvband;
  p.nc = plan->nc;
  p.ng = plan->ng;
  p.wx_stride = 0;
  p.occ = 1.0;
  p.aqsm = reinterpret_cast<const double2*>(aqsmtemp);
  p.aqsn = reinterpret_cast<const double2*>(aqsntemp);
  p.ieps = reinterpret_cast<const double2*>(I_eps_array);
  p.wt = reinterpret_cast<const double2*>(wtilde_array);
  p.vcoul = vcoul;
  p.wx = wx_array;
  p.igp_of = plan->igp_of;
  // counters, status and four gate words (ints 16-19 of the 256-byte
  // counter block) cleared; no copy ever sets a gate word to the epoch
  SIGMA_CUDA_TRY(cudaMemsetAsync(plan->counters, 0, 256, s));
  unsigned* gate = reinterpret_cast<unsigned*>(plan->counters + 16);
  GppWork w = plan->schy;
  w.order_ks = 1;
  w.ready = gate;
  w.epoch = 1;
  w.ready_first = 1;
  w.ready_gs = std::max(1, w.n_splits);  // every later split on word 2
  w.ready_m = gate + 3;
  w.ready_status = plan->prep.status;
  w.ready_polls = wait_polls;
  SIGMA_CUDA_TRY(launch_sch_fp64y(p, w, plan->schy_grid, s));
  int dev_status = 0;
  SIGMA_CUDA_TRY(cudaMemcpyAsync(&dev_status, plan->prep.status, sizeof(int), cudaMemcpyDeviceToHost, s));
  SIGMA_CUDA_TRY(cudaStreamSynchronize(s));
  return dev_status;
}

// ---------------------------------------------------------------- host drop-in
namespace sigma {
namespace {

sigma_gpp_plan g_cached_plan = nullptr;

// Copy stream and gate words of the FP64 host drop-in, whose host-to-device
// copies run beside the sum (one per process, guarded by api_mutex()).
constexpr int kGateChunks = 8;               // words for the K splits after the first
constexpr int kGateWords = kGateChunks + 3;  // + two for split 0 + one for aqsm
struct CopyLane {
  int device = -1;
  cudaStream_t cs = nullptr;
  cudaEvent_t ev_s = nullptr, ev_done = nullptr;
  unsigned* host_words = nullptr;  // pinned, kGateWords
  unsigned epoch = 0;
};
CopyLane g_lane;

void drop_lane() {
  if (g_lane.device < 0) return;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(g_lane.device);
  if (g_lane.cs) cudaStreamDestroy(g_lane.cs);
  if (g_lane.ev_s) cudaEventDestroy(g_lane.ev_s);
  if (g_lane.ev_done) cudaEventDestroy(g_lane.ev_done);
  if (g_lane.host_words) cudaFreeHost(g_lane.host_words);
  cudaSetDevice(cur);
  g_lane = CopyLane();
}

int lane_for(int dev, CopyLane** out) {
  if (g_lane.device != dev) {
    drop_lane();
    g_lane.device = dev;
    SIGMA_CUDA_TRY(cudaStreamCreateWithFlags(&g_lane.cs, cudaStreamNonBlocking));
    SIGMA_CUDA_TRY(cudaEventCreateWithFlags(&g_lane.ev_s, cudaEventDisableTiming));
    SIGMA_CUDA_TRY(cudaEventCreateWithFlags(&g_lane.ev_done, cudaEventDisableTiming));
    SIGMA_CUDA_TRY(cudaHostAlloc(reinterpret_cast<void**>(&g_lane.host_words),
                                 sizeof(unsigned) * kGateWords, cudaHostAllocDefault));
  }
  *out = &g_lane;
  return SIGMA_OK;
}

void drop_cached_plan() {
  if (g_cached_plan) sigma_gpp_plan_destroy(g_cached_plan);
  g_cached_plan = nullptr;
  drop_lane();
}

struct HookOnce {
  HookOnce() { register_shutdown_hook(drop_cached_plan); }
};

int cached_plan(int nb, int nvband, int nc, int ng, const int* inv, const int* indinv,
                int precision, sigma_gpp_plan* out) {
  static HookOnce once;
  int dev = 0;
  SIGMA_CUDA_TRY(cudaGetDevice(&dev));
  sigma_gpp_plan c = g_cached_plan;
  if (c && c->device == dev && c->nb == nb && c->nvband == nvband && c->nc == nc && c->ng == ng &&
      c->precision == precision &&
      std::memcmp(c->host_inv.data(), inv, sizeof(int) * ng) == 0 &&
      std::memcmp(c->host_indinv.data(), indinv, sizeof(int) * nc) == 0) {
    *out = c;
    return SIGMA_OK;
  }
  drop_cached_plan();
  sigma_gpp_plan p = nullptr;
  int st = sigma_gpp_plan_create(&p, nb, nvband, nc, ng, 0, kNW, inv, indinv, nc, precision);
  if (st != SIGMA_OK) return st;
  g_cached_plan = p;
  *out = p;
  return SIGMA_OK;
}

int gpp_host(int precision, int nb, int nvband, int nc, int ng, int nstart, int nend,
             const int* inv, const int* indinv, const double* wx, double occ,
             const sigma_complex128* aqsm, const sigma_complex128* aqsn,
             const sigma_complex128* ieps, const sigma_complex128* wt, const double* vcoul,
             sigma_complex128* achtemp, sigma_complex128* asxtemp, sigma_complex128* acht_n1_loc,
             void* stream) {
  if (!inv || !indinv || !wx || !aqsm || !aqsn || !ieps || !wt || !vcoul || !achtemp || !asxtemp)
    return SIGMA_ERR_NULL;
  int st = gpp_check_shape(nb, nvband, nc, ng, nstart, nend);
  if (st != SIGMA_OK) return st;
  std::lock_guard<std::mutex> lk(api_mutex());
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || device_sm_count() <= 0) {
    cudaGetLastError();
    return SIGMA_ERR_NO_DEVICE;
  }
  sigma_gpp_plan plan = nullptr;
  st = cached_plan(nb, nvband, nc, ng, inv, indinv, precision, &plan);
  if (st != SIGMA_OK) return st;

  const size_t band_bytes = sizeof(sigma_complex128) * (size_t)nb * nc;
  const size_t col_bytes = sizeof(sigma_complex128) * (size_t)ng * nc;
  size_t off[10];
  size_t total = 0;
  const size_t sizes[10] = {band_bytes, band_bytes, col_bytes, col_bytes, sizeof(double) * (size_t)nc,
                            sizeof(double) * kNW, sizeof(sigma_complex128) * kNW,
                            sizeof(sigma_complex128) * kNW, sizeof(sigma_complex128) * (size_t)nb,
                            sizeof(unsigned) * kGateWords};
  for (int i = 0; i < 10; ++i) {
    off[i] = total;
    total += align_up(sizes[i], 256);
  }
  void* arena = nullptr;
  st = arena_get(kArenaGppInputs, total, &arena);
  if (st != SIGMA_OK) return st;
  char* a = static_cast<char*>(arena);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (precision == SIGMA_PREC_FP64 && plan->schy.n_items > 0) {
    // FP64 with the shared-frequency pass: the inputs travel on a copy
    // stream while the sum runs, each piece followed by a gate word the
    // pass's items wait for.  The items run with the K split slowest, and
    // the pieces follow them: split 0 of aqsn and of the columns the first
    // wave of items takes, aqsm (read only in the items' epilogues), split 0
    // of the other columns, then groups of splits of aqsn and all columns.
    CopyLane* lane = nullptr;
    st = lane_for(dev, &lane);
    if (st != SIGMA_OK) return st;
    const GppWork& y = plan->schy;
    const int ncb = y.n_col_blocks, nsp = y.n_splits;
    const int first = std::min(ncb, (plan->schy_grid + y.n_band_blocks - 1) / y.n_band_blocks);
    const int gs = std::max(1, (nsp - 1 + kGateChunks - 1) / kGateChunks);  // splits per later word
    const int groups = (nsp - 1 + gs - 1) / gs;
    const int m_word = 2 + groups;
    unsigned epoch = ++lane->epoch;
    if (epoch == 0) epoch = ++lane->epoch;
    for (int c = 0; c <= m_word; ++c) lane->host_words[c] = epoch;
    unsigned* gate = reinterpret_cast<unsigned*>(a + off[9]);
    // gate words cleared and counters zeroed on the caller's stream; the
    // copies start after that and after the work already queued there (no
    // operation of the copy stream needs a multiprocessor, so the sum,
    // which holds them all while it waits, cannot block a copy)
    SIGMA_CUDA_TRY(cudaMemsetAsync(gate, 0, sizes[9], s));
    SIGMA_CUDA_TRY(cudaMemsetAsync(plan->counters, 0, 4 * sizeof(int), s));
    SIGMA_CUDA_TRY(cudaEventRecord(lane->ev_s, s));
    SIGMA_CUDA_TRY(cudaStreamWaitEvent(lane->cs, lane->ev_s, 0));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + off[4], vcoul, sizes[4], cudaMemcpyHostToDevice, lane->cs));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + off[5], wx, sizes[5], cudaMemcpyHostToDevice, lane->cs));
    const size_t pitch = sizeof(sigma_complex128) * (size_t)nc;
    // rows [r0, r1) x g-vectors [k0, k1) of a [rows][nc] array
    auto block = [&](int dst, const sigma_complex128* src, int r0, int r1, int k0, int k1) -> int {
      if (r1 <= r0 || k1 <= k0) return SIGMA_OK;
      const size_t o = pitch * (size_t)r0 + sizeof(sigma_complex128) * (size_t)k0;
      SIGMA_CUDA_TRY(cudaMemcpy2DAsync(a + off[dst] + o, pitch, reinterpret_cast<const char*>(src) + o,
                                       pitch, sizeof(sigma_complex128) * (size_t)(k1 - k0), r1 - r0,
                                       cudaMemcpyHostToDevice, lane->cs));
      return SIGMA_OK;
    };
    auto word = [&](int c) -> int {
      SIGMA_CUDA_TRY(cudaMemcpyAsync(gate + c, lane->host_words + c, sizeof(unsigned),
                                     cudaMemcpyHostToDevice, lane->cs));
      return SIGMA_OK;
    };
    const int k_split0 = std::min(y.split_len, nc);
    const int g_first = std::min(first * kBPY, ng);
    int r = SIGMA_OK;
    if (r == SIGMA_OK) r = block(1, aqsn, 0, nb, 0, k_split0);
    if (r == SIGMA_OK) r = block(2, ieps, 0, g_first, 0, k_split0);
    if (r == SIGMA_OK) r = block(3, wt, 0, g_first, 0, k_split0);
    if (r == SIGMA_OK) r = word(0);
    if (r == SIGMA_OK) {
      SIGMA_CUDA_TRY(cudaMemcpyAsync(a + off[0], aqsm, sizes[0], cudaMemcpyHostToDevice, lane->cs));
      r = word(m_word);
    }
    if (r == SIGMA_OK) r = block(2, ieps, g_first, ng, 0, k_split0);
    if (r == SIGMA_OK) r = block(3, wt, g_first, ng, 0, k_split0);
    if (r == SIGMA_OK) r = word(1);
    for (int g = 0; g < groups && r == SIGMA_OK; ++g) {
      const int k0 = std::min(nc, (1 + g * gs) * y.split_len);
      const int k1 = std::min(nc, (1 + (g + 1) * gs) * y.split_len);
      r = block(1, aqsn, 0, nb, k0, k1);
      if (r == SIGMA_OK) r = block(2, ieps, 0, ng, k0, k1);
      if (r == SIGMA_OK) r = block(3, wt, 0, ng, k0, k1);
      if (r == SIGMA_OK) r = word(2 + g);
    }
    if (r != SIGMA_OK) return r;
    SIGMA_CUDA_TRY(cudaEventRecord(lane->ev_done, lane->cs));

    GppDev p;
    p.nb = nb;
    p.nvband = nvband;
    p.nc = nc;
    p.ng = ng;
    p.wx_stride = 0;
    p.occ = occ;
    p.aqsm = reinterpret_cast<const double2*>(a + off[0]);
    p.aqsn = reinterpret_cast<const double2*>(a + off[1]);
    p.ieps = reinterpret_cast<const double2*>(a + off[2]);
    p.wt = reinterpret_cast<const double2*>(a + off[3]);
    p.vcoul = reinterpret_cast<const double*>(a + off[4]);
    p.wx = reinterpret_cast<const double*>(a + off[5]);
    p.igp_of = plan->igp_of;
    GppWork w = plan->schy;
    w.order_ks = 1;
    w.ready = gate;
    w.epoch = epoch;
    w.ready_first = first;
    w.ready_gs = gs;
    w.ready_m = gate + m_word;
    w.ready_status = plan->prep.status;
    SIGMA_CUDA_TRY(launch_sch_fp64y(p, w, plan->schy_grid, s));
    SIGMA_CUDA_TRY(cudaStreamWaitEvent(s, lane->ev_done, 0));
    if (plan->ssx.n_items > 0) SIGMA_CUDA_TRY(launch_ssx_fp64(p, plan->ssx, plan->ssx_grid, s));
    auto* d_ach = reinterpret_cast<double2*>(a + off[6]);
    auto* d_asx = reinterpret_cast<double2*>(a + off[7]);
    auto* d_n1 = reinterpret_cast<double2*>(a + off[8]);
    SIGMA_CUDA_TRY(launch_gpp_reduce(plan->schy, plan->ssx, nb, plan->acht_n1, d_ach, d_asx,
                                     acht_n1_loc ? d_n1 : nullptr, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(achtemp, d_ach, sizes[6], cudaMemcpyDeviceToHost, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(asxtemp, d_asx, sizes[7], cudaMemcpyDeviceToHost, s));
    if (acht_n1_loc)
      SIGMA_CUDA_TRY(cudaMemcpyAsync(acht_n1_loc, d_n1, sizes[8], cudaMemcpyDeviceToHost, s));
    int dev_status = 0;
    SIGMA_CUDA_TRY(cudaMemcpyAsync(&dev_status, plan->prep.status, sizeof(int), cudaMemcpyDeviceToHost, s));
    SIGMA_CUDA_TRY(cudaStreamSynchronize(s));
    return dev_status == 0 ? SIGMA_OK : dev_status;
  }
  const void* src[6] = {aqsm, aqsn, ieps, wt, vcoul, wx};
  for (int i = 0; i < 6; ++i)
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + off[i], src[i], sizes[i], cudaMemcpyHostToDevice, s));
  auto* d_ach = reinterpret_cast<sigma_complex128*>(a + off[6]);
  auto* d_asx = reinterpret_cast<sigma_complex128*>(a + off[7]);
  auto* d_n1 = reinterpret_cast<sigma_complex128*>(a + off[8]);
  st = sigma_gpp_execute(plan, reinterpret_cast<const double*>(a + off[5]), 0, occ,
                         reinterpret_cast<const sigma_complex128*>(a + off[0]),
                         reinterpret_cast<const sigma_complex128*>(a + off[1]),
                         reinterpret_cast<const sigma_complex128*>(a + off[2]),
                         reinterpret_cast<const sigma_complex128*>(a + off[3]),
                         reinterpret_cast<const double*>(a + off[4]), d_ach, d_asx,
                         acht_n1_loc ? d_n1 : nullptr, stream);
  if (st != SIGMA_OK) return st;
  SIGMA_CUDA_TRY(cudaMemcpyAsync(achtemp, d_ach, sizes[6], cudaMemcpyDeviceToHost, s));
  SIGMA_CUDA_TRY(cudaMemcpyAsync(asxtemp, d_asx, sizes[7], cudaMemcpyDeviceToHost, s));
  if (acht_n1_loc)
    SIGMA_CUDA_TRY(cudaMemcpyAsync(acht_n1_loc, d_n1, sizes[8], cudaMemcpyDeviceToHost, s));
  int dev_status = 0;
  SIGMA_CUDA_TRY(cudaMemcpyAsync(&dev_status, plan->prep.status, sizeof(int), cudaMemcpyDeviceToHost, s));
  SIGMA_CUDA_TRY(cudaStreamSynchronize(s));
  if (dev_status == 0 && plan->ff) dev_status = sigma_ff_plan_status(plan->ff, stream);
  return dev_status == 0 ? SIGMA_OK : dev_status;
}

}  // namespace
}  // namespace sigma

extern "C" int sigma_gpp_fp64(int number_bands, int nvband, int ncouls, int ngpown, int nstart,
                              int nend, const int* inv_igp_index, const int* indinv,
                              const double* wx_array, double occ, const sigma_complex128* aqsmtemp,
                              const sigma_complex128* aqsntemp,
                              const sigma_complex128* I_eps_array,
                              const sigma_complex128* wtilde_array, const double* vcoul,
                              sigma_complex128* achtemp, sigma_complex128* asxtemp,
                              sigma_complex128* acht_n1_loc, void* stream) {
  return sigma::gpp_host(SIGMA_PREC_FP64, number_bands, nvband, ncouls, ngpown, nstart, nend,
                         inv_igp_index, indinv, wx_array, occ, aqsmtemp, aqsntemp, I_eps_array,
                         wtilde_array, vcoul, achtemp, asxtemp, acht_n1_loc, stream);
}

extern "C" int sigma_gpp_mixed(int number_bands, int nvband, int ncouls, int ngpown, int nstart,
                               int nend, const int* inv_igp_index, const int* indinv,
                               const double* wx_array, double occ,
                               const sigma_complex128* aqsmtemp, const sigma_complex128* aqsntemp,
                               const sigma_complex128* I_eps_array,
                               const sigma_complex128* wtilde_array, const double* vcoul,
                               sigma_complex128* achtemp, sigma_complex128* asxtemp,
                               sigma_complex128* acht_n1_loc, void* stream) {
  return sigma::gpp_host(SIGMA_PREC_MIXED, number_bands, nvband, ncouls, ngpown, nstart, nend,
                         inv_igp_index, indinv, wx_array, occ, aqsmtemp, aqsntemp, I_eps_array,
                         wtilde_array, vcoul, achtemp, asxtemp, acht_n1_loc, stream);
}

extern "C" int sigma_gpp_mixed_checked(int number_bands, int nvband, int ncouls, int ngpown, int nstart,
                                       int nend, const int* inv_igp_index, const int* indinv,
                                       const double* wx_array, double occ,
                                       const sigma_complex128* aqsmtemp, const sigma_complex128* aqsntemp,
                                       const sigma_complex128* I_eps_array,
                                       const sigma_complex128* wtilde_array, const double* vcoul,
                                       sigma_complex128* achtemp, sigma_complex128* asxtemp,
                                       sigma_complex128* acht_n1_loc, void* stream, double* rel_err_out) {
  int st = sigma::gpp_host(SIGMA_PREC_MIXED, number_bands, nvband, ncouls, ngpown, nstart, nend,
                           inv_igp_index, indinv, wx_array, occ, aqsmtemp, aqsntemp, I_eps_array,
                           wtilde_array, vcoul, achtemp, asxtemp, acht_n1_loc, stream);
  if (st != SIGMA_OK || !rel_err_out) return st;
  sigma_complex128 a64[sigma::kNW], x64[sigma::kNW];
  st = sigma::gpp_host(SIGMA_PREC_FP64, number_bands, nvband, ncouls, ngpown, nstart, nend, inv_igp_index,
                       indinv, wx_array, occ, aqsmtemp, aqsntemp, I_eps_array, wtilde_array, vcoul, a64,
                       x64, nullptr, stream);
  if (st != SIGMA_OK) return st;
  auto rel = [](sigma_complex128 x, sigma_complex128 r) {
    const double d = std::hypot(x.re - r.re, x.im - r.im), m = std::hypot(r.re, r.im);
    return m > 0.0 ? d / m : (d > 0.0 ? HUGE_VAL : 0.0);
  };
  for (int iw = 0; iw < sigma::kNW; ++iw) {
    rel_err_out[iw] = rel(achtemp[iw], a64[iw]);
    rel_err_out[sigma::kNW + iw] = rel(asxtemp[iw], x64[iw]);
  }
  return SIGMA_OK;
}

extern "C" int sigma_gpp_tensor(int number_bands, int nvband, int ncouls, int ngpown, int nstart,
                                int nend, const int* inv_igp_index, const int* indinv,
                                const double* wx_array, double occ,
                                const sigma_complex128* aqsmtemp, const sigma_complex128* aqsntemp,
                                const sigma_complex128* I_eps_array,
                                const sigma_complex128* wtilde_array, const double* vcoul,
                                sigma_complex128* achtemp, sigma_complex128* asxtemp,
                                sigma_complex128* acht_n1_loc, void* stream) {
  return sigma::gpp_host(SIGMA_PREC_TENSOR, number_bands, nvband, ncouls, ngpown, nstart, nend,
                         inv_igp_index, indinv, wx_array, occ, aqsmtemp, aqsntemp, I_eps_array,
                         wtilde_array, vcoul, achtemp, asxtemp, acht_n1_loc, stream);
}
