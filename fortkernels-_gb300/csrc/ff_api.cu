// C ABI of the FF schDt contraction: plans, device execution, host drop-in.
#include <algorithm>
#include <cstring>
#include <vector>

#include "sigma_ff.h"
#include "ff_internal.cuh"
#include "ff_ozaki.cuh"
#include "ff_plan.h"
#include "runtime.h"

struct sigma_ff_plan_s {
  int device = 0;
  int nb = 0, nc = 0, ng = 0, nf = 0, mode = 0;
  int grid = 0;
  sigma::FfDev dev{};
  sigma::FfWork work{};
  sigma::OzakiPrep oz{};
  void* block = nullptr;
  bool timing = false;
  std::vector<cudaEvent_t> events;  // 3 per recorded execution
  int recorded = 0;
};

namespace sigma {
namespace {

constexpr int kFfMaxTimed = 256;
size_t up256(size_t v) { return (v + 255) / 256 * 256; }

int ff_map_columns(int nc, int ng, const int* inv, const int* indinv, std::vector<int>& igp_of) {
  igp_of.resize(ng);
  for (int g = 0; g < ng; ++g) {
    const int ind = inv[g];
    if (ind < 0 || ind >= nc) return SIGMA_ERR_INDEX_RANGE;
    const int igp = indinv[ind];
    if (igp < 0 || igp >= nc) return SIGMA_ERR_INDEX_RANGE;
    igp_of[g] = igp;
  }
  return SIGMA_OK;
}

int ff_check_shape(int nb, int nc, int ng, int nf) {
  // ngpown > ncouls is rejected as FFKer_cori/ffKernel.cpp:320-325 rejects it
  if (nb <= 0 || nc <= 0 || ng <= 0 || nf <= 0 || ng > nc) return SIGMA_ERR_INVALID_SHAPE;
  return SIGMA_OK;
}

}  // namespace
}  // namespace sigma

namespace sigma {

// Plan over an already validated column map (igp_of[my_igp], -1 = column
// left out).  Shared by the FF contraction and the static remainders.
int ff_plan_build(sigma_ff_plan* out, int number_bands, int ncouls, int ngpown, int nfreq,
                  const std::vector<int>& igp_of, int mode, void* shared_tiles,
                  const int* row_kend, int split_tiles_hint, int items_per_cta) {
  *out = nullptr;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return SIGMA_ERR_NO_DEVICE;
  }
  const int sms = device_sm_count();
  if (sms <= 0) return SIGMA_ERR_NO_DEVICE;

  auto* p = new sigma_ff_plan_s();
  p->device = dev;
  p->nb = number_bands;
  p->nc = ncouls;
  p->ng = ngpown;
  p->nf = nfreq;
  p->mode = mode;
  FfDev& d = p->dev;
  d.nb = number_bands;
  d.nc = ncouls;
  d.ng = ngpown;
  d.nf = nfreq;
  d.ngp = (ngpown + kFfRows - 1) / kFfRows * kFfRows;
  FfWork& w = p->work;
  w.n_row_blocks = nfreq * (d.ngp / kFfRows);
  w.n_col_blocks = (number_bands + kFfCols - 1) / kFfCols;
  const int ktile = 16;
  const int per_sm = mode == SIGMA_FF_FP64 ? ff_fp64_blocks_per_sm() : 1;
  p->grid = sms * per_sm;
  OzakiTables tables;
  if (mode == SIGMA_FF_OZAKI_BF16) {
    ozaki_size(p->oz, d, p->grid, row_kend, &tables, split_tiles_hint, items_per_cta);
    if (p->oz.max_seg > ozaki_max_segments()) {  // ngpown below ~18: too many frequencies per tile
      delete p;
      return SIGMA_ERR_UNSUPPORTED;
    }
    if (p->oz.n_items < p->grid) p->grid = std::max(1, p->oz.n_items);
    w.n_splits = 1;
    w.split_len = ncouls;
    w.n_items = 0;
  } else {
    const long long base = (long long)w.n_row_blocks * w.n_col_blocks;
    const long long want = (long long)p->grid * (mode == SIGMA_FF_FP64 ? 16 : 8);
    long long s = (want + base - 1) / base;
    if (s < 1) s = 1;
    int len = (int)((ncouls + s - 1) / s);
    len = (len + ktile - 1) / ktile * ktile;
    w.split_len = len;
    w.n_splits = (ncouls + len - 1) / len;
    w.n_items = (int)(base * w.n_splits);
  }
  if (mode == SIGMA_FF_FP64 && w.n_items < p->grid) p->grid = w.n_items;

  const size_t b_igp = up256(sizeof(int) * ngpown);
  const size_t b_cnt = 256;
  const size_t b_part = up256(sizeof(double2) * (size_t)w.n_items * kFfCols);
  size_t b_oz = 0;
  if (mode == SIGMA_FF_OZAKI_BF16)
    b_oz = shared_tiles ? ozaki_partial_bytes(p->oz) : ozaki_prep_bytes(p->oz);
  cudaError_t e = cudaMalloc(&p->block, b_igp + b_cnt + b_part + b_oz);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_last_cuda_error(e, "cudaMalloc(ff plan)", __LINE__);
    delete p;
    return SIGMA_ERR_ALLOC;
  }
  char* base = static_cast<char*>(p->block);
  d.igp_of = reinterpret_cast<int*>(base);
  w.counter = reinterpret_cast<int*>(base + b_igp);
  w.status = w.counter + 1;
  w.partial = reinterpret_cast<double2*>(base + b_igp + b_cnt);
  if (mode == SIGMA_FF_OZAKI_BF16) {
    if (shared_tiles)
      ozaki_bind(p->oz, shared_tiles, base + b_igp + b_cnt + b_part);
    else
      ozaki_prep_bind(p->oz, base + b_igp + b_cnt + b_part);
  }
  e = cudaMemcpy(const_cast<int*>(d.igp_of), igp_of.data(), sizeof(int) * ngpown,
                 cudaMemcpyHostToDevice);
  if (e == cudaSuccess && mode == SIGMA_FF_OZAKI_BF16) e = ozaki_upload_tables(p->oz, tables);
  if (e != cudaSuccess) {
    set_last_cuda_error(e, "cudaMemcpy(ff igp_of)", __LINE__);
    cudaFree(p->block);
    delete p;
    return SIGMA_ERR_CUDA;
  }
  *out = p;
  return SIGMA_OK;
}

}  // namespace sigma

extern "C" int sigma_ff_plan_create(sigma_ff_plan* out, int number_bands, int ncouls, int ngpown,
                                    int nfreq, const int* inv_igp_index, const int* indinv,
                                    int mode) {
  using namespace sigma;
  if (!out || !inv_igp_index || !indinv) return SIGMA_ERR_NULL;
  *out = nullptr;
  int st = ff_check_shape(number_bands, ncouls, ngpown, nfreq);
  if (st != SIGMA_OK) return st;
  if (mode != SIGMA_FF_FP64 && mode != SIGMA_FF_OZAKI_BF16) return SIGMA_ERR_UNSUPPORTED;
  std::vector<int> igp_of;
  st = ff_map_columns(ncouls, ngpown, inv_igp_index, indinv, igp_of);
  if (st != SIGMA_OK) return st;
  return ff_plan_build(out, number_bands, ncouls, ngpown, nfreq, igp_of, mode);
}

extern "C" int sigma_ff_plan_destroy(sigma_ff_plan plan) {
  if (!plan) return SIGMA_OK;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(plan->device);
  for (cudaEvent_t ev : plan->events) cudaEventDestroy(ev);
  if (plan->block) cudaFree(plan->block);
  cudaSetDevice(cur);
  delete plan;
  return SIGMA_OK;
}

extern "C" int sigma_ff_plan_set_timing(sigma_ff_plan plan, int enable) {
  if (!plan) return SIGMA_ERR_NULL;
  if (enable && plan->events.empty()) {
    plan->events.resize(3 * sigma::kFfMaxTimed);
    for (auto& ev : plan->events) SIGMA_CUDA_TRY(cudaEventCreate(&ev));
  }
  plan->timing = enable != 0;
  plan->recorded = 0;
  return SIGMA_OK;
}

extern "C" int sigma_ff_plan_timing(sigma_ff_plan plan, int* executions, double* main_ms,
                                    double* other_ms, int* launches_per_execution) {
  if (!plan) return SIGMA_ERR_NULL;
  double tm = 0.0, to = 0.0;
  const int n = plan->recorded;
  for (int i = 0; i < n; ++i) {
    cudaEvent_t* ev = &plan->events[3 * i];
    SIGMA_CUDA_TRY(cudaEventSynchronize(ev[2]));
    float a = 0.f, t = 0.f;
    SIGMA_CUDA_TRY(cudaEventElapsedTime(&a, ev[0], ev[1]));
    SIGMA_CUDA_TRY(cudaEventElapsedTime(&t, ev[0], ev[2]));
    tm += a;
    to += t - a;
  }
  if (executions) *executions = n;
  if (main_ms) *main_ms = tm;
  if (other_ms) *other_ms = to;
  if (launches_per_execution) *launches_per_execution = plan->mode == SIGMA_FF_FP64 ? 2 : 4;
  plan->recorded = 0;
  return SIGMA_OK;
}

namespace sigma {
const OzakiPrep* ff_plan_ozaki(sigma_ff_plan plan) {
  return plan && plan->mode == SIGMA_FF_OZAKI_BF16 ? &plan->oz : nullptr;
}
const FfDev* ff_plan_dev(sigma_ff_plan plan) { return plan ? &plan->dev : nullptr; }

int ff_plan_tile_bytes(int number_bands, int ncouls, int ngpown, int nfreq, size_t* bytes) {
  FfDev d{};
  d.nb = number_bands;
  d.nc = ncouls;
  d.ng = ngpown;
  d.nf = nfreq;
  OzakiPrep oz{};
  const int sms = device_sm_count();
  if (sms <= 0) return SIGMA_ERR_NO_DEVICE;
  ozaki_size(oz, d, sms);
  if (oz.max_seg > ozaki_max_segments()) return SIGMA_ERR_UNSUPPORTED;
  *bytes = ozaki_tile_bytes(oz);
  return SIGMA_OK;
}
}  // namespace sigma

extern "C" int sigma_ff_plan_bands(sigma_ff_plan plan, int* number_bands) {
  if (!plan || !number_bands) return SIGMA_ERR_NULL;
  *number_bands = plan->nb;
  return SIGMA_OK;
}

extern "C" int sigma_ff_plan_status(sigma_ff_plan plan, void* stream) {
  if (!plan) return SIGMA_ERR_NULL;
  int st = 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  SIGMA_CUDA_TRY(cudaMemcpyAsync(&st, plan->work.status, sizeof(int), cudaMemcpyDeviceToHost, s));
  SIGMA_CUDA_TRY(cudaStreamSynchronize(s));
  return st;
}

namespace sigma {

int ff_execute_weighted(sigma_ff_plan plan, const sigma_complex128* I_epsR,
                        const sigma_complex128* aqsntemp, const sigma_complex128* aqsmtemp,
                        const double* vcoul, double vfac, sigma_complex128* schDt_matrix,
                        void* stream, const float2* epsr32, bool reuse_a, const double* vcoul2,
                        double vfac2, sigma_complex128* out2, bool operands_ready) {
  if (!plan) return SIGMA_ERR_NULL;
  if ((!I_epsR && !epsr32 && !reuse_a) || !aqsntemp || !aqsmtemp || !schDt_matrix) return SIGMA_ERR_NULL;
  if ((epsr32 || reuse_a || operands_ready) && plan->mode != SIGMA_FF_OZAKI_BF16) return SIGMA_ERR_UNSUPPORTED;
  if (operands_ready && !reuse_a) return SIGMA_ERR_UNSUPPORTED;
  if ((out2 != nullptr) != (vcoul2 != nullptr) || (out2 && vcoul)) return SIGMA_ERR_UNSUPPORTED;
  if (out2 && plan->mode == SIGMA_FF_FP64) {
    // the FP64 form contracts twice
    const int r = ff_execute_weighted(plan, I_epsR, aqsntemp, aqsmtemp, nullptr, vfac, schDt_matrix, stream);
    if (r != SIGMA_OK) return r;
    return ff_execute_weighted(plan, I_epsR, aqsntemp, aqsmtemp, vcoul2, vfac * vfac2, out2, stream);
  }
  int dev = 0;
  SIGMA_CUDA_TRY(cudaGetDevice(&dev));
  if (dev != plan->device) return SIGMA_ERR_UNSUPPORTED;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  FfDev d = plan->dev;
  d.epsr = reinterpret_cast<const double2*>(I_epsR);
  d.aqsn = reinterpret_cast<const double2*>(aqsntemp);
  d.aqsm = reinterpret_cast<const double2*>(aqsmtemp);
  d.vcoul = vcoul;
  d.vfac = vfac;
  d.epsr32 = epsr32;
  d.vcoul2 = vcoul2;
  d.vfac2 = vfac2;
  OzakiPrep oz = plan->oz;
  oz.stab = vcoul2 ? oz.stab_buf : nullptr;
  cudaEvent_t* ev = nullptr;
  if (plan->timing && plan->recorded < kFfMaxTimed) ev = &plan->events[3 * plan->recorded++];
  SIGMA_CUDA_TRY(cudaMemsetAsync(plan->work.counter, 0, 2 * sizeof(int), s));
  if (plan->mode == SIGMA_FF_FP64) {
    if (ev) SIGMA_CUDA_TRY(cudaEventRecord(ev[0], s));
    SIGMA_CUDA_TRY(launch_ff_fp64(d, plan->work, plan->grid, s));
    if (ev) SIGMA_CUDA_TRY(cudaEventRecord(ev[1], s));
    SIGMA_CUDA_TRY(launch_ff_reduce(d, plan->work, reinterpret_cast<double2*>(schDt_matrix), s));
  } else {
    // operands_ready: the A and B slices and the epilogue factors were
    // written by the caller's producer pass
    if (!operands_ready) SIGMA_CUDA_TRY(launch_ozaki_prep(d, oz, s, !reuse_a));
    if (ev) SIGMA_CUDA_TRY(cudaEventRecord(ev[0], s));
    SIGMA_CUDA_TRY(launch_ozaki_gemm(d, plan->work, oz, plan->grid, s));
    if (ev) SIGMA_CUDA_TRY(cudaEventRecord(ev[1], s));
    SIGMA_CUDA_TRY(launch_ozaki_reduce(d, oz, reinterpret_cast<double2*>(schDt_matrix), s,
                                       reinterpret_cast<double2*>(out2)));
  }
  if (ev) SIGMA_CUDA_TRY(cudaEventRecord(ev[2], s));
  return SIGMA_OK;
}

}  // namespace sigma

extern "C" int sigma_ff_execute(sigma_ff_plan plan, const sigma_complex128* I_epsR,
                                const sigma_complex128* aqsntemp, const sigma_complex128* aqsmtemp,
                                sigma_complex128* schDt_matrix, void* stream) {
  return sigma::ff_execute_weighted(plan, I_epsR, aqsntemp, aqsmtemp, nullptr, 1.0, schDt_matrix,
                                    stream);
}

extern "C" int sigma_ff_schdt(int number_bands, int ncouls, int ngpown, int nfreq,
                              const int* inv_igp_index, const int* indinv,
                              const sigma_complex128* I_epsR, const sigma_complex128* aqsntemp,
                              const sigma_complex128* aqsmtemp, sigma_complex128* schDt_matrix,
                              int mode, void* stream) {
  using namespace sigma;
  if (!inv_igp_index || !indinv || !I_epsR || !aqsntemp || !aqsmtemp || !schDt_matrix)
    return SIGMA_ERR_NULL;
  int st = ff_check_shape(number_bands, ncouls, ngpown, nfreq);
  if (st != SIGMA_OK) return st;
  std::lock_guard<std::mutex> lk(api_mutex());
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || device_sm_count() <= 0) {
    cudaGetLastError();
    return SIGMA_ERR_NO_DEVICE;
  }
  sigma_ff_plan plan = nullptr;
  st = sigma_ff_plan_create(&plan, number_bands, ncouls, ngpown, nfreq, inv_igp_index, indinv, mode);
  if (st != SIGMA_OK) return st;
  const size_t eps_b = sizeof(sigma_complex128) * (size_t)nfreq * ngpown * ncouls;
  const size_t band_b = sizeof(sigma_complex128) * (size_t)number_bands * ncouls;
  const size_t out_b = sizeof(sigma_complex128) * (size_t)number_bands * nfreq;
  const size_t o1 = up256(eps_b), o2 = o1 + up256(band_b), o3 = o2 + up256(band_b);
  void* arena = nullptr;
  st = arena_get(kArenaFfInputs, o3 + up256(out_b), &arena);
  if (st != SIGMA_OK) {
    sigma_ff_plan_destroy(plan);
    return st;
  }
  char* a = static_cast<char*>(arena);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc = SIGMA_OK;
  auto run = [&]() -> int {
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a, I_epsR, eps_b, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o1, aqsntemp, band_b, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o2, aqsmtemp, band_b, cudaMemcpyHostToDevice, s));
    int r = sigma_ff_execute(plan, reinterpret_cast<const sigma_complex128*>(a),
                             reinterpret_cast<const sigma_complex128*>(a + o1),
                             reinterpret_cast<const sigma_complex128*>(a + o2),
                             reinterpret_cast<sigma_complex128*>(a + o3), stream);
    if (r != SIGMA_OK) return r;
    SIGMA_CUDA_TRY(cudaMemcpyAsync(schDt_matrix, a + o3, out_b, cudaMemcpyDeviceToHost, s));
    return sigma_ff_plan_status(plan, stream);
  };
  rc = run();
  sigma_ff_plan_destroy(plan);
  return rc;
}
