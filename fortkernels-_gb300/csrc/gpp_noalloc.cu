// GPP FP64 evaluation for callers that cannot allocate GPU memory.
//
// Some callers cannot call cudaMalloc: code running inside a framework whose
// memory pool owns the whole device, a plug-in loaded into a process that
// forbids allocations after start-up, or a hard real-time loop where an
// allocation could stall.  sigma_gpp_fp64_noalloc serves them.  It runs the
// same FP64 kernels as sigma_gpp_execute, but every scratch buffer they need
// (item counters, the column map, per-item partial sums, per-band results)
// lives in one file-scope __device__ array of fixed size, so the call makes
// no allocation of any kind.  Every GPU that loads the library holds that
// array until the process exits.
#include <cstring>
#include <mutex>

#include "sigma_gpp.h"
#include "sigma_internal.cuh"
#include "runtime.h"

namespace sigma {
int sch_blocks_per_sm_fp64();
int ssx_blocks_per_sm_fp64();

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;   // 32 MiB
constexpr int kNoAllocMaxColumns = 65536;                    // ngpown limit (column map)
constexpr int kNoAllocItemsPerSlot = 16;
constexpr int kSsxColumns = 256;                             // columns per occupied-band item

// The scratch array.  In host code this name is only a stand-in for the
// device symbol: its address must come from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_mu;
void* g_scratch_ptr[64] = {};  // device address of g_noalloc_scratch, per device

size_t up256(size_t v) { return (v + 255) / 256 * 256; }

void size_pass(GppWork& w, int band_count, int bn, int bp, int nc, int ng, int grid,
               int per_slot) {
  w.band_begin = 0;
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
  long long s = ((long long)per_slot * grid + base - 1) / base;
  if (s < 1) s = 1;
  int len = (int)((nc + s - 1) / s);
  len = (len + kCK - 1) / kCK * kCK;
  w.split_len = len;
  w.n_splits = (nc + len - 1) / len;
  w.n_items = (int)(base * w.n_splits);
}

// One-time set-up for the current device: the device address of the scratch
// array.  The caller holds g_mu.
int scratch_address(int dev, void** out) {
  if (dev < 0 || dev >= 64) return SIGMA_ERR_UNSUPPORTED;
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      set_last_cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)", __LINE__);
      return SIGMA_ERR_CUDA;
    }
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return SIGMA_OK;
}

}  // namespace
}  // namespace sigma

extern "C" int sigma_gpp_fp64_noalloc(int number_bands, int nvband, int ncouls, int ngpown,
                                      const int* inv_igp_index, const int* indinv,
                                      const double* wx_array, double occ,
                                      const sigma_complex128* aqsmtemp,
                                      const sigma_complex128* aqsntemp,
                                      const sigma_complex128* I_eps_array,
                                      const sigma_complex128* wtilde_array, const double* vcoul,
                                      sigma_complex128* achtemp, sigma_complex128* asxtemp,
                                      sigma_complex128* acht_n1_loc, void* stream) {
  using namespace sigma;
  if (!inv_igp_index || !indinv || !wx_array || !aqsmtemp || !aqsntemp || !I_eps_array ||
      !wtilde_array || !vcoul || !achtemp || !asxtemp)
    return SIGMA_ERR_NULL;
  if (number_bands <= 0 || ncouls <= 0 || ngpown <= 0 || ngpown > ncouls || nvband < 0 ||
      nvband > number_bands)
    return SIGMA_ERR_INVALID_SHAPE;
  if (ngpown > kNoAllocMaxColumns) {
    set_last_error_text("sigma_gpp_fp64_noalloc: ngpown exceeds the 65536-column limit of the "
                        "static scratch");
    return SIGMA_ERR_WORKSPACE;
  }

  std::lock_guard<std::mutex> lk(g_mu);
  // Column map of BGW-Kernels/gppKer.cpp:322-328, built in a fixed-size host
  // buffer (no heap allocation; g_mu serialises its use) and validated like
  // sigma_gpp_plan_create.
  static int igp_of[kNoAllocMaxColumns];
  for (int my_igp = 0; my_igp < ngpown; ++my_igp) {
    const int indigp = inv_igp_index[my_igp];
    if (indigp < 0 || indigp > ncouls) return SIGMA_ERR_INDEX_RANGE;
    const int igp = indigp == ncouls ? ncouls - 1 : indinv[indigp];
    if (igp == ncouls) return SIGMA_ERR_INDEX_RANGE;
    igp_of[my_igp] = (igp > ncouls || igp < 0) ? -1 : igp;
  }

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return SIGMA_ERR_NO_DEVICE;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // The column map comes from a reused host buffer and the scratch from one
  // shared array: a captured call would replay stale contents, so capture is
  // refused before anything is queued.
  cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &capturing) != cudaSuccess) {
    cudaGetLastError();
    return SIGMA_ERR_CUDA;
  }
  if (capturing != cudaStreamCaptureStatusNone) {
    set_last_error_text("sigma_gpp_fp64_noalloc: the stream is being captured; this entry point "
                        "does not run inside a CUDA graph");
    return SIGMA_ERR_UNSUPPORTED;
  }
  void* scratch = nullptr;
  int st = scratch_address(dev, &scratch);
  if (st != SIGMA_OK) return st;
  const int sms = device_sm_count();
  if (sms <= 0) return SIGMA_ERR_NO_DEVICE;

  GppWork sch{}, ssx{};
  // wx_array is one frequency set for every band: the shared-factor main pass
  int sch_grid = sms * sch_blocks_per_sm_fp64y();
  int ssx_grid = sms * ssx_blocks_per_sm_fp64();
  size_pass(sch, number_bands, kBNY, kBPY, ncouls, ngpown, sch_grid, kNoAllocItemsPerSlot);
  size_pass(ssx, nvband, kSsxBN, kSsxColumns, ncouls, ngpown, ssx_grid, 8);
  if (sch.n_items < sch_grid) sch_grid = sch.n_items;
  if (ssx.n_items < ssx_grid) ssx_grid = ssx.n_items;

  // scratch layout: counters | column map | per-band results | partials
  const size_t o_cnt = 0;
  const size_t o_igp = 256;
  const size_t o_n1 = o_igp + up256(sizeof(int) * ngpown);
  const size_t o_sch = o_n1 + up256(sizeof(double2) * (size_t)(number_bands + nvband) * kNW);
  const size_t o_ssx = o_sch + up256(sizeof(double2) * (size_t)sch.n_items * kBNY * kNW);
  const size_t need = o_ssx + up256(sizeof(double2) * (size_t)ssx.n_items * kSsxBN * kNW);
  if (need > kNoAllocScratchBytes) {
    set_last_error_text("sigma_gpp_fp64_noalloc: problem needs more than the 32 MiB static scratch");
    return SIGMA_ERR_WORKSPACE;
  }
  char* base = static_cast<char*>(scratch);
  int* counters = reinterpret_cast<int*>(base + o_cnt);
  sch.counter = counters;
  ssx.counter = counters + 1;
  sch.partial = reinterpret_cast<double2*>(base + o_sch);
  ssx.partial = reinterpret_cast<double2*>(base + o_ssx);
  double2* acht_n1 = reinterpret_cast<double2*>(base + o_n1);

  // The array keeps the previous call's contents: the item counters must
  // start at zero; every other byte the kernels read is written first.  The
  // column map is copied from pageable host memory, which the runtime stages
  // before cudaMemcpyAsync returns, so igp_of may be reused by the next call.
  SIGMA_CUDA_TRY(cudaMemsetAsync(counters, 0, 256, s));
  SIGMA_CUDA_TRY(cudaMemcpyAsync(base + o_igp, igp_of, sizeof(int) * ngpown,
                                 cudaMemcpyHostToDevice, s));

  GppDev p;
  p.nb = number_bands;
  p.nvband = nvband;
  p.nc = ncouls;
  p.ng = ngpown;
  p.wx_stride = 0;
  p.occ = occ;
  p.aqsm = reinterpret_cast<const double2*>(aqsmtemp);
  p.aqsn = reinterpret_cast<const double2*>(aqsntemp);
  p.ieps = reinterpret_cast<const double2*>(I_eps_array);
  p.wt = reinterpret_cast<const double2*>(wtilde_array);
  p.vcoul = vcoul;
  p.wx = wx_array;
  p.igp_of = reinterpret_cast<const int*>(base + o_igp);

  if (sch.n_items > 0) SIGMA_CUDA_TRY(launch_sch_fp64y(p, sch, sch_grid, s));
  if (ssx.n_items > 0) SIGMA_CUDA_TRY(launch_ssx_fp64(p, ssx, ssx_grid, s));
  SIGMA_CUDA_TRY(launch_gpp_reduce(sch, ssx, number_bands, acht_n1,
                                   reinterpret_cast<double2*>(achtemp),
                                   reinterpret_cast<double2*>(asxtemp),
                                   reinterpret_cast<double2*>(acht_n1_loc), s));
  return SIGMA_OK;
}
