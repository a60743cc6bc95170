// Static remainder of the GPP sum (reduce_achstemp of BGW-Kernels/gppKer.cpp,
// formula of gppkernel.deslippe.09.30.2014.f90:195-228) on the FF contraction
// kernels: one frequency, rows = columns my_igp of I_eps, the epilogue
// weight -0.5 vcoul[igp] per column and skipped columns left out.
#include <mutex>
#include <vector>

#include "sigma_gpp.h"
#include "sigma_ff.h"
#include "ff_plan.h"
#include "sigma_internal.cuh"
#include "runtime.h"

namespace {
size_t up256(size_t v) { return (v + 255) / 256 * 256; }

// achstemp = sum over bands of achstemp_n1, one warp, fixed-order
// compensated sums and a butterfly (same value on every lane).
__global__ void band_total_kernel(const double2* n1v, int nb, double2* total) {
  const int lane = threadIdx.x;
  sigma::Comp sx, sy;
  for (int n = lane; n < nb; n += 32) {
    sx.add(n1v[n].x);
    sy.add(n1v[n].y);
  }
  double rx = sx.value(), ry = sy.value();
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double t, e;
    sigma::two_sum_d(rx, __shfl_xor_sync(0xffffffffu, rx, o), t, e);
    rx = t + e;
    sigma::two_sum_d(ry, __shfl_xor_sync(0xffffffffu, ry, o), t, e);
    ry = t + e;
  }
  if (lane == 0) *total = make_double2(rx, ry);
}

int static_plan(sigma_ff_plan* out, int number_bands, int ncouls, int ngpown, const int* inv_igp_index,
                const int* indinv, int mode) {
  using namespace sigma;
  int st = gpp_check_shape(number_bands, 0, ncouls, ngpown, 0, kNW);
  if (st != SIGMA_OK) return st;
  if (mode != SIGMA_FF_FP64 && mode != SIGMA_FF_OZAKI_BF16) return SIGMA_ERR_UNSUPPORTED;
  std::vector<int> igp_of;
  int valid = 0;
  st = gpp_map_columns(ncouls, ngpown, inv_igp_index, indinv, ncouls, igp_of, valid);
  if (st != SIGMA_OK) return st;
  return ff_plan_build(out, number_bands, ncouls, ngpown, 1, igp_of, mode);
}
}  // namespace

extern "C" int sigma_gpp_static_plan_create(sigma_ff_plan* plan, int number_bands, int ncouls,
                                            int ngpown, const int* inv_igp_index, const int* indinv,
                                            int mode) {
  if (!plan || !inv_igp_index || !indinv) return SIGMA_ERR_NULL;
  *plan = nullptr;
  return static_plan(plan, number_bands, ncouls, ngpown, inv_igp_index, indinv, mode);
}

extern "C" int sigma_gpp_static_execute(sigma_ff_plan plan, const sigma_complex128* aqsmtemp,
                                        const sigma_complex128* aqsntemp,
                                        const sigma_complex128* I_eps_array, const double* vcoul,
                                        sigma_complex128* achstemp, sigma_complex128* achstemp_n1,
                                        void* stream) {
  using namespace sigma;
  if (!plan || !vcoul || !achstemp || !achstemp_n1) return SIGMA_ERR_NULL;
  int nb = 0;
  {
    int st = sigma_ff_plan_bands(plan, &nb);
    if (st != SIGMA_OK) return st;
  }
  int st = ff_execute_weighted(plan, I_eps_array, aqsntemp, aqsmtemp, vcoul, -0.5, achstemp_n1, stream);
  if (st != SIGMA_OK) return st;
  band_total_kernel<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(
      reinterpret_cast<const double2*>(achstemp_n1), nb, reinterpret_cast<double2*>(achstemp));
  SIGMA_CUDA_TRY(cudaGetLastError());
  return SIGMA_OK;
}

extern "C" int sigma_gpp_achstemp(int number_bands, int ncouls, int ngpown, const int* inv_igp_index,
                                  const int* indinv, const sigma_complex128* aqsmtemp,
                                  const sigma_complex128* aqsntemp,
                                  const sigma_complex128* I_eps_array, const double* vcoul,
                                  sigma_complex128* achstemp, sigma_complex128* achstemp_n1, int mode,
                                  void* stream) {
  using namespace sigma;
  if (!inv_igp_index || !indinv || !aqsmtemp || !aqsntemp || !I_eps_array || !vcoul || !achstemp)
    return SIGMA_ERR_NULL;
  {
    // argument errors come before any device work
    int st = gpp_check_shape(number_bands, 0, ncouls, ngpown, 0, kNW);
    if (st != SIGMA_OK) return st;
    if (mode != SIGMA_FF_FP64 && mode != SIGMA_FF_OZAKI_BF16) return SIGMA_ERR_UNSUPPORTED;
    std::vector<int> igp_of;
    int valid = 0;
    st = gpp_map_columns(ncouls, ngpown, inv_igp_index, indinv, ncouls, igp_of, valid);
    if (st != SIGMA_OK) return st;
  }
  std::lock_guard<std::mutex> lk(api_mutex());
  sigma_ff_plan plan = nullptr;
  int st = static_plan(&plan, number_bands, ncouls, ngpown, inv_igp_index, indinv, mode);
  if (st != SIGMA_OK) return st;
  const size_t eps_b = sizeof(sigma_complex128) * (size_t)ngpown * ncouls;
  const size_t band_b = sizeof(sigma_complex128) * (size_t)number_bands * ncouls;
  const size_t v_b = sizeof(double) * (size_t)ncouls;
  const size_t out_b = sizeof(sigma_complex128) * (size_t)number_bands;
  const size_t o1 = up256(eps_b), o2 = o1 + up256(band_b), o3 = o2 + up256(band_b),
               o4 = o3 + up256(v_b), o5 = o4 + up256(out_b);
  void* arena = nullptr;
  st = arena_get(kArenaFfInputs, o5 + 256, &arena);
  if (st != SIGMA_OK) {
    sigma_ff_plan_destroy(plan);
    return st;
  }
  char* a = static_cast<char*>(arena);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::vector<sigma_complex128> per_band(number_bands);
  auto run = [&]() -> int {
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a, I_eps_array, eps_b, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o1, aqsntemp, band_b, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o2, aqsmtemp, band_b, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o3, vcoul, v_b, cudaMemcpyHostToDevice, s));
    int r = sigma_gpp_static_execute(plan, reinterpret_cast<const sigma_complex128*>(a + o2),
                                     reinterpret_cast<const sigma_complex128*>(a + o1),
                                     reinterpret_cast<const sigma_complex128*>(a),
                                     reinterpret_cast<const double*>(a + o3),
                                     reinterpret_cast<sigma_complex128*>(a + o5),
                                     reinterpret_cast<sigma_complex128*>(a + o4), stream);
    if (r != SIGMA_OK) return r;
    SIGMA_CUDA_TRY(cudaMemcpyAsync(per_band.data(), a + o4, out_b, cudaMemcpyDeviceToHost, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(achstemp, a + o5, sizeof(sigma_complex128), cudaMemcpyDeviceToHost, s));
    return sigma_ff_plan_status(plan, stream);
  };
  const int rc = run();
  sigma_ff_plan_destroy(plan);
  if (rc != SIGMA_OK) return rc;
  if (achstemp_n1)
    for (int n1 = 0; n1 < number_bands; ++n1) achstemp_n1[n1] = per_band[n1];
  return SIGMA_OK;
}
