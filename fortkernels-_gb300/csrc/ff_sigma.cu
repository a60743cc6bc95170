// Full-frequency sigma around the schDt contraction: the band loop of
// ffkernel.deslippe.best.f90 (:201-626) in the C layouts of
// FFKer_cori/ffKernel.cpp.
//
// Every g-vector sum of that loop is a column-weighted contraction of one
// frequency slab of I_epsR or I_epsA:
//   C_X[n1][f] = sum_{my_igp} vcoul[igp] conj(aqsm[n1][igp])
//                  * sum_{ig} aqsn[n1][ig] X[f][my_igp][ig]
// and the loop only takes linear combinations of two neighbouring slabs
// (fact1 X[f] + fact2 X[f+1]), so
//   static CH   achsDtemp   = -0.5 sum_n1 C_R[n1][0]                   (:240-253)
//   SX          ssxDittt    = fact1 C_R[n1][f] + fact2 C_R[n1][f+1]    (:323-346)
//                            (C_A for wx < 0, :355-383)
//   delta terms schDttt     = fact1 (C_R - C_A)[n1][f] + fact2 (...)[f+1] (:551-601)
// The two weighted contractions run as the FF contraction with the vcoul
// column weight (either FP64 or split-BF16 tensor-core form); schDt itself
// is the unweighted contraction of I_epsR.  A small FP64 kernel then applies
// the per-(band, evaluation frequency) algebra of the loop, and a fixed-order
// compensated reduction sums the bands.
#include <cmath>
#include <mutex>
#include <vector>

#include "sigma_ff.h"
#include "ff_plan.h"
#include "sigma_internal.cuh"
#include "runtime.h"

namespace sigma {
namespace {

size_t up256(size_t v) { return (v + 255) / 256 * 256; }

constexpr int kOut = 5;  // asxDtemp, achDtemp, achDtemp_cor, achDtemp_corb, ach2Dtemp

struct FfSigmaArgs {
  int nb, nvband, nf, ne;
  const double* ekq;
  const double* grid;
  const double2* brd;
  const double* pref;
  double pref_zb, fmin, fstep, occ;
  const double2* cr;   // [nb][nf] vcoul-weighted contraction of I_epsR
  const double2* ca;   // [nb][nf] ... of I_epsA
  const double2* sdt;  // [nb][nf] schDt_matrix
  double2* per;        // [nb][kOut][ne] per-band contributions
};

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ double2 cmuld(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
// -i p z
__device__ __forceinline__ double2 minus_ip(double p, double2 z) { return make_double2(p * z.y, -p * z.x); }

// Last grid interval [g[k], g[k+1]) holding w; nf - 2 when none does (both
// interval searches of the Fortran end there, :288-311 and :536-545).
__device__ __forceinline__ int grid_interval(double w, const double* g, int nf) {
  int k = -1;
  for (int j = 0; j < nf - 1; ++j)
    if (w >= g[j] && w < g[j + 1]) k = j;
  return k < 0 ? nf - 2 : k;
}

__global__ void ff_sigma_band_kernel(FfSigmaArgs a) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.nb * a.ne) return;
  const int n1 = t / a.ne, iw = t % a.ne;
  const bool occ_band = n1 < a.nvband;
  const double e = a.fmin - a.ekq[n1] + iw * a.fstep;  // wx
  const double2* S = a.sdt + (size_t)n1 * a.nf;
  const double2* CR = a.cr + (size_t)n1 * a.nf;
  const double2* CA = a.ca + (size_t)n1 * a.nf;
  double2 asx = make_double2(0, 0), sch = make_double2(0, 0), cor = make_double2(0, 0),
          corb = make_double2(0, 0), sch2 = make_double2(0, 0);

  // SX of the occupied bands (:279-389)
  if (occ_band) {
    const bool pos = e >= 0.0;
    const int f = grid_interval(pos ? e : -e, a.grid, a.nf);
    const double d = a.grid[f + 1] - a.grid[f];
    const double f1 = pos ? (a.grid[f + 1] - e) / d : (a.grid[f + 1] + e) / d;
    const double f2 = pos ? (e - a.grid[f]) / d : (-a.grid[f] - e) / d;
    const double2* C = pos ? CR : CA;
    asx = cscale(cadd(cscale(C[f], f1), cscale(C[f + 1], f2)), a.occ);
  }
  // CH from schDt (:459-521)
  for (int f = 0; f < a.nf; ++f) {
    const double2 sd = S[f];
    const double zb = a.grid[f];
    const double2 coh = make_double2(zb - a.brd[f].x, -a.brd[f].y);
    const double2 cr = make_double2((occ_band ? -zb : zb) - a.brd[f].x, -a.brd[f].y);
    if (f != a.nf - 1) {
      const double2 wc = make_double2(e - coh.x, -coh.y), wr = make_double2(e - cr.x, -cr.y);
      sch = cadd(sch, minus_ip(a.pref[f], cdiv(sd, wc)));
      corb = cadd(corb, minus_ip(a.pref[f], cdiv(sd, wr)));
    }
    if (f != 0) {
      const double zr = zb, zl = a.grid[f - 1];
      const double2 left = S[f - 1];
      const double2 avg = cscale(cadd(sd, left), 0.5);
      const double2 lin = csub(sd, left);
      const double2 lin2 = cscale(lin, 1.0 / (zr - zl));
      double tt = fabs((e - zr) / (e - zl));
      tt = fmin(fmax(tt, 1e-4), 1e4);
      tt = -log(tt);
      sch2 = cadd(sch2, minus_ip(a.pref_zb, cscale(avg, tt)));
      double2 lin3;
      if (occ_band) {
        double t4 = fabs((e + zr) / (e + zl));
        t4 = fmin(fmax(t4, 1e-4), 1e4);
        t4 = log(t4);
        lin3 = cscale(cadd(left, cscale(lin2, -a.fmin - a.ekq[n1] + iw * a.fstep - zl)), t4);
      } else {
        lin3 = cscale(cadd(left, cscale(lin2, e - zl)), tt);
      }
      lin3 = cadd(lin3, lin);
      cor = cadd(cor, minus_ip(a.pref_zb, lin3));
    }
  }
  // delta-function terms (:530-613)
  if (e >= 0.0) {
    const int f = grid_interval(e, a.grid, a.nf);
    const double d = a.grid[f + 1] - a.grid[f];
    const double f1 = -0.5 * (a.grid[f + 1] - e) / d, f2 = -0.5 * (e - a.grid[f]) / d;
    const double2 v = cadd(cscale(csub(CR[f], CA[f]), f1), cscale(csub(CR[f + 1], CA[f + 1]), f2));
    sch2 = cadd(sch2, v);
    if (!occ_band) cor = cadd(cor, v);
  } else if (occ_band) {
    const double w = -e;
    const int f = grid_interval(w, a.grid, a.nf);
    const double d = a.grid[f + 1] - a.grid[f];
    const double f1 = (a.grid[f + 1] - w) / d, f2 = (w - a.grid[f]) / d;
    const double2 v = cadd(cscale(csub(CR[f], CA[f]), f1), cscale(csub(CR[f + 1], CA[f + 1]), f2));
    cor = cadd(cor, cscale(v, -0.5));
  }
  double2* o = a.per + (size_t)n1 * kOut * a.ne + iw;
  o[0 * a.ne] = asx;
  o[1 * a.ne] = sch;
  o[2 * a.ne] = cor;
  o[3 * a.ne] = corb;
  o[4 * a.ne] = sch2;
}

// One warp per output value: fixed-order compensated sum over the bands.
// Output 0 is achsDtemp = -0.5 sum_n1 C_R[n1][0]; outputs 1 + k*ne + iw the
// five arrays.
__global__ void ff_sigma_sum_kernel(int nb, int nf, int ne, const double2* cr, const double2* per,
                                    double2* out) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= 1 + kOut * ne) return;
  Comp sx, sy;
  for (int n = lane; n < nb; n += 32) {
    const double2 v = warp == 0 ? cr[(size_t)n * nf] : per[(size_t)n * kOut * ne + (warp - 1)];
    sx.add(v.x);
    sy.add(v.y);
  }
  double rx = sx.value(), ry = sy.value();
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double t, e;
    two_sum_d(rx, __shfl_xor_sync(0xffffffffu, rx, o), t, e);
    rx = t + e;
    two_sum_d(ry, __shfl_xor_sync(0xffffffffu, ry, o), t, e);
    ry = t + e;
  }
  if (lane == 0) out[warp] = warp == 0 ? make_double2(-0.5 * rx, -0.5 * ry) : make_double2(rx, ry);
}

}  // namespace
}  // namespace sigma

using sigma::FfSigmaArgs;
using sigma::kOut;
using sigma::up256;
using sigma::ff_sigma_band_kernel;
using sigma::ff_sigma_sum_kernel;

struct sigma_ff_sigma_plan_s {
  int device = 0, nb = 0, nvband = 0, nf = 0, ne = 0;
  sigma_ff_plan ff = nullptr;
  void* block = nullptr;
  double2 *cr = nullptr, *ca = nullptr, *sd = nullptr, *per = nullptr;
};

extern "C" int sigma_ff_sigma_plan_create(sigma_ff_sigma_plan* out, int number_bands, int nvband,
                                          int ncouls, int ngpown, int nfreq, int nfreqeval,
                                          const int* inv_igp_index, const int* indinv, int mode) {
  using namespace sigma;
  if (!out || !inv_igp_index || !indinv) return SIGMA_ERR_NULL;
  *out = nullptr;
  if (number_bands <= 0 || ncouls <= 0 || ngpown <= 0 || ngpown > ncouls || nfreq < 2 ||
      nfreqeval <= 0 || nvband < 0 || nvband > number_bands)
    return SIGMA_ERR_INVALID_SHAPE;
  if (mode != SIGMA_FF_FP64 && mode != SIGMA_FF_OZAKI_BF16) return SIGMA_ERR_UNSUPPORTED;
  // column map of the Fortran loop: igp = indinv[inv_igp_index[my_igp]];
  // columns with igp outside [0, ncouls) are left out (:324-327)
  std::vector<int> igp_of(ngpown);
  for (int g = 0; g < ngpown; ++g) {
    const int ind = inv_igp_index[g];
    if (ind < 0 || ind >= ncouls) return SIGMA_ERR_INDEX_RANGE;
    const int igp = indinv[ind];
    igp_of[g] = (igp < 0 || igp >= ncouls) ? -1 : igp;
  }
  auto* p = new sigma_ff_sigma_plan_s();
  int st = ff_plan_build(&p->ff, number_bands, ncouls, ngpown, nfreq, igp_of, mode);
  if (st != SIGMA_OK) {
    delete p;
    return st;
  }
  cudaGetDevice(&p->device);
  p->nb = number_bands;
  p->nvband = nvband;
  p->nf = nfreq;
  p->ne = nfreqeval;
  const size_t mat = up256(sizeof(double2) * (size_t)number_bands * nfreq);
  const size_t per = up256(sizeof(double2) * (size_t)number_bands * kOut * nfreqeval);
  cudaError_t e = cudaMalloc(&p->block, 3 * mat + per);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_last_cuda_error(e, "cudaMalloc(ff sigma plan)", __LINE__);
    sigma_ff_plan_destroy(p->ff);
    delete p;
    return SIGMA_ERR_ALLOC;
  }
  char* b = static_cast<char*>(p->block);
  p->cr = reinterpret_cast<double2*>(b);
  p->ca = reinterpret_cast<double2*>(b + mat);
  p->sd = reinterpret_cast<double2*>(b + 2 * mat);
  p->per = reinterpret_cast<double2*>(b + 3 * mat);
  *out = p;
  return SIGMA_OK;
}

extern "C" int sigma_ff_sigma_plan_destroy(sigma_ff_sigma_plan p) {
  if (!p) return SIGMA_OK;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(p->device);
  if (p->block) cudaFree(p->block);
  sigma_ff_plan_destroy(p->ff);
  cudaSetDevice(cur);
  delete p;
  return SIGMA_OK;
}

extern "C" int sigma_ff_sigma_plan_set_timing(sigma_ff_sigma_plan p, int enable) {
  if (!p) return SIGMA_ERR_NULL;
  return sigma_ff_plan_set_timing(p->ff, enable);
}

extern "C" int sigma_ff_sigma_plan_timing(sigma_ff_sigma_plan p, int* contractions,
                                          double* contraction_ms, double* other_ms) {
  if (!p) return SIGMA_ERR_NULL;
  int launches = 0;
  return sigma_ff_plan_timing(p->ff, contractions, contraction_ms, other_ms, &launches);
}

extern "C" int sigma_ff_sigma_plan_status(sigma_ff_sigma_plan p, void* stream) {
  if (!p) return SIGMA_ERR_NULL;
  return sigma_ff_plan_status(p->ff, stream);
}

extern "C" int sigma_ff_sigma_execute(sigma_ff_sigma_plan p, const sigma_complex128* aqsmtemp,
                                      const sigma_complex128* aqsntemp,
                                      const sigma_complex128* I_epsR,
                                      const sigma_complex128* I_epsA, const double* vcoul,
                                      const double* ekq, const double* dFreqGrid,
                                      const sigma_complex128* dFreqBrd, const double* pref,
                                      double pref_zb, double freqevalmin, double freqevalstep,
                                      double occ, const sigma_complex128* schDt_matrix,
                                      sigma_complex128* out, void* stream) {
  using namespace sigma;
  if (!p) return SIGMA_ERR_NULL;
  if (!aqsmtemp || !aqsntemp || !I_epsR || !I_epsA || !vcoul || !ekq || !dFreqGrid || !dFreqBrd ||
      !pref || !out)
    return SIGMA_ERR_NULL;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  auto C = [](double2* x) { return reinterpret_cast<sigma_complex128*>(x); };
  // schDt (weight 1) and C_R (weight vcoul) are one contraction of I_epsR
  // with two epilogue sums when schDt is not given
  const double2* sd = reinterpret_cast<const double2*>(schDt_matrix);
  int r;
  if (!schDt_matrix) {
    r = ff_execute_weighted(p->ff, I_epsR, aqsntemp, aqsmtemp, nullptr, 1.0, C(p->sd), stream,
                            nullptr, false, vcoul, 1.0, C(p->cr));
    sd = p->sd;
  } else {
    r = ff_execute_weighted(p->ff, I_epsR, aqsntemp, aqsmtemp, vcoul, 1.0, C(p->cr), stream);
  }
  if (r != SIGMA_OK) return r;
  r = ff_execute_weighted(p->ff, I_epsA, aqsntemp, aqsmtemp, vcoul, 1.0, C(p->ca), stream);
  if (r != SIGMA_OK) return r;
  FfSigmaArgs g;
  g.nb = p->nb;
  g.nvband = p->nvband;
  g.nf = p->nf;
  g.ne = p->ne;
  g.ekq = ekq;
  g.grid = dFreqGrid;
  g.brd = reinterpret_cast<const double2*>(dFreqBrd);
  g.pref = pref;
  g.pref_zb = pref_zb;
  g.fmin = freqevalmin;
  g.fstep = freqevalstep;
  g.occ = occ;
  g.cr = p->cr;
  g.ca = p->ca;
  g.sdt = sd;
  g.per = p->per;
  // one thread per (band, evaluation frequency), FP64-bound: one warp per
  // block spreads the few thousand threads over every SM
  const int threads = 32, items = p->nb * p->ne;
  ff_sigma_band_kernel<<<(items + threads - 1) / threads, threads, 0, s>>>(g);
  SIGMA_CUDA_TRY(cudaGetLastError());
  const int warps = 1 + kOut * p->ne;
  ff_sigma_sum_kernel<<<(warps * 32 + 255) / 256, 256, 0, s>>>(
      p->nb, p->nf, p->ne, p->cr, p->per, reinterpret_cast<double2*>(out));
  SIGMA_CUDA_TRY(cudaGetLastError());
  return SIGMA_OK;
}

extern "C" int sigma_ff_sigma(int number_bands, int nvband, int ncouls, int ngpown, int nfreq,
                              int nfreqeval, const int* inv_igp_index, const int* indinv,
                              const sigma_complex128* aqsmtemp, const sigma_complex128* aqsntemp,
                              const sigma_complex128* I_epsR, const sigma_complex128* I_epsA,
                              const double* vcoul, const double* ekq, const double* dFreqGrid,
                              const sigma_complex128* dFreqBrd, const double* pref, double pref_zb,
                              double freqevalmin, double freqevalstep, double occ,
                              const sigma_complex128* schDt_matrix, sigma_complex128* achsDtemp,
                              sigma_complex128* asxDtemp, sigma_complex128* achDtemp,
                              sigma_complex128* achDtemp_cor, sigma_complex128* achDtemp_corb,
                              sigma_complex128* ach2Dtemp, int mode, void* stream) {
  using namespace sigma;
  if (!inv_igp_index || !indinv || !aqsmtemp || !aqsntemp || !I_epsR || !I_epsA || !vcoul || !ekq ||
      !dFreqGrid || !dFreqBrd || !pref || !achsDtemp || !asxDtemp || !achDtemp || !achDtemp_cor ||
      !achDtemp_corb || !ach2Dtemp)
    return SIGMA_ERR_NULL;
  if (nfreq >= 2)
    for (int f = 0; f + 1 < nfreq; ++f)
      if (!(dFreqGrid[f + 1] > dFreqGrid[f])) return SIGMA_ERR_INVALID_SHAPE;  // ascending grid
  std::lock_guard<std::mutex> lk(api_mutex());
  sigma_ff_sigma_plan plan = nullptr;
  int st = sigma_ff_sigma_plan_create(&plan, number_bands, nvband, ncouls, ngpown, nfreq, nfreqeval,
                                      inv_igp_index, indinv, mode);
  if (st != SIGMA_OK) return st;
  const int nb = number_bands, nf = nfreq, ne = nfreqeval;
  const size_t eps_b = sizeof(sigma_complex128) * (size_t)nf * ngpown * ncouls;
  const size_t band_b = sizeof(sigma_complex128) * (size_t)nb * ncouls;
  const size_t mat_b = sizeof(double2) * (size_t)nb * nf;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += up256(bytes);
    return o;
  };
  const size_t o_r = take(eps_b), o_a = take(eps_b), o_n = take(band_b), o_m = take(band_b),
               o_v = take(sizeof(double) * ncouls), o_ekq = take(sizeof(double) * nb),
               o_grid = take(sizeof(double) * nf), o_brd = take(sizeof(double2) * nf),
               o_pref = take(sizeof(double) * nf), o_sd = take(mat_b),
               o_out = take(sizeof(double2) * (1 + kOut * ne));
  void* arena = nullptr;
  st = arena_get(kArenaFfInputs, off, &arena);
  if (st != SIGMA_OK) {
    sigma_ff_sigma_plan_destroy(plan);
    return st;
  }
  char* a = static_cast<char*>(arena);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::vector<double2> out(1 + kOut * ne);
  auto D = [&](size_t o) { return reinterpret_cast<sigma_complex128*>(a + o); };
  auto run = [&]() -> int {
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_r, I_epsR, eps_b, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_a, I_epsA, eps_b, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_n, aqsntemp, band_b, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_m, aqsmtemp, band_b, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_v, vcoul, sizeof(double) * ncouls, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_ekq, ekq, sizeof(double) * nb, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_grid, dFreqGrid, sizeof(double) * nf, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_brd, dFreqBrd, sizeof(double2) * nf, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_pref, pref, sizeof(double) * nf, cudaMemcpyHostToDevice, s));
    if (schDt_matrix)
      SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_sd, schDt_matrix, mat_b, cudaMemcpyHostToDevice, s));
    int r = sigma_ff_sigma_execute(plan, D(o_m), D(o_n), D(o_r), D(o_a),
                                   reinterpret_cast<const double*>(a + o_v),
                                   reinterpret_cast<const double*>(a + o_ekq),
                                   reinterpret_cast<const double*>(a + o_grid), D(o_brd),
                                   reinterpret_cast<const double*>(a + o_pref), pref_zb, freqevalmin,
                                   freqevalstep, occ, schDt_matrix ? D(o_sd) : nullptr, D(o_out), stream);
    if (r != SIGMA_OK) return r;
    SIGMA_CUDA_TRY(cudaMemcpyAsync(out.data(), a + o_out, sizeof(double2) * out.size(),
                                   cudaMemcpyDeviceToHost, s));
    return sigma_ff_sigma_plan_status(plan, stream);
  };
  const int rc = run();
  sigma_ff_sigma_plan_destroy(plan);
  if (rc != SIGMA_OK) return rc;
  auto put = [](sigma_complex128* dst, double2 v) {
    dst->re = v.x;
    dst->im = v.y;
  };
  put(achsDtemp, out[0]);
  for (int iw = 0; iw < ne; ++iw) {
    put(asxDtemp + iw, out[1 + 0 * ne + iw]);
    put(achDtemp + iw, out[1 + 1 * ne + iw]);
    put(achDtemp_cor + iw, out[1 + 2 * ne + iw]);
    put(achDtemp_corb + iw, out[1 + 3 * ne + iw]);
    put(ach2Dtemp + iw, out[1 + 4 * ne + iw]);
  }
  return SIGMA_OK;
}
