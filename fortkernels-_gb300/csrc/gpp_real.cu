// Real-valued GPP (gppKer_real.cpp:17-155, 296-390; gppKerFort_real.f90):
// the GPP sum with real arrays, one frequency set for every band.
//
// Term of every band: scha = aqsm[n1][igp] aqsn[n1][ig] delw I_eps, with
// delw = wtilde / (wx - wtilde) and the pole guard of the complex path
// (b = 0), so scha = aqsm[n1][igp] * aqsn[n1][ig] * Y_iw[my_igp][ig] with the
// band-independent factor Y_iw = I_eps wtilde c / c^2 (c = wx - wtilde; 0 when
// dropped).  The main pass forms Y in FP64 per staged chunk and stages it, and
// aqsn, as float-float pairs; every term aqsn Y is then a float-float product
// on the FP32 pipe, the high halves of two g-vectors' terms are added exactly
// (TwoSum) and their sum added exactly to the chunk's float-float sum, the
// rounding errors and low halves summed in FP32; after each chunk that sum is
// renormalised and its high half widened and added to the FP64 sums, kept in
// shared memory (1/32 FP64 operation per term, against one DFMA).  A chunk
// with a value outside the float-float range forms its factors again in FP64
// and runs FP64 multiply-adds.  Occupied bands add
//   ssx = Omega2 / wx^2 (kept), -G / (2 (wx + wtilde)) (dropped with
//   delw^2 > to1), 0 otherwise,
// in FP64 (G = I_eps wtilde, Omega2 = wtilde G).  Partial sums use the
// complex path's fixed slots and reduction (imaginary parts zero); the
// outputs are their real parts.
//
// Where the reference's unoccupied loop adds a stale scha[ig] from an
// earlier frequency or g-vector block for a dropped term
// (gppKer_real.cpp:367-371 writes scha only when the guard passes), this
// path adds 0, the value the guard stands for.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "sigma_gpp.h"
#include "sigma_internal.cuh"
#include "floatfloat.cuh"
#include "runtime.h"

namespace sigma {
namespace {

constexpr int kRBN = 64, kRBP = 32;   // bands x columns per main-pass item
constexpr int kRCK = 32;             // g-vectors per staged chunk

struct GppRealDev {
  int nb, nvband, nc, ng;
  double occ;
  const double *aqsm, *aqsn, *ieps, *wt, *vcoul, *wx;
  const int* igp_of;
};

// Rows padded by one element: the staging writes run along g-vectors (the
// coalesced direction of the global reads), so unpadded rows, whose strides
// are multiples of 128 bytes, put a warp's writes in one bank.
struct RealSmem {
  // each thread's FP64 sums (4 bands x 2 columns x 3 frequencies), one slot
  // row per output: a warp's accesses are contiguous
  double acc[(kRBN / 16) * (kRBP / 16) * kNW][kThreads];
  float2 yf[kRCK][kNW * kRBP + 1];  // [k][iw * kRBP + column]: Y as float-float
  float2 nf[kRCK][kRBN + 1];        // aqsn as float-float
};

// Y = I_eps wtilde c / c^2 (c = wx - wtilde) of one (column, g-vector)
// element in FP64, 0 where the guard drops the term or the element is
// padding; the reciprocal to the FP64 rounding unit.
__device__ __forceinline__ double real_y(double wt, double g, double thr, double wx) {
  const double c = __dsub_rn(wx, wt);
  const double wv = __dmul_rn(c, c);
  return keep_nonneg(wv, thr) ? g * (c * rcp_f64(wv)) : 0.0;
}

// A chunk holding a factor or an aqsn element outside the float-float range:
// FP64 multiply-adds of the thread's register tile, its factors formed again
// from the inputs and aqsn read again, added to the thread's FP64 sums.  Out
// of line: the common path carries none of its registers.
static __device__ __noinline__ void real_wide_chunk(const GppRealDev& p, double (*acc)[kThreads], int tid,
                                                    int ig0, int ig_end, int n1_0, int p0, double wx0,
                                                    double wx1, double wx2) {
  constexpr int TB = kRBN / 16, TC = kRBP / 16;
  const int tx = tid & 15, ty = tid >> 4;
  double aw[TB][TC][kNW];
  for (int i = 0; i < TB; ++i)
    for (int j = 0; j < TC; ++j)
      for (int iw = 0; iw < kNW; ++iw) aw[i][j][iw] = 0.0;
  for (int k = 0; k < kRCK; ++k) {
    const int ig = ig0 + k;
    double y[TC][kNW];
    for (int j = 0; j < TC; ++j) {
      const int my_igp = p0 + tx + 16 * j;
      for (int iw = 0; iw < kNW; ++iw) y[j][iw] = 0.0;
      if (ig < ig_end && my_igp < p.ng) {
        const size_t off = (size_t)my_igp * p.nc + ig;
        const double wt = p.wt[off], g = p.ieps[off] * wt, thr = guard_thr(wt, 0.0);
        y[j][0] = real_y(wt, g, thr, wx0);
        y[j][1] = real_y(wt, g, thr, wx1);
        y[j][2] = real_y(wt, g, thr, wx2);
      }
    }
    for (int i = 0; i < TB; ++i) {
      const int n1 = n1_0 + ty + 16 * i;
      const double nn = (ig < ig_end && n1 < p.nb) ? p.aqsn[(size_t)n1 * p.nc + ig] : 0.0;
      for (int j = 0; j < TC; ++j)
        for (int iw = 0; iw < kNW; ++iw) aw[i][j][iw] = fma(nn, y[j][iw], aw[i][j][iw]);
    }
  }
  for (int i = 0; i < TB; ++i)
    for (int j = 0; j < TC; ++j)
      for (int iw = 0; iw < kNW; ++iw) acc[(i * TC + j) * kNW + iw][tid] += aw[i][j][iw];
}

__global__ void __launch_bounds__(kThreads, 2) sch_real_kernel(GppRealDev p, GppWork w) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  RealSmem& sm = *reinterpret_cast<RealSmem*>(smem_raw);
  __shared__ int s_item;
  constexpr int TB = kRBN / 16, TC = kRBP / 16;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const double wx0 = p.wx[0], wx1 = p.wx[1], wx2 = p.wx[2];
  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(w.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= w.n_items) break;
    const ItemCoord ic = decode_item(w, item);
    const int n1_0 = ic.bb * kRBN, p0 = ic.cb * kRBP;
    const int ig_begin = ic.s * w.split_len, ig_end = min(ig_begin + w.split_len, p.nc);
    // FP64 sums in shared memory (each thread its own slots); per-chunk
    // float-float sums in registers: the high halves of two g-vectors' terms
    // added exactly (TwoSum), their sum added exactly to the high half, the
    // errors and low halves to the low half; after each chunk the pair
    // renormalised (Fast2Sum), its high half added to the FP64 sum and its
    // low half carried on
    float ach[TB][TC][kNW], acl[TB][TC][kNW];
#pragma unroll
    for (int i = 0; i < TB; ++i)
#pragma unroll
      for (int j = 0; j < TC; ++j)
#pragma unroll
        for (int iw = 0; iw < kNW; ++iw) {
          sm.acc[(i * TC + j) * kNW + iw][tid] = 0.0;
          ach[i][j][iw] = 0.f;
          acl[i][j][iw] = 0.f;
        }

    for (int ig0 = ig_begin; ig0 < ig_end; ig0 += kRCK) {
      __syncthreads();
      bool chunk_wide = false;  // a value of the chunk outside the float-float range
      for (int e = tid; e < kRCK * kRBP; e += kThreads) {
        const int k = e % kRCK, pl = e / kRCK;
        const int ig = ig0 + k, my_igp = p0 + pl;
        double y0 = 0.0, y1 = 0.0, y2 = 0.0;
        if (ig < ig_end && my_igp < p.ng) {
          const size_t off = (size_t)my_igp * p.nc + ig;
          const double wt = p.wt[off], g = p.ieps[off] * wt, thr = guard_thr(wt, 0.0);
          y0 = real_y(wt, g, thr, wx0);
          y1 = real_y(wt, g, thr, wx1);
          y2 = real_y(wt, g, thr, wx2);
        }
        const double ys[kNW] = {y0, y1, y2};
#pragma unroll
        for (int iw = 0; iw < kNW; ++iw) {
          const FF f = ff_of_rn(ys[iw]);
          sm.yf[k][iw * kRBP + pl] = make_float2(f.hi, f.lo);
          chunk_wide = chunk_wide || !ff_range(ys[iw], 0.0);
        }
      }
      for (int e = tid; e < kRCK * kRBN; e += kThreads) {
        const int k = e % kRCK, bl = e / kRCK;
        const int ig = ig0 + k, n1 = n1_0 + bl;
        const double v = (ig < ig_end && n1 < p.nb) ? p.aqsn[(size_t)n1 * p.nc + ig] : 0.0;
        const FF f = ff_of_rn(v);
        sm.nf[k][bl] = make_float2(f.hi, f.lo);
        chunk_wide = chunk_wide || !ff_range(v, 0.0);
      }
      chunk_wide = __syncthreads_or(chunk_wide);
      if (!chunk_wide) {
        // the terms of two g-vectors: float-float products, their high
        // halves added exactly, the sum added exactly to the chunk's
        // float-float sum
        static_assert(kRCK % 2 == 0, "g-vector pairs");
#pragma unroll 1
        for (int k = 0; k < kRCK; k += 2) {
          float2 y[2][TC][kNW];
#pragma unroll
          for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int j = 0; j < TC; ++j)
#pragma unroll
              for (int iw = 0; iw < kNW; ++iw) y[h][j][iw] = sm.yf[k + h][iw * kRBP + tx + 16 * j];
#pragma unroll
          for (int i = 0; i < TB; ++i) {
            const float2 n0 = sm.nf[k][ty + 16 * i], n1v = sm.nf[k + 1][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < TC; ++j)
#pragma unroll
              for (int iw = 0; iw < kNW; ++iw) {
                const FF t0 = ff_mul_raw(FF{n0.x, n0.y}, FF{y[0][j][iw].x, y[0][j][iw].y});
                const FF t1 = ff_mul_raw(FF{n1v.x, n1v.y}, FF{y[1][j][iw].x, y[1][j][iw].y});
                float s, e, hs, he;
                two_sum_f(t0.hi, t1.hi, s, e);
                two_sum_f(ach[i][j][iw], s, hs, he);
                ach[i][j][iw] = hs;
                acl[i][j][iw] += ((e + t0.lo) + t1.lo) + he;
              }
          }
        }
#pragma unroll
        for (int i = 0; i < TB; ++i)
#pragma unroll
          for (int j = 0; j < TC; ++j)
#pragma unroll
            for (int iw = 0; iw < kNW; ++iw) {
              const float s = __fadd_rn(ach[i][j][iw], acl[i][j][iw]);
              acl[i][j][iw] = __fsub_rn(acl[i][j][iw], __fsub_rn(s, ach[i][j][iw]));
              ach[i][j][iw] = 0.f;
              sm.acc[(i * TC + j) * kNW + iw][tid] += f32_widen(s);
            }
      } else {
        real_wide_chunk(p, sm.acc, tid, ig0, ig_end, n1_0, p0, wx0, wx1, wx2);
      }
    }
    double acc[TB][TC][kNW];
#pragma unroll
    for (int i = 0; i < TB; ++i)
#pragma unroll
      for (int j = 0; j < TC; ++j)
#pragma unroll
        for (int iw = 0; iw < kNW; ++iw) acc[i][j][iw] = sm.acc[(i * TC + j) * kNW + iw][tid] + f32_widen(acl[i][j][iw]);
    // epilogue: x aqsm[n1][igp] * 0.5 * vcoul[igp], half-warp butterfly over columns
#pragma unroll
    for (int i = 0; i < TB; ++i) {
      const int bl = ty + 16 * i, n1 = n1_0 + bl;
      double part[kNW] = {0.0, 0.0, 0.0};
#pragma unroll
      for (int j = 0; j < TC; ++j) {
        const int my_igp = p0 + tx + 16 * j;
        const int igp = my_igp < p.ng ? p.igp_of[my_igp] : -1;
        if (n1 < p.nb && igp >= 0) {
          const double f = p.aqsm[(size_t)n1 * p.nc + igp] * 0.5 * p.vcoul[igp];
#pragma unroll
          for (int iw = 0; iw < kNW; ++iw) part[iw] = fma(acc[i][j][iw], f, part[iw]);
        }
      }
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw)
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) part[iw] += __shfl_xor_sync(0xffffffffu, part[iw], o);
      if (tx == 0)
#pragma unroll
        for (int iw = 0; iw < kNW; ++iw)
          w.partial[ic.pidx * kRBN * kNW + bl * kNW + iw] = make_double2(part[iw], 0.0);
    }
  }
}

// Occupied bands: thread = column, kSsxBN bands per item.
__global__ void __launch_bounds__(kThreads) ssx_real_kernel(GppRealDev p, GppWork w) {
  __shared__ int s_item;
  __shared__ double red[kSsxBN][kNW][kThreads / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  double iwx2[kNW];
#pragma unroll
  for (int iw = 0; iw < kNW; ++iw) iwx2[iw] = 1.0 / (p.wx[iw] * p.wx[iw]);
  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(w.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= w.n_items) break;
    const ItemCoord ic = decode_item(w, item);
    const int n1_0 = ic.bb * kSsxBN;
    const int nbl = min(kSsxBN, p.nvband - n1_0);
    const int my_igp = ic.cb * kSsxBP + tid;
    const int ig_begin = ic.s * w.split_len, ig_end = min(ig_begin + w.split_len, p.nc);
    double acc[kSsxBN][kNW];
#pragma unroll
    for (int i = 0; i < kSsxBN; ++i)
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) acc[i][iw] = 0.0;
    if (my_igp < p.ng) {
      for (int ig = ig_begin; ig < ig_end; ++ig) {
        const size_t off = (size_t)my_igp * p.nc + ig;
        const double wt = p.wt[off];
        const double g = p.ieps[off] * wt;
        const double om = wt * g;
        const double thr = guard_thr(wt, 0.0), thr2 = guard_thr2(wt, 0.0);
        double sv[kNW];
#pragma unroll
        for (int iw = 0; iw < kNW; ++iw) {
          const double c = __dsub_rn(p.wx[iw], wt);
          const double wv = __dmul_rn(c, c);
          const bool keep = keep_nonneg(wv, thr);
          const bool br2 = !keep && gt_nonneg(wv, 0.0) && gt_nonneg(thr2, wv);
          const double s2 = -0.5 * g / (p.wx[iw] + wt);
          sv[iw] = keep ? om * iwx2[iw] : (br2 ? s2 : 0.0);
        }
#pragma unroll
        for (int i = 0; i < kSsxBN; ++i)
          if (i < nbl) {
            const double an = p.aqsn[(size_t)(n1_0 + i) * p.nc + ig];
#pragma unroll
            for (int iw = 0; iw < kNW; ++iw) acc[i][iw] = fma(an, sv[iw], acc[i][iw]);
          }
      }
    }
    const int igp = my_igp < p.ng ? p.igp_of[my_igp] : -1;
#pragma unroll
    for (int i = 0; i < kSsxBN; ++i)
#pragma unroll
      for (int iw = 0; iw < kNW; ++iw) {
        double v = 0.0;
        if (i < nbl && igp >= 0) v = acc[i][iw] * p.aqsm[(size_t)(n1_0 + i) * p.nc + igp] * p.occ * p.vcoul[igp];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[i][iw][warp] = v;
      }
    __syncthreads();
    if (tid < kSsxBN * kNW) {
      const int i = tid / kNW, iw = tid % kNW;
      Comp sx;
      for (int q = 0; q < kThreads / 32; ++q) sx.add(red[i][iw][q]);
      w.partial[ic.pidx * kSsxBN * kNW + tid] = make_double2(sx.value(), 0.0);
    }
  }
}

__global__ void real_parts_kernel(const double2* ach, const double2* asx, const double2* n1, int nb,
                                  double* ach_out, double* asx_out, double* n1_out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < kNW) {
    ach_out[t] = ach[t].x;
    asx_out[t] = asx[t].x;
  }
  if (n1_out && t < nb) n1_out[t] = n1[t].x;
}

size_t up256(size_t v) { return (v + 255) / 256 * 256; }

}  // namespace
}  // namespace sigma

struct sigma_gpp_real_plan_s {
  int device = 0, nb = 0, nvband = 0, nc = 0, ng = 0;
  int sch_grid = 0, ssx_grid = 0;
  sigma::GppWork sch{}, ssx{};
  void* block = nullptr;
  int* igp_of = nullptr;
  int* counters = nullptr;
  double2* acht_n1 = nullptr;  // [nb + nvband][3]
  double2* outc = nullptr;     // achtemp[3], asxtemp[3], acht_n1_loc[nb] (complex workspace)
};

extern "C" int sigma_gpp_real_plan_create(sigma_gpp_real_plan* out, int number_bands, int nvband,
                                          int ncouls, int ngpown, int nstart, int nend,
                                          const int* inv_igp_index, const int* indinv,
                                          int indinv_len) {
  using namespace sigma;
  if (!out || !inv_igp_index || !indinv) return SIGMA_ERR_NULL;
  *out = nullptr;
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
  auto* p = new sigma_gpp_real_plan_s();
  p->device = dev;
  p->nb = number_bands;
  p->nvband = nvband;
  p->nc = ncouls;
  p->ng = ngpown;
  p->sch_grid = 2 * sms;  // two CTAs per SM
  p->ssx_grid = sms * 4;
  gpp_size_work(p->sch, 0, number_bands, kRBN, kRBP, ncouls, ngpown, p->sch_grid, 24);
  gpp_size_work(p->ssx, 0, nvband, kSsxBN, kSsxBP, ncouls, ngpown, p->ssx_grid, 8);
  if (p->sch.n_items < p->sch_grid) p->sch_grid = std::max(1, p->sch.n_items);
  if (p->ssx.n_items < p->ssx_grid) p->ssx_grid = std::max(1, p->ssx.n_items);
  const size_t b_igp = up256(sizeof(int) * ngpown), b_cnt = 256;
  const size_t b_n1 = up256(sizeof(double2) * (size_t)(number_bands + nvband) * kNW);
  const size_t b_out = up256(sizeof(double2) * (size_t)(2 * kNW + number_bands));
  const size_t b_sch = up256(sizeof(double2) * (size_t)p->sch.n_items * kRBN * kNW);
  const size_t b_ssx = up256(sizeof(double2) * (size_t)p->ssx.n_items * kSsxBN * kNW);
  cudaError_t e = cudaMalloc(&p->block, b_igp + b_cnt + b_n1 + b_out + b_sch + b_ssx);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_last_cuda_error(e, "cudaMalloc(real plan)", __LINE__);
    delete p;
    return SIGMA_ERR_ALLOC;
  }
  char* b = static_cast<char*>(p->block);
  p->igp_of = reinterpret_cast<int*>(b);
  p->counters = reinterpret_cast<int*>(b + b_igp);
  p->acht_n1 = reinterpret_cast<double2*>(b + b_igp + b_cnt);
  p->outc = reinterpret_cast<double2*>(b + b_igp + b_cnt + b_n1);
  p->sch.partial = reinterpret_cast<double2*>(b + b_igp + b_cnt + b_n1 + b_out);
  p->ssx.partial = reinterpret_cast<double2*>(b + b_igp + b_cnt + b_n1 + b_out + b_sch);
  p->sch.counter = p->counters;
  p->ssx.counter = p->counters + 1;
  e = cudaMemcpy(p->igp_of, igp_of.data(), sizeof(int) * ngpown, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    set_last_cuda_error(e, "cudaMemcpy(real igp_of)", __LINE__);
    cudaFree(p->block);
    delete p;
    return SIGMA_ERR_CUDA;
  }
  *out = p;
  return SIGMA_OK;
}

extern "C" int sigma_gpp_real_plan_destroy(sigma_gpp_real_plan p) {
  if (!p) return SIGMA_OK;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(p->device);
  if (p->block) cudaFree(p->block);
  cudaSetDevice(cur);
  delete p;
  return SIGMA_OK;
}

extern "C" int sigma_gpp_real_execute(sigma_gpp_real_plan plan, const double* wx_array, double occ,
                                      const double* aqsmtemp, const double* aqsntemp,
                                      const double* I_eps_array, const double* wtilde_array,
                                      const double* vcoul, double* achtemp, double* asxtemp,
                                      double* acht_n1_loc, void* stream) {
  using namespace sigma;
  if (!plan) return SIGMA_ERR_NULL;
  if (!wx_array || !aqsmtemp || !aqsntemp || !I_eps_array || !wtilde_array || !vcoul || !achtemp ||
      !asxtemp)
    return SIGMA_ERR_NULL;
  int dev = 0;
  SIGMA_CUDA_TRY(cudaGetDevice(&dev));
  if (dev != plan->device) return SIGMA_ERR_UNSUPPORTED;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  GppRealDev p{plan->nb, plan->nvband, plan->nc, plan->ng, occ, aqsmtemp, aqsntemp, I_eps_array,
               wtilde_array, vcoul, wx_array, plan->igp_of};
  SIGMA_CUDA_TRY(cudaMemsetAsync(plan->counters, 0, 2 * sizeof(int), s));
  if (plan->sch.n_items > 0) {
    SIGMA_CUDA_TRY(cudaFuncSetAttribute(sch_real_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)sizeof(RealSmem)));
    // two CTAs per SM hold ~180 KB of shared memory between them
    SIGMA_CUDA_TRY(cudaFuncSetAttribute(sch_real_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                        cudaSharedmemCarveoutMaxShared));
    sch_real_kernel<<<plan->sch_grid, kThreads, sizeof(RealSmem), s>>>(p, plan->sch);
    SIGMA_CUDA_TRY(cudaGetLastError());
  }
  if (plan->ssx.n_items > 0) {
    ssx_real_kernel<<<plan->ssx_grid, kThreads, 0, s>>>(p, plan->ssx);
    SIGMA_CUDA_TRY(cudaGetLastError());
  }
  double2* ach_c = plan->outc;
  double2* asx_c = plan->outc + kNW;
  double2* n1_c = plan->outc + 2 * kNW;
  SIGMA_CUDA_TRY(launch_gpp_reduce(plan->sch, plan->ssx, plan->nb, plan->acht_n1, ach_c, asx_c,
                                   acht_n1_loc ? n1_c : nullptr, s));
  const int nthreads = 256, n = std::max(plan->nb, kNW);
  real_parts_kernel<<<(n + nthreads - 1) / nthreads, nthreads, 0, s>>>(ach_c, asx_c, n1_c, plan->nb,
                                                                       achtemp, asxtemp, acht_n1_loc);
  SIGMA_CUDA_TRY(cudaGetLastError());
  return SIGMA_OK;
}

extern "C" int sigma_gpp_real_fp64(int number_bands, int nvband, int ncouls, int ngpown, int nstart,
                                   int nend, const int* inv_igp_index, const int* indinv,
                                   const double* wx_array, double occ, const double* aqsmtemp,
                                   const double* aqsntemp, const double* I_eps_array,
                                   const double* wtilde_array, const double* vcoul, double* achtemp,
                                   double* asxtemp, double* acht_n1_loc, void* stream) {
  using namespace sigma;
  if (!inv_igp_index || !indinv || !wx_array || !aqsmtemp || !aqsntemp || !I_eps_array ||
      !wtilde_array || !vcoul || !achtemp || !asxtemp)
    return SIGMA_ERR_NULL;
  int st = gpp_check_shape(number_bands, nvband, ncouls, ngpown, nstart, nend);
  if (st != SIGMA_OK) return st;
  std::lock_guard<std::mutex> lk(api_mutex());
  sigma_gpp_real_plan plan = nullptr;
  st = sigma_gpp_real_plan_create(&plan, number_bands, nvband, ncouls, ngpown, nstart, nend,
                                  inv_igp_index, indinv, ncouls);
  if (st != SIGMA_OK) return st;
  const size_t bb = sizeof(double) * (size_t)number_bands * ncouls;
  const size_t cb = sizeof(double) * (size_t)ngpown * ncouls;
  size_t off = 0;
  auto take = [&](size_t n) {
    const size_t o = off;
    off += up256(n);
    return o;
  };
  const size_t o_m = take(bb), o_n = take(bb), o_e = take(cb), o_w = take(cb),
               o_v = take(sizeof(double) * ncouls), o_x = take(sizeof(double) * kNW),
               o_a = take(sizeof(double) * kNW), o_s = take(sizeof(double) * kNW),
               o_1 = take(sizeof(double) * number_bands);
  void* arena = nullptr;
  st = arena_get(kArenaMisc, off, &arena);
  if (st != SIGMA_OK) {
    sigma_gpp_real_plan_destroy(plan);
    return st;
  }
  char* a = static_cast<char*>(arena);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  auto D = [&](size_t o) { return reinterpret_cast<double*>(a + o); };
  auto run = [&]() -> int {
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_m, aqsmtemp, bb, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_n, aqsntemp, bb, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_e, I_eps_array, cb, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_w, wtilde_array, cb, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_v, vcoul, sizeof(double) * ncouls, cudaMemcpyHostToDevice, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(a + o_x, wx_array, sizeof(double) * kNW, cudaMemcpyHostToDevice, s));
    int r = sigma_gpp_real_execute(plan, D(o_x), occ, D(o_m), D(o_n), D(o_e), D(o_w), D(o_v), D(o_a),
                                   D(o_s), acht_n1_loc ? D(o_1) : nullptr, stream);
    if (r != SIGMA_OK) return r;
    SIGMA_CUDA_TRY(cudaMemcpyAsync(achtemp, a + o_a, sizeof(double) * kNW, cudaMemcpyDeviceToHost, s));
    SIGMA_CUDA_TRY(cudaMemcpyAsync(asxtemp, a + o_s, sizeof(double) * kNW, cudaMemcpyDeviceToHost, s));
    if (acht_n1_loc)
      SIGMA_CUDA_TRY(cudaMemcpyAsync(acht_n1_loc, a + o_1, sizeof(double) * number_bands,
                                     cudaMemcpyDeviceToHost, s));
    SIGMA_CUDA_TRY(cudaStreamSynchronize(s));
    return SIGMA_OK;
  };
  const int rc = run();
  sigma_gpp_real_plan_destroy(plan);
  return rc;
}
