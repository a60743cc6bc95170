// FF schDt contraction on tcgen05 tensor cores (sm_103a), split-BF16 form.
//
// tempz = I_epsR * aqsn^T (ffkernel.deslippe.best.f90:404) is one real GEMM
// per tile with the complex parts laid along K (ff_ozaki.cuh), so a TMEM lane
// holds Re and Im of tempz for its row and 64 bands.
//
// Splitting: each FP64 value x is rounded to FP32 and split exactly into three
// BF16 slices x = s1 + s2 + s3 (8 significant bits each; the subtractions
// are exact in FP32).  A*B ~ A1*B1 + (A1*B2 + A2*B1 + A1*B3 + A2*B2 + A3*B1);
// products of order 2^-24 and below are dropped.  The leading product and
// the five corrections accumulate in two TMEM accumulators so that the
// corrections' roundings are 2^-8 smaller.
//
// Accumulation: the tensor core's FP32 accumulation rounds every MMA step
// toward zero (a measured relative bias that grows linearly with the number
// of steps: 1.8e-5 over 1024 steps at the production K).  So accumulators
// live only 8 K-steps: TMEM holds two accumulator pairs, and while the
// tensor cores fill one, four drain warps read the other (tcgen05.ld) into
// round-to-nearest FP32 running sums held in registers.
//
// Roles (224 threads): warp 4 lane 0 streams 48 KB K-tiles (three A and three
// B slices of 32 K values in the 64-byte swizzle, one bulk copy per operand)
// into a four-stage shared ring, up to three tiles ahead of the tensor
// cores; warp 6 waits for each tile's stage (and for the accumulator pair
// to be drained) and releases warp 5 through a named barrier; warp 5 lane 0
// issues 12 tcgen05.mma (M=128, N=128, K=16) per tile and releases each
// stage with tcgen05.commit; warps 0-3 drain TMEM and run the epilogue,
// which multiplies tempz by conj(aqsm[n1][igp(my_igp)]) and sums the tile's
// rows per frequency (:408-418) with a reduce-scatter butterfly.  Items are
// work entries x band blocks, scheduled statically.
#include <algorithm>

#include <cuda_bf16.h>

#include "ff_ozaki.cuh"
#include "sigma_tma.cuh"

namespace sigma {
namespace {

using namespace tma;

constexpr int kOzThreads = 224;
constexpr int kDrainThreads = 128;
constexpr int kTmaWarp = 4, kMmaWarp = 5, kGateWarp = 6;
constexpr int kGateTiles = 2;  // tiles per release of the MMA warp
constexpr int kChunksPerRow = kOzKTile / 8;                      // 16-byte chunks per tile row
constexpr uint32_t kSliceBytes = kOzSliceBytes;                  // 8 KB
constexpr uint32_t kOperandBytes = kOzOperandBytes;              // 24 KB
constexpr uint32_t kStageBytes = 2 * kOperandBytes;              // 48 KB
constexpr int kStages = 4;
constexpr uint32_t kSmemBytes = kStages * kStageBytes + 2048;    // + alignment slack and 1 KB past the ring
constexpr uint32_t kTmemCols = 512;                     // 2 x (leading + correction) accumulators
constexpr int kChunkStages = 4;                         // K tiles per accumulator lifetime (8 K-steps)
constexpr int kMaxSeg = 8;                              // frequencies per row block (host checks)
constexpr uint32_t kIdesc = idesc_bf16_f32(128, 128);

__global__ void __launch_bounds__(256) ozaki_prep_a_kernel(FfDev p, OzakiPrep oz) {
  const long long total = (long long)oz.n_row_blocks * oz.kt * 128 * kChunksPerRow;
  const int rows = p.nf * p.ng;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int ch = (int)(t % kChunksPerRow);
    const int r = (int)((t / kChunksPerRow) & 127);
    const long long rest = t / (kChunksPerRow * 128);
    const int kt = (int)(rest % oz.kt);
    const int rb = (int)(rest / oz.kt);
    if (kt >= oz.kt_lim[rb]) continue;  // zero tile, not read by the contraction
    const int R = rb * kOzRows + r;
    const int k0 = kt * kOzKTile + ch * 8;
    float re[8], im[8];  // each value rounded to FP32 before it is sliced
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int k = k0 + j;
      float2 v = make_float2(0.f, 0.f);
      if (R < rows && k < p.nc) {
        if (p.epsr32) {
          v = p.epsr32[(size_t)R * p.nc + k];
        } else {
          const double2 d = p.epsr[(size_t)R * p.nc + k];
          v = make_float2(__double2float_rn(d.x), __double2float_rn(d.y));
        }
      }
      re[j] = v.x;
      im[j] = v.y;
    }
    unsigned char* base = oz.a_tiles + (size_t)rb * 2 * oz.kt * kOperandBytes;
    oz_put_row_chunk(base + (size_t)kt * kOperandBytes, r, ch, re);
    oz_put_row_chunk(base + (size_t)(oz.kt + kt) * kOperandBytes, r, ch, im);
  }
}

__global__ void __launch_bounds__(256) ozaki_prep_b_kernel(FfDev p, OzakiPrep oz) {
  const long long total = oz_prep_b_count(oz);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x)
    oz_prep_b_elem(p, oz, t);
}

__global__ void __launch_bounds__(256) ozaki_weights_kernel(FfDev p, OzakiPrep oz) {
  const long long total = oz_weights_count(oz);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x)
    oz_weights_elem(p, oz, t);
}

struct OzItem {
  int rb, cb, t0, nst;  // row block, band block, first K' tile, tiles
  size_t pidx;
};
// Items run band block fastest, then the work entries (row block, then the
// K split slowest): the CTAs running at one time share A tiles (8 band
// blocks read each) and touch only one K split of the B operand, which then
// stays in L2 (the whole B operand is 200 MB at the production shape, one
// split a quarter of it).  pidx, the partial-sum slot, does not depend on
// the order.
__device__ __forceinline__ OzItem oz_decode(const OzakiPrep& oz, int item) {
  OzItem t;
  t.cb = item % oz.n_col_blocks;
  const int4 e = oz.entries[item / oz.n_col_blocks];
  t.rb = e.x;
  t.t0 = e.z;
  t.nst = e.w;
  t.pidx = ((size_t)t.rb * oz.n_col_blocks + t.cb) * oz.max_pieces + e.y;
  return t;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void drain_barrier() {
  asm volatile("bar.sync 1, 128;" ::: "memory");
}
// The MMA warp and the gate warp meet once per kGateTiles tiles; the
// barrier's OR reduction carries the gate warp's failure flag to the MMA
// warp (a shared-memory flag read by the issuing thread between its MMAs
// would stall the tensor pipe).
__device__ __forceinline__ bool mma_gate_sync(bool flag) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 q, %1, 0;\n\t"
      "bar.red.or.pred p, 2, 64, q;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)flag)
      : "memory");
  return r != 0;
}

// One item of a group's table (kGroup): its job, tile run and partial slot.
__device__ __forceinline__ OzItem oz_group_item(const OzGroup& g, int item, int& job) {
  const int4 e = g.items[item];
  job = e.x;
  const OzakiPrep& oz = g.jobs[e.x].oz;
  OzItem t;
  t.rb = e.y >> 16;
  t.cb = e.y & 0xFFFF;
  t.t0 = e.z;
  t.nst = e.w & 0xFFFF;
  t.pidx = ((size_t)t.rb * oz.n_col_blocks + t.cb) * oz.max_pieces + (e.w >> 16);
  return t;
}

// kGroup: the items of every job of the group `g` (one table, one static
// schedule), each item with its own job's operands and epilogue; else the
// one contraction (p, oz).  The roles and their waits are the same.
template <bool kGroup>
__global__ void __launch_bounds__(kOzThreads, 1) ozaki_gemm_kernel(FfDev p, FfWork w, OzakiPrep oz, OzGroup grp) {
  extern __shared__ unsigned char smem_raw[];
  // full[kStages], empty[kStages], accf[2], acce[2], done
  __shared__ __align__(8) unsigned long long bars[2 * kStages + 5];
  __shared__ uint32_t tmem_slot;
  __shared__ float2 s_red[2][4][kMaxSeg][kOzCols];

  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t sbase = (raw + 1023u) & ~1023u;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t full0 = smem_u32(&bars[0]), empty0 = smem_u32(&bars[kStages]);
  const uint32_t accf0 = smem_u32(&bars[2 * kStages]), acce0 = smem_u32(&bars[2 * kStages + 2]);
  const int n_items = kGroup ? grp.total : oz.n_items;
  int* const status = kGroup ? grp.status : w.status;

  if (warp == 0) tmem_alloc(smem_u32(&tmem_slot), kTmemCols);
  const uint32_t done0 = smem_u32(&bars[2 * kStages + 4]);
  if (tid == 0) {
    for (int i = 0; i < 2 * kStages + 2; ++i) mbar_init(smem_u32(&bars[i]), 1);
    mbar_init(acce0, 4);
    mbar_init(acce0 + 8u, 4);
    mbar_init(done0, 1);
    fence_mbar_init();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == kTmaWarp) {
    // ------------------------------------------------ bulk copies into the stage ring
    if (lane == 0) {
      uint32_t g = 0;  // tiles issued by this CTA
      bool ok = true;
      for (int item = blockIdx.x; ok && item < n_items; item += gridDim.x) {
        int job = 0;
        const OzItem it = kGroup ? oz_group_item(grp, item, job) : oz_decode(oz, item);
        const int nst = it.nst;
        const unsigned char* at = kGroup ? grp.jobs[job].oz.a_tiles : oz.a_tiles;
        const unsigned char* bt = kGroup ? grp.jobs[job].oz.b_tiles : oz.b_tiles;
        const int two_kt = 2 * (kGroup ? grp.jobs[job].oz.kt : oz.kt);
        const unsigned char* a_src = at + ((size_t)it.rb * two_kt + it.t0) * kOperandBytes;
        const unsigned char* b_src = bt + ((size_t)it.cb * two_kt + it.t0) * kOperandBytes;
        for (int s = 0; s < nst; ++s, ++g) {
          const uint32_t b = g % kStages, use = g / kStages;
          // stage b is free once the MMAs of its previous tile have completed
          if (use > 0 && !mbar_wait(empty0 + 8u * b, (use - 1) & 1u, status)) {
            ok = false;  // no further copies
            break;
          }
          const uint32_t bar = full0 + 8u * b;
          const uint32_t dst = sbase + b * kStageBytes;
          mbar_expect_tx(bar, kStageBytes);
          bulk_load(dst, a_src + (size_t)s * kOperandBytes, kOperandBytes, bar);
          bulk_load(dst + kOperandBytes, b_src + (size_t)s * kOperandBytes, kOperandBytes, bar);
        }
      }
      // after a failure: the copies of the last (up to kStages) tiles may
      // still be landing; wait for them before the CTA releases its ring
      if (!ok)
        for (uint32_t t = g > (uint32_t)kStages ? g - kStages : 0u; t < g; ++t)
          mbar_wait_own(full0 + 8u * (t % kStages), (t / kStages) & 1u);
    }
    __syncwarp();
  } else if (warp == kGateWarp) {
    // ------------------------------------------------ release of the MMA warp
    // Waits for each tile's stage (and, at an accumulator lifetime's first
    // tile, for the drain of that accumulator pair), and meets the MMA warp
    // at a named barrier once per kGateTiles tiles.  The issuing thread itself never polls shared
    // memory: a poll between its MMAs stalls the tensor pipe (measured: 89
    // instead of 64 cycles per MMA).
    // After a wait gives up it keeps meeting the MMA warp at the same named
    // barriers (whose count must match) without waiting, and passes the
    // failure on through them so the MMA warp issues nothing more.
    uint32_t ph_acce0 = 0, ph_acce1 = 0;
    bool used0 = false, used1 = false, failed = false;
    uint32_t g = 0, gc = 0;
    // group: the next item's tile count is loaded one item ahead
    int nst_next = kGroup && blockIdx.x < n_items ? (grp.items[blockIdx.x].w & 0xFFFF) : 0;
    for (int item = blockIdx.x; item < n_items; item += gridDim.x) {
      int nst;
      if (kGroup) {
        nst = nst_next;
        if (item + (int)gridDim.x < n_items) nst_next = grp.items[item + gridDim.x].w & 0xFFFF;
      } else {
        nst = oz_decode(oz, item).nst;
      }
      for (int s = 0; s < nst; ++s, ++g) {
        const int cs = s % kChunkStages;
        const uint32_t tb = gc & 1u;
        if (lane == 0 && !failed) {
          if (cs == 0) {  // first tile of an accumulator lifetime: pair tb must be drained
            if (tb == 0 && used0) {
              failed = !mbar_wait(acce0, ph_acce0, status);
              ph_acce0 ^= 1u;
            }
            if (tb == 1 && used1) {
              failed = failed || !mbar_wait(acce0 + 8u, ph_acce1, status);
              ph_acce1 ^= 1u;
            }
          }
          const uint32_t b = g % kStages;
          failed = failed || !mbar_wait(full0 + 8u * b, (g / kStages) & 1u, status);
        }
        if (cs == 0) {
          if (tb == 0) used0 = true; else used1 = true;
        }
        if (cs == kChunkStages - 1 || s == nst - 1) ++gc;
        if (s % kGateTiles == kGateTiles - 1 || s == nst - 1) {
          __syncwarp();
          mma_gate_sync(failed);
        }
      }
    }
    // every accumulator pair in use drained
    if (lane == 0 && !failed) {
      if (used0) mbar_wait(acce0, ph_acce0, status);
      if (used1) mbar_wait(acce0 + 8u, ph_acce1, status);
    }
    __syncwarp();
  } else if (warp == kMmaWarp) {
    // ------------------------------------------------ tensor-core issue (lane 0)
    uint32_t g = 0;   // tiles consumed by this CTA
    uint32_t gc = 0;  // accumulator lifetimes started
    bool failed = false;
    // group: the next item's tile count is loaded one item ahead
    int nst_next = kGroup && blockIdx.x < n_items ? (grp.items[blockIdx.x].w & 0xFFFF) : 0;
    for (int item = blockIdx.x; item < n_items; item += gridDim.x) {
      int nst;
      if (kGroup) {
        nst = nst_next;
        if (item + (int)gridDim.x < n_items) nst_next = grp.items[item + gridDim.x].w & 0xFFFF;
      } else {
        nst = oz_decode(oz, item).nst;
      }
      for (int s = 0; s < nst; ++s, ++g) {
        const int cs = s % kChunkStages;
        const uint32_t tb = gc & 1u;
        // stages full, accumulator pair free (or the gate warp gave up)
        if (s % kGateTiles == 0) failed = mma_gate_sync(false) || failed;
        if (lane == 0 && !failed) {
          tc_fence_after();
          const uint32_t b = g % kStages;
          const uint32_t a_addr = sbase + b * kStageBytes;
          const uint32_t b_addr = a_addr + kOperandBytes;
          const uint32_t d_big = tmem + tb * 256u, d_small = d_big + 128u;
#pragma unroll
          for (int kk = 0; kk < kOzKTile / 16; ++kk) {
            const uint64_t a1 = sw64_desc(a_addr + kk * 32);
            const uint64_t a2 = sw64_desc(a_addr + kSliceBytes + kk * 32);
            const uint64_t a3 = sw64_desc(a_addr + 2 * kSliceBytes + kk * 32);
            const uint64_t b1 = sw64_desc(b_addr + kk * 32);
            const uint64_t b2 = sw64_desc(b_addr + kSliceBytes + kk * 32);
            const uint64_t b3 = sw64_desc(b_addr + 2 * kSliceBytes + kk * 32);
            const uint32_t acc = (cs > 0 || kk > 0) ? 1u : 0u;
            mma_f16(d_big, a1, b1, kIdesc, acc);
            mma_f16(d_small, a1, b2, kIdesc, acc);
            mma_f16(d_small, a2, b1, kIdesc, 1u);
            mma_f16(d_small, a1, b3, kIdesc, 1u);
            mma_f16(d_small, a2, b2, kIdesc, 1u);
            mma_f16(d_small, a3, b1, kIdesc, 1u);
          }
          mma_commit(empty0 + 8u * b);  // stage b free once these MMAs complete
          if (cs == kChunkStages - 1 || s == nst - 1) mma_commit(accf0 + 8u * tb);  // pair tb complete
        }
        if (cs == kChunkStages - 1 || s == nst - 1) ++gc;
        __syncwarp();
      }
    }
    // after a failure: the MMAs already issued complete before the tensor
    // memory is released
    if (lane == 0 && failed) {
      mma_commit(done0);
      mbar_wait_own(done0, 0);
    }
    __syncwarp();
  } else {
    // ------------------------------------------------ drain + epilogue (warps 0-3)
    uint32_t ph_accf0 = 0, ph_accf1 = 0;
    uint32_t gc = 0;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    for (int item = blockIdx.x; item < n_items; item += gridDim.x) {
      int job = 0;
      const OzItem it = kGroup ? oz_group_item(grp, item, job) : oz_decode(oz, item);
      // the item's contraction: its shape, epilogue factors and partial slots
      const int e_nf = kGroup ? grp.jobs[job].d.nf : p.nf, e_ng = kGroup ? grp.jobs[job].d.ng : p.ng;
      const int rows = e_nf * e_ng;
      const int nchunks = (it.nst + kChunkStages - 1) / kChunkStages;
      float acc[128];
#pragma unroll
      for (int i = 0; i < 128; ++i) acc[i] = 0.f;
      for (int c = 0; c < nchunks; ++c) {
        const uint32_t tb = gc & 1u;
        if (tb == 0) {
          mbar_wait(accf0, ph_accf0, status);
          ph_accf0 ^= 1u;
        } else {
          mbar_wait(accf0 + 8u, ph_accf1, status);
          ph_accf1 ^= 1u;
        }
        tc_fence_after();
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          float big[32], small[32];
          tmem_ld32(lane_base + tb * 256u + q * 32, big);
          tmem_ld32(lane_base + tb * 256u + 128u + q * 32, small);
#pragma unroll
          for (int i = 0; i < 32; ++i) acc[q * 32 + i] += big[i] + small[i];
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(acce0 + 8u * tb);
        ++gc;
      }

      // epilogue: row R of this lane, 64 bands; tempz * weight * conj(aqsm[n1][igp])
      const int R = it.rb * kOzRows + warp * 32 + lane;
      const bool row_ok = R < rows;
      const int f = row_ok ? R / e_ng : 0;
      const int g = row_ok ? R % e_ng : 0;
      const int f_first = (it.rb * kOzRows) / e_ng;
      const int f_last = (min(it.rb * kOzRows + kOzRows, rows) - 1) / e_ng;
      const float2* e_wtab = kGroup ? grp.jobs[job].oz.wtab : oz.wtab;
      const int e_nbpad = kGroup ? grp.jobs[job].oz.nb_pad : oz.nb_pad;
      const float* e_stab = kGroup ? grp.jobs[job].oz.stab : oz.stab;
      // the row's 64 factors: 32 contiguous 16-byte loads in four batches
      const float4* wrow =
          reinterpret_cast<const float4*>(e_wtab + (size_t)g * e_nbpad + (size_t)it.cb * kOzCols);
#pragma unroll
      for (int n0 = 0; n0 < 64; n0 += 16) {
        float4 wv[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) wv[j] = row_ok ? __ldg(wrow + n0 / 2 + j) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int n = n0 + 2 * j + h;
            const float mr = h ? wv[j].z : wv[j].x, mi = h ? wv[j].w : wv[j].y;
            const float cr = acc[n], ci = acc[64 + n];
            acc[n] = fmaf(cr, mr, ci * mi);
            acc[64 + n] = fmaf(ci, mr, -cr * mi);
          }
        }
      }
      // one or two outputs: the second's rows carry the extra column factor stab
      const bool two = e_stab != nullptr;
      const float sc = (two && row_ok) ? e_stab[g] : 0.f;
      for (int seg = 0; seg <= f_last - f_first; ++seg) {
        const bool mine = row_ok && (f - f_first) == seg;
        // 16 bands at a time: a reduce-scatter butterfly over the warp leaves
        // lanes 2j and 2j+1 with the sum of band j of the batch
#pragma unroll
        for (int b0 = 0; b0 < 64; b0 += 16) {
#pragma unroll 1
          for (int out = 0; out < 2; ++out) {
            if (out == 1 && !two) break;
            const float m = out == 0 ? 1.f : sc;
            float xr[16], xi[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) {
              xr[i] = mine ? acc[b0 + i] * m : 0.f;
              xi[i] = mine ? acc[64 + b0 + i] * m : 0.f;
            }
#pragma unroll
            for (int o = 16, h = 8; o >= 2; o >>= 1, h >>= 1) {
              const bool up = (lane & o) != 0;
#pragma unroll
              for (int i = 0; i < h; ++i) {
                const float sr = up ? xr[i] : xr[i + h];
                const float si = up ? xi[i] : xi[i + h];
                const float rr = __shfl_xor_sync(0xffffffffu, sr, o);
                const float ri = __shfl_xor_sync(0xffffffffu, si, o);
                xr[i] = (up ? xr[i + h] : xr[i]) + rr;
                xi[i] = (up ? xi[i + h] : xi[i]) + ri;
              }
            }
            xr[0] += __shfl_xor_sync(0xffffffffu, xr[0], 1);
            xi[0] += __shfl_xor_sync(0xffffffffu, xi[0], 1);
            if ((lane & 1) == 0) s_red[out][warp][seg][b0 + (lane >> 1)] = make_float2(xr[0], xi[0]);
          }
        }
      }
      drain_barrier();
      const int nseg = f_last - f_first + 1;
      for (int e = tid; e < (two ? 2 : 1) * nseg * kOzCols; e += kDrainThreads) {
        const int out = e / (nseg * kOzCols), r = e % (nseg * kOzCols);
        const int seg = r / kOzCols, n = r % kOzCols;
        double sr = 0.0, si = 0.0;
        for (int q = 0; q < 4; ++q) {
          sr += (double)s_red[out][q][seg][n].x;
          si += (double)s_red[out][q][seg][n].y;
        }
        double2* part = kGroup ? (out ? grp.jobs[job].oz.partial2 : grp.jobs[job].oz.partial)
                               : (out ? oz.partial2 : oz.partial);
        const int max_seg = kGroup ? grp.jobs[job].oz.max_seg : oz.max_seg;
        part[(it.pidx * max_seg + seg) * kOzCols + n] = make_double2(sr, si);
      }
      drain_barrier();
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

// schDt[n1][ifreq]: one warp per entry, fixed-order compensated sum over the
// row blocks that hold frequency ifreq and over their work entries.
__device__ __forceinline__ void reduce_entry(const FfDev& p, const OzakiPrep& oz, const double2* partial,
                                             double2* schdt, int warp, int lane) {
  const int n = warp / p.nf, f = warp % p.nf;
  const int cb = n / kOzCols, c = n % kOzCols;
  const int rb_lo = (f * p.ng) / kOzRows, rb_hi = ((f + 1) * p.ng - 1) / kOzRows;
  Comp sx, sy;
  int q0 = 0;  // entries of the row blocks before rb, lanes take every 32nd
  for (int rb = rb_lo; rb <= rb_hi; ++rb) {
    const int np = oz.pieces[rb];
    const int seg = f - (rb * kOzRows) / p.ng;
    for (int j = (lane - q0 % 32 + 32) % 32; j < np; j += 32) {
      const size_t pidx = ((size_t)rb * oz.n_col_blocks + cb) * oz.max_pieces + j;
      const double2 v = partial[(pidx * oz.max_seg + seg) * kOzCols + c];
      sx.add(v.x);
      sy.add(v.y);
    }
    q0 += np;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double a = __shfl_xor_sync(0xffffffffu, sx.s, o), b = __shfl_xor_sync(0xffffffffu, sx.c, o);
    const double c2 = __shfl_xor_sync(0xffffffffu, sy.s, o), d = __shfl_xor_sync(0xffffffffu, sy.c, o);
    double t, e;
    two_sum_d(sx.s, a, t, e);
    sx.s = t;
    sx.c = __dadd_rn(__dadd_rn(sx.c, b), e);
    two_sum_d(sy.s, c2, t, e);
    sy.s = t;
    sy.c = __dadd_rn(__dadd_rn(sy.c, d), e);
  }
  if (lane == 0) schdt[(size_t)n * p.nf + f] = make_double2(sx.value(), sy.value());
}

__global__ void ozaki_reduce_kernel(FfDev p, OzakiPrep oz, const double2* partial, double2* schdt) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= p.nb * p.nf) return;
  reduce_entry(p, oz, partial, schdt, warp, threadIdx.x & 31);
}

// Group form: warps r_warp_off .. + nb * nf of each job reduce its entries.
__global__ void ozaki_group_reduce_kernel(OzGroup g) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= g.r_warps) return;
  int lo = 0, hi = g.n_jobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (g.jobs[mid].r_warp_off <= warp) lo = mid; else hi = mid - 1;
  }
  const OzGroupJob& J = g.jobs[lo];
  reduce_entry(J.d, J.oz, J.oz.partial, J.out, warp - J.r_warp_off, threadIdx.x & 31);
}

}  // namespace

void ozaki_size(OzakiPrep& oz, const FfDev& d, int grid, const int* row_kend, OzakiTables* tables,
                int split_tiles_hint, int items_per_cta) {
  oz.kt = (d.nc + kOzKTile - 1) / kOzKTile;
  const int rows = d.nf * d.ng;
  oz.n_row_blocks = (rows + kOzRows - 1) / kOzRows;
  oz.n_col_blocks = (d.nb + kOzCols - 1) / kOzCols;
  oz.max_seg = (kOzRows + d.ng - 2) / d.ng + 1;
  const int two_kt = 2 * oz.kt;
  std::vector<int> kl(oz.n_row_blocks, oz.kt);
  long long active = 0;  // K' tiles over all row blocks that can be nonzero
  for (int rb = 0; rb < oz.n_row_blocks; ++rb) {
    if (row_kend) {
      int k = 0;
      for (int r = rb * kOzRows; r < std::min(rows, rb * kOzRows + kOzRows); ++r)
        k = std::max(k, std::min(row_kend[r], d.nc));
      kl[rb] = (k + kOzKTile - 1) / kOzKTile;
    }
    active += 2LL * kl[rb];
  }
  // about 20 items per CTA: as many K splits as the active tiles need
  const long long want = (long long)(items_per_cta > 0 ? items_per_cta : 20) * grid * two_kt;
  const long long have = std::max(1LL, active * oz.n_col_blocks);
  long long s = (want + have - 1) / have;
  if (split_tiles_hint > 0) s = (two_kt + split_tiles_hint - 1) / split_tiles_hint;
  if (s < 1) s = 1;
  if (s > two_kt) s = two_kt;
  oz.split_tiles = (int)((two_kt + s - 1) / s);
  oz.n_splits = (two_kt + oz.split_tiles - 1) / oz.split_tiles;
  // entries: per split, per row block, the split's tiles within [0, kl) and
  // [kt, kt + kl) (one run when they touch)
  std::vector<int4> ent;
  std::vector<int> pieces(oz.n_row_blocks, 0);
  for (int sp = 0; sp < oz.n_splits; ++sp) {
    const int a = sp * oz.split_tiles, b = std::min(two_kt, a + oz.split_tiles);
    for (int rb = 0; rb < oz.n_row_blocks; ++rb) {
      const int runs[2][2] = {{0, kl[rb]}, {oz.kt, oz.kt + kl[rb]}};
      int lo[2], hi[2], n = 0;
      for (const auto& run : runs) {
        const int x = std::max(a, run[0]), y = std::min(b, run[1]);
        if (x >= y) continue;
        if (n > 0 && hi[n - 1] == x) {
          hi[n - 1] = y;
        } else {
          lo[n] = x;
          hi[n] = y;
          ++n;
        }
      }
      for (int i = 0; i < n; ++i) ent.push_back(make_int4(rb, pieces[rb]++, lo[i], hi[i] - lo[i]));
    }
  }
  oz.n_entries = (int)ent.size();
  oz.n_items = oz.n_entries * oz.n_col_blocks;
  oz.max_pieces = std::max(1, *std::max_element(pieces.begin(), pieces.end()));
  oz.ng = d.ng;
  oz.nb_pad = oz.n_col_blocks * kOzCols;
  if (tables) {
    tables->entries = std::move(ent);
    tables->pieces = std::move(pieces);
    tables->kt_lim = std::move(kl);
  }
}

int ozaki_max_segments() { return kMaxSeg; }

size_t ozaki_tile_bytes(const OzakiPrep& oz) {
  return ((size_t)oz.n_row_blocks + oz.n_col_blocks) * 2 * oz.kt * kOperandBytes + 1024;
}

static size_t up256(size_t v) { return (v + 255) / 256 * 256; }

static size_t ozaki_partial_only_bytes(const OzakiPrep& oz) {
  return up256(sizeof(double2) * (size_t)oz.n_row_blocks * oz.n_col_blocks * oz.max_pieces *
               oz.max_seg * kOzCols);
}
static size_t ozaki_wtab_bytes(const OzakiPrep& oz) {
  return up256(sizeof(float2) * (size_t)oz.ng * oz.nb_pad);
}

size_t ozaki_partial_bytes(const OzakiPrep& oz) {
  return 2 * ozaki_partial_only_bytes(oz) + ozaki_wtab_bytes(oz) + up256(sizeof(float) * (size_t)oz.ng) +
         up256(sizeof(int4) * (size_t)std::max(oz.n_entries, 1)) +
         2 * up256(sizeof(int) * (size_t)oz.n_row_blocks) + 256;
}

size_t ozaki_prep_bytes(const OzakiPrep& oz) { return ozaki_tile_bytes(oz) + ozaki_partial_bytes(oz); }

void ozaki_bind(OzakiPrep& oz, void* tiles, void* partial) {
  uintptr_t b = (reinterpret_cast<uintptr_t>(tiles) + 1023) & ~uintptr_t(1023);
  oz.a_tiles = reinterpret_cast<unsigned char*>(b);
  oz.b_tiles = oz.a_tiles + (size_t)oz.n_row_blocks * 2 * oz.kt * kOperandBytes;
  uintptr_t pp = (reinterpret_cast<uintptr_t>(partial) + 255) & ~uintptr_t(255);
  oz.partial = reinterpret_cast<double2*>(pp);
  pp += ozaki_partial_only_bytes(oz);
  oz.partial2 = reinterpret_cast<double2*>(pp);
  pp += ozaki_partial_only_bytes(oz);
  oz.wtab = reinterpret_cast<float2*>(pp);
  pp += ozaki_wtab_bytes(oz);
  oz.stab_buf = reinterpret_cast<float*>(pp);
  oz.stab = nullptr;
  pp += up256(sizeof(float) * (size_t)oz.ng);
  oz.entries = reinterpret_cast<const int4*>(pp);
  pp += up256(sizeof(int4) * (size_t)std::max(oz.n_entries, 1));
  oz.pieces = reinterpret_cast<const int*>(pp);
  pp += up256(sizeof(int) * (size_t)oz.n_row_blocks);
  oz.kt_lim = reinterpret_cast<const int*>(pp);
}

void ozaki_prep_bind(OzakiPrep& oz, void* base) {
  ozaki_bind(oz, base, static_cast<char*>(base) + ozaki_tile_bytes(oz));
}

cudaError_t ozaki_upload_tables(const OzakiPrep& oz, const OzakiTables& t) {
  cudaError_t e = cudaSuccess;
  if (!t.entries.empty())
    e = cudaMemcpy(const_cast<int4*>(oz.entries), t.entries.data(), sizeof(int4) * t.entries.size(),
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(const_cast<int*>(oz.pieces), t.pieces.data(), sizeof(int) * t.pieces.size(),
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(const_cast<int*>(oz.kt_lim), t.kt_lim.data(), sizeof(int) * t.kt_lim.size(),
                   cudaMemcpyHostToDevice);
  return e;
}

cudaError_t launch_ozaki_prep(const FfDev& d, const OzakiPrep& oz, cudaStream_t s, bool with_a) {
  cudaError_t e;
  if (with_a) {
    ozaki_prep_a_kernel<<<152 * 16, 256, 0, s>>>(d, oz);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  ozaki_prep_b_kernel<<<152 * 4, 256, 0, s>>>(d, oz);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  ozaki_weights_kernel<<<152 * 2, 256, 0, s>>>(d, oz);
  return cudaGetLastError();
}

namespace {
// Zero slices of the A rows in [rows, n_row_blocks * 128) for the K tiles the
// contraction reads (rows a producer of A rows does not write).
__global__ void __launch_bounds__(256) ozaki_zero_rows_kernel(OzakiPrep oz, int rows) {
  const int last = oz.n_row_blocks - 1;
  const int r0 = rows - last * kOzRows;
  if (r0 >= kOzRows) return;
  const long long total = (long long)(kOzRows - r0) * oz.kt * kChunksPerRow;
  const float z[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int ch = (int)(t % kChunksPerRow);
    const int kt = (int)((t / kChunksPerRow) % oz.kt);
    const int r = r0 + (int)(t / ((long long)kChunksPerRow * oz.kt));
    if (kt >= oz.kt_lim[last]) continue;
    oz_put_a(oz, last * kOzRows + r, kt * kOzKTile + ch * 8, z, z);
  }
}
}  // namespace

cudaError_t launch_ozaki_zero_rows(const OzakiPrep& oz, int rows, cudaStream_t s) {
  if (rows >= oz.n_row_blocks * kOzRows) return cudaSuccess;
  ozaki_zero_rows_kernel<<<152, 256, 0, s>>>(oz, rows);
  return cudaGetLastError();
}

cudaError_t launch_ozaki_gemm(const FfDev& d, const FfWork& w, const OzakiPrep& oz, int grid,
                              cudaStream_t s) {
  cudaError_t e =
      cudaFuncSetAttribute(ozaki_gemm_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
  if (e != cudaSuccess) return e;
  ozaki_gemm_kernel<false><<<grid, kOzThreads, kSmemBytes, s>>>(d, w, oz, OzGroup{});
  return cudaGetLastError();
}

void ozaki_group_items(int job, const OzakiPrep& oz, const OzakiTables& t, std::vector<int4>& items) {
  for (int it = 0; it < oz.n_items; ++it) {
    const int4 e = t.entries[it / oz.n_col_blocks];
    const int cb = it % oz.n_col_blocks;
    items.push_back(make_int4(job, (e.x << 16) | cb, e.z, e.w | (e.y << 16)));
  }
}

cudaError_t launch_ozaki_group_gemm(const OzGroup& g, int grid, cudaStream_t s) {
  if (g.total <= 0) return cudaSuccess;
  cudaError_t e =
      cudaFuncSetAttribute(ozaki_gemm_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
  if (e != cudaSuccess) return e;
  ozaki_gemm_kernel<true><<<std::min(grid, g.total), kOzThreads, kSmemBytes, s>>>(FfDev{}, FfWork{}, OzakiPrep{},
                                                                                  g);
  return cudaGetLastError();
}

cudaError_t launch_ozaki_group_reduce(const OzGroup& g, cudaStream_t s) {
  if (g.r_warps <= 0) return cudaSuccess;
  ozaki_group_reduce_kernel<<<(g.r_warps * 32 + 255) / 256, 256, 0, s>>>(g);
  return cudaGetLastError();
}

cudaError_t launch_ozaki_reduce(const FfDev& d, const OzakiPrep& oz, double2* schdt, cudaStream_t s,
                                double2* schdt2) {
  const int warps = d.nb * d.nf;
  const int blocks = (warps * 32 + 255) / 256;
  ozaki_reduce_kernel<<<blocks, 256, 0, s>>>(d, oz, oz.partial, schdt);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || !schdt2) return e;
  ozaki_reduce_kernel<<<blocks, 256, 0, s>>>(d, oz, oz.partial2, schdt2);
  return cudaGetLastError();
}

}  // namespace sigma
