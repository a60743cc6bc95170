// The split-BF16 tcgen05 contraction kernel: roles, stage ring, TMEM drains
// and epilogue (ff_ozaki.cu launches it for the FF and GPP contractions).
#pragma once

#include "ff_ozaki.cuh"
#include "sigma_tma.cuh"

namespace sigma {
namespace ozk {

using namespace tma;

constexpr int kOzThreads = 224;
constexpr int kDrainThreads = 128;
constexpr int kTmaWarp = 4, kMmaWarp = 5, kGateWarp = 6;
constexpr int kGateTiles = 2;  // tiles per release of the MMA warp
constexpr uint32_t kSliceBytes = kOzSliceBytes;                  // 8 KB
constexpr uint32_t kOperandBytes = kOzOperandBytes;              // 24 KB
constexpr uint32_t kStageBytes = 2 * kOperandBytes;              // 48 KB
constexpr int kStages = 4;
constexpr uint32_t kRingBytes = kStages * kStageBytes + 1024;    // + slack to align the ring to 1 KB
constexpr uint32_t kTmemCols = 512;                     // 2 x (leading + correction) accumulators
constexpr int kChunkStages = 4;                         // K tiles per accumulator lifetime (8 K-steps)
constexpr int kMaxSeg = 8;                              // frequencies per row block (host checks)
constexpr uint32_t kIdesc = idesc_bf16_f32(128, 128);

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
// The launch's items [begin, end) of the single plan's or the group's item
// order, and the epilogue's staging shape: outs output sums (1, or 2 with a
// second column factor) of segs frequency segments per row block.
struct OzLaunch {
  int begin, end;
  int outs, segs;
};
// Dynamic shared memory of a launch: the ring, then the epilogue staging
// s_red[outs][4 warps][segs][kOzCols].
__host__ __device__ constexpr uint32_t oz_red_bytes(int outs, int segs) {
  return (uint32_t)(outs * 4 * segs * kOzCols) * (uint32_t)sizeof(float2);
}
__host__ __device__ constexpr uint32_t oz_smem_bytes(int outs, int segs) {
  return kRingBytes + oz_red_bytes(outs, segs);
}

template <bool kGroup>
__global__ void __launch_bounds__(kOzThreads, 1) ozaki_gemm_kernel(FfDev p, FfWork w, OzakiPrep oz, OzGroup grp,
                                                                  OzLaunch L) {
  extern __shared__ unsigned char smem_raw[];
  // full[kStages], empty[kStages], accf[2], acce[2], done
  __shared__ __align__(8) unsigned long long bars[2 * kStages + 5];
  __shared__ uint32_t tmem_slot;

  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t sbase = (raw + 1023u) & ~1023u;
  // epilogue staging after the ring (16-byte aligned: the ring is 1 KB aligned)
  float2* const s_red = reinterpret_cast<float2*>(smem_raw + (sbase - raw) + kStages * kStageBytes);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t full0 = smem_u32(&bars[0]), empty0 = smem_u32(&bars[kStages]);
  const uint32_t accf0 = smem_u32(&bars[2 * kStages]), acce0 = smem_u32(&bars[2 * kStages + 2]);
  const int n_items = L.end;
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
      for (int item = L.begin + blockIdx.x; ok && item < n_items; item += gridDim.x) {
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
    int nst_next = kGroup && L.begin + (int)blockIdx.x < n_items ? (grp.items[L.begin + blockIdx.x].w & 0xFFFF) : 0;
    for (int item = L.begin + blockIdx.x; item < n_items; item += gridDim.x) {
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
    int nst_next = kGroup && L.begin + (int)blockIdx.x < n_items ? (grp.items[L.begin + blockIdx.x].w & 0xFFFF) : 0;
    for (int item = L.begin + blockIdx.x; item < n_items; item += gridDim.x) {
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
    for (int item = L.begin + blockIdx.x; item < n_items; item += gridDim.x) {
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
            if ((lane & 1) == 0) s_red[((out * 4 + warp) * L.segs + seg) * kOzCols + b0 + (lane >> 1)] = make_float2(xr[0], xi[0]);
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
          const float2 v = s_red[((out * 4 + q) * L.segs + seg) * kOzCols + n];
          sr += (double)v.x;
          si += (double)v.y;
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

}  // namespace ozk
}  // namespace sigma
