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
#include "ozaki_gemm.cuh"
#include "sigma_tma.cuh"

namespace sigma {
namespace {

using namespace tma;
using namespace ozk;

constexpr int kChunksPerRow = kOzKTile / 8;                      // 16-byte chunks per tile row

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
  const OzLaunch L{0, oz.n_items, oz.stab ? 2 : 1, oz.max_seg};
  const uint32_t smem = oz_smem_bytes(L.outs, L.segs);
  cudaError_t e = cudaFuncSetAttribute(ozaki_gemm_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  ozaki_gemm_kernel<false><<<grid, kOzThreads, smem, s>>>(d, w, oz, OzGroup{}, L);
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
  const OzLaunch L{0, g.total, g.outs, g.segs};
  const uint32_t smem = oz_smem_bytes(L.outs, L.segs);
  cudaError_t e = cudaFuncSetAttribute(ozaki_gemm_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  ozaki_gemm_kernel<true><<<std::min(grid, g.total), kOzThreads, smem, s>>>(FfDev{}, FfWork{}, OzakiPrep{}, g, L);
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
