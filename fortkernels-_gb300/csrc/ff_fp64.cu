// FF schDt contraction, FP64 form (sm_103a), and the fixed-order reduction
// shared by both FF forms.
//
// tempz[(ifreq, my_igp), n1] = sum_ig I_epsR[ifreq][my_igp][ig] * aqsn[n1][ig] is a
// complex GEMM (M = nfreq*ngpown, N = number_bands, K = ncouls); the reference
// writes it as zgemm('t','n', ...) (ffkernel.deslippe.best.f90:404).  Here a
// persistent grid takes (row block, band block, K split) items; each CTA
// stages 16-wide K chunks of both operands through shared memory and every
// thread keeps a 4 x 4 complex register tile.  Each complex multiply-add is
// three real products: with the chunk's sums a.x + a.y and b.x + b.y staged
// beside the operands, P1 = sum a.x b.x, P2 = sum a.y b.y,
// P3 = sum (a.x + a.y)(b.x + b.y) and sum a b = (P1 - P2) + i (P3 - P1 - P2):
// 3 DFMA instead of 4 (FP64 roundings of the sums stay near 1e-16 of the
// partial sums).  The epilogue fuses the second
// half of the source loop (:408-418): each tile multiplies its tempz values
// by conj(aqsm[n1][igp(my_igp)]) and sums its rows, so tempz never reaches
// memory.
#include "ff_internal.cuh"

namespace sigma {
namespace {

constexpr int kK = 16;            // complex K per staged chunk
constexpr int kFfThreads = 256;   // 16 x 16 threads, 4 x 4 complex per thread

struct FfSmem {
  double2 a[kK][kFfRows + 1];
  double2 b[kK][kFfCols + 1];
  double as[kK][kFfRows + 1];  // a.x + a.y
  double bs[kK][kFfCols + 1];  // b.x + b.y
  double2 red[16][kFfCols];
};

__global__ void __launch_bounds__(kFfThreads, 1) ff_fp64_kernel(FfDev p, FfWork w) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  FfSmem& sm = *reinterpret_cast<FfSmem*>(smem_raw);
  __shared__ int s_item;
  const int tid = threadIdx.x, tc = tid & 15, tr = tid >> 4;
  const int blocks_per_freq = p.ngp / kFfRows;

  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(w.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= w.n_items) break;
    const FfItem it = ff_decode(w, item);
    const int f = it.rb / blocks_per_freq;
    const int g0 = (it.rb % blocks_per_freq) * kFfRows;
    const int n0 = it.cb * kFfCols;
    const int k_begin = it.s * w.split_len;
    const int k_end = min(k_begin + w.split_len, p.nc);

    double p1[4][4], p2[4][4], p3[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) p1[i][j] = p2[i][j] = p3[i][j] = 0.0;

    for (int k0 = k_begin; k0 < k_end; k0 += kK) {
      __syncthreads();
      for (int e = tid; e < kK * kFfRows; e += kFfThreads) {
        const int r = e / kK, k = e % kK;
        const int g = g0 + r, kk = k0 + k;
        double2 v = make_double2(0.0, 0.0);
        if (g < p.ng && kk < k_end) v = p.epsr[((size_t)f * p.ng + g) * p.nc + kk];
        sm.a[k][r] = v;
        sm.as[k][r] = __dadd_rn(v.x, v.y);
      }
      for (int e = tid; e < kK * kFfCols; e += kFfThreads) {
        const int c = e / kK, k = e % kK;
        const int n = n0 + c, kk = k0 + k;
        double2 v = make_double2(0.0, 0.0);
        if (n < p.nb && kk < k_end) v = p.aqsn[(size_t)n * p.nc + kk];
        sm.b[k][c] = v;
        sm.bs[k][c] = __dadd_rn(v.x, v.y);
      }
      __syncthreads();
#pragma unroll 4
      for (int k = 0; k < kK; ++k) {
        double2 a[4], b[4];
        double asum[4], bsum[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          a[i] = sm.a[k][tr + 16 * i];
          asum[i] = sm.as[k][tr + 16 * i];
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          b[j] = sm.b[k][tc + 16 * j];
          bsum[j] = sm.bs[k][tc + 16 * j];
        }
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            p1[i][j] = fma(a[i].x, b[j].x, p1[i][j]);
            p2[i][j] = fma(a[i].y, b[j].y, p2[i][j]);
            p3[i][j] = fma(asum[i], bsum[j], p3[i][j]);
          }
      }
    }

    // epilogue: tempz * conj(aqsm[n1][igp]) summed over the tile's rows
    double2 part[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) part[j] = make_double2(0.0, 0.0);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int g = g0 + tr + 16 * i;
      if (g >= p.ng) continue;
      const int igp = p.igp_of[g];
      if (igp < 0) continue;
      const double wgt = ff_column_weight(p, igp);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int n = n0 + tc + 16 * j;
        if (n >= p.nb) continue;
        double2 m = p.aqsm[(size_t)n * p.nc + igp];  // conj(m) applied below
        m.x *= wgt;
        m.y *= wgt;
        const double tre = __dsub_rn(p1[i][j], p2[i][j]);
        const double tim = __dsub_rn(__dsub_rn(p3[i][j], p1[i][j]), p2[i][j]);
        part[j].x += tre * m.x + tim * m.y;
        part[j].y += tim * m.x - tre * m.y;
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) sm.red[tr][tc + 16 * j] = part[j];
    __syncthreads();
    if (tid < kFfCols) {
      double sx = 0.0, sy = 0.0;
      for (int q = 0; q < 16; ++q) {
        sx += sm.red[q][tid].x;
        sy += sm.red[q][tid].y;
      }
      w.partial[it.pidx * kFfCols + tid] = make_double2(sx, sy);
    }
  }
}

// schDt[n1][ifreq]: one warp per entry sums its row blocks and K splits in a
// fixed order with compensated FP64.
__global__ void ff_reduce_kernel(FfDev p, FfWork w, double2* schdt) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= p.nb * p.nf) return;
  const int n = warp / p.nf, f = warp % p.nf;
  const int blocks_per_freq = p.ngp / kFfRows;
  const int cb = n / kFfCols, c = n % kFfCols;
  const int count = blocks_per_freq * w.n_splits;
  Comp sx, sy;
  for (int q = lane; q < count; q += 32) {
    const int rb = f * blocks_per_freq + q / w.n_splits, s = q % w.n_splits;
    const size_t pidx = ((size_t)rb * w.n_col_blocks + cb) * w.n_splits + s;
    const double2 v = w.partial[pidx * kFfCols + c];
    sx.add(v.x);
    sy.add(v.y);
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

}  // namespace

int ff_fp64_blocks_per_sm() {
  int n = 0;
  cudaFuncSetAttribute(ff_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(FfSmem));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ff_fp64_kernel, kFfThreads, sizeof(FfSmem));
  return n > 0 ? n : 1;
}

cudaError_t launch_ff_fp64(const FfDev& p, const FfWork& w, int grid, cudaStream_t s) {
  cudaError_t e =
      cudaFuncSetAttribute(ff_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, sizeof(FfSmem));
  if (e != cudaSuccess) return e;
  ff_fp64_kernel<<<grid, kFfThreads, sizeof(FfSmem), s>>>(p, w);
  return cudaGetLastError();
}

cudaError_t launch_ff_reduce(const FfDev& p, const FfWork& w, double2* schdt, cudaStream_t s) {
  const int warps = p.nb * p.nf;
  const int threads = 256;
  const int blocks = (warps * 32 + threads - 1) / threads;
  ff_reduce_kernel<<<blocks, threads, 0, s>>>(p, w, schdt);
  return cudaGetLastError();
}

}  // namespace sigma
