// FF schDt contraction on tcgen05 tensor cores with split BF16 operands.
#pragma once

#include <vector>

#include <cuda_bf16.h>

#include "ff_internal.cuh"
#include "sigma_tma.cuh"

namespace sigma {

constexpr int kOzKTile = 32;    // K elements per staged tile (one 64-byte swizzle row)
constexpr int kOzRows = 128;    // complex rows (ifreq, my_igp) per tile, frequencies flattened
constexpr int kOzCols = 64;     // complex bands per tile

// Operands in the shared-memory image the tensor cores read (K-major,
// 128-byte swizzle).  The complex product is one real product with the real
// and imaginary parts laid along K:
//   A'[R][k']   = Re I_epsR[R][k]          (k' <  K)   Im I_epsR[R][k]  (k' >= K)
//   B'[n][k']   = Re aqsn[n][k], -Im ...   (rows 0..63: real part of the product)
//   B'[64+n][k']= Im aqsn[n][k],  Re ...   (rows 64..127: imaginary part)
// so C'[R][n] = Re tempz and C'[R][64+n] = Im tempz sit in one TMEM lane.
// One 24 KB block per (row block, K' tile) holds three 8 KB BF16 slices.
struct OzakiPrep {
  unsigned char* a_tiles;   // [n_row_blocks][2*kt][3][128][32] bf16
  unsigned char* b_tiles;   // [n_col_blocks][2*kt][3][128][32] bf16
  int kt;                   // K tiles per real/imaginary half (ncouls padded to 32)
  int n_row_blocks;         // ceil(nfreq * ngpown / 128)
  int n_col_blocks;         // ceil(number_bands / 64)
  int n_splits, split_tiles;  // K' split into n_splits ranges of split_tiles tiles
  // Work entries, the K split slowest: each is one row block's tiles within
  // one split that can hold nonzero A values (row blocks whose rows are zero
  // past some K have fewer); items are entries x band blocks.
  int n_entries, n_items;
  int max_pieces;           // entries per row block at most (partial slots)
  const int4* entries;      // [n_entries]: row block, piece, first K' tile, tiles
  const int* pieces;        // [n_row_blocks]: entries of each row block
  const int* kt_lim;        // [n_row_blocks]: K tiles (per half) that can be nonzero
  int max_seg;              // frequencies one row block can touch
  double2* partial;         // [row block][col block][piece][max_seg][64]
  // Epilogue factors, formed per execution: wtab[g][n] = aqsm[n][igp(g)] *
  // column weight, in FP32 (0 for a skipped column or a padded band), so a
  // drain lane reads its row's 64 factors as contiguous 16-byte loads.
  float2* wtab;             // [ng][nb_pad]
  int ng, nb_pad;
  // Optional second output (FfDev::vcoul2 set): the same contraction with
  // the extra column factor stab[g] = vfac2 * vcoul2[igp(g)] in FP32, summed
  // into partial2 by the same epilogue.  stab points at stab_buf then.
  float* stab;
  float* stab_buf;          // [ng]
  double2* partial2;
};

constexpr uint32_t kOzSliceBytes = 128 * kOzKTile * 2;  // one BF16 slice of a 128-row K tile, 8 KB
constexpr uint32_t kOzOperandBytes = 3 * kOzSliceBytes;  // the three slices, 24 KB

// x = s1 + s2 + s3 exactly, each a BF16 value (8 significant bits).
__device__ __forceinline__ void oz_split3(float x, unsigned short& a, unsigned short& b,
                                          unsigned short& c) {
  const __nv_bfloat16 s1 = __float2bfloat16_rn(x);
  const float t1 = x - __bfloat162float(s1);
  const __nv_bfloat16 s2 = __float2bfloat16_rn(t1);
  const float t2 = t1 - __bfloat162float(s2);
  const __nv_bfloat16 s3 = __float2bfloat16_rn(t2);
  a = __bfloat16_as_ushort(s1);
  b = __bfloat16_as_ushort(s2);
  c = __bfloat16_as_ushort(s3);
}

// Slices of 8 consecutive K values of one row: three 16-byte chunks (one
// per slice tile of a 24 KB block).  Two values per paired conversion
// (cvt.rn.bf16x2.f32 rounds each as __float2bfloat16_rn does, so the slices
// are those of oz_split3), the pairs already packed.
struct OzChunk {
  uint4 s[3];
};
__device__ __forceinline__ OzChunk oz_slice_chunk(const float (&v)[8]) {
  uint32_t sl[3][4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const __nv_bfloat162 h1 = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
    const float2 f1 = __bfloat1622float2(h1);
    const float r0 = v[2 * j] - f1.x, r1 = v[2 * j + 1] - f1.y;  // exact
    const __nv_bfloat162 h2 = __floats2bfloat162_rn(r0, r1);
    const float2 f2 = __bfloat1622float2(h2);
    const __nv_bfloat162 h3 = __floats2bfloat162_rn(r0 - f2.x, r1 - f2.y);
    sl[0][j] = *reinterpret_cast<const uint32_t*>(&h1);
    sl[1][j] = *reinterpret_cast<const uint32_t*>(&h2);
    sl[2][j] = *reinterpret_cast<const uint32_t*>(&h3);
  }
  OzChunk c;
#pragma unroll
  for (int s = 0; s < 3; ++s) c.s[s] = make_uint4(sl[s][0], sl[s][1], sl[s][2], sl[s][3]);
  return c;
}
// The slices of -v: each slice negated (round to nearest even is symmetric).
__device__ __forceinline__ OzChunk oz_negate_chunk(const OzChunk& c) {
  OzChunk n;
#pragma unroll
  for (int s = 0; s < 3; ++s)
    n.s[s] = make_uint4(c.s[s].x ^ 0x80008000u, c.s[s].y ^ 0x80008000u, c.s[s].z ^ 0x80008000u,
                        c.s[s].w ^ 0x80008000u);
  return n;
}
__device__ __forceinline__ void oz_store_chunk(unsigned char* blk, int r, int ch, const OzChunk& c) {
#pragma unroll
  for (int s = 0; s < 3; ++s)
    *reinterpret_cast<uint4*>(blk + s * kOzSliceBytes + tma::sw64_offset(r, ch * 8)) = c.s[s];
}
__device__ __forceinline__ void oz_put_row_chunk(unsigned char* blk, int r, int ch, const float (&v)[8]) {
  oz_store_chunk(blk, r, ch, oz_slice_chunk(v));
}

// The slices of A'[R][k0 .. k0+8): real parts re (K' = k) and imaginary
// parts im (K' = ncouls_padded + k); k0 a multiple of 8.  A producer of FP32
// A rows writes these instead of the operand the slicing pre-pass reads.
__device__ __forceinline__ void oz_put_a(const OzakiPrep& oz, int R, int k0, const float (&re)[8],
                                         const float (&im)[8]);

// Work sizing and buffers of the split-BF16 form (partials + slices).
// row_kend (nullable, [nfreq * ngpown]): the A row's entries at K >= row_kend
// are zero, so the tiles past its row block's largest value are skipped.
// The entry tables (host copies) are uploaded by ozaki_upload_tables.
struct OzakiTables {
  std::vector<int4> entries;
  std::vector<int> pieces, kt_lim;
};
// split_tiles_hint > 0 sets the K' tiles per split (a group sizes every
// job's items alike); otherwise about items_per_cta (0: 20) items per CTA
// of `grid`.
void ozaki_size(OzakiPrep& oz, const FfDev& d, int grid, const int* row_kend = nullptr,
                OzakiTables* tables = nullptr, int split_tiles_hint = 0, int items_per_cta = 0);
cudaError_t ozaki_upload_tables(const OzakiPrep& oz, const OzakiTables& t);
int ozaki_max_segments();
size_t ozaki_prep_bytes(const OzakiPrep& oz);  // slice images + partials
size_t ozaki_tile_bytes(const OzakiPrep& oz);   // slice images (1024-aligned inside)
size_t ozaki_partial_bytes(const OzakiPrep& oz);
void ozaki_prep_bind(OzakiPrep& oz, void* base);
// Slice images and partials in separate buffers (images may be a workspace
// shared by plans that run one after another on one stream).
void ozaki_bind(OzakiPrep& oz, void* tiles, void* partial);
// with_a = false keeps the A slices already in the workspace
cudaError_t launch_ozaki_prep(const FfDev& d, const OzakiPrep& oz, cudaStream_t s, bool with_a = true);
// Zero slices of A rows [rows, n_row_blocks * 128): the rows past nf * ngpown
// that a producer of A rows leaves unwritten.
cudaError_t launch_ozaki_zero_rows(const OzakiPrep& oz, int rows, cudaStream_t s);
cudaError_t launch_ozaki_gemm(const FfDev& d, const FfWork& w, const OzakiPrep& oz, int grid,
                              cudaStream_t s);
cudaError_t launch_ozaki_reduce(const FfDev& d, const OzakiPrep& oz, double2* schdt, cudaStream_t s,
                                double2* schdt2 = nullptr);

// A group of contractions run as one launch per stage (the batched tensor
// form): each job is one contraction with its own operands, layout and
// partial buffers; the GEMM's items of every job are listed in one table,
// the reduction splits its warps among the jobs.  The jobs' operands (A and
// B slices, epilogue factors) are written by the caller's producer pass.
struct OzGroupJob {
  FfDev d;
  OzakiPrep oz;
  double2* out;            // [nb][nf] (reduction output)
  int r_warp_off;          // first warp of the reduction stage (nb * nf warps)
};
struct OzGroup {
  const OzGroupJob* jobs;  // device array
  int n_jobs;
  const int4* items;       // [total]: job, row block << 16 | band block, first K' tile, tiles | piece << 16
  int total;
  int r_warps;
  int outs, segs;          // epilogue staging: outputs per job (1 or 2), max_seg over the jobs
  int* status;
};
// Host side of a group: the item table of job `job` appended to `items`
// (its entries in the order of ozaki_size, band blocks fastest).
void ozaki_group_items(int job, const OzakiPrep& oz, const OzakiTables& t, std::vector<int4>& items);
cudaError_t launch_ozaki_group_gemm(const OzGroup& g, int grid, cudaStream_t s);
cudaError_t launch_ozaki_group_reduce(const OzGroup& g, cudaStream_t s);

__device__ __forceinline__ void oz_put_a(const OzakiPrep& oz, int R, int k0, const float (&re)[8],
                                         const float (&im)[8]) {
  const int rb = R / kOzRows, r = R % kOzRows, kt = k0 / kOzKTile, ch = (k0 % kOzKTile) / 8;
  unsigned char* base = oz.a_tiles + (size_t)rb * 2 * oz.kt * kOzOperandBytes;
  oz_put_row_chunk(base + (size_t)kt * kOzOperandBytes, r, ch, re);
  oz_put_row_chunk(base + (size_t)(oz.kt + kt) * kOzOperandBytes, r, ch, im);
}

// B' rows: [Re | -Im] (real part of the product) and [Im | Re] (imaginary
// part); element t of oz_prep_b_count: one (band block, K tile, band, 8-value
// chunk) of aqsn rounded to FP32 and written as slices.
__device__ __forceinline__ long long oz_prep_b_count(const OzakiPrep& oz) {
  return (long long)oz.n_col_blocks * oz.kt * 64 * (kOzKTile / 8);
}
__device__ __forceinline__ void oz_prep_b_elem(const FfDev& p, const OzakiPrep& oz, long long t) {
  constexpr int kChunks = kOzKTile / 8;
  const int ch = (int)(t % kChunks);
  const int nl = (int)((t / kChunks) & 63);
  const long long rest = t / (kChunks * 64);
  const int kt = (int)(rest % oz.kt);
  const int cb = (int)(rest / oz.kt);
  const int n = cb * kOzCols + nl;
  const int k0 = kt * kOzKTile + ch * 8;
  float re[8], im[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int k = k0 + j;
    const double2 v = (n < p.nb && k < p.nc) ? p.aqsn[(size_t)n * p.nc + k] : make_double2(0.0, 0.0);
    re[j] = __double2float_rn(v.x);
    im[j] = __double2float_rn(v.y);
  }
  unsigned char* base = oz.b_tiles + (size_t)cb * 2 * oz.kt * kOzOperandBytes;
  unsigned char* lo = base + (size_t)kt * kOzOperandBytes;            // K' < K: real parts of aqsn
  unsigned char* hi = base + (size_t)(oz.kt + kt) * kOzOperandBytes;  // K' >= K: imaginary parts
  const OzChunk cre = oz_slice_chunk(re), cim = oz_slice_chunk(im);
  oz_store_chunk(lo, nl, ch, cre);
  oz_store_chunk(lo, 64 + nl, ch, cim);
  oz_store_chunk(hi, nl, ch, oz_negate_chunk(cim));
  oz_store_chunk(hi, 64 + nl, ch, cre);
}

// Epilogue factors, element t of oz_weights_count: wtab[g][n] = aqsm[n][igp(g)]
// * weight(g), rounded to FP32 from the FP64 product.
__device__ __forceinline__ long long oz_weights_count(const OzakiPrep& oz) {
  return (long long)oz.ng * oz.nb_pad;
}
__device__ __forceinline__ void oz_weights_elem(const FfDev& p, const OzakiPrep& oz, long long t) {
  const int g = (int)(t / oz.nb_pad), n = (int)(t % oz.nb_pad);
  const int igp = p.igp_of[g];
  float2 v = make_float2(0.f, 0.f);
  if (igp >= 0 && n < p.nb) {
    const double wgt = ff_column_weight(p, igp);
    const double2 md = p.aqsm[(size_t)n * p.nc + igp];
    v = make_float2(__double2float_rn(md.x * wgt), __double2float_rn(md.y * wgt));
  }
  oz.wtab[t] = v;
  if (oz.stab && n == 0) oz.stab[g] = igp >= 0 ? (float)(p.vfac2 * p.vcoul2[igp]) : 0.f;
}

}  // namespace sigma
