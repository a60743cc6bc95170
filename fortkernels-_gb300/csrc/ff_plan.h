// Internal entry points of the FF plan shared with the static remainders.
#pragma once

#include <vector>

#include <cuda_runtime.h>

#include "sigma_ff.h"

namespace sigma {

// Plan over an already validated column map (igp_of[my_igp] in [0, ncouls),
// or -1 for a column left out of every sum).
// shared_tiles (split-BF16 form only): a workspace of at least
// ff_plan_tile_bytes() holding the slice images instead of the plan's own
// allocation, for plans that run one after another on one stream.
// row_kend (split-BF16 form only, nullable): per I_epsR row (ifreq * ngpown
// + my_igp) the K from which the row is zero in every execution; the
// contraction skips those K tiles.
// split_tiles_hint (split-BF16 form, > 0): K' tiles per work split, so
// that the plans of a group have items of about the same size; otherwise
// items_per_cta (> 0; default 20) GEMM items per resident CTA.
int ff_plan_build(sigma_ff_plan* out, int number_bands, int ncouls, int ngpown, int nfreq,
                  const std::vector<int>& igp_of, int mode, void* shared_tiles = nullptr,
                  const int* row_kend = nullptr, int split_tiles_hint = 0, int items_per_cta = 0);
int ff_plan_tile_bytes(int number_bands, int ncouls, int ngpown, int nfreq, size_t* bytes);

// The split-BF16 plan's operand layout (slice images, K tiles, row limits),
// for kernels that write the A slices themselves and then execute with
// reuse_a; nullptr for an FP64 plan.
struct OzakiPrep;
const OzakiPrep* ff_plan_ozaki(sigma_ff_plan plan);
// The plan's device view (shape, column map; operand pointers unset).
struct FfDev;
const FfDev* ff_plan_dev(sigma_ff_plan plan);

// sigma_ff_execute with the column weight vfac * vcoul[igp] (vcoul a device
// array, or nullptr for weight 1).
// With epsr32 set (split-BF16 form only) the contraction reads that FP32
// operand [nf][ng][nc] instead of I_epsR (which may then be NULL).  With
// reuse_a (split-BF16 form only) it contracts the operand slices the
// previous execution left in the plan's slice workspace (the same operand
// again, no other plan on that workspace in between); I_epsR and epsr32 are
// then not read.
// With out2 and vcoul2 set (vcoul then NULL) the same contraction also
// yields out2, the sum with the extra column factor vfac2 * vcoul2[igp]: one
// tensor-core pass with a second epilogue reduction (the FP64 form
// contracts twice).
int ff_execute_weighted(sigma_ff_plan plan, const sigma_complex128* I_epsR,
                        const sigma_complex128* aqsntemp, const sigma_complex128* aqsmtemp,
                        const double* vcoul, double vfac, sigma_complex128* schDt_matrix,
                        void* stream, const float2* epsr32 = nullptr, bool reuse_a = false,
                        const double* vcoul2 = nullptr, double vfac2 = 1.0,
                        sigma_complex128* out2 = nullptr, bool operands_ready = false);

}  // namespace sigma
