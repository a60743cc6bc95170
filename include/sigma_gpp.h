/* sigma_gpp.h - GPP (generalized plasmon-pole) sigma sum on GB300.
 *
 * Computes, for bands n1 in [0, number_bands), columns my_igp in [0, ngpown)
 * (igp = indinv[inv_igp_index[my_igp]], clamped to ncouls-1 when the index is
 * ncouls, column skipped when igp < 0 or igp > ncouls), g-vectors ig in
 * [0, ncouls) and the three frequencies iw:
 *
 *   wdiff  = wx[iw] - wtilde[my_igp][ig]
 *   delw   = wtilde * conj(wdiff) / |wdiff|^2
 *   scha   = conj(aqsm[n1][igp]) * aqsn[n1][ig] * delw * I_eps[my_igp][ig]
 *            kept when |wdiff|^2 > 0.25 and |delw|^2 < 1/(4e-6)   (pole guard)
 *   achtemp[iw]     += 0.5 * vcoul[igp] * sum_ig scha
 *   acht_n1_loc[n1] += 0.5 * vcoul[igp] * sum_ig scha(iw = 2)
 *   asxtemp[iw]     += occ * vcoul[igp] * sum_ig ssxa        (bands n1 < nvband)
 *
 * with ssxa the occupied-band screened-exchange term of ssxt_scht_solver.
 * Reference: BGW-Kernels/gppKer.cpp:19-65 (ssxt_scht_solver), :130-159
 * (flagOCC_solver), :303-439 (band loop, hot loop :387-413, epilogue
 * :416-424, reduction :431-439), index map :322-328, frequencies :310-314.
 *
 * Outputs are overwritten, not accumulated (the reference zero-initialises
 * them, :222-232, :255).  wx_array holds the caller's frequencies: three per
 * band with stride wx_band_stride, or stride 0 for one set shared by every
 * band (the mini-app's case: e_n1kq is one constant, :201, :312).
 *
 * Arrays (row-major, interleaved complex128):
 *   aqsmtemp, aqsntemp          [number_bands][ncouls]
 *   I_eps_array, wtilde_array   [ngpown][ncouls]
 *   vcoul                       [ncouls]
 *   inv_igp_index               [ngpown]
 *   indinv                      [indinv_len]  (>= ncouls; indinv[ncouls] is never read)
 *   achtemp, asxtemp            [3]
 *   acht_n1_loc                 [number_bands]  (may be NULL)
 */
#ifndef SIGMA_GPP_H
#define SIGMA_GPP_H

#include "sigma_common.h"
#include "sigma_ff.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------------
 * Host-pointer drop-in.  Takes the arrays gppKer.cpp builds in main()
 * (BGW-Kernels/gppKer.cpp:222-299) and replaces its loop nest :303-439 with
 * one call.  The library copies the inputs into its cached device buffers,
 * runs the kernels on `stream` (NULL: the legacy default stream) and copies
 * the outputs back; it returns after the stream has drained.  The FP64 form
 * copies on an internal stream ordered after the work already queued on
 * `stream`, in pieces that the sum waits for one by one, so the copies
 * overlap the sum; the other forms copy on `stream` first.  indinv has
 * ncouls entries, as in the reference; wx_array has 3 entries shared by every
 * band.  Host buffers in pinned memory copy fastest.
 *
 * State: the drop-ins keep ONE cached plan (the last shape, index maps and
 * form), one input arena and one copy stream with its gate words per
 * process, for the device that was current at the last call.  Calls are
 * serialised by a library mutex.  A call on another device, or with another
 * shape or form, drops that state and builds it anew (a plan costs a few
 * milliseconds and device allocations), so a process that alternates
 * between devices or shapes re-plans on every call: use one process per
 * device (the replica layout), or the plan API (sigma_gpp_plan_create /
 * sigma_gpp_execute), which keeps one plan per shape and device.
 * sigma_shutdown() frees the cached state.
 * ------------------------------------------------------------------------- */
int sigma_gpp_fp64(int number_bands, int nvband, int ncouls, int ngpown, int nstart, int nend,
                   const int* inv_igp_index, const int* indinv, const double* wx_array,
                   double occ, const sigma_complex128* aqsmtemp,
                   const sigma_complex128* aqsntemp, const sigma_complex128* I_eps_array,
                   const sigma_complex128* wtilde_array, const double* vcoul,
                   sigma_complex128* achtemp, sigma_complex128* asxtemp,
                   sigma_complex128* acht_n1_loc, void* stream);

/* Same contract; FP32 bulk arithmetic with the pole-guard decisions taken as
 * the FP64 path takes them and compensated FP64 reductions.  Every output is
 * within 1e-6 relative of the FP64 result on the production value ranges. */
int sigma_gpp_mixed(int number_bands, int nvband, int ncouls, int ngpown, int nstart, int nend,
                    const int* inv_igp_index, const int* indinv, const double* wx_array,
                    double occ, const sigma_complex128* aqsmtemp,
                    const sigma_complex128* aqsntemp, const sigma_complex128* I_eps_array,
                    const sigma_complex128* wtilde_array, const double* vcoul,
                    sigma_complex128* achtemp, sigma_complex128* asxtemp,
                    sigma_complex128* acht_n1_loc, void* stream);

/* sigma_gpp_mixed with its error reported: when rel_err_out (double[6]) is
 * not NULL, the FP64 form also runs on the same inputs and
 *   rel_err_out[iw]     = |achtemp[iw] - achtemp_fp64[iw]| / |achtemp_fp64[iw]|
 *   rel_err_out[3 + iw] = the same for asxtemp (0 where both are 0),
 * the mixed outputs being the ones returned.  The check costs one FP64
 * evaluation (about 90 times the mixed one at the production shape), so it
 * is a validation mode.  sigma_gpp_mixed keeps the argument list of
 * sigma_gpp_fp64 (no extra argument) so that the two are interchangeable
 * where the reference's loop is replaced (BGW-Kernels/gppKer.cpp:303-439). */
int sigma_gpp_mixed_checked(int number_bands, int nvband, int ncouls, int ngpown, int nstart, int nend,
                            const int* inv_igp_index, const int* indinv, const double* wx_array,
                            double occ, const sigma_complex128* aqsmtemp,
                            const sigma_complex128* aqsntemp, const sigma_complex128* I_eps_array,
                            const sigma_complex128* wtilde_array, const double* vcoul,
                            sigma_complex128* achtemp, sigma_complex128* asxtemp,
                            sigma_complex128* acht_n1_loc, void* stream, double* rel_err_out);

/* Same contract, tensor-core form (SIGMA_PREC_TENSOR): one frequency set for
 * every band (wx_array[3]); the band sum runs as a complex GEMM on tcgen05
 * tensor cores with split-BF16 operands.  ngpown must be at least ~18 (the
 * contraction tiles hold at most 8 frequency segments; smaller returns
 * SIGMA_ERR_UNSUPPORTED). */
int sigma_gpp_tensor(int number_bands, int nvband, int ncouls, int ngpown, int nstart, int nend,
                     const int* inv_igp_index, const int* indinv, const double* wx_array,
                     double occ, const sigma_complex128* aqsmtemp,
                     const sigma_complex128* aqsntemp, const sigma_complex128* I_eps_array,
                     const sigma_complex128* wtilde_array, const double* vcoul,
                     sigma_complex128* achtemp, sigma_complex128* asxtemp,
                     sigma_complex128* acht_n1_loc, void* stream);

/* ---------------------------------------------------------------------------
 * Device-resident path.  A plan validates the index maps on the host (where
 * the reference would read out of bounds it returns SIGMA_ERR_INDEX_RANGE),
 * uploads the column map and owns the partial-sum buffers; executing it is
 * asynchronous on `stream`, allocates nothing and can be captured in a CUDA
 * graph.  Inputs and outputs of sigma_gpp_execute are device pointers.
 * One plan may be executed by one stream at a time (its partial buffers are
 * reused by every execution).
 * ------------------------------------------------------------------------- */
typedef struct sigma_gpp_plan_s* sigma_gpp_plan;

int sigma_gpp_plan_create(sigma_gpp_plan* plan, int number_bands, int nvband, int ncouls,
                          int ngpown, int nstart, int nend, const int* inv_igp_index,
                          const int* indinv, int indinv_len, int precision);

int sigma_gpp_execute(sigma_gpp_plan plan, const double* wx_array, int wx_band_stride, double occ,
                      const sigma_complex128* aqsmtemp, const sigma_complex128* aqsntemp,
                      const sigma_complex128* I_eps_array, const sigma_complex128* wtilde_array,
                      const double* vcoul, sigma_complex128* achtemp, sigma_complex128* asxtemp,
                      sigma_complex128* acht_n1_loc, void* stream);

int sigma_gpp_plan_destroy(sigma_gpp_plan plan);

/* Waits for `stream` and returns the device-side status of the plan's last
 * execution: SIGMA_OK, or SIGMA_ERR_TIMEOUT when a bounded wait inside a
 * kernel gave up (results of that execution are then not valid). */
int sigma_gpp_plan_status(sigma_gpp_plan plan, void* stream);

/* Self-test of the device-side bounded wait (no counterpart in the
 * reference, whose loops never wait on the device).  Runs the FP64 plan's
 * shared-frequency main pass on the given device arrays the way the host
 * drop-in runs it beside its copies, but with gate words that nothing ever
 * writes and each wait bounded by `wait_polls` polls (256 ns apart), then
 * waits for `stream` and returns the device status: SIGMA_ERR_TIMEOUT when
 * the waits gave up as designed (the kernel drops its items and returns; the
 * CUDA context stays usable).  The next sigma_gpp_execute of the plan, or the
 * next host drop-in call, starts from a cleared status.  FP64 plans with one
 * frequency set only (SIGMA_ERR_UNSUPPORTED otherwise). */
int sigma_gpp_selftest_gate_timeout(sigma_gpp_plan plan, const double* wx_array,
                                    const sigma_complex128* aqsmtemp, const sigma_complex128* aqsntemp,
                                    const sigma_complex128* I_eps_array,
                                    const sigma_complex128* wtilde_array, const double* vcoul,
                                    int wait_polls, void* stream);

/* Per-launch timing, the device-side counterpart of the reference's chrono
 * timer around its band loop (BGW-Kernels/gppKer.cpp:301, 441).  While
 * enabled, each execution records CUDA events on its stream around the main
 * (all-band) kernel, the occupied-band kernel and the remaining launches
 * (pre-pass, reductions); up to 256 executions are kept.  sigma_gpp_plan_timing
 * waits for them, returns the summed milliseconds of each part and the number
 * of kernels one execution launches, and clears the record. */
int sigma_gpp_plan_set_timing(sigma_gpp_plan plan, int enable);
int sigma_gpp_plan_timing(sigma_gpp_plan plan, int* executions, double* main_ms,
                          double* occupied_ms, double* other_ms, int* launches_per_execution);

/* Number of valid columns (my_igp whose igp survives the reference's range
 * test) and of terms number_bands * valid_columns * ncouls * 3. */
int sigma_gpp_plan_info(sigma_gpp_plan plan, int* valid_columns, long long* terms);

/* ---------------------------------------------------------------------------
 * Batched evaluation: many sigma instances (q-points, band windows) of
 * different number_bands / ncouls / ngpown / nvband at once.  The reference
 * evaluates one instance per run of its driver; here every instance's work
 * items go into one device work queue per pass, drained by one persistent
 * kernel (main pass, then occupied-band pass), with per-instance pre-passes
 * and reductions around them.  The whole sequence can be captured once into
 * a CUDA graph and replayed.
 * ------------------------------------------------------------------------- */
typedef struct sigma_gpp_instance {
  int number_bands, nvband, ncouls, ngpown;
  const int* inv_igp_index;        /* host [ngpown] */
  const int* indinv;               /* host [ncouls] */
  const double* wx_array;          /* device: [3], or [number_bands][wx_band_stride] */
  int wx_band_stride;
  double occ;
  const sigma_complex128* aqsmtemp;      /* device [number_bands][ncouls] */
  const sigma_complex128* aqsntemp;      /* device [number_bands][ncouls] */
  const sigma_complex128* I_eps_array;   /* device [ngpown][ncouls] */
  const sigma_complex128* wtilde_array;  /* device [ngpown][ncouls] */
  const double* vcoul;                   /* device [ncouls] */
  sigma_complex128* achtemp;             /* device out [3] */
  sigma_complex128* asxtemp;             /* device out [3] */
  sigma_complex128* acht_n1_loc;         /* device out [number_bands], may be NULL */
} sigma_gpp_instance;

typedef struct sigma_gpp_batch_s* sigma_gpp_batch;

/* Validates every instance like sigma_gpp_plan_create and sizes the queues.
 * tile_shape (may be NULL) picks the FP64 main-pass tile per instance, -1
 * for the library's choice (least padding).  A batch whose instances all
 * share one frequency set per instance (wx_band_stride 0) runs the
 * shared-frequency kernel: tiles 3 = 64 bands x 32 columns, 4 = 32 x 64,
 * 5 = 32 x 32, 6 = 64 x 16 (5 and 6: two CTAs per SM when every instance
 * takes one of them); otherwise the per-band kernel: 0 = 32 x 32,
 * 1 = 16 x 64, 2 = 64 x 16.  A tile of the other family is
 * SIGMA_ERR_UNSUPPORTED.  The tuning table of fortkernels-_gb300/autotune.py
 * chooses per shape class.  The mixed form has one tile shape.  precision
 * SIGMA_PREC_TENSOR needs one frequency set per instance and ngpown >= ~18
 * (SIGMA_ERR_UNSUPPORTED otherwise); with at most 8 occupied bands per
 * instance every stage is one launch for all instances (the split-BF16
 * GEMM over one work table listing every instance's items), each instance
 * keeping its own slice images (about 36 B per column and g-vector plus
 * 24 B per band and g-vector of device memory); otherwise each instance's
 * contraction runs in stream order over one shared workspace.  Every form
 * reduces all instances with two launches. */
int sigma_gpp_batch_create(sigma_gpp_batch* batch, int n_instances, const sigma_gpp_instance* inst,
                           int precision, const int* tile_shape);

/* sigma_gpp_batch_create with the work sizing given (0 for the default of
 * each): items_per_cta, the FP64 and mixed main pass's work items per
 * resident CTA (each item a band block x column block x g-vector split;
 * default 16), and tensor_split_tiles, the tensor form's contraction items'
 * length in K tiles of 32 g-vectors (real and imaginary halves counted
 * apart), the same for every instance (default: each instance's items
 * sized as its single-instance plan's, about 20 per CTA).  Results do not
 * depend on items_per_cta beyond the order of the g-vector sums; the tensor
 * form's error depends on tensor_split_tiles through where its K splits
 * fall.  fortkernels-_gb300/autotune.py tunes both with the tile shapes. */
int sigma_gpp_batch_create_tuned(sigma_gpp_batch* batch, int n_instances, const sigma_gpp_instance* inst,
                                 int precision, const int* tile_shape, int items_per_cta,
                                 int tensor_split_tiles);

/* Launches the batch on `stream` (asynchronous; allocates nothing). */
int sigma_gpp_batch_execute(sigma_gpp_batch batch, void* stream);

/* First call captures sigma_gpp_batch_execute into a CUDA graph on `stream`
 * (which must not be the legacy NULL stream); every call launches the graph. */
int sigma_gpp_batch_launch_graph(sigma_gpp_batch batch, void* stream);

/* Terms of the whole batch, work items of the main pass, kernels per execution. */
int sigma_gpp_batch_info(sigma_gpp_batch batch, long long* terms, int* items, int* launches);

/* Waits for `stream`; SIGMA_OK or SIGMA_ERR_TIMEOUT from a bounded device wait. */
int sigma_gpp_batch_status(sigma_gpp_batch batch, void* stream);

int sigma_gpp_batch_destroy(sigma_gpp_batch batch);

/* One-shot form: create, execute, wait, destroy. */
int sigma_gpp_batched(int n_instances, const sigma_gpp_instance* inst, int precision, void* stream);

/* ---------------------------------------------------------------------------
 * FP64 evaluation that allocates nothing.  This entry point has no
 * counterpart in the reference; it exists for callers that cannot allocate
 * GPU memory: code inside a framework whose memory pool owns the device, a
 * plug-in in a process that forbids allocation after start-up, or a
 * real-time loop where an allocation could stall.
 *
 * Same result as sigma_gpp_execute with an FP64 plan (within 1e-12 relative;
 * the g-vector split differs), same arrays, all device pointers except the
 * host index maps (indinv with ncouls entries; wx_array: 3 device doubles
 * shared by every band).  Its scratch (item counters, column map, partial
 * sums) is one fixed 32 MiB __device__ array inside the library, held by
 * every GPU that loads the library until the process exits; the call makes
 * no cudaMalloc, cudaFree or other allocation.
 *   - Limits: ngpown <= 65536, and the partial sums of the problem must fit
 *     the 32 MiB (the production shape 512 x 1638 x 32768 uses ~17 MB);
 *     larger problems return SIGMA_ERR_WORKSPACE with a message in
 *     sigma_last_error_message().
 *   - The first call on a device looks up the array's device address
 *     (cudaGetSymbolAddress).
 *   - A call on a stream that is being captured into a CUDA graph returns
 *     SIGMA_ERR_UNSUPPORTED and queues nothing: the column map is copied
 *     from a reused host buffer and the scratch is shared, so a captured
 *     call could not be replayed.
 *   - Every call shares the one array.  Calls that overlap on the GPU (on
 *     different streams, or from threads that do not wait for each other's
 *     stream) race on it and give wrong results; serialise them.
 *   - The column map is copied from pageable host memory, so the call may
 *     wait for work already queued on `stream`.
 * Asynchronous on `stream` otherwise; outputs are valid once it drains.
 * ------------------------------------------------------------------------- */
int sigma_gpp_fp64_noalloc(int number_bands, int nvband, int ncouls, int ngpown,
                           const int* inv_igp_index, const int* indinv, const double* wx_array,
                           double occ, const sigma_complex128* aqsmtemp,
                           const sigma_complex128* aqsntemp, const sigma_complex128* I_eps_array,
                           const sigma_complex128* wtilde_array, const double* vcoul,
                           sigma_complex128* achtemp, sigma_complex128* asxtemp,
                           sigma_complex128* acht_n1_loc, void* stream);

/* ---------------------------------------------------------------------------
 * Static remainder of the GPP sum (the exact static COH term):
 *
 *   achstemp_n1[n1] = sum_{my_igp} -0.5 vcoul[igp] conj(aqsm[n1][igp])
 *                       * sum_{ig} aqsn[n1][ig] I_eps[my_igp][ig]
 *   achstemp = sum_{n1} achstemp_n1[n1]
 *
 * Replaces reduce_achstemp (BGW-Kernels/gppKer.cpp:67-128), called there
 * once per band inside the band loop (:308).  The formula is the Fortran
 * kernel's (gppkernel.deslippe.09.30.2014.f90:195-228); the C++ function
 * reads the single element I_eps[my_igp][igp] instead of the g-vector sum,
 * never resets schstemp between columns, and discards its result.  Index map
 * and skipped columns as sigma_gpp_fp64 (BGW-Kernels/gppKer.cpp:322-328).
 * The sums are one complex GEMM (bands x columns x g-vectors) with the
 * conj(aqsm) vcoul reduction fused, run in either form of the FF
 * contraction: mode SIGMA_FF_FP64 or SIGMA_FF_OZAKI_BF16 (sigma_ff.h).
 *
 * Host pointers: aqsmtemp / aqsntemp [number_bands][ncouls], I_eps_array
 * [ngpown][ncouls], vcoul [ncouls]; achstemp [1] and achstemp_n1
 * [number_bands] (may be NULL) are written.  Returns after `stream` drains.
 * ------------------------------------------------------------------------- */
int sigma_gpp_achstemp(int number_bands, int ncouls, int ngpown, const int* inv_igp_index,
                       const int* indinv, const sigma_complex128* aqsmtemp,
                       const sigma_complex128* aqsntemp, const sigma_complex128* I_eps_array,
                       const double* vcoul, sigma_complex128* achstemp,
                       sigma_complex128* achstemp_n1, int mode, void* stream);

/* Device-resident form: a plan of the contraction (an FF plan with one
 * frequency and the GPP column map; destroy it with sigma_ff_plan_destroy,
 * time it with sigma_ff_plan_set_timing / sigma_ff_plan_timing) and an
 * asynchronous execution on device arrays.  achstemp [1] and achstemp_n1
 * [number_bands] are device outputs (both required). */
int sigma_gpp_static_plan_create(sigma_ff_plan* plan, int number_bands, int ncouls, int ngpown,
                                 const int* inv_igp_index, const int* indinv, int mode);
int sigma_gpp_static_execute(sigma_ff_plan plan, const sigma_complex128* aqsmtemp,
                             const sigma_complex128* aqsntemp, const sigma_complex128* I_eps_array,
                             const double* vcoul, sigma_complex128* achstemp,
                             sigma_complex128* achstemp_n1, void* stream);

/* ---------------------------------------------------------------------------
 * Real-valued GPP (gppKer_real.cpp:17-155, 296-390, gppKerFort_real.f90):
 * the same sums with real arrays, one frequency set for every band
 * (wx_array[3]), FP64.  Term scha = aqsm[n1][igp] aqsn[n1][ig] delw I_eps
 * (no conjugate), delw = wtilde / (wx - wtilde), the complex path's pole
 * guard; occupied bands add ssx = Omega2 / wx^2 or -Omega2 cden delw / cden^2,
 * cden = 4 wtilde^2 (delw + 1/2).  Arrays: aqsmtemp / aqsntemp
 * [number_bands][ncouls], I_eps_array / wtilde_array [ngpown][ncouls],
 * vcoul [ncouls] (all double); outputs achtemp[3], asxtemp[3] and
 * acht_n1_loc[number_bands] (may be NULL), overwritten.  Where the
 * reference adds a stale scha[ig] for a term its guard drops (:367-371
 * write it only when kept), this path adds 0.
 * ------------------------------------------------------------------------- */
int sigma_gpp_real_fp64(int number_bands, int nvband, int ncouls, int ngpown, int nstart, int nend,
                        const int* inv_igp_index, const int* indinv, const double* wx_array,
                        double occ, const double* aqsmtemp, const double* aqsntemp,
                        const double* I_eps_array, const double* wtilde_array, const double* vcoul,
                        double* achtemp, double* asxtemp, double* acht_n1_loc, void* stream);

/* Device-resident form (device arrays, asynchronous on `stream`). */
typedef struct sigma_gpp_real_plan_s* sigma_gpp_real_plan;
int sigma_gpp_real_plan_create(sigma_gpp_real_plan* plan, int number_bands, int nvband, int ncouls,
                               int ngpown, int nstart, int nend, const int* inv_igp_index,
                               const int* indinv, int indinv_len);
int sigma_gpp_real_execute(sigma_gpp_real_plan plan, const double* wx_array, double occ,
                           const double* aqsmtemp, const double* aqsntemp, const double* I_eps_array,
                           const double* wtilde_array, const double* vcoul, double* achtemp,
                           double* asxtemp, double* acht_n1_loc, void* stream);
int sigma_gpp_real_plan_destroy(sigma_gpp_real_plan plan);

/* ---------------------------------------------------------------------------
 * gppsum = 1 ("half sum") GPP (gppKerSeq.cpp, the reference's sequential
 * driver, run as `gppKerSeq nb nvband ncouls npg 1`), FP64.  Replaces its
 * band loop :407-492 with the solvers it drives: noflagOCC_solver :193-261
 * (non-occupied bands, in 512-wide g-vector blocks :457-470),
 * flagOCC_solver :76-191 (occupied bands) and reduce_achstemp :13-72 (the
 * static remainder `achstemp`, which the reference computes and never
 * prints).  Each column my_igp sums g-vectors below its igp with the
 * Hermitian partner term; the reference's own conventions are kept: its
 * inverted pole test for the non-occupied bands (a term is kept where
 * |wdiff|^2 < 0.25 or |delw|^2 > limitone), the g-vectors its block loop
 * skips (ig mod 512 == 511 and ig == igp - 1; ig == igp alone when igp is a
 * positive multiple of 512), the occupied loop's stop at the first
 * |Omega2| < to1, and the unpaired term at ig == igp - 1.  Exact poles give
 * non-finite results, as in the reference.
 *
 * sigma_gpp_halfsum_fp64 takes host arrays in gppKerSeq.cpp's own
 * g-vector-major layout: aqsmtemp / aqsntemp [ncouls][number_bands],
 * I_eps_array / wtilde_array [ncouls][ngpown] (the reference's row-pointer
 * arrays, stored contiguously), vcoul [ncouls], wx_array [3].  Outputs are
 * overwritten: achtemp[3], asxtemp[3], acht_n1_loc[number_bands] (may be
 * NULL), achstemp[1] (may be NULL: the static remainder is then not run).
 * ------------------------------------------------------------------------- */
enum {
  SIGMA_HALFSUM_STATIC = 1,     /* plan also evaluates the static remainder achstemp */
  SIGMA_HALFSUM_GVEC_MAJOR = 2, /* execute takes gppKerSeq.cpp's [ncouls][...] layout */
  SIGMA_HALFSUM_TENSOR = 4      /* the band sums as split-BF16 tcgen05 contractions (FP32-class
                                   error, ~1e-7 relative); occupied bands stay FP64; needs
                                   ngpown of at least ~18, as sigma_gpp_tensor */
};
int sigma_gpp_halfsum_fp64(int number_bands, int nvband, int ncouls, int ngpown, int nstart,
                           int nend, const int* inv_igp_index, const int* indinv,
                           const double* wx_array, double occ, const sigma_complex128* aqsmtemp,
                           const sigma_complex128* aqsntemp, const sigma_complex128* I_eps_array,
                           const sigma_complex128* wtilde_array, const double* vcoul,
                           sigma_complex128* achtemp, sigma_complex128* asxtemp,
                           sigma_complex128* acht_n1_loc, sigma_complex128* achstemp,
                           void* stream);

/* The same with the band sums on the tensor cores (SIGMA_HALFSUM_TENSOR). */
int sigma_gpp_halfsum_tensor(int number_bands, int nvband, int ncouls, int ngpown, int nstart,
                             int nend, const int* inv_igp_index, const int* indinv,
                             const double* wx_array, double occ, const sigma_complex128* aqsmtemp,
                             const sigma_complex128* aqsntemp, const sigma_complex128* I_eps_array,
                             const sigma_complex128* wtilde_array, const double* vcoul,
                             sigma_complex128* achtemp, sigma_complex128* asxtemp,
                             sigma_complex128* acht_n1_loc, sigma_complex128* achstemp,
                             void* stream);

/* Device-resident form.  Without SIGMA_HALFSUM_GVEC_MAJOR execute takes the
 * library's band-major layout (aqsmtemp / aqsntemp [number_bands][ncouls],
 * I_eps_array / wtilde_array [ngpown][ncouls], as gppKer.cpp); with it, the
 * layout above, transposed on the device into plan-owned buffers.  achstemp
 * needs SIGMA_HALFSUM_STATIC (else SIGMA_ERR_UNSUPPORTED). */
typedef struct sigma_gpp_halfsum_plan_s* sigma_gpp_halfsum_plan;
int sigma_gpp_halfsum_plan_create(sigma_gpp_halfsum_plan* plan, int number_bands, int nvband,
                                  int ncouls, int ngpown, int nstart, int nend,
                                  const int* inv_igp_index, const int* indinv, int indinv_len,
                                  int flags);
int sigma_gpp_halfsum_execute(sigma_gpp_halfsum_plan plan, const double* wx_array, double occ,
                              const sigma_complex128* aqsmtemp, const sigma_complex128* aqsntemp,
                              const sigma_complex128* I_eps_array,
                              const sigma_complex128* wtilde_array, const double* vcoul,
                              sigma_complex128* achtemp, sigma_complex128* asxtemp,
                              sigma_complex128* acht_n1_loc, sigma_complex128* achstemp,
                              void* stream);
int sigma_gpp_halfsum_plan_destroy(sigma_gpp_halfsum_plan plan);

#ifdef __cplusplus
}
#endif

#endif /* SIGMA_GPP_H */
