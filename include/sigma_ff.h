/* sigma_ff.h - full-frequency (FF) sigma: the schDt contraction on GB300.
 *
 *   schDt[n1][ifreq] = sum_{my_igp} conj(aqsm[n1][igp])
 *                        * sum_{ig} I_epsR[ifreq][my_igp][ig] * aqsn[n1][ig]
 *   igp = indinv[inv_igp_index[my_igp]]
 *
 * This is the contraction of ffkernel.deslippe.best.f90:402-418 (a zgemm
 * tempz = I_epsR^T aqsn followed by a conj(aqsm) reduction over my_igp, kept
 * commented out in the reference) in the C layouts of FFKer_cori/ffKernel.cpp:
 * I_epsR[ifreq][my_igp][ig] (:366, :430), aqsn/aqsm[n1][ig] (:360-363, :416),
 * schDt_matrix[n1][ifreq] as achDtemp_Kernel reads it (:165).  The live
 * reference code zeroes schDt_matrix instead (FFKer_cori/ffKernel.cpp:421-422).
 * No vcoul factor, as in the source.  Every igp must lie in [0, ncouls)
 * (the reference applies no clamp here); otherwise SIGMA_ERR_INDEX_RANGE.
 *
 * Arrays (row-major, interleaved complex128):
 *   I_epsR        [nfreq][ngpown][ncouls]
 *   aqsntemp      [number_bands][ncouls]
 *   aqsmtemp      [number_bands][ncouls]
 *   schDt_matrix  [number_bands][nfreq]   (output, overwritten)
 */
#ifndef SIGMA_FF_H
#define SIGMA_FF_H

#include "sigma_common.h"

#ifdef __cplusplus
extern "C" {
#endif

enum sigma_ff_mode {
  SIGMA_FF_FP64 = 0,        /* complex FP64 GEMM on the FP64 pipe */
  SIGMA_FF_OZAKI_BF16 = 1   /* each FP64 operand rounded to FP32 and split exactly into 3 BF16
                               slices; the 6 leading slice products run on tcgen05 tensor cores
                               with FP32 accumulation in tensor memory (leading product and
                               corrections in separate accumulators); FP64 final reduction */
};

/* Host-pointer drop-in for the commented zgemm + reduction of
 * ffkernel.deslippe.best.f90:402-418: copies the inputs to the device on
 * `stream`, evaluates, copies schDt_matrix back and returns after the stream
 * has drained. */
int sigma_ff_schdt(int number_bands, int ncouls, int ngpown, int nfreq,
                   const int* inv_igp_index, const int* indinv,
                   const sigma_complex128* I_epsR, const sigma_complex128* aqsntemp,
                   const sigma_complex128* aqsmtemp, sigma_complex128* schDt_matrix, int mode,
                   void* stream);

/* Device-resident plan: validates the index maps on the host, owns the
 * partial-sum (and, for the Ozaki mode, BF16 slice) buffers.  Execution is
 * asynchronous and allocates nothing; arrays are device pointers. */
typedef struct sigma_ff_plan_s* sigma_ff_plan;

int sigma_ff_plan_create(sigma_ff_plan* plan, int number_bands, int ncouls, int ngpown, int nfreq,
                         const int* inv_igp_index, const int* indinv, int mode);
int sigma_ff_execute(sigma_ff_plan plan, const sigma_complex128* I_epsR,
                     const sigma_complex128* aqsntemp, const sigma_complex128* aqsmtemp,
                     sigma_complex128* schDt_matrix, void* stream);
int sigma_ff_plan_destroy(sigma_ff_plan plan);

/* Per-launch timing like sigma_gpp_plan_set_timing: the contraction kernel
 * (main) and everything else (slicing pre-pass, reduction). */
int sigma_ff_plan_set_timing(sigma_ff_plan plan, int enable);
int sigma_ff_plan_timing(sigma_ff_plan plan, int* executions, double* main_ms, double* other_ms,
                         int* launches_per_execution);

/* number_bands the plan was made for. */
int sigma_ff_plan_bands(sigma_ff_plan plan, int* number_bands);

/* Waits for `stream`; SIGMA_OK or SIGMA_ERR_TIMEOUT when a bounded device
 * wait of the last execution gave up. */
int sigma_ff_plan_status(sigma_ff_plan plan, void* stream);

/* ---------------------------------------------------------------------------
 * Full-frequency sigma: the band loop of ffkernel.deslippe.best.f90
 * (:201-626) around the contraction, in the C layouts above plus
 *   I_epsA [nfreq][ngpown][ncouls], vcoul [ncouls], ekq [number_bands],
 *   dFreqGrid [nfreq] (ascending), dFreqBrd [nfreq] (complex), pref [nfreq].
 * Outputs (host, overwritten): achsDtemp [1] (static CH, :240-253),
 * asxDtemp (SX of the occupied bands, :279-389), achDtemp (sigma1),
 * achDtemp_corb (sigma3), ach2Dtemp (sigma2 + delta terms) and achDtemp_cor
 * (sigma4 + delta terms), each [nfreqeval] (:459-613), with
 * wx = freqevalmin - ekq[n1] + iw * freqevalstep, band n1 occupied when
 * n1 < nvband.  These replace achsDtemp_Kernel, asxDtemp_Kernel,
 * achDtemp_Kernel and achDtemp_cor_Kernel (FFKer_cori/ffKernel.cpp:107-245)
 * with the Fortran's semantics where the C++ port departs from them
 * (frequency index of the static term, the (iw-1) * freqevalstep of wx,
 * I_epsA for wx < 0 in SX, the separate achDtemp array, the interval
 * search at grid points and outside the grid).
 * schDt_matrix [number_bands][nfreq]: used as given (achDtemp_Kernel's
 * input); NULL computes it from I_epsR with the contraction of this header
 * (the Fortran zeroes it: its contraction is commented out).
 * Columns whose igp = indinv[inv_igp_index[my_igp]] falls outside
 * [0, ncouls) are left out, as the Fortran cycles them.  mode picks the
 * contraction form (SIGMA_FF_FP64 or SIGMA_FF_OZAKI_BF16) of the three
 * g-vector contractions; the rest runs in FP64.  Returns after `stream`
 * drains.
 * ------------------------------------------------------------------------- */
int sigma_ff_sigma(int number_bands, int nvband, int ncouls, int ngpown, int nfreq, int nfreqeval,
                   const int* inv_igp_index, const int* indinv, const sigma_complex128* aqsmtemp,
                   const sigma_complex128* aqsntemp, const sigma_complex128* I_epsR,
                   const sigma_complex128* I_epsA, const double* vcoul, const double* ekq,
                   const double* dFreqGrid, const sigma_complex128* dFreqBrd, const double* pref,
                   double pref_zb, double freqevalmin, double freqevalstep, double occ,
                   const sigma_complex128* schDt_matrix, sigma_complex128* achsDtemp,
                   sigma_complex128* asxDtemp, sigma_complex128* achDtemp,
                   sigma_complex128* achDtemp_cor, sigma_complex128* achDtemp_corb,
                   sigma_complex128* ach2Dtemp, int mode, void* stream);

/* Device-resident form: a plan (column map validated on the host, the FF
 * contraction plan and the per-band workspace) and an asynchronous
 * execution on device arrays.  dFreqGrid must be ascending (the host
 * drop-in checks it).  out is device complex[1 + 5 * nfreqeval]:
 * achsDtemp, then asxDtemp, achDtemp, achDtemp_cor, achDtemp_corb,
 * ach2Dtemp, nfreqeval values each.  Timing counts the contraction kernels
 * (two or three per execution) and everything else. */
typedef struct sigma_ff_sigma_plan_s* sigma_ff_sigma_plan;
int sigma_ff_sigma_plan_create(sigma_ff_sigma_plan* plan, int number_bands, int nvband, int ncouls,
                               int ngpown, int nfreq, int nfreqeval, const int* inv_igp_index,
                               const int* indinv, int mode);
int sigma_ff_sigma_execute(sigma_ff_sigma_plan plan, const sigma_complex128* aqsmtemp,
                           const sigma_complex128* aqsntemp, const sigma_complex128* I_epsR,
                           const sigma_complex128* I_epsA, const double* vcoul, const double* ekq,
                           const double* dFreqGrid, const sigma_complex128* dFreqBrd,
                           const double* pref, double pref_zb, double freqevalmin,
                           double freqevalstep, double occ, const sigma_complex128* schDt_matrix,
                           sigma_complex128* out, void* stream);
int sigma_ff_sigma_plan_set_timing(sigma_ff_sigma_plan plan, int enable);
int sigma_ff_sigma_plan_timing(sigma_ff_sigma_plan plan, int* contractions, double* contraction_ms,
                               double* other_ms);
int sigma_ff_sigma_plan_status(sigma_ff_sigma_plan plan, void* stream);
int sigma_ff_sigma_plan_destroy(sigma_ff_sigma_plan plan);

#ifdef __cplusplus
}
#endif

#endif /* SIGMA_FF_H */
