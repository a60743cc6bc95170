/* sigma_tools.h - workload generation and measurement helpers.
 *
 * The reference drivers fill their inputs with constants inside main()
 * (BGW-Kernels/gppKer.cpp:275-299, FFKer_cori/ffKernel.cpp:398-433).  These
 * helpers generate the seeded synthetic inputs of the production shapes
 * directly in device memory, bit-identical to the host generator in
 * fortkernels-_gb300/workload.py (SplitMix64 as a counter-based stream), and
 * measure the FP64 / FP32 FMA throughput the roofline is quoted against.
 */
#ifndef SIGMA_TOOLS_H
#define SIGMA_TOOLS_H

#include "sigma_common.h"

#ifdef __cplusplus
extern "C" {
#endif

/* dst[i * dst_stride] = lo + span * u(draw_offset + i * draw_stride), i < count,
 * where u(k) is draw k of stream (seed, array_id) as a double in [0, 1).
 * dst is a device pointer.  Asynchronous on `stream`. */
int sigma_fill_uniform(double* dst, long long count, long long dst_stride,
                       unsigned long long seed, unsigned long long array_id,
                       long long draw_offset, long long draw_stride, double lo, double span,
                       void* stream);

/* Moves a fraction of the wtilde elements (interleaved complex128, device) to
 * re = wx[k] + offset, offset in (-width, width), k among the nw frequencies,
 * using draws 3e, 3e+1, 3e+2 of stream (seed, array_id) for element e; the
 * same rule as workload.stress_wtilde. */
int sigma_fill_stress(double* wtilde, long long count, unsigned long long seed,
                      unsigned long long array_id, const double* wx_host, int nw,
                      double fraction, double width, void* stream);

/* Measured issue-limited throughput of dependent-free DFMA and FFMA streams
 * on the current device, in TFLOP/s (an FMA counts as 2 flop).  Runs a few
 * milliseconds of kernels on `stream` and synchronises it. */
int sigma_measure_fma_peaks(double* fp64_tflops, double* fp32_tflops, void* stream);

/* The library's two FP64 reciprocal routines on n positive device values w
 * (a check of their error bounds; no counterpart in the reference):
 * out[3i] = rcp_f64(w[i]) (hardware seed, cubic Newton step; within the FP64
 * rounding unit), out[3i+1] = rcp_f64_seed32(w[i]) (FP32 seed, one Newton
 * step; within 2^-44.8 relative, from below, for normal w whose reciprocal
 * is normal), out[3i+2] = the correctly rounded IEEE 1/w.  out is a device
 * array of 3n doubles.  Asynchronous on `stream`. */
int sigma_eval_reciprocals(const double* w, double* out, long long n, void* stream);

/* The float-float split of n device doubles x (a check of the split the
 * FP32-class forms and the FP64 forms' float-float factors build on; no
 * counterpart in the reference): out[2i] = hi (x truncated to 24
 * significant bits), out[2i+1] = lo (the remaining bits rounded to FP32), so
 * |x - hi - lo| <= 2^-48 |x| for 2^-74 <= |x| < 2^128.  out is a device
 * array of 2n floats.  Asynchronous on `stream`. */
int sigma_eval_split(const double* x, float* out, long long n, void* stream);

/* The rounded float-float split the FP64 forms' float-float terms use (no
 * counterpart in the reference): out[2i] = hi (x rounded to the nearest
 * FP32 value, ties to even), out[2i+1] = lo (x - hi rounded to FP32), so
 * |x - hi - lo| <= 2^-48 |x| and |lo| <= 2^-24 |x| for 2^-74 <= |x| < 2^128
 * (an infinite hi from FLT_MAX + 1/2 ulp up).  out is a device array of 2n
 * floats.  Asynchronous on `stream`. */
int sigma_eval_split_round(const double* x, float* out, long long n, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SIGMA_TOOLS_H */
