/* sigma_common.h - types and status codes shared by the sigma GPP / FF C ABI.
 *
 * The library replaces the hot loops of the BerkeleyGW sigma mini-apps in
 * rgayatri23/FortKernels- (GPP: BGW-Kernels/gppKer.cpp; FF:
 * ffkernel.deslippe.best.f90 and FFKer_cori/ffKernel.cpp) with GB300 (sm_103a)
 * CUDA kernels behind plain C entry points: raw pointers, int shapes, int
 * status.  Every complex array is interleaved complex128, the layout of
 * std::complex<double> and of the reference's GPUComplex (Complex.h:18-26).
 */
#ifndef SIGMA_COMMON_H
#define SIGMA_COMMON_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sigma_complex128 {
  double re;
  double im;
} sigma_complex128;

/* Status codes.  The reference exits the process on bad arguments
 * (BGW-Kernels/gppKer.cpp:164-169, FFKer_cori/ffKernel.cpp:320-325); the
 * library returns one of these instead and never calls exit(). */
enum sigma_status {
  SIGMA_OK = 0,
  SIGMA_ERR_INVALID_SHAPE = -1, /* a size is <= 0, ngpown > ncouls, nend-nstart != 3, ... */
  SIGMA_ERR_INDEX_RANGE = -2,   /* an inv_igp_index / indinv entry the reference would read out of bounds */
  SIGMA_ERR_ALLOC = -3,         /* device or pinned allocation failed */
  SIGMA_ERR_CUDA = -4,          /* a CUDA runtime call failed */
  SIGMA_ERR_TIMEOUT = -5,       /* a bounded device wait gave up (batched work queue) */
  SIGMA_ERR_NULL = -6,          /* a required pointer is NULL */
  SIGMA_ERR_NO_DEVICE = -7,     /* no CUDA device, or the library was not built for it */
  SIGMA_ERR_UNSUPPORTED = -8,   /* argument combination this build does not handle */
  SIGMA_ERR_WORKSPACE = -9      /* caller-provided workspace is too small */
};

/* Arithmetic forms. */
enum sigma_precision {
  SIGMA_PREC_FP64 = 0,  /* plain FP64: every term in double precision */
  SIGMA_PREC_MIXED = 1, /* FP32 bulk, FP64 pole-guard decisions, compensated FP64 reductions */
  SIGMA_PREC_TENSOR = 2 /* one frequency set for all bands only: the band sum as a complex GEMM
                           on tcgen05 tensor cores (split-BF16 operands, FP32 accumulation
                           drained into FP32 sums, FP64 partials), frequency factors and
                           pole-guard decisions in FP64; occupied bands as in the mixed form */
};

/* Human-readable name of a status code (static string). */
const char* sigma_status_string(int status);

/* Text of the last CUDA failure the library saw (thread-local copy; empty
 * when there was none). */
const char* sigma_last_error_message(void);

/* Frees the library's cached device buffers and plans on every device.
 * Safe to call more than once. */
int sigma_shutdown(void);

/* Library build tag (static string). */
const char* sigma_version(void);

#ifdef __cplusplus
}
#endif

#endif /* SIGMA_COMMON_H */
