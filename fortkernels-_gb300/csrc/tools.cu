// Seeded device fills (bit-identical to workload.py) and FMA peak probes.
#include "sigma_tools.h"
#include "sigma_internal.cuh"
#include "floatfloat.cuh"

namespace sigma {
namespace {

constexpr unsigned long long kGolden = 0x9E3779B97F4A7C15ull;
constexpr unsigned long long kSeedK = 0xD1342543DE82EF95ull;

__host__ __device__ __forceinline__ unsigned long long fmix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ double u01(unsigned long long s0, long long k) {
  const unsigned long long z = fmix64(s0 + (unsigned long long)(k + 1) * kGolden);
  return (double)(z >> 11) * 0x1.0p-53;
}

__global__ void fill_kernel(double* dst, long long count, long long dst_stride,
                            unsigned long long s0, long long off, long long stride, double lo,
                            double span) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x)
    dst[i * dst_stride] = __dadd_rn(lo, __dmul_rn(span, u01(s0, off + i * stride)));
}

__global__ void stress_kernel(double2* wt, long long count, unsigned long long s0, double w0,
                              double w1, double w2, int nw, double fraction, double width) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < count;
       e += (long long)gridDim.x * blockDim.x) {
    if (u01(s0, 3 * e) < fraction) {
      const double uk = u01(s0, 3 * e + 1), uo = u01(s0, 3 * e + 2);
      long long k = (long long)(uk * nw);
      if (k > nw - 1) k = nw - 1;
      const double off = __dmul_rn(__dsub_rn(__dmul_rn(2.0, uo), 1.0), width);
      const double wx = k == 0 ? w0 : (k == 1 ? w1 : w2);
      wt[e].x = __dadd_rn(wx, off);
    }
  }
}

// FMA throughput probe: eight independent dependency chains per thread whose
// operands are all distinct registers (constant operands shared by every
// chain cost throughput on this part).
template <typename T>
__global__ void fma_probe_kernel(double* out, int iters) {
  T a0 = (T)(threadIdx.x * 1e-3), a1 = a0 + (T)1, a2 = a0 + (T)2, a3 = a0 + (T)3;
  T a4 = a0 + (T)4, a5 = a0 + (T)5, a6 = a0 + (T)6, a7 = a0 + (T)7;
  T b0 = (T)0.999999, b1 = (T)0.9999991, b2 = (T)0.9999992, b3 = (T)0.9999993;
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, b0, a4); a1 = fma(a1, b1, a5); a2 = fma(a2, b2, a6); a3 = fma(a3, b3, a7);
    a4 = fma(a4, b1, a0); a5 = fma(a5, b2, a1); a6 = fma(a6, b3, a2); a7 = fma(a7, b0, a3);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = (double)(a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7);
}

}  // namespace
}  // namespace sigma

extern "C" int sigma_fill_uniform(double* dst, long long count, long long dst_stride,
                                  unsigned long long seed, unsigned long long array_id,
                                  long long draw_offset, long long draw_stride, double lo,
                                  double span, void* stream) {
  using namespace sigma;
  if (!dst) return SIGMA_ERR_NULL;
  if (count < 0 || dst_stride < 1) return SIGMA_ERR_INVALID_SHAPE;
  if (count == 0) return SIGMA_OK;
  const unsigned long long s0 = fmix64(seed * kSeedK + array_id);
  long long blocks = (count + 255) / 256;
  if (blocks > 65536) blocks = 65536;
  fill_kernel<<<(int)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      dst, count, dst_stride, s0, draw_offset, draw_stride, lo, span);
  SIGMA_CUDA_TRY(cudaGetLastError());
  return SIGMA_OK;
}

extern "C" int sigma_fill_stress(double* wtilde, long long count, unsigned long long seed,
                                 unsigned long long array_id, const double* wx_host, int nw,
                                 double fraction, double width, void* stream) {
  using namespace sigma;
  if (!wtilde || !wx_host) return SIGMA_ERR_NULL;
  if (nw < 1 || nw > 3 || count < 0) return SIGMA_ERR_INVALID_SHAPE;
  if (count == 0) return SIGMA_OK;
  const unsigned long long s0 = fmix64(seed * kSeedK + array_id);
  long long blocks = (count + 255) / 256;
  if (blocks > 65536) blocks = 65536;
  stress_kernel<<<(int)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      reinterpret_cast<double2*>(wtilde), count, s0, wx_host[0], nw > 1 ? wx_host[1] : 0.0,
      nw > 2 ? wx_host[2] : 0.0, nw, fraction, width);
  SIGMA_CUDA_TRY(cudaGetLastError());
  return SIGMA_OK;
}

extern "C" int sigma_measure_fma_peaks(double* fp64_tflops, double* fp32_tflops, void* stream) {
  using namespace sigma;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int sms = 0, dev = 0;
  SIGMA_CUDA_TRY(cudaGetDevice(&dev));
  SIGMA_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int threads = 256, blocks = sms * 8;
  double* out = nullptr;
  SIGMA_CUDA_TRY(cudaMallocAsync(&out, sizeof(double) * threads * blocks, s));
  cudaEvent_t e0, e1;
  SIGMA_CUDA_TRY(cudaEventCreate(&e0));
  SIGMA_CUDA_TRY(cudaEventCreate(&e1));
  double res[2] = {0.0, 0.0};
  for (int which = 0; which < 2; ++which) {
    const int iters = which == 0 ? 1000 : 40000;
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
      SIGMA_CUDA_TRY(cudaEventRecord(e0, s));
      if (which == 0)
        fma_probe_kernel<double><<<blocks, threads, 0, s>>>(out, iters);
      else
        fma_probe_kernel<float><<<blocks, threads, 0, s>>>(out, iters);
      SIGMA_CUDA_TRY(cudaGetLastError());
      SIGMA_CUDA_TRY(cudaEventRecord(e1, s));
      SIGMA_CUDA_TRY(cudaEventSynchronize(e1));
      float ms = 0.f;
      SIGMA_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
      if (rep > 0 && ms < best) best = ms;
    }
    const double fmas = (double)blocks * threads * iters * 8.0;
    res[which] = 2.0 * fmas / (best * 1e-3) / 1e12;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  SIGMA_CUDA_TRY(cudaFreeAsync(out, s));
  SIGMA_CUDA_TRY(cudaStreamSynchronize(s));
  if (fp64_tflops) *fp64_tflops = res[0];
  if (fp32_tflops) *fp32_tflops = res[1];
  return SIGMA_OK;
}

namespace sigma {
namespace {
__global__ void reciprocals_kernel(const double* w, double* out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double x = w[i];
    out[3 * i] = rcp_f64(x);
    out[3 * i + 1] = rcp_f64_seed32(x);
    out[3 * i + 2] = __drcp_rn(x);  // IEEE 1/x, correctly rounded
  }
}
__global__ void split_kernel(const double* x, float* out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const FF s = ff_of(x[i]);
    out[2 * i] = s.hi;
    out[2 * i + 1] = s.lo;
  }
}
__global__ void split_round_kernel(const double* x, float* out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const FF s = ff_of_rn(x[i]);
    out[2 * i] = s.hi;
    out[2 * i + 1] = s.lo;
  }
}
}  // namespace
}  // namespace sigma

extern "C" int sigma_eval_split(const double* x, float* out, long long n, void* stream) {
  using namespace sigma;
  if (!x || !out) return SIGMA_ERR_NULL;
  if (n <= 0) return SIGMA_ERR_INVALID_SHAPE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 16);
  split_kernel<<<(int)blocks, 256, 0, s>>>(x, out, n);
  SIGMA_CUDA_TRY(cudaGetLastError());
  return SIGMA_OK;
}

extern "C" int sigma_eval_split_round(const double* x, float* out, long long n, void* stream) {
  using namespace sigma;
  if (!x || !out) return SIGMA_ERR_NULL;
  if (n <= 0) return SIGMA_ERR_INVALID_SHAPE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 16);
  split_round_kernel<<<(int)blocks, 256, 0, s>>>(x, out, n);
  SIGMA_CUDA_TRY(cudaGetLastError());
  return SIGMA_OK;
}

extern "C" int sigma_eval_reciprocals(const double* w, double* out, long long n, void* stream) {
  using namespace sigma;
  if (!w || !out) return SIGMA_ERR_NULL;
  if (n <= 0) return SIGMA_ERR_INVALID_SHAPE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 16);
  reciprocals_kernel<<<(int)blocks, 256, 0, s>>>(w, out, n);
  SIGMA_CUDA_TRY(cudaGetLastError());
  return SIGMA_OK;
}
