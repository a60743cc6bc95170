// Library runtime: status strings, the last CUDA error, per-device caches of
// device buffers used by the host-pointer entry points, and shutdown.
#include <mutex>
#include <string>
#include <vector>
#include <cstdio>

#include "sigma_internal.cuh"
#include "runtime.h"

namespace sigma {
namespace {

std::mutex g_err_mu;
std::string g_last_error;

}  // namespace

void set_last_cuda_error(cudaError_t err, const char* what, int line) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  char buf[512];
  snprintf(buf, sizeof buf, "%s (%s) at line %d: %s", cudaGetErrorName(err), what, line,
           cudaGetErrorString(err));
  g_last_error = buf;
}

void set_last_error_text(const char* text) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_last_error = text;
}

std::mutex& api_mutex() {
  static std::mutex mu;
  return mu;
}

// ---------------------------------------------------------------- device info
int device_sm_count() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  static std::vector<int> cache(64, -1);
  if (dev < 0 || dev >= (int)cache.size()) return 0;
  if (cache[dev] < 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    cache[dev] = n;
  }
  return cache[dev];
}

// ---------------------------------------------------------------- device arena
namespace {
struct Arena {
  void* ptr = nullptr;
  size_t bytes = 0;
};
std::vector<Arena>& arenas() {
  static std::vector<Arena> a(64 * kArenaSlots);
  return a;
}
std::vector<ShutdownHook>& hooks() {
  static std::vector<ShutdownHook> h;
  return h;
}
}  // namespace

int arena_get(int slot, size_t bytes, void** out) {
  int dev = 0;
  SIGMA_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64 || slot < 0 || slot >= kArenaSlots) return SIGMA_ERR_UNSUPPORTED;
  Arena& a = arenas()[dev * kArenaSlots + slot];
  if (a.bytes < bytes) {
    if (a.ptr) {
      cudaDeviceSynchronize();
      cudaFree(a.ptr);
      a.ptr = nullptr;
      a.bytes = 0;
    }
    // round up to 64 MiB steps so growing workloads do not reallocate each call
    const size_t step = size_t(64) << 20;
    const size_t want = (bytes + step - 1) / step * step;
    cudaError_t e = cudaMalloc(&a.ptr, want);
    if (e != cudaSuccess) {
      cudaGetLastError();
      set_last_cuda_error(e, "cudaMalloc(arena)", __LINE__);
      a.ptr = nullptr;
      return SIGMA_ERR_ALLOC;
    }
    a.bytes = want;
  }
  *out = a.ptr;
  return SIGMA_OK;
}

void register_shutdown_hook(ShutdownHook h) { hooks().push_back(h); }

}  // namespace sigma

extern "C" {

const char* sigma_status_string(int status) {
  switch (status) {
    case SIGMA_OK: return "ok";
    case SIGMA_ERR_INVALID_SHAPE: return "invalid shape";
    case SIGMA_ERR_INDEX_RANGE: return "index out of range";
    case SIGMA_ERR_ALLOC: return "allocation failed";
    case SIGMA_ERR_CUDA: return "CUDA error";
    case SIGMA_ERR_TIMEOUT: return "device wait timed out";
    case SIGMA_ERR_NULL: return "null pointer";
    case SIGMA_ERR_NO_DEVICE: return "no usable CUDA device";
    case SIGMA_ERR_UNSUPPORTED: return "unsupported argument combination";
    case SIGMA_ERR_WORKSPACE: return "workspace too small";
    default: return "unknown status";
  }
}

const char* sigma_last_error_message(void) {
  static thread_local std::string copy;
  std::lock_guard<std::mutex> lk(sigma::g_err_mu);
  copy = sigma::g_last_error;
  return copy.c_str();
}

int sigma_shutdown(void) {
  std::lock_guard<std::mutex> lk(sigma::api_mutex());
  for (auto& h : sigma::hooks()) h();
  int cur = 0;
  cudaGetDevice(&cur);
  auto& a = sigma::arenas();
  for (size_t i = 0; i < a.size(); ++i) {
    if (a[i].ptr) {
      cudaSetDevice((int)(i / sigma::kArenaSlots));
      cudaFree(a[i].ptr);
      a[i].ptr = nullptr;
      a[i].bytes = 0;
    }
  }
  cudaSetDevice(cur);
  return SIGMA_OK;
}

const char* sigma_version(void) { return "sigma-gb300 1.0 (sm_103a)"; }

}  // extern "C"
