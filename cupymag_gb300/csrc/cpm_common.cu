// Library-level helpers: error strings, device queries, version.
#include <cstdarg>
#include <cstdio>

#include "cpm_common.cuh"

namespace cpm {

static thread_local char g_err[1024] = "";

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int check_launch(const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    return CPM_CUDA_ERROR;
  }
  return CPM_OK;
}

int device_id() {
  int d = 0;
  cudaGetDevice(&d);
  return d;
}

int sm_count() {
  static int cache_dev = -1, cache_sms = 0;
  const int d = device_id();
  if (d != cache_dev) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, d);
    cache_sms = v;
    cache_dev = d;
  }
  return cache_sms;
}

}  // namespace cpm

extern "C" const char *cpm_version(void) { return "cupymag_gb300 0.1.0 (sm_103a)"; }

extern "C" const char *cpm_last_error_string(void) { return cpm::g_err; }

extern "C" int cpm_device_sm_count(int device) {
  int v = 0;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return -1;
  return v;
}
