// Error state and device queries of the C ABI.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <string>

#include "tatva_gb300.h"

namespace tg {

static thread_local std::string g_last_error;

int set_error(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_check(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return TG_OK;
  return set_error(TG_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

}  // namespace tg

extern "C" const char* tg_last_error(void) { return tg::g_last_error.c_str(); }

extern "C" int tg_version(void) { return 1; }

extern "C" int tg_device_sm_count(void) {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

// Streams owned by this library's CUDA runtime (for callers whose own stream
// handles come from another runtime instance).
extern "C" int tg_stream_create(void** stream) {
  if (!stream) return tg::set_error(TG_ERR_VALUE, "stream must not be NULL");
  cudaStream_t s = nullptr;
  const int rc = tg::cuda_check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "tg_stream_create");
  *stream = rc == TG_OK ? (void*)s : nullptr;
  return rc;
}

extern "C" int tg_stream_destroy(void* stream) {
  if (!stream) return TG_OK;
  return tg::cuda_check(cudaStreamDestroy((cudaStream_t)stream), "tg_stream_destroy");
}

extern "C" int tg_stream_synchronize(void* stream) {
  return tg::cuda_check(cudaStreamSynchronize((cudaStream_t)stream), "tg_stream_synchronize");
}

extern "C" int tg_device_synchronize(void) {
  return tg::cuda_check(cudaDeviceSynchronize(), "tg_device_synchronize");
}
