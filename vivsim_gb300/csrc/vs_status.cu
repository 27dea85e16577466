// Status codes and the per-thread last-error message of the C ABI.
#include <stdarg.h>
#include <stdio.h>

#include <string>

#include "vs_common.cuh"

namespace vs {

static thread_local std::string g_last_error;

void set_error(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

int cuda_status(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return VS_OK;
  set_error("%s: %s (%s)", where, cudaGetErrorString(e), cudaGetErrorName(e));
  return VS_ERR_CUDA;
}

}  // namespace vs

extern "C" {

const char* vs_last_error(void) { return vs::g_last_error.c_str(); }

const char* vs_status_string(int status) {
  switch (status) {
    case VS_OK: return "ok";
    case VS_ERR_INVALID_ARG: return "invalid argument";
    case VS_ERR_CUDA: return "CUDA error";
    case VS_ERR_UNSUPPORTED: return "unsupported";
    case VS_ERR_RANGE: return "index out of range";
    case VS_ERR_TIMEOUT: return "device wait timed out";
    case VS_ERR_NONFINITE: return "non-finite populations";
    case VS_ERR_TIMEOUT_INFLIGHT: return "device wait timed out with a bulk copy still in flight";
    default: return "unknown status";
  }
}

int vs_version(void) { return 100; }

}  // extern "C"
