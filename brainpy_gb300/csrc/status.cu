// status.cu -- error reporting of the C ABI.
#include <string>

#include "common.cuh"

namespace bp {

static thread_local std::string g_last_error;

void set_error(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

void clear_error() { g_last_error.clear(); }

bp_status check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("%s: launch failed: %s", what, cudaGetErrorString(e));
    return BP_ECUDA;
  }
  return BP_OK;
}

int device_sm_count() {
  static int cache[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return kNumSMs;
  if (cache[dev] == 0) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cache[dev] = sms > 0 ? sms : kNumSMs;
  }
  return cache[dev];
}

}  // namespace bp

extern "C" {

const char* bp_status_string(bp_status s) {
  switch (s) {
    case BP_OK: return "BP_OK";
    case BP_EINVAL: return "BP_EINVAL: invalid argument";
    case BP_ESHAPE: return "BP_ESHAPE: shape mismatch";
    case BP_EDTYPE: return "BP_EDTYPE: unsupported dtype";
    case BP_ENOMEM: return "BP_ENOMEM: buffer or workspace too small";
    case BP_ETIMEOUT: return "BP_ETIMEOUT: bounded device wait expired";
    case BP_ECUDA: return "BP_ECUDA: CUDA error";
    case BP_ENOTSUP: return "BP_ENOTSUP: not supported";
  }
  return "unknown bp_status";
}

const char* bp_last_error(void) { return bp::g_last_error.c_str(); }

int32_t bp_version(void) { return 0x000100; }

}  // extern "C"
