// common.cpp - error text, status names and device checks of the C ABI.
#include "common.h"

#include <cstring>

namespace csmv {

static thread_local char g_last_error[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

csmv_status check_device(int device, int* n_sms) {
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    set_error("no CUDA device: %s", e == cudaSuccess ? "count is 0" : cudaGetErrorString(e));
    return CSMV_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= count) {
    set_error("device %d out of range (%d devices)", device, count);
    return CSMV_ERR_INVALID_ARG;
  }
  cudaDeviceProp prop;
  CSMV_CUDA(cudaGetDeviceProperties(&prop, device));
  if (prop.major != 10 || prop.minor != 3) {
    set_error("device %d is sm_%d%d; this library is built for sm_103a only", device,
              prop.major, prop.minor);
    return CSMV_ERR_NO_DEVICE;
  }
  if (n_sms) *n_sms = prop.multiProcessorCount;
  return CSMV_OK;
}

}  // namespace csmv

extern "C" const char* csmv_last_error(void) { return csmv::g_last_error; }

extern "C" const char* csmv_status_str(csmv_status s) {
  switch (s) {
    case CSMV_OK: return "ok";
    case CSMV_ERR_INVALID_ARG: return "invalid argument";
    case CSMV_ERR_CUDA: return "CUDA error";
    case CSMV_ERR_OOM: return "out of memory";
    case CSMV_ERR_TIMEOUT: return "bounded device wait timed out";
    case CSMV_ERR_CAPACITY: return "capacity exceeded";
    case CSMV_ERR_NO_DEVICE: return "no sm_103 device";
    case CSMV_ERR_STATE: return "call out of order";
    case CSMV_ERR_IO: return "file error";
  }
  return "unknown status";
}

extern "C" int csmv_abi_version(void) { return CSMV_ABI_VERSION; }

extern "C" csmv_status csmv_pinned_alloc(size_t bytes, void** out) {
  if (!out || bytes == 0) return CSMV_ERR_INVALID_ARG;
  *out = nullptr;
  return csmv::cuda_status(cudaMallocHost(out, bytes), "cudaMallocHost");
}

extern "C" void csmv_pinned_free(void* p) {
  if (p) cudaFreeHost(p);
}
