// common.h - host-side helpers shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>

#include "../../include/csmv.h"

namespace csmv {

void set_error(const char* fmt, ...) __attribute__((format(printf, 1, 2)));

// Record a CUDA failure and turn it into a status (never aborts the process).
inline csmv_status cuda_status(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return CSMV_OK;
  set_error("%s: %s", what, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? CSMV_ERR_OOM : CSMV_ERR_CUDA;
}

#define CSMV_CUDA(call)                                         \
  do {                                                          \
    csmv_status st__ = ::csmv::cuda_status((call), #call);      \
    if (st__ != CSMV_OK) return st__;                           \
  } while (0)

// Checks that `device` exists and is an sm_103 part; returns the SM count.
csmv_status check_device(int device, int* n_sms);

// The bank's account count; true when it commits in groups (prevalidate 3, stamp protocol), the
// mode that takes a stream's lock_last classes (bank_engine.cu).
bool bank_group_commit(const csmv_bank_t* h, uint32_t* n_accounts);

}  // namespace csmv
