/*
 * ref_shim.h - host shims so the reference's device functions compile with g++ as plain host
 * code for the oracle's parity pin. TEST INFRASTRUCTURE ONLY (built into oracle/_ref/).
 *
 * The reference sources are compiled where they lie (never copied); this header stands in for
 * the CUDA runtime pieces they touch: qualifiers, atomics, fences, clock64, and the warp
 * collectives (__ballot_sync/__shfl_sync/__syncwarp), which run on a 32-thread barrier emulator
 * (one host thread per lane) in ref_glue.cpp.
 */
#ifndef CSMV_REF_SHIM_H_
#define CSMV_REF_SHIM_H_

#include <assert.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>

/* skip the real CUDA runtime header and the reference's PTX helper header */
#define __CUDA_RUNTIME_H__
#define SERVER_COMM_H_

typedef unsigned int uint;
typedef unsigned short ushort;

#define __device__
#define __global__
#define __host__
#define __forceinline__ inline
#define __shared__ static

typedef int cudaError_t;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind { cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2 };
static inline const char* cudaGetErrorString(cudaError_t) { return "host shim"; }
static inline cudaError_t cudaMalloc(void** p, size_t n) {
  *p = calloc(1, n);
  return *p ? 0 : 2;
}
static inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) {
  memcpy(d, s, n);
  return 0;
}
static inline cudaError_t cudaFree(void* p) {
  free(p);
  return 0;
}

static inline long long int clock64() { return 0; }
static inline void __threadfence() { std::atomic_thread_fence(std::memory_order_seq_cst); }
static inline int atomicAdd(int* p, int v) { return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST); }
static inline unsigned atomicAdd(unsigned* p, unsigned v) {
  return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST);
}
static inline int atomicCAS(int* p, int cmp, int val) {
  __atomic_compare_exchange_n(p, &cmp, val, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
  return cmp;
}

/* warp emulator (ref_glue.cpp) */
unsigned ref_emu_lane(void);
unsigned ref_emu_ballot(int pred);
int ref_emu_shfl(int v, int src);
void ref_emu_sync(void);
static const int warpSize = 32;
static inline unsigned __activemask() { return 0xFFFFFFFFu; }
static inline unsigned __ballot_sync(unsigned, int pred) { return ref_emu_ballot(pred); }
static inline int __shfl_sync(unsigned, int v, int src) { return ref_emu_shfl(v, src); }
static inline void __syncwarp() { ref_emu_sync(); }

/* the helpers of sync_lib/common.h the API files use */
static inline unsigned get_lane_id() { return ref_emu_lane(); }
static inline unsigned vote_ballot(unsigned b) { return ref_emu_ballot(b != 0); }
static inline unsigned count_bit(unsigned m) { return (unsigned)__builtin_popcount(m); }
static inline unsigned set_bits(unsigned mask, unsigned val, unsigned pos, unsigned len) {
  unsigned f = len >= 32 ? 0xFFFFFFFFu : ((1u << len) - 1u);
  return (mask & ~(f << pos)) | ((val & f) << pos);
}
static inline unsigned find_nth_bit(unsigned mask, unsigned base, unsigned offset) {
  (void)base; /* only used as fns(mask, 0, 1): lowest set bit */
  unsigned n = 0;
  for (unsigned i = 0; i < 32; i++)
    if ((mask >> i) & 1u)
      if (++n == offset) return i;
  return 0xFFFFFFFFu;
}
struct ref_dim3 {
  unsigned x, y, z;
};
extern thread_local ref_dim3 threadIdx;

#endif
