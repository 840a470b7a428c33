// csmv_prims.cuh - memory-model primitives and bounded waits for the sm_103a commit path.
//
// The reference (sync_lib/common.h:12-173) wraps pre-Volta PTX (bfind, fns, popc, shfl.sync
// with a full mask from divergent code, ld/st.global.cg). Here every cross-warp hand-off is an
// explicit acquire/release pair at the narrowest scope that covers it (.cta for the
// shared-memory mailbox, .gpu for the commit order and the clock), and every spin has an
// iteration budget after which it records an error and returns instead of hanging the GPU.
#pragma once
#include <cstdint>

namespace csmv {

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// ---- global (gpu scope) -------------------------------------------------------------------
__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_acquire_gpu(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_gpu(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_release_gpu(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_relaxed_gpu(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_gpu(uint32_t* p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_gpu(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_gpu(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
// two 8-byte version slots in one 16-byte access; each element is single-copy atomic
__device__ __forceinline__ void ld_relaxed_gpu_v2(const unsigned long long* p,
                                                  unsigned long long& a,
                                                  unsigned long long& b) {
  asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];"
               : "=l"(a), "=l"(b)
               : "l"(p)
               : "memory");
}
__device__ __forceinline__ void fence_acq_rel_gpu() {
  asm volatile("fence.acq_rel.gpu;" ::: "memory");
}


// Global words shared only by the threads of one CTA (one SM): CTA scope lets the SM's L1 serve
// them. Each 8-byte access is single-copy atomic.
__device__ __forceinline__ unsigned long long ld_relaxed_cta_global(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.cta.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_cta_global(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.cta.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// ---- shared (cta scope) -------------------------------------------------------------------
__device__ __forceinline__ uint32_t ld_acquire_cta(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.cta.shared.u32 %0, [%1];"
               : "=r"(v)
               : "r"((uint32_t)__cvta_generic_to_shared(p))
               : "memory");
  return v;
}
__device__ __forceinline__ void st_release_cta(uint32_t* p, uint32_t v) {
  asm volatile("st.release.cta.shared.u32 [%0], %1;" ::"r"((uint32_t)__cvta_generic_to_shared(p)),
               "r"(v)
               : "memory");
}

// ---- device error word ----------------------------------------------------------------------
enum : uint32_t {
  ERR_NONE = 0,
  ERR_WAIT_TURN = 1,     // commit-order turn never came
  ERR_WAIT_CLOCK = 2,    // clock never reached the predecessor's timestamp
  ERR_WAIT_REPLY = 3,    // a client warp's request got no reply
  ERR_WAIT_REQUEST = 4,  // the server saw no progress from its clients
  ERR_CAPACITY = 5,      // read/write set or batch capacity exceeded
  ERR_DATA = 6,          // malformed transaction (bad size / address)
  ERR_LIVELOCK = 7,      // a round exhausted its attempt budget without committing
  ERR_WAIT_FLOW = 8      // a dataflow-lane transaction's inputs never arrived
};

__device__ __forceinline__ void raise_error(uint32_t* err, uint32_t code) {
  atomicCAS(err, 0u, code);
}

// Bounded poll: returns true when pred() holds, false when the budget ran out or another warp
// raised an error (which is then left in *err). The first polls spin (the commit-order hand-offs
// are latency-critical), later ones back off with nanosleep up to 256 ns.
template <class Pred>
__device__ __forceinline__ bool bounded_wait(Pred pred, uint32_t* err, uint32_t code,
                                             uint32_t limit_log2) {
  uint32_t ns = 32;
  const uint64_t limit = 1ull << limit_log2;
  for (uint64_t it = 0; it < limit; ++it) {
    if (pred()) return true;
    if ((it & 15u) == 15u && ld_relaxed_gpu(err) != 0) return false;
    if (it >= 64) {
      __nanosleep(ns);
      if (ns < 256) ns <<= 1;
    }
  }
  raise_error(err, code);
  return false;
}

// bounded_wait for a latency-critical reply: 1024 polls back to back (the device error word
// every 256th), then short sleeps of at most 64 ns.
template <class Pred>
__device__ __forceinline__ bool bounded_wait_fast(Pred pred, uint32_t* err, uint32_t code,
                                                  uint32_t limit_log2) {
  const uint64_t limit = 1ull << limit_log2;
  for (uint64_t it = 0; it < limit; ++it) {
    if (pred()) return true;
    if ((it & 255u) == 255u && ld_relaxed_gpu(err) != 0) return false;
    if (it >= 1024) __nanosleep(64);
  }
  raise_error(err, code);
  return false;
}

// 4-byte asynchronous global->shared copy (lands in shared memory; wait with cp_async_wait_all).
__device__ __forceinline__ void cp_async4(void* smem_dst, const void* gmem_src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(smem_dst)),
               "l"(gmem_src)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}
// Cluster scope through generic addresses (the caller's shared memory or another CTA's of the
// cluster, as mapped by cluster.map_shared_rank): mailboxes of a thread-block cluster.
__device__ __forceinline__ uint32_t ld_acquire_cluster(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.cluster.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_cluster(uint32_t* p, uint32_t v) {
  asm volatile("st.release.cluster.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// Mailbox handshakes at the scope the mailbox is shared at.
template <bool CLUSTER>
__device__ __forceinline__ uint32_t mail_acquire(const uint32_t* p) {
  return CLUSTER ? ld_acquire_cluster(p) : ld_acquire_cta(p);
}
template <bool CLUSTER>
__device__ __forceinline__ void mail_release(uint32_t* p, uint32_t v) {
  if (CLUSTER)
    st_release_cluster(p, v);
  else
    st_release_cta(p, v);
}

// System scope: words shared with the host through mapped (zero-copy) host memory.
__device__ __forceinline__ uint32_t ld_acquire_sys(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_sys(uint32_t* p, uint32_t v) {
  asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// 16-byte asynchronous global->shared copy through L2 (both addresses 16-byte aligned).
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(smem_dst)),
               "l"(gmem_src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// wait until at most N of this thread's committed groups are still in flight
template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

}  // namespace csmv
