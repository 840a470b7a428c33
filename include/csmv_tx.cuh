// csmv_tx.cuh - device-side transaction API of the GB300 CSMV engine.
//
// Same seven entry points as the reference's per-thread API
// (csmv_optimizations/batchedAtrInsert/csmv_sh/API.cuh:139-151): TXBegin, TXRead, TXReadOnly,
// TXWrite, TXPreValidation, TXAddToRecord (server side, in the engine) and TXWriteBack, with the
// same meaning and abort convention (*isAborted / a zero commit timestamp), re-laid for sm_103a:
//
//  * Versions are packed 64-bit slots (ts << 32 | value), `depth` per item, item-major, so an
//    item's whole version list (depth 4 = 32 bytes) is one DRAM sector and one (ts, value)
//    pair is read with a single single-copy-atomic access. An empty slot has ts 0xFFFFFFFF.
//    The newest version visible at snapshot ts is the slot with the largest ts <= snapshot;
//    none means the reference's DataAge abort (bank/csmv_sh/API.cu:20-24).
//  * Read and write sets live in registers (fixed maximum sizes), not in a 4 KB-per-thread
//    global array as in the reference (bank/csmv_sh/API.cuh:84-95).
//  * The warp-collective calls must be reached by all 32 lanes (full-mask __shfl_sync /
//    __ballot_sync); a lane that takes no part passes active = false.
#pragma once
#include <cstdint>

#include "../csmv-gpu-stm_gb300/csrc/csmv_prims.cuh"

namespace csmv {

constexpr uint32_t kEmptyTs = 0xFFFFFFFFu;

struct VersionStore {
  unsigned long long* slots;  // [n_items * depth]
  uint32_t n_items;
};

template <int MAXR>
struct ReadSet {
  uint32_t n = 0;
  uint32_t addr[MAXR] = {};
};

template <int MAXW>
struct WriteSet {
  uint32_t n = 0;
  uint32_t addr[MAXW] = {};
  int32_t val[MAXW] = {};
};

__device__ __forceinline__ unsigned long long pack_version(uint32_t ts, int32_t v) {
  return ((unsigned long long)ts << 32) | (uint32_t)v;
}
__device__ __forceinline__ uint32_t version_ts(unsigned long long s) { return (uint32_t)(s >> 32); }
__device__ __forceinline__ int32_t version_val(unsigned long long s) { return (int32_t)(uint32_t)s; }

// Newest version with ts <= snap among the item's DEPTH slots. Returns false (DataAge) when
// every kept version is newer than the snapshot.
template <int DEPTH>
__device__ __forceinline__ bool read_version(const unsigned long long* item, uint32_t snap,
                                             int32_t& out) {
  static_assert(DEPTH % 2 == 0, "depth is even (16-byte loads)");
  unsigned long long s[DEPTH];
#pragma unroll
  for (int d = 0; d < DEPTH; d += 2) ld_relaxed_gpu_v2(item + d, s[d], s[d + 1]);
  bool found = false;
  uint32_t bts = 0;
  int32_t bv = 0;
#pragma unroll
  for (int d = 0; d < DEPTH; d++) {
    uint32_t t = version_ts(s[d]);
    bool ok = (t != kEmptyTs) && (t <= snap) && (!found || t > bts);
    if (ok) {
      found = true;
      bts = t;
      bv = version_val(s[d]);
    }
  }
  out = bv;
  return found;
}

// TXBegin (bank/csmv_sh/API.cu:275-291, batched form :392-397): empty sets, snapshot = clock.
// The acquire load makes every write-back with ts <= snapshot visible to this thread.
template <int MAXR, int MAXW>
__device__ __forceinline__ uint32_t TXBegin(const uint32_t* clock, ReadSet<MAXR>& rs,
                                            WriteSet<MAXW>& ws) {
  rs.n = 0;
  ws.n = 0;
  return ld_acquire_gpu(clock);
}

// TXWrite (bank/csmv_sh/API.cu:69-85): buffer (addr, value), overwriting an earlier write.
template <int MAXW>
__device__ __forceinline__ bool TXWrite(uint32_t addr, int32_t value, WriteSet<MAXW>& ws) {
#pragma unroll
  for (int i = 0; i < MAXW; i++)
    if (i < (int)ws.n && ws.addr[i] == addr) {
      ws.val[i] = value;
      return true;
    }
  if (ws.n >= (uint32_t)MAXW) return false;
#pragma unroll
  for (int i = 0; i < MAXW; i++)
    if (i == (int)ws.n) {
      ws.addr[i] = addr;
      ws.val[i] = value;
    }
  ws.n++;
  return true;
}

// TXRead (bank/csmv_sh/API.cu:5-41): read-your-writes from the write set, else the version
// rule; the address joins the read set. Sets *isAborted on DataAge.
template <int DEPTH, int MAXR, int MAXW>
__device__ __forceinline__ int32_t TXRead(const VersionStore& vs, uint32_t addr, uint32_t ts,
                                          ReadSet<MAXR>& rs, const WriteSet<MAXW>& ws,
                                          bool* isAborted) {
  int32_t v = 0;
  bool hit = false;
#pragma unroll
  for (int i = 0; i < MAXW; i++)
    if (i < (int)ws.n && ws.addr[i] == addr) {
      v = ws.val[i];
      hit = true;
    }
  if (!hit && !read_version<DEPTH>(vs.slots + (size_t)addr * DEPTH, ts, v)) {
    *isAborted = true;
    return 0;
  }
#pragma unroll
  for (int i = 0; i < MAXR; i++)
    if (i == (int)rs.n) rs.addr[i] = addr;
  if (rs.n < (uint32_t)MAXR) rs.n++;
  return v;
}

// Read of the latest committed version in the stamp protocol: an item's commit word holds the
// timestamp of its last committed writer (published only after that writer's version is in
// the list), and the read returns that version. The stamp joins the read set; commit-time
// validation then only checks that it has not moved. When the version of the stamp is not yet
// visible (the word and the slots were fetched concurrently), the word is fetched again with
// acquire semantics and the slots after it.
template <int DEPTH>
__device__ __forceinline__ bool read_stamped(const unsigned long long* item, uint32_t stamp,
                                             int32_t& out) {
  unsigned long long s[DEPTH];
#pragma unroll
  for (int d = 0; d < DEPTH; d += 2) ld_relaxed_gpu_v2(item + d, s[d], s[d + 1]);
  bool found = false;
#pragma unroll
  for (int d = 0; d < DEPTH; d++)
    if (version_ts(s[d]) == stamp) {
      out = version_val(s[d]);
      found = true;
    }
  return found;
}

// Latest committed version of an item and its stamp (the read of TXReadLatest without the read
// set). Returns false when the stamp's version could not be found.
template <int DEPTH>
__device__ __forceinline__ bool read_latest(const VersionStore& vs,
                                            const unsigned long long* commit_words, uint32_t addr,
                                            uint32_t& stamp, int32_t& v) {
  const unsigned long long* item = vs.slots + (size_t)addr * DEPTH;
  stamp = (uint32_t)ld_relaxed_gpu(commit_words + addr);
  if (read_stamped<DEPTH>(item, stamp, v)) return true;
  stamp = (uint32_t)ld_acquire_gpu(commit_words + addr);
  return read_stamped<DEPTH>(item, stamp, v);
}

template <int DEPTH, int MAXR>
__device__ __forceinline__ int32_t TXReadLatest(const VersionStore& vs,
                                                const unsigned long long* commit_words,
                                                uint32_t addr, ReadSet<MAXR>& rs,
                                                uint32_t& stamp, bool* isAborted) {
  int32_t v = 0;
  if (!read_latest<DEPTH>(vs, commit_words, addr, stamp, v)) *isAborted = true;
#pragma unroll
  for (int i = 0; i < MAXR; i++)
    if (i == (int)rs.n) rs.addr[i] = addr;
  if (rs.n < (uint32_t)MAXR) rs.n++;
  return v;
}

// TXReadOnly (bank/csmv_sh/API.cu:43-67): the version rule without read-set logging.
template <int DEPTH>
__device__ __forceinline__ int32_t TXReadOnly(const VersionStore& vs, uint32_t addr, uint32_t ts,
                                              bool* isAborted) {
  int32_t v = 0;
  if (!read_version<DEPTH>(vs.slots + (size_t)addr * DEPTH, ts, v)) *isAborted = true;
  return v;
}

// TXPreValidation (batchedAtrInsert/csmv_sh/API.cu:94-191), warp-collective. Lane l's conflict
// bit i is set when a lower active lane i writes an address lane l read; lanes then resolve in
// lane order: commit iff no conflicting lower lane committed (a conflict with an aborted lane is
// dropped) - the fixpoint the reference reaches with its TA/A/C shuffle rounds. Returns the
// warp's commit mask (same value in every lane).
template <int MAXR, int MAXW>
__device__ __forceinline__ uint32_t TXPreValidation(const ReadSet<MAXR>& rs,
                                                    const WriteSet<MAXW>& ws, bool active) {
  const uint32_t me = lane_id();
  uint32_t conflict = 0;
  for (uint32_t i = 0; i < 31; i++) {
    uint32_t nw = __shfl_sync(0xFFFFFFFFu, active ? ws.n : 0u, i);
#pragma unroll
    for (int j = 0; j < MAXW; j++) {
      uint32_t a = __shfl_sync(0xFFFFFFFFu, ws.addr[j], i);
      bool hit = false;
#pragma unroll
      for (int k = 0; k < MAXR; k++) hit |= (k < (int)rs.n) && (rs.addr[k] == a);
      if (active && i < me && (uint32_t)j < nw && hit) conflict |= 1u << i;
    }
  }
  uint32_t commit = 0;
  for (uint32_t i = 0; i < 32; i++) {
    uint32_t b = __ballot_sync(0xFFFFFFFFu, me == i && active && (conflict & commit) == 0);
    commit |= b;
  }
  return commit;
}

// Lanes below this one (among the active lanes) whose write sets share an address with this
// lane's write set, warp-collective. The stamp protocol lets only the lowest writer of an
// address in a warp try for its lock, so the warp's outcome never depends on which lane's atomic
// the memory system serves first.
template <int MAXW>
__device__ __forceinline__ uint32_t TXWriteOverlap(const WriteSet<MAXW>& ws, bool active) {
  const uint32_t me = lane_id();
  uint32_t overlap = 0;
  for (uint32_t i = 0; i < 31; i++) {
    const uint32_t nw = __shfl_sync(0xFFFFFFFFu, active ? ws.n : 0u, i);
#pragma unroll
    for (int j = 0; j < MAXW; j++) {
      const uint32_t a = __shfl_sync(0xFFFFFFFFu, ws.addr[j], i);
      bool hit = false;
#pragma unroll
      for (int k = 0; k < MAXW; k++) hit |= (k < (int)ws.n) && (ws.addr[k] == a);
      if (active && i < me && (uint32_t)j < nw && hit) overlap |= 1u << i;
    }
  }
  return overlap;
}

// Slot to overwrite with a new version: an empty slot first, else the oldest - the slot the
// reference frees by advancing tail (bank/csmv_sh/API.cu:157-161). Lowest index on ties.
template <int DEPTH>
__device__ __forceinline__ int victim_slot(const unsigned long long* item) {
  unsigned long long s[DEPTH];
#pragma unroll
  for (int d = 0; d < DEPTH; d += 2) ld_relaxed_gpu_v2(item + d, s[d], s[d + 1]);
  int v = 0;
  uint32_t key = version_ts(s[0]) + 1u;
#pragma unroll
  for (int d = 1; d < DEPTH; d++) {
    uint32_t k = version_ts(s[d]) + 1u;
    if (k < key) {
      key = k;
      v = d;
    }
  }
  return v;
}

// TXWriteBack (bank/csmv_sh/API.cu:147-190): install every buffered write as version `ts`.
// The reference needs three fence-separated phases (tail, slot, head) because a reader could
// see a half-written version; a packed slot is written by one 8-byte store, so one fence at
// the end (by the caller, before it publishes the clock) suffices. Callers hold the commit
// for these items: validation guarantees no other committed writer of them is in flight.
template <int DEPTH, int MAXW>
__device__ __forceinline__ void TXWriteBack(uint32_t ts, const VersionStore& vs,
                                            const WriteSet<MAXW>& ws) {
#pragma unroll
  for (int i = 0; i < MAXW; i++) {
    if (i < (int)ws.n) {
      unsigned long long* item = vs.slots + (size_t)ws.addr[i] * DEPTH;
      int d = victim_slot<DEPTH>(item);
      st_relaxed_gpu(item + d, pack_version(ts, ws.val[i]));
    }
  }
}

}  // namespace csmv
