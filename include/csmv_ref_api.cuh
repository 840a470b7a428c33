// csmv_ref_api.cuh - the reference's per-thread device API, with its argument lists, on the GB300
// version store.
//
// A driver written against the reference's header (csmv_optimizations/batchedAtrInsert/csmv_sh/
// API.cuh:139-151) compiles against this one unchanged in its calls:
//   uint TXBegin(uint tid, writeSet* ws, readSet* rs)
//   int  TXRead(VertionedDataItem* data, int addr, uint ts, readSet* rs, writeSet* ws, uint tid,
//               bool* isAborted)
//   int  TXReadOnly(...same...)
//   bool TXWrite(VertionedDataItem* data, int value, int addr, writeSet* ws, uint tid)
//   bool TXPreValidation(uint tid, readSet* rs, writeSet* ws)                 (warp-collective)
//   int  TXAddToRecord(TMmetadata*, TXRecord*, readSet*, writeSet*, Statistics*, time_rate*,
//                      int ts, int tid)                                         (warp-collective)
//   void TXWriteBack(int ts, VertionedDataItem* data, writeSet ws)              (warp-collective)
// with the same meaning: read sets and write sets are per-thread records in global memory
// indexed by tid; an abort is *isAborted = true or a TXAddToRecord result of 0; ts = -1 asks
// TXAddToRecord for nothing (the lane has already decided); the clock advances in commit order.
//
// What differs underneath (and why):
//  * VertionedDataItem is the packed item of this project: CSMV_REF_DEPTH 64-bit (ts << 32 |
//    value) slots, newest version = largest ts, empty slot ts 0xFFFFFFFF - one single-copy-atomic
//    access per version instead of the reference's head/tail ring of separate arrays
//    (bank/csmv_sh/API.cuh:61-67), so a reader never sees a half-written version;
//  * TXAddToRecord runs in the calling warp against a commit-record ring and metadata in global
//    memory (the reference's "gb" form, bank/csmv_gb/API.cuh:12), inside a commit section
//    taken by the warp's lowest live lane; there is no separate server kernel to spin on, and
//    every wait is bounded (CSMV_REF_SPIN polls; a wait that runs out aborts the attempt and
//    sets csmv_ref_error);
//  * the record ring's RecordAge rule and the plain validation rule are the reference's
//    (bank/csmv_sh/API.cu:88-144): a read set conflicts with any record newer than the snapshot
//    that wrote one of its addresses, and a snapshot older than the ring's oldest record aborts.
// The caller allocates the items (n x sizeof(VertionedDataItem)), the read and write sets (one per
// thread), a TMmetadata and a TXRecord ring of CSMV_REF_RECORDS entries, all zeroed except the
// items' initial versions (value at ts 0, the other slots empty: csmv_ref_init_item), and sets
// csmv_ref_clock and csmv_ref_error to 0 before the kernel runs. The header defines these two
// device variables: include it in one translation unit of a program.
#pragma once
#include <cstdint>

#include "csmv_tx.cuh"

#ifndef CSMV_REF_DEPTH
#define CSMV_REF_DEPTH 4
#endif
#ifndef CSMV_REF_MAX_READS
#define CSMV_REF_MAX_READS 64  // the reference reserves 1024 per thread (API.cuh:18)
#endif
#ifndef CSMV_REF_RECORDS
#define CSMV_REF_RECORDS 4096  // power of two
#endif
#ifndef CSMV_REF_SPIN
#define CSMV_REF_SPIN (1u << 22)
#endif
#define CSMV_REF_MAX_WRITES 2  // MaxWriteSetSize of the bank (API.cuh:17)

typedef unsigned int uint;
typedef unsigned short ushort;

struct VertionedDataItem {
  unsigned long long slot[CSMV_REF_DEPTH];
};
struct TMmetadata {
  uint lock;      // commit section: 0 free, 1 held
  uint frontier;  // timestamp of the last record appended
  uint pad[30];
};
struct TXRecord {
  uint transactionNumber;
  ushort n_writes;
  uint writeSet[CSMV_REF_MAX_WRITES];
};
struct readSet {
  ushort size;
  uint addrs[CSMV_REF_MAX_READS];
};
struct writeSet {
  ushort size;
  uint addrs[CSMV_REF_MAX_WRITES];
  int value[CSMV_REF_MAX_WRITES];
};
struct Statistics {
  int nbCommits;
  int nbAbortsRecordAge;
  int nbAbortsReadWrite;
  int nbAbortsPreValid;
  int nbAbortsDataAge;
};
struct time_rate {  // the reference's per-thread timing fields; kept for the signatures only
  long long int total, runtime, commit, dataWrite, val1, val2, recordWrite, wait, preValidation,
      wastedTime;
  long int comparisons, nbReadOnly, nbUpdates;
};

__device__ uint csmv_ref_clock;  // every commit with ts <= csmv_ref_clock is written back
__device__ uint csmv_ref_error;  // set to 1 when a bounded wait of this API ran out

__host__ __device__ inline VertionedDataItem csmv_ref_init_item(int value) {
  VertionedDataItem it;
  it.slot[0] = (unsigned long long)(uint32_t)value;  // ts 0
  for (int d = 1; d < CSMV_REF_DEPTH; d++) it.slot[d] = 0xFFFFFFFFull << 32;
  return it;
}

// TXBegin (batchedAtrInsert/csmv_sh/API.cu:392-397): empty sets, snapshot = clock.
__device__ inline uint TXBegin(uint tid, writeSet* ws, readSet* rs) {
  rs[tid].size = 0;
  ws[tid].size = 0;
  return csmv::ld_acquire_gpu(&csmv_ref_clock);
}

// TXRead (API.cu:12-48): read-your-writes, else the newest version <= ts (none: DataAge abort);
// the address joins the read set.
__device__ inline int TXRead(VertionedDataItem* data, int addr, uint timestamp, readSet* rs,
                             writeSet* ws, uint tid, bool* isAborted) {
  for (int i = 0; i < ws[tid].size; i++)
    if ((uint)addr == ws[tid].addrs[i]) {
      if (rs[tid].size < CSMV_REF_MAX_READS) rs[tid].addrs[rs[tid].size++] = (uint)addr;
      return ws[tid].value[i];
    }
  int32_t v = 0;
  if (!csmv::read_version<CSMV_REF_DEPTH>(data[addr].slot, timestamp, v)) {
    *isAborted = true;
    return 0;
  }
  if (rs[tid].size < CSMV_REF_MAX_READS)
    rs[tid].addrs[rs[tid].size++] = (uint)addr;
  else
    *isAborted = true;  // read set full: the transaction cannot be validated
  return v;
}

// TXReadOnly (API.cu:50-73): the version rule without read-set logging.
__device__ inline int TXReadOnly(VertionedDataItem* data, int addr, uint timestamp, readSet* rs,
                                 writeSet* ws, uint tid, bool* isAborted) {
  (void)rs;
  (void)ws;
  (void)tid;
  int32_t v = 0;
  if (!csmv::read_version<CSMV_REF_DEPTH>(data[addr].slot, timestamp, v)) *isAborted = true;
  return v;
}

// TXWrite (API.cu:75-91): buffer (addr, value), overwriting an earlier write of the address.
__device__ inline bool TXWrite(VertionedDataItem* data, int value, int addr, writeSet* ws, uint tid) {
  (void)data;
  for (int i = 0; i < ws[tid].size; i++)
    if ((uint)addr == ws[tid].addrs[i]) {
      ws[tid].value[i] = value;
      return true;
    }
  if (ws[tid].size >= CSMV_REF_MAX_WRITES) return false;
  ws[tid].addrs[ws[tid].size] = (uint)addr;
  ws[tid].value[ws[tid].size] = value;
  ws[tid].size++;
  return true;
}

// TXPreValidation (batchedAtrInsert/csmv_sh/API.cu:94-191), warp-collective over the lanes that
// call it together: a lane passes unless a lower passing lane writes an address it read.
__device__ inline bool TXPreValidation(uint tid, readSet* rs, writeSet* ws) {
  const uint32_t active = __activemask();
  const uint32_t me = csmv::lane_id();
  uint32_t conflict = 0;
  // every lane compares its read set with the write sets of the lower active lanes, whose tids
  // come through shuffles of the whole active group
  for (uint32_t i = 0; i < 32; i++) {
    if (!((active >> i) & 1u)) continue;
    const uint32_t ot = __shfl_sync(active, tid, i);
    if (i >= me) continue;
    for (int j = 0; j < ws[ot].size; j++)
      for (int k = 0; k < rs[tid].size; k++)
        if (rs[tid].addrs[k] == ws[ot].addrs[j]) conflict |= 1u << i;
  }
  uint32_t pass = 0;
  for (uint32_t i = 0; i < 32; i++) {
    if (!((active >> i) & 1u)) continue;
    pass |= __ballot_sync(active, me == i && (conflict & pass) == 0u);
  }
  return (pass >> me) & 1u;
}

// Validation of one transaction's read set against the records with ts in (snap, frontier]
// (bank/csmv_sh/API.cu:88-144): RecordAge when the ring no longer reaches back to snap.
__device__ inline bool csmv_ref_validate(const TXRecord* rec, uint snap, uint frontier,
                                         const readSet& rs, Statistics* stats) {
  if ((unsigned long long)snap + CSMV_REF_RECORDS < (unsigned long long)frontier) {
    atomicAdd(&stats->nbAbortsRecordAge, 1);
    return false;
  }
  for (uint t = snap + 1; t <= frontier; t++) {
    const TXRecord& r = rec[t & (CSMV_REF_RECORDS - 1)];
    for (int j = 0; j < r.n_writes; j++)
      for (int k = 0; k < rs.size; k++)
        if (rs.addrs[k] == r.writeSet[j]) {
          atomicAdd(&stats->nbAbortsReadWrite, 1);
          return false;
        }
  }
  return true;
}

// TXAddToRecord (batchedAtrInsert/csmv_sh/API.cu:266-389), warp-collective over the lanes that
// call it together: lanes with timestamp >= 0 are validated inside one commit section taken by
// the warp's lowest such lane, the survivors take consecutive commit timestamps in lane order and
// append their records. Returns the lane's commit timestamp, 0 for an abort (or for ts = -1).
__device__ inline int TXAddToRecord(TMmetadata* metadata, TXRecord* TxRecords, readSet* read_log,
                                    writeSet* write_log, Statistics* stats, time_rate* times,
                                    int timestamp, int tid) {
  (void)times;
  const uint32_t active = __activemask();
  const uint32_t me = csmv::lane_id();
  const uint32_t want = __ballot_sync(active, timestamp >= 0);
  if (want == 0u) return 0;
  const uint32_t leader = (uint32_t)(__ffs(want) - 1);
  bool got = true;
  if (me == leader) {
    got = false;
    for (uint32_t it = 0; it < CSMV_REF_SPIN && !got; it++) {
      got = atomicCAS(&metadata->lock, 0u, 1u) == 0u;
      if (!got) __nanosleep(64);
    }
  }
  got = __shfl_sync(active, got, leader);
  if (!got) {  // the commit section never came: abort, the caller retries
    if (me == leader) atomicExch(&csmv_ref_error, 1u);
    return 0;
  }
  __threadfence();
  const uint frontier = *(volatile uint*)&metadata->frontier;
  const bool live = timestamp >= 0 && csmv_ref_validate(TxRecords, (uint)timestamp, frontier,
                                                        read_log[tid], stats);
  const uint32_t pass = __ballot_sync(active, live);
  int ts = 0;
  if (live) {
    ts = (int)(frontier + 1u + __popc(pass & csmv::lanemask_lt()));
    TXRecord& r = TxRecords[(uint)ts & (CSMV_REF_RECORDS - 1)];
    r.transactionNumber = (uint)ts;
    r.n_writes = write_log[tid].size;
    for (int i = 0; i < write_log[tid].size; i++) r.writeSet[i] = write_log[tid].addrs[i];
    atomicAdd(&stats->nbCommits, 1);
  }
  __threadfence();
  __syncwarp(active);
  if (me == leader) {
    metadata->frontier = frontier + __popc(pass);
    __threadfence();
    atomicExch(&metadata->lock, 0u);
  }
  return ts;
}

// TXWriteBack (batchedAtrInsert/csmv_sh/API.cu:231-263), warp-collective over the lanes that call
// it together: every committed lane (ts > 0) installs its writes (victim = empty, else oldest
// slot), then the lowest committed lane waits (bounded) until the clock reaches its batch and
// advances it over the batch's timestamps.
__device__ inline void TXWriteBack(int newtimestamp, VertionedDataItem* data, writeSet write_log) {
  const uint32_t active = __activemask();
  const uint32_t wb = __ballot_sync(active, newtimestamp > 0);
  if (newtimestamp > 0)
    for (int i = 0; i < write_log.size; i++) {
      unsigned long long* item = data[write_log.addrs[i]].slot;
      const int d = csmv::victim_slot<CSMV_REF_DEPTH>(item);
      csmv::st_relaxed_gpu(item + d, csmv::pack_version((uint32_t)newtimestamp, write_log.value[i]));
    }
  __threadfence();
  __syncwarp(active);
  if (wb == 0u) return;
  const uint32_t leader = (uint32_t)(__ffs(wb) - 1);
  const int first = __shfl_sync(active, newtimestamp, leader);
  if (csmv::lane_id() == leader) {
    bool moved = false;
    for (uint32_t it = 0; it < CSMV_REF_SPIN && !moved; it++) {
      if (csmv::ld_acquire_gpu(&csmv_ref_clock) == (uint)first - 1u) {
        csmv::st_release_gpu(&csmv_ref_clock, (uint)first - 1u + __popc(wb));
        moved = true;
      } else {
        __nanosleep(32);
      }
    }
    if (!moved) atomicExch(&csmv_ref_error, 1u);
  }
  __syncwarp(active);
}
