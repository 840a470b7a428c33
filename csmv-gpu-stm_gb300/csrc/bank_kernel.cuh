// bank_kernel.cuh - persistent CSMV commit kernel for the bank workload (sm_103a).
//
// Reference structure (bank/csmv_sh/exe.cu:89-338, sync_lib/*): client warps in many blocks send
// (tid, snapshot) messages through a global-memory ring to ONE server block; a leader warp hands
// 32-message chunks to worker warps, which validate against a commit-record ring in that block's
// shared memory, take a commit timestamp with a CAS on w_hp, answer through a global scoreboard,
// and client warps write back and advance a global clock one warp at a time.
//
// GB300 structure (one kernel, every CTA alike, all CTAs co-resident via cooperative launch):
//  * warps 1..nc of a CTA are client warps, warp 0 is that CTA's commit server; client and server
//    talk through shared-memory mailboxes (the csmv_sh form: no global message ring, no leader);
//  * two commit protocols share the kernel:
//    - stamp (CSMV_VALIDATE_STAMP, the default): every item carries a 64-bit commit word
//      {stamp = ts of its last committed writer, owner = warp holding its write lock}. A client
//      warp locks its candidates' write items (one CAS each), posts the count to its server, which
//      draws consecutive commit timestamps for every ready warp of the CTA with ONE atomicAdd and
//      replies; the client then validates its reads against the commit words (stamp <= snapshot,
//      no foreign lock), writes back, and releases each lock by publishing the new stamp. Lock ->
//      timestamp -> validate is the order that makes this serialisable (the TL2 argument); no
//      warp waits for any other CTA, so there is no global serial section;
//    - ring (CSMV_VALIDATE_RING / RING_LANE, the reference algorithm): the server takes a ticket
//      on a global commit order, and when its turn comes validates its batch against the
//      commit-record ring (snapshot, frontier], gives survivors consecutive timestamps, appends
//      their records and passes the turn on with one release store;
//  * the clock (snapshot source) covers every timestamp whose write-back is complete: a
//    completion bitmap indexed by timestamp, advanced by whichever warp completes the prefix.
#pragma once
#include <cstddef>
#include <cstdint>

#include "../../include/csmv.h"
#include "../../include/csmv_tx.cuh"
#include <cooperative_groups.h>

#include "csmv_prims.cuh"

namespace csmv {

constexpr uint32_t kSnapFlag = 0x80000000u;
constexpr uint32_t kHole = 0xFFFFFFFFu;  // log entry of a timestamp whose transaction aborted
constexpr uint32_t kPendingFlag = 0x80000000u;  // lock word: holder's commit timestamp is known
// Group commit: lock word of a holder that holds every lock of its group and is drawing its
// timestamps (bit 31 clear). A holder without it is still acquiring, so its timestamps will be
// drawn after any validator that sees it - that validator may ignore its lock.
constexpr uint32_t kReadyFlag = 0x40000000u;
constexpr int kMaxClientWarps = 15;
constexpr int kHashSize = 4096;  // shared-memory hash entries (power of two)
constexpr int kBatchDescs = 32;

enum StatIdx {
  ST_COMMIT_UPDATE,
  ST_COMMIT_RO,
  ST_COMMIT_NOWRITE,
  ST_ABORT_DATA_AGE,
  ST_ABORT_RECORD_AGE,
  ST_ABORT_READ_WRITE,
  ST_ABORT_PREVALID,
  ST_ABORT_WRITE_WRITE,
  ST_SECTIONS,
  ST_ROUNDS,
  ST_COUNT
};

// Global words of the commit order, each on its own 128-byte line.
struct alignas(128) GlobalSync {
  alignas(128) unsigned long long turn;  // ring protocol: low 32 ticket served, high 32 last ts
  alignas(128) uint32_t ticket;          // ring protocol: next ticket
  alignas(128) uint32_t clock;           // every commit with ts <= clock is written back
  alignas(128) uint32_t ts_next;         // stamp protocol: last timestamp handed out
  alignas(128) uint32_t round_next;      // next unclaimed round of the stream (main queue)
  alignas(128) uint32_t round_deferred;  // next unclaimed round of the deferred queue
  alignas(128) uint32_t error;           // first device error (ERR_*)
  alignas(128) uint32_t section;         // baseline arm: next ticket of the commit section
  alignas(128) uint32_t section_serving; // baseline arm: the ticket whose warp holds the section
};

struct BankParams {
  const uint32_t* op;
  const uint32_t* off;
  const uint32_t* addr;
  uint32_t n_rounds;
  uint32_t n_items;
  unsigned long long* slots;
  unsigned long long* cw;  // per item: stamp | lock << 32; lock = 0 free, warp id + 1 while the
                           // holder's timestamp is unknown, kPendingFlag | ts once it is known
  uint4* ring;             // {ts, n_writes, w0, w1}
  uint32_t ring_mask;
  uint32_t* done;          // completion bitmap, one bit per timestamp (ring of done_mask+1 words)
  uint32_t done_mask;
  GlobalSync* gs;
  uint32_t* log_txn;
  uint32_t* outcome;
  int32_t* result;
  unsigned long long* stats;  // [ST_COUNT]
  uint32_t log;
  uint32_t log_base;  // last commit ts before this run: log_txn is indexed by ts-1-log_base
  uint32_t log_cap;   // entries of log_txn (aborted stamp-protocol commits leave holes)
  uint32_t nc;        // client warps per CTA
  uint32_t validate, writeback, batch, prevalidate;
  uint32_t spin_log2;
  uint32_t* txn_aborts;     // optional [n_rounds*32]: failed attempts of each transaction
  uint32_t split_round;     // rounds [split_round, n_rounds) form the deferred queue (0 = none)
  uint32_t deferred_warps;  // client warps (lowest global ids) that serve the deferred queue
  const uint32_t* lane_start;  // optional [deferred_warps + 1]: the deferred queue as one lane of
                               // rounds per deferred warp, each served in order by its warp
  uint32_t* grp;            // group commit with log: bit (ts-1-log_base) = ts ends a commit group
  uint32_t* txn_waits;      // optional [n_rounds*32]: 1 when the transaction's group waited for a
                            // lock another warp held (group commit)
  uint32_t* tk;             // group commit: per account {next ticket, ticket served} of its
                            // lock's wait queue
  uint32_t grace;            // group commit: polls a head keeps trying its other locks
  uint32_t read_wait;        // group commit: polls for an earlier group's lock on a foreign read
                             // before the lane gives up (0 = 4096)
  const uint8_t* lock_last;  // group commit, optional [n_items]: heat class of each account
                             // (0 = none); classed accounts are locked after all others, the
                             // hottest last
  const uint32_t* backoff;  // optional [n_rounds*32]: longest pause (ns) before a retry of each
                            // transaction (a scheduler's per-transaction backoff)
};

template <int MAXR, int MAXW>
struct MailSlot {
  uint32_t req, rep;      // request / reply sequence numbers
  uint32_t snap, cand;    // request: snapshot, candidate lanes (stamp: locked lanes)
  uint32_t ok, bid;       // reply: committed lanes (ring), batch descriptor of the clock advance
  uint32_t base, pad;     // reply (stamp): last timestamp before this warp's range
  uint32_t tsl[32];       // reply (ring): commit timestamp of each committed lane
  uint32_t rs[MAXR][32];  // read sets, transposed (lane-contiguous: no bank conflicts)
  uint32_t ws[MAXW][32];
  int32_t wv[MAXW][32];
  uint32_t n[32];         // nreads | nwrites << 8
  uint32_t txn[32];
};

struct BatchDesc {
  uint32_t first_ts, last_ts, remaining, pad;
};

template <int MAXR, int MAXW>
struct CtaShared {
  uint32_t done_warps;
  uint32_t next_bid;
  uint32_t pad[2];
  unsigned long long stat[ST_COUNT];
  BatchDesc batch[kBatchDescs];
  alignas(16) uint32_t hkey[kHashSize];  // cleared with 16-byte stores
  alignas(16) uint32_t hval[kHashSize];
  uint32_t conflict[32];  // ring: per-warp conflict lanes
  uint32_t recage[32];    // ring: per-warp record-age lanes
  uint32_t snaps[32];     // ring: snapshot of each batch warp
  MailSlot<MAXR, MAXW> mail[1];  // nc slots (dynamic shared memory)
};

using CtaShared8x2 = CtaShared<8, 2>;
static_assert(offsetof(CtaShared8x2, hkey) % 16 == 0, "hash table must be 16-byte aligned");

template <int MAXR, int MAXW>
__host__ __device__ constexpr size_t cta_shared_bytes(uint32_t nc) {
  return sizeof(CtaShared<MAXR, MAXW>) + (nc - 1) * sizeof(MailSlot<MAXR, MAXW>);
}

// Group commit (prevalidate == 3): per-client-warp table of the accounts the warp's round may
// write (at most 64: two per lane), their writer lanes, lock state and latest committed value,
// plus each lane's chain outputs. Lives in dynamic shared memory after the mailboxes.
constexpr int kGrpSlots = 128;  // power of two, >= 2 x 64
constexpr uint32_t kGrpEmpty = 0xFFFFFFFFu;
struct GroupScratch {
  uint32_t key[kGrpSlots];    // account (kGrpEmpty = free)
  uint32_t wmask[kGrpSlots];  // lanes whose transfer may write it
  uint32_t busy[kGrpSlots];   // 1 when its lock was held by another warp at the first try
  int32_t base[kGrpSlots];    // its latest committed value, read under the warp's lock
  int32_t out0[32], out1[32]; // per lane: value written to its debit / credit account
  uint32_t wa0[32], wa1[32];  // per lane: its debit / credit account
  // the chain walk's inputs per lane: table slots of its accounts, the part of its amount sum
  // read outside the table, the slots of its other table reads, and its amount divisor
  uint32_t cs[32];            // slot of a0 | slot of a1 << 8 | table reads << 16 | always << 24
  uint32_t facc[32];
  unsigned long long tr[32];  // up to 8 slots, one byte each
  uint32_t md[32], mm[32];    // divisor and its multiply-shift magic
};

__host__ __device__ constexpr size_t group_scratch_offset(size_t cta_bytes) {
  return (cta_bytes + 15u) & ~size_t(15u);
}

__device__ __forceinline__ uint32_t grp_hash(uint32_t a) { return (a * 0x9E3779B1u) >> 25; }

// Slot of account x in the warp's table, inserting it (lanes of one warp insert concurrently).
__device__ __forceinline__ int grp_insert(GroupScratch& gx, uint32_t x) {
  uint32_t h = grp_hash(x);
  for (uint32_t probe = 0; probe < (uint32_t)kGrpSlots; probe++) {
    const uint32_t prev = atomicCAS(&gx.key[h], kGrpEmpty, x);
    if (prev == kGrpEmpty || prev == x) return (int)h;
    h = (h + 1u) & (kGrpSlots - 1u);
  }
  return -1;  // unreachable: at most 64 keys
}

__device__ __forceinline__ int grp_find(const GroupScratch& gx, uint32_t x) {
  uint32_t h = grp_hash(x);
  for (uint32_t probe = 0; probe < (uint32_t)kGrpSlots; probe++) {
    const uint32_t k = gx.key[h];
    if (k == x) return (int)h;
    if (k == kGrpEmpty) return -1;
    h = (h + 1u) & (kGrpSlots - 1u);
  }
  return -1;
}

__device__ __forceinline__ uint32_t hash_addr(uint32_t a) {
  a *= 0x9E3779B1u;
  return (a ^ (a >> 15)) & (kHashSize - 1);
}

__device__ __forceinline__ void stat_add(unsigned long long* s, int idx, uint32_t v) {
  if (v) atomicAdd(&s[idx], (unsigned long long)v);
}

__device__ __forceinline__ uint32_t* owner_word(unsigned long long* cw, uint32_t x) {
  return reinterpret_cast<uint32_t*>(cw + x) + 1;  // high half of the little-endian word
}

// Writes of a transfer given the values it read (include/csmv.h): amount from amt0 and the extra
// reads, debit a0 / credit a1 when funds suffice (always for CSMV_KIND_TRANSFER_ALWAYS).
template <int MAXR>
__device__ __forceinline__ bool transfer_writes(uint32_t op, uint32_t nr, const int32_t (&v)[MAXR],
                                                int32_t& w0, int32_t& w1) {
  uint32_t acc = CSMV_OP_AMT0(op) - 1u;
#pragma unroll
  for (int k = 2; k < MAXR; k++)
    if (k < (int)nr) acc += (uint32_t)v[k];
  const uint32_t amt = 1u + acc % CSMV_OP_AMOD(op);
  w0 = (int32_t)((uint32_t)v[0] - amt);
  w1 = (int32_t)((uint32_t)v[1] + amt);
  return CSMV_OP_KIND(op) == CSMV_KIND_TRANSFER_ALWAYS || v[0] >= (int32_t)amt;
}

// acc % d for a divisor fixed over a round, without a hardware divide: q = umulhi(acc, m) with
// m = floor((2^32 - 1) / d) is floor(acc / d) or one less, so one correction gives the remainder.
struct ModMagic {
  uint32_t d, m;
  __device__ __forceinline__ explicit ModMagic(uint32_t div) : d(div), m(0xFFFFFFFFu / div) {}
  __device__ __forceinline__ uint32_t mod(uint32_t acc) const {
    uint32_t r = acc - __umulhi(acc, m) * d;
    return r >= d ? r - d : r;
  }
};

template <int MAXR>
__device__ __forceinline__ bool transfer_writes(uint32_t op, uint32_t nr, const int32_t (&v)[MAXR],
                                                const ModMagic& mm, int32_t& w0, int32_t& w1) {
  uint32_t acc = CSMV_OP_AMT0(op) - 1u;
#pragma unroll
  for (int k = 2; k < MAXR; k++)
    if (k < (int)nr) acc += (uint32_t)v[k];
  const uint32_t amt = 1u + mm.mod(acc);
  w0 = (int32_t)((uint32_t)v[0] - amt);
  w1 = (int32_t)((uint32_t)v[1] + amt);
  return CSMV_OP_KIND(op) == CSMV_KIND_TRANSFER_ALWAYS || v[0] >= (int32_t)amt;
}

// Install versions (ts, value) into an item whose lock the caller holds: `n` insertions applied
// to the item's slots in registers (victim = empty, else oldest), then stored back.
template <int DEPTH>
struct SlotEditor {
  unsigned long long s[DEPTH];
  __device__ __forceinline__ void load(const unsigned long long* item) {
#pragma unroll
    for (int d = 0; d < DEPTH; d += 2) ld_relaxed_gpu_v2(item + d, s[d], s[d + 1]);
  }
  __device__ __forceinline__ void insert(uint32_t ts, int32_t v) {
    int vic = 0;
    uint32_t key = version_ts(s[0]) + 1u;
#pragma unroll
    for (int d = 1; d < DEPTH; d++) {
      const uint32_t k = version_ts(s[d]) + 1u;
      if (k < key) {
        key = k;
        vic = d;
      }
    }
#pragma unroll
    for (int d = 0; d < DEPTH; d++)
      if (d == vic) s[d] = pack_version(ts, v);
  }
  __device__ __forceinline__ void store(unsigned long long* item) const {
#pragma unroll
    for (int d = 0; d < DEPTH; d++) st_relaxed_gpu(item + d, s[d]);
  }
  // value of the version with timestamp ts (false when the slots do not hold it)
  __device__ __forceinline__ bool find(uint32_t ts, int32_t& v) const {
    bool f = false;
#pragma unroll
    for (int d = 0; d < DEPTH; d++)
      if (version_ts(s[d]) == ts) {
        v = version_val(s[d]);
        f = true;
      }
    return f;
  }
};

// ---------------------------------------------------------------------------------------------
// clock: completion bitmap
// ---------------------------------------------------------------------------------------------

// Mark timestamps [lo, hi] complete (their write-back is visible), then move the clock over the
// longest complete prefix. Any warp may advance: a CAS keeps the clock monotonic, and the warp
// that passes the end of a bitmap word clears it for the next lap. Called by one lane.
// A range is published atomically for the clock: its bitmap words are set from the highest down,
// fenced, and the scan below reads words with acquire loads in ascending order, so a scan that
// sees the range's lowest bits sees all of them - the clock never stops inside a range (a group
// commit's intermediate versions are never installed, and no snapshot may fall between them).
static __device__ void complete_range(uint32_t* done, uint32_t done_mask, GlobalSync* gs, uint32_t lo,
                               uint32_t hi) {
  __threadfence();
  for (uint32_t w = hi >> 5;; w--) {
    const uint32_t t0 = max(lo, w << 5), t1 = min(hi, (w << 5) + 31u);
    const uint32_t span = t1 - t0 + 1u, bit = t0 & 31u;
    const uint32_t m = (span == 32u ? 0xFFFFFFFFu : ((1u << span) - 1u)) << bit;
    atomicOr(&done[w & done_mask], m);
    if (w == (lo >> 5)) break;
    __threadfence();
  }
  // store-buffering pattern with the warp completing the range below ours: with SC fences on
  // both sides at least one of us sees the other's bits, so the clock never stalls
  __threadfence();
  for (uint32_t attempt = 0; attempt < 4096; attempt++) {
    const uint32_t c = ld_acquire_gpu(&gs->clock);
    uint32_t n = c;
    // scan to the first incomplete timestamp, never a fixed number of words: a scan cut short
    // could end inside a range and publish a clock no snapshot may take (at most the whole
    // bitmap, which holds every timestamp in flight)
    for (uint32_t words = 0; words <= done_mask; words++) {
      const uint32_t t = n + 1, bit = t & 31u;
      const uint32_t w = ld_acquire_gpu(&done[(t >> 5) & done_mask]) >> bit;
      const uint32_t ones = (w == 0xFFFFFFFFu) ? 32u : (uint32_t)(__ffs(~w) - 1);
      const uint32_t run = min(ones, 32u - bit);
      n += run;
      if (run < 32u - bit) break;
    }
    if (n == c) return;  // c+1 not complete yet: its owner will advance past us
    __threadfence();
    if (atomicCAS(&gs->clock, c, n) == c) {
      // clear every word whose last timestamp this advance passed
      for (uint32_t wd = (c + 1) >> 5; wd <= (n >> 5); wd++)
        if (wd * 32u + 31u <= n) st_relaxed_gpu(&done[wd & done_mask], 0u);
    }
  }
}

// ---------------------------------------------------------------------------------------------
// ring protocol: per-batch clock advance in timestamp order (the reference's leader spin,
// batchedAtrInsert/csmv_sh/API.cu:257-261, once per batch instead of once per warp)
// ---------------------------------------------------------------------------------------------
template <int MAXR, int MAXW>
__device__ __forceinline__ void batch_done(const BankParams& p, CtaShared<MAXR, MAXW>& sm,
                                           uint32_t bid) {
  BatchDesc& d = sm.batch[bid];
  const uint32_t first = d.first_ts, last = d.last_ts;
  __threadfence();
  if (atomicSub(&d.remaining, 1u) == 1u) {
    __threadfence();
    if (bounded_wait([&] { return ld_acquire_gpu(&p.gs->clock) == first - 1u; }, &p.gs->error,
                     ERR_WAIT_CLOCK, p.spin_log2))
      st_release_gpu(&p.gs->clock, last);
  }
}

// ---------------------------------------------------------------------------------------------
// group commit (prevalidate == 3, stamp protocol)
// ---------------------------------------------------------------------------------------------

// Lock of account x by a 64-bit CAS of its commit word from (stamp, free) to (stamp, owner):
// the lock and, in the same atomic, a check that `stamp` (the version the caller read) is still
// the latest. When only the stamp moved, the lock is taken at the new stamp and *stale is set
// (the caller re-reads the value under the lock). False when another warp holds the lock.
__device__ __forceinline__ unsigned long long lock_word(uint32_t stamp, uint32_t owner) {
  return ((unsigned long long)owner << 32) | stamp;
}

__device__ __forceinline__ bool group_cas_lock(unsigned long long* cw, uint32_t x, uint32_t me,
                                               uint32_t& stamp, bool& stale) {
  for (int r = 0; r < 8; r++) {
    const unsigned long long exp = stamp;
    const unsigned long long old = atomicCAS(cw + x, exp, exp | ((unsigned long long)me << 32));
    if (old == exp) return true;
    if ((old >> 32) != 0ull) return false;
    stamp = (uint32_t)old;
    stale = true;
  }
  return false;
}

// Lock queues. Waiters for account x queue first-come first-served on the account's ticket pair
// (tk[2x] = next ticket, tk[2x + 1] = ticket being served): a warp takes a ticket, waits until it
// is served (its turn), then takes the lock as soon as its holder releases it, and serves the
// next ticket - so only the head of the queue polls the commit word, and a waiter far from the
// account's L2 slice is not overtaken forever by nearer ones (a plain polling race hands a hot
// lock to whoever sees the release first). A round's fast path (group_cas_lock) may still take a
// free lock ahead of the queue. A waiter never leaves the queue while its run is healthy (the
// tickets behind it would wait forever): the waits are bounded only by the device error word and
// by 2^spin_log2 polls, after which the run fails with ERR_WAIT_TURN.
__device__ __forceinline__ bool group_take_turn(const BankParams& p, uint32_t x) {
  uint32_t* next = p.tk + 2u * (size_t)x;
  uint32_t* serving = next + 1;
  const uint32_t mine = atomicAdd(next, 1u);
  const uint64_t limit = 1ull << min(p.spin_log2, 22u);  // at most a few seconds
  for (uint64_t it = 0; it < limit; it++) {
    const uint32_t now = ld_acquire_gpu(serving);
    if (now == mine) return true;
    if ((it & 63u) == 63u && ld_relaxed_gpu(&p.gs->error) != 0u) return false;
    __nanosleep(min(64u * (mine - now), 1024u));  // farther back in the queue: poll less often
  }
  raise_error(&p.gs->error, ERR_WAIT_TURN);
  return false;
}

__device__ __forceinline__ void group_pass_turn(const BankParams& p, uint32_t x) {
  atomicAdd(p.tk + 2u * (size_t)x + 1u, 1u);
}

// At the head of x's queue: waits for the holder's release and takes the lock, with the account's
// version slots (ed) and latest value (v) read as it is taken. The poll that finds the lock free
// is an acquire load, so the slots loaded after it hold the version of the stamp it saw, and a
// CAS that succeeds at that stamp proves them current (*stale stays false).
template <int DEPTH>
__device__ __forceinline__ bool group_lock_at_turn(const BankParams& p, uint32_t x, uint32_t me,
                                                   uint32_t& stamp, bool& stale,
                                                   SlotEditor<DEPTH>& ed, int32_t& v) {
  const uint64_t limit = 1ull << min(p.spin_log2, 22u);
  for (uint64_t it = 0; it < limit; it++) {
    const unsigned long long w = ld_acquire_gpu(&p.cw[x]);
    if ((w >> 32) == 0ull) {
      ed.load(p.slots + (size_t)x * DEPTH);
      if (atomicCAS(&p.cw[x], w, w | ((unsigned long long)me << 32)) == w) {
        stamp = (uint32_t)w;
        stale = !ed.find(stamp, v);
        return true;
      }
      continue;  // a fast-path CAS took it first: poll again
    }
    if ((it & 63u) == 63u && ld_relaxed_gpu(&p.gs->error) != 0u) break;
    __nanosleep(32);
  }
  raise_error(&p.gs->error, ERR_WAIT_TURN);
  return false;
}

// x's lock seen free as the word w (an acquire load): its slots are read and the lock taken by a
// CAS at that stamp (false when another warp took it first).
template <int DEPTH>
__device__ __forceinline__ bool group_take_seen(const BankParams& p, uint32_t x, uint32_t me,
                                                unsigned long long w, uint32_t& stamp, bool& stale,
                                                SlotEditor<DEPTH>& ed, int32_t& v) {
  ed.load(p.slots + (size_t)x * DEPTH);
  if (atomicCAS(&p.cw[x], w, w | ((unsigned long long)me << 32)) != w) return false;
  stamp = (uint32_t)w;
  stale = !ed.find(stamp, v);
  return true;
}

// Queue for x's lock and take it (the turn is served on, also when the wait failed).
template <int DEPTH>
__device__ __forceinline__ bool group_wait_lock(const BankParams& p, uint32_t x, uint32_t me,
                                                uint32_t& stamp, bool& stale,
                                                SlotEditor<DEPTH>& ed, int32_t& v) {
  if (!group_take_turn(p, x)) return false;
  const bool got = group_lock_at_turn<DEPTH>(p, x, me, stamp, stale, ed, v);
  group_pass_turn(p, x);
  return got;
}

// One attempt of a transfer round as a commit group, warp-collective. Every active lane's
// transfer may write its two accounts; the warp locks each such account once (its lowest writer
// lane does), in one total order (step 2), waiting for a lock held elsewhere while it holds only
// smaller ones (no cycle of waits is possible). Every access of this mode to a commit word is a
// full 8-byte access. The locked accounts' latest values are read under the locks; the commit
// server then gives the group consecutive timestamps in lane order; every read of an account the group does not lock (a foreign read) is validated
// against its commit word, as the stamp protocol validates any transaction; the lanes that pass
// run in lane order as a chain through the locked accounts (each reads the value left by the
// nearest lower lane that wrote it, else the locked value), so a dependent transfer never
// aborts for a lower lane of its own group; and each locked account gets ONE new version, the
// last group member's write. Intermediate versions of a group are never observable: snapshots
// come from the clock, which passes a group's timestamps at once (complete_range), and latest
// reads follow the stamp, which is published with the last version. A lane that fails
// validation leaves a hole at its timestamp and is retried; when a lock wait runs out the whole
// attempt is dropped before any timestamp is drawn (*gave_up). Returns the committed lanes.
template <int DEPTH, int MAXR, int MAXW, bool CLUSTER>
__device__ uint32_t group_attempt(const BankParams& p, CtaShared<MAXR, MAXW>& sm,
                                  MailSlot<MAXR, MAXW>& ms, GroupScratch& gx, uint32_t me,
                                  uint32_t t, uint32_t op, uint32_t nr,
                                  const uint32_t (&a)[MAXR], bool act, uint32_t& seq,
                                  bool patient, bool& gave_up, bool& failed, bool& waited,
                                  bool& sat_out) {
  constexpr uint32_t FULL = 0xFFFFFFFFu;
  const uint32_t lane = lane_id();
  const VersionStore vs{p.slots, p.n_items};
  gave_up = false;
  sat_out = false;
  // 1. the accounts the round may write, with their writer lanes
  for (uint32_t i = lane; i < (uint32_t)kGrpSlots; i += 32) {
    gx.key[i] = kGrpEmpty;
    gx.wmask[i] = 0u;
    gx.busy[i] = 0u;
  }
  __syncwarp();
  int s0 = -1, s1 = -1;
  if (act) {
    s0 = grp_insert(gx, a[0]);
    s1 = a[1] == a[0] ? s0 : grp_insert(gx, a[1]);
    atomicOr(&gx.wmask[s0], 1u << lane);
    if (s1 != s0) atomicOr(&gx.wmask[s1], 1u << lane);
    gx.wa0[lane] = a[0];
    gx.wa1[lane] = a[1];
  }
  __syncwarp();
  int rsl[MAXR];  // table slot of each read, -1 for a foreign read
#pragma unroll
  for (int k = 0; k < MAXR; k++)
    rsl[k] = (!act || k >= (int)nr) ? -1 : k == 0 ? s0 : k == 1 ? s1 : grp_find(gx, a[k]);
  const bool lead0 = act && (uint32_t)(__ffs(gx.wmask[s0]) - 1) == lane;
  const bool lead1 = act && s1 != s0 && (uint32_t)(__ffs(gx.wmask[s1]) - 1) == lane;

  // 2. locks, waiting (bounded) for locks held elsewhere, in one total order: accounts with no
  //    heat class (lock_last 0) ascending, then the classed (hot) ones by class and account, the
  //    hottest last. A group first tries every lock at once; when one is held elsewhere it
  //    settles the smallest missing lock while holding only smaller ones, queueing on a cold
  //    account's tickets. A group with hot accounts that did not get every lock at once
  //    releases all and queues, holding nothing, for its LAST lock in the order (its hottest
  //    account); at the head of that queue it takes its other locks - cold ones queued, hot
  //    ones by polling - and the hottest last, so a hot lock is held only for the commit
  //    itself, and the next group in line takes its other locks while the current holder
  //    commits. Waits follow the order turns < cold locks < hot locks, a group holds at most
  //    one turn, and a hot lock is held only by a group that holds every smaller lock it needs
  //    or is committing: no cycle of waits. A leader keeps the account's version slots from its
  //    read: the write-back edits them in registers.
  const uint32_t c0 = (lead0 && p.lock_last != nullptr) ? p.lock_last[a[0]] : 0u;
  const uint32_t c1 = (lead1 && p.lock_last != nullptr) ? p.lock_last[a[1]] : 0u;
  // order key: (tier | class, account); tier bit 31 set for hot accounts
  const uint32_t kh0 = c0 ? 0x80000000u | c0 : 0u, kh1 = c1 ? 0x80000000u | c1 : 0u;
  auto key_min = [&](bool m0, bool m1, uint32_t& fh, uint32_t& fl) {  // smallest key of a set
    const uint32_t h = min(m0 ? kh0 : 0xFFFFFFFFu, m1 ? kh1 : 0xFFFFFFFFu);
    fh = __reduce_min_sync(FULL, h);
    fl = __reduce_min_sync(FULL, min((m0 && kh0 == fh) ? a[0] : kGrpEmpty,
                                     (m1 && kh1 == fh) ? a[1] : kGrpEmpty));
  };
  auto above = [](uint32_t h, uint32_t l, uint32_t fh, uint32_t fl) {
    return h > fh || (h == fh && l > fl);
  };
  uint32_t st0 = 0, st1 = 0;
  int32_t bv0 = 0, bv1 = 0;
  SlotEditor<DEPTH> ed0, ed1;
  bool stale0 = false, stale1 = false, h0 = false, h1 = false;
  if (lead0) {
    st0 = (uint32_t)ld_acquire_gpu(&p.cw[a[0]]);
    ed0.load(p.slots + (size_t)a[0] * DEPTH);
  }
  if (lead1) {
    st1 = (uint32_t)ld_acquire_gpu(&p.cw[a[1]]);
    ed1.load(p.slots + (size_t)a[1] * DEPTH);
  }
  if (lead0) stale0 = !ed0.find(st0, bv0);
  if (lead1) stale1 = !ed1.find(st1, bv1);
  if (lead0) h0 = group_cas_lock(p.cw, a[0], me, st0, stale0);
  if (lead1) h1 = group_cas_lock(p.cw, a[1], me, st1, stale1);
  if (lead0 && !h0) gx.busy[s0] = 1u;
  if (lead1 && !h1) gx.busy[s1] = 1u;
  __syncwarp();
  waited = act && (gx.busy[s0] | gx.busy[s1]) != 0u;
  bool all = false, ok = true;
  int turn = -1;  // which of my accounts' queue turn this lane holds (the group holds at most one)
  if (__any_sync(FULL, (lead0 && !h0) || (lead1 && !h1)) && __any_sync(FULL, c0 || c1)) {
    // hot path: release all, queue (holding nothing) for the group's hottest account, and at
    // the head of its queue take the other locks by CAS whenever they look free (never waiting
    // for them) until the hottest lock itself is free, then take it. The lanes whose other
    // accounts are still held elsewhere then sit this attempt out. A round that sat out twice
    // running is patient: at the head it waits for its other locks in order, the hottest last.
    // Every waiting group holds only locks below the one it waits for (a head's held locks are
    // below its queued one), so keys rise along any chain of waits: no cycle.
    if (h0) st_relaxed_gpu(&p.cw[a[0]], (unsigned long long)st0);
    if (h1) st_relaxed_gpu(&p.cw[a[1]], (unsigned long long)st1);
    h0 = h1 = false;
    // the group's last lock: the largest key among its hot accounts
    const uint32_t qh = __reduce_max_sync(FULL, max(kh0, kh1));
    const uint32_t ql = __reduce_max_sync(FULL, max((c0 && kh0 == qh) ? a[0] : 0u,
                                                    (c1 && kh1 == qh) ? a[1] : 0u));
    bool r = true;
    if (c0 && kh0 == qh && a[0] == ql) {
      r = group_take_turn(p, a[0]);
      if (r) turn = 0;
    } else if (c1 && kh1 == qh && a[1] == ql) {
      r = group_take_turn(p, a[1]);
      if (r) turn = 1;
    }
    ok = !__any_sync(FULL, !r);
    const uint64_t limit = 1ull << min(p.spin_log2, 22u);
    for (uint64_t it = 0; ok && !patient && it < limit; it++) {
      // one round of loads in flight together: the queued lock's word and the other missing
      // ones; the queued lock is taken as soon as it is seen free, the others only when the
      // queued one is still held
      const bool o0 = lead0 && !h0 && turn != 0, o1 = lead1 && !h1 && turn != 1;
      unsigned long long wq = ~0ull, w0 = ~0ull, w1 = ~0ull;
      if (turn == 0) wq = ld_acquire_gpu(&p.cw[a[0]]);
      if (turn == 1) wq = ld_acquire_gpu(&p.cw[a[1]]);
      if (o0) w0 = ld_relaxed_gpu(&p.cw[a[0]]);
      if (o1) w1 = ld_relaxed_gpu(&p.cw[a[1]]);
      if (__any_sync(FULL, turn >= 0 && (wq >> 32) == 0ull)) {
        if (turn == 0 && (wq >> 32) == 0ull) h0 = group_take_seen<DEPTH>(p, a[0], me, wq, st0, stale0, ed0, bv0);
        if (turn == 1 && (wq >> 32) == 0ull) h1 = group_take_seen<DEPTH>(p, a[1], me, wq, st1, stale1, ed1, bv1);
      } else {
        if (o0 && (w0 >> 32) == 0ull) h0 = group_cas_lock(p.cw, a[0], me, st0, stale0);
        if (o1 && (w1 >> 32) == 0ull) h1 = group_cas_lock(p.cw, a[1], me, st1, stale1);
      }
      if (__any_sync(FULL, (turn == 0 && h0) || (turn == 1 && h1))) {
        all = true;
        // a short grace for the other locks still held elsewhere (bounded: no wait cycle can
        // form, at worst their lanes sit out)
        for (uint32_t g = 0; g < p.grace &&
                             __any_sync(FULL, (lead0 && !h0 && turn != 0) || (lead1 && !h1 && turn != 1));
             g++) {
          __nanosleep(32);
          if (lead0 && !h0 && turn != 0 && (ld_relaxed_gpu(&p.cw[a[0]]) >> 32) == 0ull)
            h0 = group_cas_lock(p.cw, a[0], me, st0, stale0);
          if (lead1 && !h1 && turn != 1 && (ld_relaxed_gpu(&p.cw[a[1]]) >> 32) == 0ull)
            h1 = group_cas_lock(p.cw, a[1], me, st1, stale1);
        }
        break;
      }
      if ((it & 63u) == 63u && __any_sync(FULL, lane == 0 && ld_relaxed_gpu(&p.gs->error) != 0u))
        break;
      __nanosleep(32);
    }
    if (ok && !patient && !all && lane == 0) raise_error(&p.gs->error, ERR_WAIT_TURN);
  }
  if (ok && !all) {
    for (uint32_t it = 0; it <= 64u; it++) {  // each pass settles the smallest missing lock
      uint32_t fh, fl;
      key_min(lead0 && !h0, lead1 && !h1, fh, fl);
      if (fl == kGrpEmpty) {
        all = true;
        break;
      }
      if (h0 && above(kh0, a[0], fh, fl)) {  // hold nothing above the lock being waited for
        st_relaxed_gpu(&p.cw[a[0]], (unsigned long long)st0);
        h0 = false;
      }
      if (h1 && above(kh1, a[1], fh, fl)) {
        st_relaxed_gpu(&p.cw[a[1]], (unsigned long long)st1);
        h1 = false;
      }
      bool r = true;  // a hot lock is polled (its queue's turn is this group's or another's)
      if (lead0 && !h0 && kh0 == fh && a[0] == fl)
        r = h0 = c0 ? group_lock_at_turn<DEPTH>(p, a[0], me, st0, stale0, ed0, bv0)
                    : group_wait_lock<DEPTH>(p, a[0], me, st0, stale0, ed0, bv0);
      else if (lead1 && !h1 && kh1 == fh && a[1] == fl)
        r = h1 = c1 ? group_lock_at_turn<DEPTH>(p, a[1], me, st1, stale1, ed1, bv1)
                    : group_wait_lock<DEPTH>(p, a[1], me, st1, stale1, ed1, bv1);
      if (__any_sync(FULL, !r)) break;
      if (lead0 && !h0 && above(kh0, a[0], fh, fl)) h0 = group_cas_lock(p.cw, a[0], me, st0, stale0);
      if (lead1 && !h1 && above(kh1, a[1], fh, fl)) h1 = group_cas_lock(p.cw, a[1], me, st1, stale1);
    }
  }
  if (turn >= 0) group_pass_turn(p, turn == 0 ? a[0] : a[1]);  // the next in line starts now
  // the accounts held; a lane sits the attempt out when one of its own is not (hot path only)
  const bool own0 = lead0 && h0, own1 = lead1 && h1;
  if (lead0) gx.busy[s0] = own0 ? 0u : 1u;
  if (lead1) gx.busy[s1] = own1 ? 0u : 1u;
  __syncwarp();
  const bool in = act && all && gx.busy[s0] == 0u && gx.busy[s1] == 0u;
  if (in) {  // a read of a table account this group does not hold becomes a foreign read
#pragma unroll
    for (int k = 2; k < MAXR; k++)
      if (rsl[k] >= 0 && gx.busy[rsl[k]] != 0u) rsl[k] = -1;
  }
  const uint32_t inc = __ballot_sync(FULL, in);
  const uint32_t actm = __ballot_sync(FULL, act);
  sat_out = all && actm != inc;
  if (!all || inc == 0u) {  // a wait ran out, or no lane can commit now: release, retry later
    if (h0) st_relaxed_gpu(&p.cw[a[0]], (unsigned long long)st0);
    if (h1) st_relaxed_gpu(&p.cw[a[1]], (unsigned long long)st1);
    gave_up = !all;
    if (all && lane == 0) stat_add(sm.stat, ST_ABORT_WRITE_WRITE, __popc(actm));
    return 0u;
  }
  // 3. latest values of the locked accounts whose slots were read before their stamp moved (the
  //    stamp cannot move while the lock is held), then the ready marks: every lock of the group
  //    is held and its timestamps are drawn next (the server's fence orders these marks before
  //    its draw: the mailbox hand-off carries them to it)
  if (__any_sync(FULL, (own0 && stale0) || (own1 && stale1))) {
    fence_acq_rel_gpu();  // the previous holders' versions are visible before they are read
    bool lost = false;
    if (own0 && stale0) {
      ed0.load(p.slots + (size_t)a[0] * DEPTH);
      lost |= !ed0.find(st0, bv0);
    }
    if (own1 && stale1) {
      ed1.load(p.slots + (size_t)a[1] * DEPTH);
      lost |= !ed1.find(st1, bv1);
    }
    if (lost) raise_error(&p.gs->error, ERR_DATA);  // the latest version must be present
  }
  if (own0) {
    gx.base[s0] = bv0;
    st_relaxed_gpu(&p.cw[a[0]], lock_word(st0, me | kReadyFlag));
  }
  if (own1) {
    gx.base[s1] = bv1;
    st_relaxed_gpu(&p.cw[a[1]], lock_word(st1, me | kReadyFlag));
  }
  __syncwarp();

  // 4. post the group to the commit server; the foreign reads run while it draws
  seq++;
  if (lane == 0) {
    ms.snap = 0u;
    ms.cand = inc;
    mail_release<CLUSTER>(&ms.req, seq);
  }
  int32_t fv[MAXR];
  uint32_t fst[MAXR];
  bool fok = true;
#pragma unroll
  for (int k = 0; k < MAXR; k++) {
    fv[k] = 0;
    fst[k] = 0u;
    if (in && k < (int)nr && rsl[k] < 0) fok &= read_latest<DEPTH>(vs, p.cw, a[k], fst[k], fv[k]);
  }
  bool ok_wait = true;
  if (lane == 0)  // the hottest lock is held: spin on the reply before sleeping between polls
    ok_wait = bounded_wait_fast([&] { return mail_acquire<CLUSTER>(&ms.rep) == seq; },
                                &p.gs->error, ERR_WAIT_REPLY, p.spin_log2);
  ok_wait = __shfl_sync(FULL, ok_wait, 0);
  if (!ok_wait) {
    failed = true;
    return 0u;
  }
  (void)mail_acquire<CLUSTER>(&ms.rep);
  const uint32_t base = ms.base, n_ts = __popc(inc);
  const uint32_t my_ts = base + 1u + __popc(inc & lanemask_lt());
  fence_acq_rel_gpu();

  // 5. the group's first timestamp in its locks, then validation of the foreign reads: the stamp
  //    read must still be the latest, and a lock of a holder ordered before us (or whose
  //    timestamps are being drawn) must be resolved first. Waits point only to earlier
  //    timestamps or to holders already drawing: no cycles.
  if (own0) st_relaxed_gpu(&p.cw[a[0]], lock_word(st0, kPendingFlag | (base + 1u)));
  if (own1) st_relaxed_gpu(&p.cw[a[1]], lock_word(st1, kPendingFlag | (base + 1u)));
  bool valid = in && fok;
  if (valid) {
    const uint32_t wait_polls = p.read_wait ? p.read_wait : 4096u;
    unsigned long long word[MAXR];
#pragma unroll
    for (int k = 0; k < MAXR; k++)
      word[k] = (k < (int)nr && rsl[k] < 0) ? ld_relaxed_gpu(&p.cw[a[k]]) : 0ull;
#pragma unroll
    for (int k = 0; k < MAXR; k++) {
      if (k >= (int)nr || rsl[k] >= 0 || !valid) continue;
      unsigned long long wd = word[k];
      bool settled = false;  // a lane that gives up leaves a hole and is retried
      for (uint32_t it = 0; it < wait_polls; it++) {
        const uint32_t own = (uint32_t)(wd >> 32);
        bool clear;
        if (own == 0u)
          clear = true;
        else if (own & kPendingFlag)
          clear = (own & ~kPendingFlag) >= my_ts;  // its group is ordered after ours
        else
          clear = !(own & kReadyFlag);  // still acquiring: its timestamps follow ours
        if (clear) {
          settled = true;
          break;
        }
        __nanosleep(32);
        wd = ld_relaxed_gpu(&p.cw[a[k]]);
      }
      // the reads were issued while the timestamps were being drawn, so a version read may even
      // be newer than ours (a group ordered after us that committed meanwhile): it must be below
      if (settled && ((uint32_t)wd != fst[k] || fst[k] >= my_ts)) {
        // a version below our timestamp was committed since the read, and no holder ordered
        // before us remains: that version is the latest as of our timestamp, so it is read
        // again (the chain below has not used the value yet) instead of aborting. A version at
        // or above our timestamp (a group ordered after us that already committed) is not.
        uint32_t s2 = 0u;
        int32_t v2 = 0;
        if ((uint32_t)wd < my_ts && read_latest<DEPTH>(vs, p.cw, a[k], s2, v2) &&
            s2 == (uint32_t)wd) {
          fst[k] = s2;
          fv[k] = v2;
        } else {
          settled = false;
        }
      }
      valid = settled;
    }
  }
  const uint32_t fin = __ballot_sync(FULL, valid);

  // 6. the chain, in lane order through the locked accounts. Every lane first computes its
  //    transfer from the values read under the locks; that result is final for a lane no lower
  //    lane writes any of its accounts to (every writer of an account also reads it, so two
  //    writers of one account are always dependent). When some lanes depend on lower ones, each
  //    stages what its transfer needs (table slots, the part of its amount sum read outside the
  //    table, its divisor) and lane 0 runs every lane from the first dependent one on, in order,
  //    over the table's values in shared memory (a transfer writes a1 last; an independent
  //    lane's inputs are unchanged, so it computes its result again).
  uint32_t dep = 0u;
#pragma unroll
  for (int k = 0; k < MAXR; k++)
    if (valid && k < (int)nr && rsl[k] >= 0) dep |= gx.wmask[rsl[k]];
  dep &= fin & lanemask_lt();
  bool has_w = false;
  if (valid) {
    int32_t v[MAXR];
#pragma unroll
    for (int k = 0; k < MAXR; k++) v[k] = (k >= (int)nr) ? 0 : rsl[k] < 0 ? fv[k] : gx.base[rsl[k]];
    int32_t w0 = 0, w1 = 0;
    has_w = transfer_writes<MAXR>(op, nr, v, w0, w1);
    gx.out0[lane] = w0;
    gx.out1[lane] = w1;
  }
  const uint32_t depm = __ballot_sync(FULL, dep != 0u);
  uint32_t hw = __ballot_sync(FULL, has_w);
  if (depm) {
    if (valid) {
      uint32_t facc = CSMV_OP_AMT0(op) - 1u, ntr = 0u;
      unsigned long long tr = 0ull;  // unused bytes name slot 0 (read, then not counted)
#pragma unroll
      for (int k = 2; k < MAXR; k++) {
        if (k >= (int)nr) continue;
        if (rsl[k] < 0) {
          facc += (uint32_t)fv[k];
        } else {
          tr = (tr & ~(0xFFull << (8u * ntr))) | ((unsigned long long)rsl[k] << (8u * ntr));
          ntr++;
        }
      }
      const uint32_t d = CSMV_OP_AMOD(op);
      gx.cs[lane] = (uint32_t)s0 | ((uint32_t)s1 << 8) | (ntr << 16) |
                    ((CSMV_OP_KIND(op) == CSMV_KIND_TRANSFER_ALWAYS ? 1u : 0u) << 24);
      gx.facc[lane] = facc;
      gx.tr[lane] = tr;
      gx.md[lane] = d;
      gx.mm[lane] = 0xFFFFFFFFu / d;
    }
    __syncwarp();
    uint32_t hwm = hw & ~depm;
    if (lane == 0) {
      // Each step's table values are loaded one step ahead, before the previous step's writes
      // land, and patched with those two writes (a1 first: it is stored last); the transfer's
      // condition selects its writes without a branch. A step is then a short chain of
      // arithmetic instead of a shared-memory round trip and a branch.
      constexpr int NT = MAXR > 2 ? MAXR - 2 : 1;
      uint32_t m = fin & (0u - (depm & (0u - depm)));  // from the first dependent lane on...
      const uint32_t below = fin & ~m & hw;              // ...after the writes of those below it
      for (uint32_t b = below; b; b &= b - 1u) {
        const uint32_t j = __ffs(b) - 1u, cs = gx.cs[j];
        gx.base[cs & 0xFFu] = gx.out0[j];
        gx.base[(cs >> 8) & 0xFFu] = gx.out1[j];
      }
      uint32_t j = m ? __ffs(m) - 1u : 0u;
      uint32_t cs = gx.cs[j], facc = gx.facc[j], d = gx.md[j], mg = gx.mm[j];
      unsigned long long tr = gx.tr[j];
      int32_t l0 = gx.base[cs & 0xFFu], l1 = gx.base[(cs >> 8) & 0xFFu], lt[NT];
#pragma unroll
      for (int q = 0; q < NT; q++) lt[q] = gx.base[(tr >> (8u * q)) & 0xFFu];
      uint32_t px0 = 0xFFFFFFFFu, px1 = 0xFFFFFFFFu;  // the previous step's slots and writes
      int32_t pw0 = 0, pw1 = 0;
      while (m) {
        m &= m - 1u;
        const uint32_t jn = m ? __ffs(m) - 1u : j;
        const uint32_t x0 = cs & 0xFFu, x1 = (cs >> 8) & 0xFFu, n = (cs >> 16) & 0xFFu;
        const int32_t v0 = x0 == px1 ? pw1 : x0 == px0 ? pw0 : l0;
        const int32_t v1 = x1 == px1 ? pw1 : x1 == px0 ? pw0 : l1;
        uint32_t acc = facc;
#pragma unroll
        for (int q = 0; q < MAXR - 2; q++) {
          const uint32_t y = (uint32_t)(tr >> (8u * q)) & 0xFFu;
          const int32_t t = y == px1 ? pw1 : y == px0 ? pw0 : lt[q];
          acc += (uint32_t)q < n ? (uint32_t)t : 0u;
        }
        const uint32_t csn = gx.cs[jn], faccn = gx.facc[jn], dn = gx.md[jn], mgn = gx.mm[jn];
        const unsigned long long trn = gx.tr[jn];
        l0 = gx.base[csn & 0xFFu];
        l1 = gx.base[(csn >> 8) & 0xFFu];
#pragma unroll
        for (int q = 0; q < NT; q++) lt[q] = gx.base[(trn >> (8u * q)) & 0xFFu];
        uint32_t r = acc - __umulhi(acc, mg) * d;  // acc mod d (one correction suffices)
        r = r >= d ? r - d : r;
        const uint32_t amt = 1u + r;
        const bool moved = (cs >> 24) != 0u || v0 >= (int32_t)amt;
        const int32_t w0 = moved ? (int32_t)((uint32_t)v0 - amt) : v0;
        const int32_t w1 = moved ? (int32_t)((uint32_t)v1 + amt) : v1;
        gx.base[x0] = w0;
        gx.base[x1] = w1;
        gx.out0[j] = w0;
        gx.out1[j] = w1;
        hwm = moved ? (hwm | (1u << j)) : (hwm & ~(1u << j));
        px0 = x0;
        px1 = x1;
        pw0 = w0;
        pw1 = w1;
        j = jn;
        cs = csn;
        facc = faccn;
        d = dn;
        mg = mgn;
        tr = trn;
      }
    }
    hw = __shfl_sync(FULL, hwm, 0);
    __syncwarp();
  }

  // 7. one version per locked account (its last writer's), then the stamp (released: the
  //    version is visible first) and the unlock
  auto install = [&](int s, uint32_t x, SlotEditor<DEPTH>& ed) -> uint32_t {
    const uint32_t wr = gx.wmask[s] & hw;
    if (!wr) return 0u;
    const uint32_t j = 31u - __clz(wr);
    const int32_t val = gx.wa1[j] == x ? gx.out1[j] : gx.out0[j];
    const uint32_t ts = base + 1u + __popc(inc & ((1u << j) - 1u));
    ed.insert(ts, val);
    ed.store(p.slots + (size_t)x * DEPTH);
    return ts;
  };
  uint32_t pub0 = 0u, pub1 = 0u;
  if (own0) pub0 = install(s0, a[0], ed0);
  if (own1) pub1 = install(s1, a[1], ed1);
  // one fence releases both words (a fence then relaxed stores is a release): two release
  // stores in a row would wait for the first to land before the second
  if (own0 || own1) fence_acq_rel_gpu();
  if (own0) st_relaxed_gpu(&p.cw[a[0]], (unsigned long long)(pub0 ? pub0 : st0));
  if (own1) st_relaxed_gpu(&p.cw[a[1]], (unsigned long long)(pub1 ? pub1 : st1));

  // 8. log, outcomes, the group's end, completion
  if (p.log && in) {
    const uint32_t li = my_ts - 1u - p.log_base;
    if (li < p.log_cap)
      p.log_txn[li] = valid ? t : kHole;
    else
      raise_error(&p.gs->error, ERR_CAPACITY);
    if (valid) {
      p.outcome[t] = my_ts;
      p.result[t] = 0;
    }
  }
  __syncwarp();
  if (lane == 0) {
    if (p.log && p.grp) {
      const uint32_t li = base + n_ts - 1u - p.log_base;
      if (li < p.log_cap) atomicOr(&p.grp[li >> 5], 1u << (li & 31u));
    }
    complete_range(p.done, p.done_mask, p.gs, base + 1u, base + n_ts);
    stat_add(sm.stat, ST_COMMIT_UPDATE, __popc(hw));
    stat_add(sm.stat, ST_COMMIT_NOWRITE, __popc(fin & ~hw));
    stat_add(sm.stat, ST_ABORT_READ_WRITE, __popc(inc & ~fin));
    stat_add(sm.stat, ST_ABORT_WRITE_WRITE, __popc(actm & ~inc));  // sat out: a lock was held
  }
  return fin;
}

// ---------------------------------------------------------------------------------------------
// client side
// ---------------------------------------------------------------------------------------------
// CLUSTER: the mailbox `ms` (and the finished-client counter) live in the shared memory of the
// cluster's leader CTA, reached through distributed shared memory; else in this CTA's.
// gx: this warp's group-commit table (prevalidate == 3), in this CTA's shared memory.
template <int DEPTH, int MAXR, int MAXW, bool CLUSTER = false>
__device__ void client_warp(const BankParams& p, CtaShared<MAXR, MAXW>& sm, uint32_t w,
                            MailSlot<MAXR, MAXW>& ms, uint32_t* done_ctr, GroupScratch* gx) {
  const uint32_t lane = lane_id();
  const VersionStore vs{p.slots, p.n_items};
  const bool stamp = p.validate == CSMV_VALIDATE_STAMP;
  const uint32_t me = blockIdx.x * p.nc + w + 1;  // lock owner id of this warp
  uint32_t seq = 0;
  bool failed = false;
  // Deferred queue (a scheduler's likely-conflicting rounds): only the first deferred_warps
  // warps of the grid take those rounds, so at most that many run at once; they join the main
  // queue when the deferred one is empty.
  // With lane_start, the deferred queue is one lane of rounds per deferred warp instead, served
  // in order by that warp alone.
  const uint32_t main_end = p.split_round ? p.split_round : p.n_rounds;
  const uint32_t gw = blockIdx.x * p.nc + w;
  bool serve_deferred = p.split_round != 0 && gw < p.deferred_warps;
  uint32_t lane_next = 0u, lane_end = 0u;
  if (serve_deferred && p.lane_start) {
    lane_next = max(p.lane_start[gw], p.split_round);  // never a round of the main queue
    lane_end = min(p.lane_start[gw + 1], p.n_rounds);
  }
  for (;;) {
    uint32_t g = 0xFFFFFFFFu;
    if (lane == 0) {
      if (serve_deferred && p.lane_start) {
        if (lane_next < lane_end)
          g = lane_next++;
        else
          serve_deferred = false;
      } else if (serve_deferred) {
        g = p.split_round + atomicAdd(&p.gs->round_deferred, 1u);
        if (g >= p.n_rounds) {
          g = 0xFFFFFFFFu;
          serve_deferred = false;
        }
      }
      if (g == 0xFFFFFFFFu) {
        g = atomicAdd(&p.gs->round_next, 1u);
        if (g >= main_end) g = 0xFFFFFFFFu;
      }
    }
    g = __shfl_sync(0xFFFFFFFFu, g, 0);
    if (g == 0xFFFFFFFFu) break;
    const uint32_t t = g * 32u + lane;
    const uint32_t op = p.op[t];
    const uint32_t kind = CSMV_OP_KIND(op), nr = CSMV_OP_NREADS(op);
    const uint32_t off = p.off[t];
    // the round's kind must be warp-uniform (the stream format guarantees it, the reference
    // decides it per warp, bank/csmv_sh/exe.cu:134-139): every branch on it holds collectives
    const bool ro = __all_sync(0xFFFFFFFFu, kind == CSMV_KIND_READONLY);
    bool bad = (ro != (kind == CSMV_KIND_READONLY)) || (!ro && (nr < 2 || nr > (uint32_t)MAXR));
    uint32_t a[MAXR];
#pragma unroll
    for (int k = 0; k < MAXR; k++) {
      a[k] = (!ro && !bad && k < (int)nr) ? p.addr[off + k] : 0u;
      bad |= a[k] >= p.n_items;
    }
    if (ro)
#pragma unroll 8
      for (uint32_t k = 0; k < nr; k++) bad |= p.addr[off + k] >= p.n_items;  // loads batch up
    if (bad) raise_error(&p.gs->error, ERR_DATA);  // no access outside the accounts
    if (__any_sync(0xFFFFFFFFu, bad)) {
      failed = true;
      break;
    }

    uint32_t pending = 0xFFFFFFFFu;
    uint32_t attempts = 0, lock_fails = 0, tries = 0, stuck = 0, sat_outs = 0;
    if (p.txn_waits) p.txn_waits[t] = 0u;
    while (pending) {
      if (lane == 0) atomicAdd(&sm.stat[ST_ROUNDS], 1ull);
      tries += (pending >> lane) & 1u;
      if (lock_fails) {  // randomized, growing back-off after a lost lock: breaks lock-step retries
        const uint32_t h = (me * 0x9E3779B1u) ^ (attempts * 0x85EBCA6Bu);
        __nanosleep((h >> 16) & ((64u << lock_fails) - 1u));
      }
      if (p.backoff && attempts > 0) {  // a scheduler's per-transaction pause before a retry
        const uint32_t bo = __reduce_max_sync(0xFFFFFFFFu, ((pending >> lane) & 1u) ? p.backoff[t] : 0u);
        if (bo) __nanosleep(((me * 0x85EBCA6Bu) ^ (attempts * 0x9E3779B1u)) % bo);
      }
      if (++attempts > (1u << 20)) {  // no round may retry forever: report and leave
        if (lane == 0) raise_error(&p.gs->error, ERR_LIVELOCK);
        failed = true;
        break;
      }
      const bool mine = (pending >> lane) & 1u;
      ReadSet<MAXR> rs;
      WriteSet<MAXW> ws;
      uint32_t snap = 0;
      if (lane == 0) snap = TXBegin(&p.gs->clock, rs, ws);
      rs.n = 0;
      ws.n = 0;
      snap = __shfl_sync(0xFFFFFFFFu, snap, 0);
      bool aborted = false;

      if (ro) {  // read-only: consistent snapshot read, commits without validation
        uint32_t s = 0;
        if (mine)
          for (uint32_t k0 = 0; k0 < nr; k0 += 8) {  // 8 independent version loads in flight
            uint32_t ad[8];
#pragma unroll
            for (int j = 0; j < 8; j++) ad[j] = k0 + j < nr ? p.addr[off + k0 + j] : 0u;
#pragma unroll
            for (int j = 0; j < 8; j++)
              if (k0 + j < nr) s += (uint32_t)TXReadOnly<DEPTH>(vs, ad[j], snap, &aborted);
          }
        const bool done = mine && !aborted;
        if (done && p.log) {
          p.outcome[t] = snap | kSnapFlag;
          p.result[t] = (int32_t)s;
        }
        const uint32_t dm = __ballot_sync(0xFFFFFFFFu, done);
        const uint32_t am = __ballot_sync(0xFFFFFFFFu, mine && aborted);
        if (lane == 0) {
          stat_add(sm.stat, ST_COMMIT_RO, __popc(dm));
          stat_add(sm.stat, ST_ABORT_DATA_AGE, __popc(am));
        }
        pending &= ~dm;
        continue;
      }

      if (stamp && p.prevalidate == 3) {  // group commit of the round's transfers
        bool gave_up = false, waited = false, sat = false;
        const uint32_t fin = group_attempt<DEPTH, MAXR, MAXW, CLUSTER>(
            p, sm, ms, *gx, me, t, op, nr, a, mine, seq, sat_outs >= 2u, gave_up, failed,
            waited, sat);
        sat_outs = sat ? sat_outs + 1u : 0u;
        if (failed) break;
        if (p.txn_waits && waited) p.txn_waits[t] = 1u;
        if (lane == 0 && gave_up) stat_add(sm.stat, ST_ABORT_WRITE_WRITE, __popc(pending));
        lock_fails = gave_up ? min(lock_fails + 1, 6u) : 0u;
        // a lock that stays held across 64 bounded waits (about 3 s) is reported, not retried on
        if (gave_up && lock_fails == 6u && ++stuck > 64u) {
          if (lane == 0) raise_error(&p.gs->error, ERR_LIVELOCK);
          failed = true;
          break;
        }
        if (!gave_up) stuck = 0;
        pending &= ~fin;
        uint32_t err = 0;
        if (lane == 0) err = ld_relaxed_gpu(&p.gs->error);
        if (__shfl_sync(0xFFFFFFFFu, err, 0) != 0) {
          failed = true;
          break;
        }
        continue;
      }

      // transfer reads. Ring protocol: the reference's rule, everything at the snapshot. Stamp
      // protocol: each item's latest committed version, with its stamp kept for validation (a
      // snapshot read would go stale whenever the clock trails a hot item's commits)
      int32_t v[MAXR];
      uint32_t stv[MAXR];
#pragma unroll
      for (int k = 0; k < MAXR; k++) {
        v[k] = 0;
        stv[k] = 0;
        if (mine && k < (int)nr) {
          if (stamp)
            v[k] = TXReadLatest<DEPTH>(vs, p.cw, a[k], rs, stv[k], &aborted);
          else
            v[k] = TXRead<DEPTH>(vs, a[k], snap, rs, ws, &aborted);
        }
      }
      const bool stale = false;
      // a transfer that commits no writes is read-only: in the stamp protocol it serialises at
      // the largest stamp it read, once a second collect finds every stamp unchanged and no
      // lock on them (a writer of one of them with a smaller timestamp would hold its lock)
      uint32_t ro_snap = snap;
      auto recheck = [&](bool active) {
        bool ok = active;
        uint32_t mx = 0;
#pragma unroll
        for (int k = 0; k < MAXR; k++) {
          if (!active || k >= (int)nr) continue;
          const unsigned long long wd = ld_relaxed_gpu(&p.cw[a[k]]);
          ok &= (uint32_t)wd == stv[k] && (uint32_t)(wd >> 32) == 0u;
          mx = max(mx, stv[k]);
        }
        ro_snap = mx;
        return ok;
      };

      // ---- stamp protocol with intra-warp chaining (prevalidate == 2): instead of aborting a
      // lane that read what a lower lane writes (TXPreValidation), the warp runs its transfers as
      // one serial chain in lane order, forwarding each lower lane's written values to the lanes
      // that read them; only reads taken from the snapshot are validated, each written account
      // is locked once (by its lowest writer), and every link of the chain gets the next commit
      // timestamp. A link whose lock or validation fails takes down the links that consumed it.
      if (stamp && p.prevalidate == 2) {
        const bool okr = mine && !aborted && !stale;
        uint32_t dep = 0;  // lower lanes whose possible writes {a0, a1} hit my reads
        for (uint32_t i = 0; i < 31; i++) {
          const bool oki = __shfl_sync(0xFFFFFFFFu, okr, i);
          const uint32_t x0 = __shfl_sync(0xFFFFFFFFu, a[0], i), x1 = __shfl_sync(0xFFFFFFFFu, a[1], i);
          bool hit = false;
#pragma unroll
          for (int k = 0; k < MAXR; k++) hit |= (k < (int)nr) && (a[k] == x0 || a[k] == x1);
          if (okr && oki && i < lane && hit) dep |= 1u << i;
        }
        const uint32_t srcs = __reduce_or_sync(0xFFFFFFFFu, dep);
        uint32_t fwd = 0, fwdk = 0;  // lanes whose values I consumed / my reads that were forwarded
        for (uint32_t m = srcs; m; m &= m - 1) {
          const uint32_t i = __ffs(m) - 1;
          int32_t w0, w1;
          const bool hw = okr && transfer_writes<MAXR>(op, nr, v, w0, w1);
          const bool hwi = __shfl_sync(0xFFFFFFFFu, hw, i);
          const uint32_t x0 = __shfl_sync(0xFFFFFFFFu, a[0], i), x1 = __shfl_sync(0xFFFFFFFFu, a[1], i);
          const int32_t y0 = __shfl_sync(0xFFFFFFFFu, w0, i), y1 = __shfl_sync(0xFFFFFFFFu, w1, i);
          if (okr && lane > i && hwi) {
#pragma unroll
            for (int k = 0; k < MAXR; k++) {
              if (k >= (int)nr) continue;
              if (a[k] == x0) {
                v[k] = y0;
                fwd |= 1u << i;
                fwdk |= 1u << k;
              } else if (a[k] == x1) {
                v[k] = y1;
                fwd |= 1u << i;
                fwdk |= 1u << k;
              }
            }
          }
        }
        int32_t w0, w1;
        const bool has_w = okr && transfer_writes<MAXR>(op, nr, v, w0, w1);
        // every transfer of the round is a link with a timestamp, also one that writes nothing:
        // a no-write transfer serialised at the stamps it read could fall inside a chain, whose
        // intermediate states are never installed
        const bool part = okr;
        const bool ro_cand = false;
        const bool snap_ok = recheck(ro_cand);
        const bool ro_fail = ro_cand && !snap_ok;
        // lock leaders: the lowest lane writing each address takes its lock
        uint32_t lead_lane[2] = {lane, lane}, lead_slot[2] = {0u, 1u};
        bool found[2] = {false, false};
        for (uint32_t i = 0; i < 32; i++) {
          const bool h = __shfl_sync(0xFFFFFFFFu, has_w, i);
          const uint32_t x0 = __shfl_sync(0xFFFFFFFFu, a[0], i), x1 = __shfl_sync(0xFFFFFFFFu, a[1], i);
#pragma unroll
          for (int k = 0; k < 2; k++) {
            if (has_w && !found[k] && h && (x0 == a[k] || x1 == a[k])) {
              lead_lane[k] = i;
              lead_slot[k] = x0 == a[k] ? 0u : 1u;
              found[k] = true;
            }
          }
        }
        bool got[2] = {false, false};
#pragma unroll
        for (int k = 0; k < 2; k++)
          if (has_w && lead_lane[k] == lane) got[k] = atomicCAS(owner_word(p.cw, a[k]), 0u, me) == 0u;
        bool lock_ok = true;
#pragma unroll
        for (int k = 0; k < 2; k++) {
          const bool g0 = __shfl_sync(0xFFFFFFFFu, got[0], lead_lane[k]);
          const bool g1 = __shfl_sync(0xFFFFFFFFu, got[1], lead_lane[k]);
          if (has_w) lock_ok &= lead_slot[k] == 0 ? g0 : g1;
        }
        uint32_t F = 0;  // failed links, cascading to the links that consumed them
        for (uint32_t i = 0; i < 32; i++)
          F |= __ballot_sync(0xFFFFFFFFu, lane == i && part && (!lock_ok || (fwd & F) != 0));
        const uint32_t partm = __ballot_sync(0xFFFFFFFFu, part);
        const uint32_t lockf = __ballot_sync(0xFFFFFFFFu, part && !lock_ok);
        const uint32_t snapm = __ballot_sync(0xFFFFFFFFu, snap_ok);
        const uint32_t agm = __ballot_sync(0xFFFFFFFFu, mine && aborted);
        const uint32_t stm = __ballot_sync(0xFFFFFFFFu, ro_fail);
        if (snap_ok && p.log) {
          p.outcome[t] = ro_snap | kSnapFlag;
          p.result[t] = 0;
        }
        if (lane == 0) {
          stat_add(sm.stat, ST_COMMIT_NOWRITE, __popc(snapm));
          stat_add(sm.stat, ST_ABORT_DATA_AGE, __popc(agm));
          stat_add(sm.stat, ST_ABORT_READ_WRITE, __popc(stm));
          stat_add(sm.stat, ST_ABORT_WRITE_WRITE, __popc(lockf));
          stat_add(sm.stat, ST_ABORT_PREVALID, __popc(F & ~lockf));
        }
        lock_fails = lockf ? min(lock_fails + 1, 6u) : 0u;
        const uint32_t cand = partm & ~F;
        const bool cand_me = (cand >> lane) & 1u;
        uint32_t C = 0, base = 0, my_ts = 0;
        if (cand) {
          seq++;
          __syncwarp();
          if (lane == 0) {
            ms.snap = snap;
            ms.cand = cand;
            mail_release<CLUSTER>(&ms.req, seq);
          }
          bool ok_wait = true;
          if (lane == 0)
            ok_wait = bounded_wait([&] { return mail_acquire<CLUSTER>(&ms.rep) == seq; }, &p.gs->error,
                                   ERR_WAIT_REPLY, p.spin_log2);
          ok_wait = __shfl_sync(0xFFFFFFFFu, ok_wait, 0);
          if (!ok_wait) {
            failed = true;
            break;
          }
          (void)mail_acquire<CLUSTER>(&ms.rep);
          base = ms.base;
          my_ts = base + 1 + __popc(cand & lanemask_lt());
          fence_acq_rel_gpu();
#pragma unroll
          for (int k = 0; k < 2; k++)
            if (got[k] && cand_me) st_relaxed_gpu(owner_word(p.cw, a[k]), kPendingFlag | my_ts);
          // validate the reads that came from the snapshot (forwarded ones are the chain's own)
          bool valid = cand_me;
          if (cand_me) {
            unsigned long long word[MAXR];
#pragma unroll
            for (int k = 0; k < MAXR; k++)
              word[k] = (k < (int)nr && !((fwdk >> k) & 1u)) ? ld_relaxed_gpu(&p.cw[a[k]]) : 0ull;
#pragma unroll
            for (int k = 0; k < MAXR; k++) {
              if (k >= (int)nr || ((fwdk >> k) & 1u) || !valid) continue;
              unsigned long long wd = word[k];
              bool settled = false;
              for (uint32_t it = 0; it < 2048; it++) {
                const uint32_t own = (uint32_t)(wd >> 32);
                if (own == 0u || own == me || ((own & kPendingFlag) && (own & ~kPendingFlag) >= my_ts)) {
                  settled = true;
                  break;
                }
                __nanosleep(32);
                wd = ld_relaxed_gpu(&p.cw[a[k]]);
              }
              valid = settled && (uint32_t)wd == stv[k];
            }
          }
          uint32_t F2 = 0;
          for (uint32_t i = 0; i < 32; i++)
            F2 |= __ballot_sync(0xFFFFFFFFu, lane == i && cand_me && (!valid || (fwd & F2) != 0));
          C = cand & ~F2;
          const bool commit = (C >> lane) & 1u;
          if (lane == 0) stat_add(sm.stat, ST_ABORT_READ_WRITE, __popc(F2));
          if (p.log && cand_me) {
            const uint32_t li = my_ts - 1 - p.log_base;
            if (li < p.log_cap)
              p.log_txn[li] = commit ? t : kHole;
            else
              raise_error(&p.gs->error, ERR_CAPACITY);
          }
          if (commit && p.log) {
            p.outcome[t] = my_ts;
            p.result[t] = 0;
          }
          // write-back by the lock leaders: ONE version per item, the last committed link's,
          // then its stamp and the unlock. The chain's timestamps are published to the clock
          // as one range, so no snapshot falls between them and the intermediate versions are
          // never read; installing them would also let one store evict two versions, and a
          // concurrent snapshot read could then see the older victim without the younger one.
          const uint32_t hwm = __ballot_sync(0xFFFFFFFFu, has_w && commit);
#pragma unroll
          for (int k = 0; k < 2; k++) {
            const bool lead = got[k];
            unsigned long long* item = p.slots + (size_t)a[k] * DEPTH;
            SlotEditor<DEPTH> ed;
            if (lead) ed.load(item);
            uint32_t last = 0;
            int32_t lv = 0;
            for (uint32_t m = hwm; m; m &= m - 1) {
              const uint32_t i = __ffs(m) - 1;
              const uint32_t x0 = __shfl_sync(0xFFFFFFFFu, a[0], i), x1 = __shfl_sync(0xFFFFFFFFu, a[1], i);
              const int32_t y0 = __shfl_sync(0xFFFFFFFFu, w0, i), y1 = __shfl_sync(0xFFFFFFFFu, w1, i);
              const uint32_t ti = __shfl_sync(0xFFFFFFFFu, my_ts, i);
              if (lead && (x0 == a[k] || x1 == a[k])) {
                lv = x1 == a[k] ? y1 : y0;  // a transfer writes a1 last
                last = ti;
              }
            }
            if (lead && last) {
              ed.insert(last, lv);
              ed.store(item);
            }
            __threadfence();
            if (lead) {
              if (last)
                st_release_gpu(&p.cw[a[k]], (unsigned long long)last);  // stamp, unlock
              else
                st_relaxed_gpu(owner_word(p.cw, a[k]), 0u);
            }
          }
          __syncwarp();
          if (lane == 0) {
            if (p.log && p.grp) {  // the chain's end, for the replay's one-version-per-group rule
              const uint32_t li = base + __popc(cand) - 1u - p.log_base;
              if (li < p.log_cap) atomicOr(&p.grp[li >> 5], 1u << (li & 31u));
            }
            complete_range(p.done, p.done_mask, p.gs, base + 1, base + __popc(cand));
          }
        } else {
          // no links: leaders release whatever they locked
#pragma unroll
          for (int k = 0; k < 2; k++)
            if (got[k]) st_relaxed_gpu(owner_word(p.cw, a[k]), 0u);
        }
        const uint32_t hw_c = __ballot_sync(0xFFFFFFFFu, has_w && ((C >> lane) & 1u));
        if (lane == 0) {
          stat_add(sm.stat, ST_COMMIT_UPDATE, __popc(hw_c));
          stat_add(sm.stat, ST_COMMIT_NOWRITE, __popc(C & ~hw_c));
        }
        pending &= ~(C | snapm);
        uint32_t err = 0;
        if (lane == 0) err = ld_relaxed_gpu(&p.gs->error);
        if (__shfl_sync(0xFFFFFFFFu, err, 0) != 0) {
          failed = true;
          break;
        }
        continue;
      }
      bool has_w = false;
      if (mine && !aborted && !stale) {
        uint32_t acc = CSMV_OP_AMT0(op) - 1u;
#pragma unroll
        for (int k = 2; k < MAXR; k++)
          if (k < (int)nr) acc += (uint32_t)v[k];
        const uint32_t amt = 1u + acc % CSMV_OP_AMOD(op);
        if (kind == CSMV_KIND_TRANSFER_ALWAYS || v[0] >= (int32_t)amt) {
          TXWrite(a[0], (int32_t)((uint32_t)v[0] - amt), ws);
          TXWrite(a[1], (int32_t)((uint32_t)v[1] + amt), ws);
          has_w = true;
        }
      }
      bool nowrite = mine && !aborted && !stale && !has_w;
      bool ro_fail = false;
      if (stamp) {
        const bool ok = recheck(nowrite);
        ro_fail = nowrite && !ok;
        nowrite = nowrite && ok;
      }
      if (nowrite && p.log) {
        p.outcome[t] = ro_snap | kSnapFlag;
        p.result[t] = 0;
      }
      const uint32_t nwm = __ballot_sync(0xFFFFFFFFu, nowrite);
      const uint32_t agm = __ballot_sync(0xFFFFFFFFu, mine && aborted);
      const uint32_t stm = __ballot_sync(0xFFFFFFFFu, ro_fail);
      uint32_t cand = __ballot_sync(0xFFFFFFFFu, has_w);
      if (lane == 0) {
        stat_add(sm.stat, ST_COMMIT_NOWRITE, __popc(nwm));
        stat_add(sm.stat, ST_ABORT_DATA_AGE, __popc(agm));
        stat_add(sm.stat, ST_ABORT_READ_WRITE, __popc(stm));
      }
      pending &= ~nwm;
      if (cand == 0) continue;
      bool cand_me = (cand >> lane) & 1u;

      if (stamp) {
        // lock the write items first (before the timestamps are drawn; only the lowest lane
        // writing an address tries), then resolve lane order among the lanes that hold their
        // locks, so no lane is dropped for a lower lane that could not lock
        // (warp-collective: every lane calls it, candidate or not)
        const uint32_t overlap = TXWriteOverlap(ws, cand_me);
        const bool attempt = cand_me && (overlap & cand) == 0;
        // locks in address order, no waiting: the higher one is tried only once the lower one is
        // held, so two warps never each hold one of the other's pair (that lock-step was a
        // livelock); a lost lock releases what was taken and backs off
        static_assert(MAXW == 2, "ordered acquisition below is written for two write items");
        const uint32_t lo_a = ws.n > 1 ? min(ws.addr[0], ws.addr[1]) : ws.addr[0];
        const uint32_t hi_a = ws.n > 1 ? max(ws.addr[0], ws.addr[1]) : ws.addr[0];
        bool got_lo = false, got_hi = ws.n < 2;
        if (attempt) {
          got_lo = atomicCAS(owner_word(p.cw, lo_a), 0u, me) == 0u;
          if (got_lo && !got_hi) got_hi = atomicCAS(owner_word(p.cw, hi_a), 0u, me) == 0u;
          if (got_lo && !got_hi) st_relaxed_gpu(owner_word(p.cw, lo_a), 0u);
        }
        const bool all = attempt && got_lo && got_hi;
        bool got[MAXW];
#pragma unroll
        for (int k = 0; k < MAXW; k++) got[k] = all && k < (int)ws.n;
        const uint32_t locked = __ballot_sync(0xFFFFFFFFu, all);
        // intra-warp resolution: always needed here, since a lane must not commit after a lower
        // lane of its own warp wrote what it read (their locks have the same owner)
        const uint32_t pass = TXPreValidation(rs, ws, (locked >> lane) & 1u);
        if (cand_me && !((pass >> lane) & 1u)) {
#pragma unroll
          for (int k = 0; k < MAXW; k++)
            if (got[k]) st_relaxed_gpu(owner_word(p.cw, ws.addr[k]), 0u);
        }
        if (lane == 0) {
          stat_add(sm.stat, ST_ABORT_WRITE_WRITE, __popc(cand & ~locked));
          stat_add(sm.stat, p.prevalidate ? ST_ABORT_PREVALID : ST_ABORT_READ_WRITE,
                   __popc(locked & ~pass));
        }
        // back off only when a lock was lost to another warp (not for own-warp overlaps)
        lock_fails = __ballot_sync(0xFFFFFFFFu, attempt && !all) ? min(lock_fails + 1, 6u) : 0u;
        cand = pass;
        cand_me = (cand >> lane) & 1u;
        if (cand == 0) continue;
      } else {
        if (p.prevalidate) {
          const uint32_t pass = TXPreValidation(rs, ws, cand_me);
          if (lane == 0) stat_add(sm.stat, ST_ABORT_PREVALID, __popc(cand & ~pass));
          cand = pass;
          cand_me = (cand >> lane) & 1u;
          if (cand == 0) continue;
        }
        if (cand_me) {  // ring protocol: the server validates from the mailbox
#pragma unroll
          for (int k = 0; k < MAXR; k++) ms.rs[k][lane] = rs.addr[k];
#pragma unroll
          for (int k = 0; k < MAXW; k++) {
            ms.ws[k][lane] = ws.addr[k];
            ms.wv[k][lane] = ws.val[k];
          }
          ms.n[lane] = rs.n | (ws.n << 8);
          ms.txn[lane] = t;
        }
      }
      // post the request into the shared-memory mailbox, wait for the reply
      seq++;
      __syncwarp();
      if (lane == 0) {
        ms.snap = snap;
        ms.cand = cand;
        mail_release<CLUSTER>(&ms.req, seq);
      }
      bool ok_wait = true;
      if (lane == 0)
        ok_wait = bounded_wait([&] { return mail_acquire<CLUSTER>(&ms.rep) == seq; }, &p.gs->error,
                               ERR_WAIT_REPLY, p.spin_log2);
      ok_wait = __shfl_sync(0xFFFFFFFFu, ok_wait, 0);
      if (!ok_wait) {
        failed = true;
        break;
      }
      (void)mail_acquire<CLUSTER>(&ms.rep);

      uint32_t okm = 0, my_ts = 0;
      if (stamp) {
        // timestamps base+1.. in lane order over the locked lanes
        const uint32_t base = ms.base;
        my_ts = base + 1 + __popc(cand & lanemask_lt());
        fence_acq_rel_gpu();
        // advertise the pending timestamp in the lock words: a validator later in the order
        // may then ignore our lock, one earlier waits for our outcome instead of aborting
#pragma unroll
        for (int k = 0; k < MAXW; k++)
          if (cand_me && k < (int)ws.n) st_relaxed_gpu(owner_word(p.cw, ws.addr[k]), kPendingFlag | my_ts);
        // validate the reads: the stamp must not be newer than the snapshot, and a lock held by
        // a transaction earlier in the order (or one whose timestamp is not known yet) must be
        // resolved first. Waits only ever point to smaller timestamps: no cycles.
        bool valid = cand_me;
        if (cand_me) {
          unsigned long long word[MAXR];
#pragma unroll
          for (int k = 0; k < MAXR; k++)
            word[k] = k < (int)rs.n ? ld_relaxed_gpu(&p.cw[rs.addr[k]]) : 0ull;
#pragma unroll
          for (int k = 0; k < MAXR; k++) {
            if (k >= (int)rs.n || !valid) continue;
            unsigned long long wd = word[k];
            bool settled = false;
            for (uint32_t it = 0; it < 2048; it++) {
              const uint32_t own = (uint32_t)(wd >> 32);
              if (own == 0u || own == me || ((own & kPendingFlag) && (own & ~kPendingFlag) >= my_ts)) {
                settled = true;
                break;
              }
              __nanosleep(32);
              wd = ld_relaxed_gpu(&p.cw[rs.addr[k]]);
            }
            valid = settled && (uint32_t)wd == stv[k];
          }
        }
        okm = __ballot_sync(0xFFFFFFFFu, valid);
        if (lane == 0) stat_add(sm.stat, ST_ABORT_READ_WRITE, __popc(cand & ~okm));
        if (p.log && cand_me) {
          const uint32_t li = my_ts - 1 - p.log_base;
          if (li < p.log_cap)
            p.log_txn[li] = valid ? t : kHole;
          else
            raise_error(&p.gs->error, ERR_CAPACITY);
        }
        if (valid) {
          TXWriteBack<DEPTH>(my_ts, vs, ws);
          if (p.log) {
            p.outcome[t] = my_ts;
            p.result[t] = 0;
          }
        }
        __threadfence();  // write-back visible before the stamps and the completion bits
#pragma unroll
        for (int k = 0; k < MAXW; k++) {
          if (cand_me && k < (int)ws.n) {
            if (valid)
              st_release_gpu(&p.cw[ws.addr[k]], (unsigned long long)my_ts);  // stamp, unlock
            else
              st_relaxed_gpu(owner_word(p.cw, ws.addr[k]), 0u);
          }
        }
        __syncwarp();
        if (lane == 0) complete_range(p.done, p.done_mask, p.gs, base + 1, base + __popc(cand));
      } else {
        okm = ms.ok;
        const uint32_t bid = ms.bid;
        const bool committed = (okm >> lane) & 1u;
        my_ts = committed ? ms.tsl[lane] : 0u;
        if (committed && p.log) {
          p.outcome[t] = my_ts;
          p.result[t] = 0;
        }
        if (p.writeback == CSMV_WRITEBACK_CLIENT && okm) {
          if (committed) TXWriteBack<DEPTH>(my_ts, vs, ws);
          __syncwarp();
          if (lane == 0) batch_done(p, sm, bid);
        }
      }
      __syncwarp();
      if (lane == 0) stat_add(sm.stat, ST_COMMIT_UPDATE, __popc(okm));
      pending &= ~okm;
      uint32_t err = 0;  // read once and broadcast: the warp leaves the loop together
      if (lane == 0) err = ld_relaxed_gpu(&p.gs->error);
      if (__shfl_sync(0xFFFFFFFFu, err, 0) != 0) {
        failed = true;
        break;
      }
    }
    if (failed) break;
    if (p.txn_aborts) p.txn_aborts[t] = tries - 1u;
  }
  __syncwarp();
  if (lane == 0) atomicAdd(done_ctr, 1u);
}

// ---------------------------------------------------------------------------------------------
// server side
// ---------------------------------------------------------------------------------------------

// Polls the mailboxes of the CTA's client warps; returns the ready mask (0 = none), sets
// *stop when every client finished or an error was raised. SM is any CTA layout with
// mail[w].{req,rep,cand,base} slots and done_warps/stat fields.
template <class SM, bool CLUSTER = false>
__device__ __forceinline__ uint32_t poll_mailboxes(uint32_t nc, GlobalSync* gs, SM& sm,
                                                   uint32_t seen, uint32_t* req, bool* stop,
                                                   bool check_error = true) {
  const uint32_t lane = lane_id();
  *req = 0;
  if (lane < nc) *req = mail_acquire<CLUSTER>(&sm.mail[lane].req);
  const uint32_t ready = __ballot_sync(0xFFFFFFFFu, lane < nc && *req != seen);
  *stop = false;
  if (ready == 0) {
    uint32_t done = 0, err = 0;
    if (lane == 0) {
      done = CLUSTER ? ld_acquire_cluster(&sm.done_warps) : *(volatile uint32_t*)&sm.done_warps;
      // the device error word is an L2 round trip: an idle server looks at it only now and
      // then, so a request that arrives is seen within a shared-memory poll
      if (check_error) err = ld_relaxed_gpu(&gs->error);
    }
    done = __shfl_sync(0xFFFFFFFFu, done, 0);
    err = __shfl_sync(0xFFFFFFFFu, err, 0);
    *stop = (done == nc) || err;
  }
  return ready;
}

// Stamp protocol server: one atomicAdd draws consecutive timestamps for every ready warp
// (batched commit-timestamp assignment, batchedAtrInsert/csmv_sh/API.cu:331-361, here per CTA
// batch instead of per warp); warp w gets (base_w, base_w + count_w].
template <class SM, bool CLUSTER = false>
__device__ void server_warp_stamp(uint32_t nc, uint32_t batch, GlobalSync* gs, SM& sm) {
  const uint32_t lane = lane_id();
  uint32_t seen = 0, idle = 0;
  for (;;) {
    uint32_t req;
    bool stop;
    uint32_t ready =
        poll_mailboxes<SM, CLUSTER>(nc, gs, sm, seen, &req, &stop, (idle & 63u) == 63u);
    if (ready == 0) {
      if (stop) break;
      if (++idle > 256u) __nanosleep(64);  // spin a while first: the reply is latency-critical
      continue;
    }
    idle = 0;
    if (batch != CSMV_BATCH_CTA) ready &= (0u - ready);  // one warp per assignment
    const bool mine = lane < nc && ((ready >> lane) & 1u);
    uint32_t cnt = 0;
    if (mine) {
      seen = req;
      cnt = __popc(sm.mail[lane].cand);
    }
    // inclusive prefix over the ready warps in warp order
    uint32_t incl = cnt;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
      if (lane >= (uint32_t)d) incl += y;
    }
    const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    uint32_t t0 = 0;
    if (lane == 0) {  // fences on both sides order the draw after the observed locks and
      __threadfence();  // before the validations that follow it
      t0 = atomicAdd(&gs->ts_next, total);
      __threadfence();
    }
    t0 = __shfl_sync(0xFFFFFFFFu, t0, 0);
    if (mine) {
      sm.mail[lane].base = t0 + incl - cnt;
      mail_release<CLUSTER>(&sm.mail[lane].rep, seen);
    }
    if (lane == 0) stat_add(sm.stat, ST_SECTIONS, 1);
  }
}

// Intra-warp resolution on the server when clients skip pre-validation (ring protocol): the
// same lane-order rule as TXPreValidation, over the sets in the mailbox.
template <int MAXR, int MAXW>
__device__ __forceinline__ uint32_t server_lane_order(const MailSlot<MAXR, MAXW>& ms,
                                                      uint32_t cand) {
  const uint32_t lane = lane_id();
  const bool active = (cand >> lane) & 1u;
  const uint32_t nrs = ms.n[lane] & 0xFFu;
  uint32_t conflict = 0;
  for (uint32_t i = 0; i < lane; i++) {
    if (!((cand >> i) & 1u)) continue;
    const uint32_t nw = ms.n[i] >> 8;
    for (uint32_t j = 0; j < nw; j++) {
      const uint32_t a = ms.ws[j][i];
      for (uint32_t k = 0; k < nrs; k++)
        if (ms.rs[k][lane] == a) conflict |= 1u << i;
    }
  }
  uint32_t commit = 0;
  for (uint32_t i = 0; i < 32; i++)
    commit |= __ballot_sync(0xFFFFFFFFu, lane == i && active && (conflict & commit) == 0);
  return commit;
}

template <int MAXR, int MAXW>
__device__ __forceinline__ void hash_clear(CtaShared<MAXR, MAXW>& sm) {
  uint4* k = reinterpret_cast<uint4*>(sm.hkey);
  for (uint32_t i = lane_id(); i < kHashSize / 4; i += 32) k[i] = make_uint4(~0u, ~0u, ~0u, ~0u);
  __syncwarp();
}

// set insert (write addresses of the batch's survivors); __match_any_sync lets one lane insert
// per distinct address when several lanes write the same (hot) item.
template <int MAXR, int MAXW>
__device__ __forceinline__ void hash_insert_set(CtaShared<MAXR, MAXW>& sm, uint32_t a, bool act) {
  const uint32_t peers = __match_any_sync(0xFFFFFFFFu, act ? a : 0xFFFFFFFFu);
  if (!act || (__ffs(peers) - 1) != (int)lane_id()) return;
  uint32_t h = hash_addr(a);
  for (uint32_t probe = 0; probe < kHashSize; probe++) {
    const uint32_t prev = atomicCAS(&sm.hkey[h], 0xFFFFFFFFu, a);
    if (prev == 0xFFFFFFFFu || prev == a) return;
    h = (h + 1) & (kHashSize - 1);
  }
}

template <int MAXR, int MAXW>
__device__ __forceinline__ bool hash_contains(const CtaShared<MAXR, MAXW>& sm, uint32_t a) {
  uint32_t h = hash_addr(a);
  for (uint32_t probe = 0; probe < kHashSize; probe++) {
    const uint32_t k = sm.hkey[h];
    if (k == a) return true;
    if (k == 0xFFFFFFFFu) return false;
    h = (h + 1) & (kHashSize - 1);
  }
  return false;
}

// multimap insert for the ring-mode read hash: (address -> candidate id), duplicates kept
template <int MAXR, int MAXW>
__device__ __forceinline__ bool hash_insert_multi(CtaShared<MAXR, MAXW>& sm, uint32_t a,
                                                  uint32_t cid) {
  uint32_t h = hash_addr(a);
  for (uint32_t probe = 0; probe < kHashSize; probe++) {
    if (atomicCAS(&sm.hkey[h], 0xFFFFFFFFu, a) == 0xFFFFFFFFu) {
      sm.hval[h] = cid;
      return true;
    }
    h = (h + 1) & (kHashSize - 1);
  }
  return false;
}

// Ring-mode scan of committed records with ts in (lo, hi]: lanes stride over records; each
// record's write addresses probe the batch read hash; a hit on a candidate whose snapshot is
// older than the record marks a conflict (collabValidation/csmv_sh/API.cu:212-253, with one scan
// per batch instead of one per lane). A record overwritten since (ts mismatch) marks RecordAge
// for every candidate older than it.
template <int MAXR, int MAXW>
__device__ void ring_scan(const BankParams& p, CtaShared<MAXR, MAXW>& sm, uint32_t lo,
                          uint32_t hi, const uint32_t* snaps, uint32_t bwarps) {
  for (uint32_t t = lo + 1 + lane_id(); t <= hi; t += 32) {
    const uint4 r = p.ring[t & p.ring_mask];
    if (r.x != t) {
      for (uint32_t m = bwarps; m; m &= m - 1) {
        const uint32_t w = __ffs(m) - 1;
        if (snaps[w] < t) atomicOr(&sm.recage[w], 0xFFFFFFFFu);
      }
      continue;
    }
    for (uint32_t j = 0; j < r.y && j < 2; j++) {
      const uint32_t a = j == 0 ? r.z : r.w;
      uint32_t h = hash_addr(a);
      for (uint32_t probe = 0; probe < kHashSize; probe++) {
        const uint32_t k = sm.hkey[h];
        if (k == 0xFFFFFFFFu) break;
        if (k == a) {
          const uint32_t cid = sm.hval[h], w = cid >> 5;
          if (snaps[w] < t) atomicOr(&sm.conflict[w], 1u << (cid & 31u));
        }
        h = (h + 1) & (kHashSize - 1);
      }
    }
  }
  __syncwarp();
}

// Ring protocol server (TXAddToRecord of the reference): batch, intra-batch conflicts, then one
// commit section per batch (per transaction for CSMV_BATCH_LANE) in ticket order.
template <int DEPTH, int MAXR, int MAXW>
__device__ void server_warp_ring(const BankParams& p, CtaShared<MAXR, MAXW>& sm) {
  const uint32_t lane = lane_id();
  const uint32_t nc = p.nc;
  uint32_t seen = 0;
  uint32_t* snaps = sm.snaps;
  const VersionStore vs{p.slots, p.n_items};

  for (;;) {
    uint32_t req;
    bool stop;
    uint32_t ready = poll_mailboxes(p.nc, p.gs, sm, seen, &req, &stop);
    if (ready == 0) {
      if (stop) break;
      __nanosleep(64);
      continue;
    }
    if (p.batch != CSMV_BATCH_CTA) ready &= (0u - ready);  // lowest ready warp only
    {  // the batch read hash must fit: cap the batch
      uint32_t capped = 0, entries = 0;
      for (uint32_t m = ready; m; m &= m - 1) {
        const uint32_t w = __ffs(m) - 1;
        if (capped && entries + 32u * MAXR > kHashSize / 2) break;
        capped |= 1u << w;
        entries += 32u * MAXR;
      }
      ready = capped;
    }
    if (lane < nc && ((ready >> lane) & 1u)) {
      seen = req;
      snaps[lane] = sm.mail[lane].snap;
    }
    __syncwarp();
    // every lane reads every batch mailbox: each takes its own acquire on the request word
    for (uint32_t m = ready; m; m &= m - 1) (void)ld_acquire_cta(&sm.mail[__ffs(m) - 1].req);

    // ---- phase A: candidates, intra-batch conflicts (outside the commit section) ----
    uint32_t surv_of_me = 0;  // lane w: survivors of client warp w
    const bool multi = __popc(ready) > 1;
    if (multi) hash_clear(sm);
    uint32_t stat_rw = 0;
    for (uint32_t m = ready; m; m &= m - 1) {
      const uint32_t w = __ffs(m) - 1;
      const MailSlot<MAXR, MAXW>& ms = sm.mail[w];
      uint32_t cand = ms.cand;
      if (!p.prevalidate) {
        const uint32_t pass = server_lane_order(ms, cand);
        stat_rw += __popc(cand & ~pass);
        cand = pass;
      }
      const bool c = (cand >> lane) & 1u;
      const uint32_t n = ms.n[lane], nrs = n & 0xFFu, nws = n >> 8;
      bool hit = false;
      if (multi && c)
        for (uint32_t k = 0; k < nrs && !hit; k++) hit = hash_contains(sm, ms.rs[k][lane]);
      const uint32_t s = __ballot_sync(0xFFFFFFFFu, c && !hit);
      stat_rw += __popc(cand & ~s);
      if (multi) {
        __syncwarp();
#pragma unroll
        for (int k = 0; k < MAXW; k++) hash_insert_set(sm, ms.ws[k][lane], ((s >> lane) & 1u) && k < (int)nws);
        __syncwarp();
      }
      if (lane == w) surv_of_me = s;
    }

    // the batch read hash and a pre-scan up to the current frontier
    hash_clear(sm);
    if (lane < nc) {
      sm.conflict[lane] = 0;
      sm.recage[lane] = 0;
    }
    __syncwarp();
    for (uint32_t m = ready; m; m &= m - 1) {
      const uint32_t w = __ffs(m) - 1;
      const uint32_t s = __shfl_sync(0xFFFFFFFFu, surv_of_me, w);
      const MailSlot<MAXR, MAXW>& ms = sm.mail[w];
      if ((s >> lane) & 1u) {
        const uint32_t nrs = ms.n[lane] & 0xFFu;
        for (uint32_t k = 0; k < nrs; k++) hash_insert_multi(sm, ms.rs[k][lane], w * 32 + lane);
      }
    }
    __syncwarp();
    uint32_t pre_hi = 0, lo = 0xFFFFFFFFu;
    for (uint32_t m = ready; m; m &= m - 1) lo = min(lo, snaps[__ffs(m) - 1]);
    if (lane == 0) pre_hi = (uint32_t)(ld_acquire_gpu(&p.gs->turn) >> 32);
    pre_hi = __shfl_sync(0xFFFFFFFFu, pre_hi, 0);
    const uint32_t floor_ts = pre_hi > p.ring_mask ? pre_hi - p.ring_mask : 0u;
    if (lo < floor_ts) lo = floor_ts;  // older snapshots fail the RecordAge rule anyway
    if (p.validate == CSMV_VALIDATE_RING && lo < pre_hi) ring_scan(p, sm, lo, pre_hi, snaps, ready);

    // ---- one commit section per batch (per transaction for CSMV_BATCH_LANE, like the
    // reference's per-lane CAS loop, bank/csmv_sh/API.cu:218-265) ----
    const bool lane_sections = p.batch == CSMV_BATCH_LANE;
    uint32_t todo_of_me = surv_of_me, done_of_me = 0;
    uint32_t scanned_hi = pre_hi;
    uint32_t stat_ra = 0, bid = 0;
    bool aborted_run = false;
    while (__any_sync(0xFFFFFFFFu, todo_of_me != 0)) {
      uint32_t sec_of_me = lane_sections ? (todo_of_me & (0u - todo_of_me)) : todo_of_me;
      todo_of_me &= ~sec_of_me;
      uint32_t ticket = 0;
      if (lane == 0) ticket = atomicAdd(&p.gs->ticket, 1u);
      ticket = __shfl_sync(0xFFFFFFFFu, ticket, 0);
      unsigned long long turn = 0;
      bool got = true;
      if (lane == 0)
        got = bounded_wait(
            [&] {
              turn = ld_acquire_gpu(&p.gs->turn);
              return (uint32_t)turn == ticket;
            },
            &p.gs->error, ERR_WAIT_TURN, p.spin_log2);
      got = __shfl_sync(0xFFFFFFFFu, got, 0);
      if (!got) {
        aborted_run = true;
        break;
      }
      const uint32_t C = (uint32_t)(__shfl_sync(0xFFFFFFFFu, turn, 0) >> 32);
      fence_acq_rel_gpu();
      if (p.validate == CSMV_VALIDATE_RING && scanned_hi < C) {
        ring_scan(p, sm, scanned_hi, C, snaps, ready);
        scanned_hi = C;
      }
      for (uint32_t m = ready; m; m &= m - 1) {
        const uint32_t w = __ffs(m) - 1;
        const MailSlot<MAXR, MAXW>& ms = sm.mail[w];
        const uint32_t s = __shfl_sync(0xFFFFFFFFu, sec_of_me, w);
        const uint32_t snap = snaps[w];
        bool bad = false, aged = false;
        if ((s >> lane) & 1u) {
          const uint32_t nrs = ms.n[lane] & 0xFFu;
          if (p.validate == CSMV_VALIDATE_RING) {
            aged = (uint64_t)snap + (p.ring_mask + 1) <= C || ((sm.recage[w] >> lane) & 1u);
            bad = !aged && ((sm.conflict[w] >> lane) & 1u);
          } else {  // plain per-lane scan of (snap, C], bank/csmv_sh/API.cu:88-144
            aged = (uint64_t)snap + (p.ring_mask + 1) <= C;
            for (uint32_t t = snap + 1; t <= C && !aged && !bad; t++) {
              const uint4 r = p.ring[t & p.ring_mask];
              if (r.x != t) {
                aged = true;
                break;
              }
              for (uint32_t k = 0; k < nrs; k++) {
                const uint32_t x = ms.rs[k][lane];
                bad |= (r.y > 0 && x == r.z) || (r.y > 1 && x == r.w);
              }
            }
          }
        }
        const uint32_t f = __ballot_sync(0xFFFFFFFFu, bad || aged);
        const uint32_t ag = __ballot_sync(0xFFFFFFFFu, aged);
        stat_ra += __popc(ag);
        stat_rw += __popc(f & ~ag);
        if (lane == w) sec_of_me = s & ~f;
      }
      // consecutive timestamps in (warp, lane) order; records and log
      uint32_t base = C;
      for (uint32_t m = ready; m; m &= m - 1) {
        const uint32_t w = __ffs(m) - 1;
        MailSlot<MAXR, MAXW>& ms = sm.mail[w];
        const uint32_t s = __shfl_sync(0xFFFFFFFFu, sec_of_me, w);
        if ((s >> lane) & 1u) {
          const uint32_t ts = base + 1 + __popc(s & lanemask_lt());
          const uint32_t nws = ms.n[lane] >> 8;
          WriteSet<MAXW> ws;
          ws.n = nws;
#pragma unroll
          for (int k = 0; k < MAXW; k++) {
            ws.addr[k] = ms.ws[k][lane];
            ws.val[k] = ms.wv[k][lane];
          }
          p.ring[ts & p.ring_mask] = make_uint4(ts, nws, ws.addr[0], ws.addr[MAXW - 1]);
          if (p.log) {
            const uint32_t li = ts - 1 - p.log_base;
            if (li < p.log_cap)
              p.log_txn[li] = ms.txn[lane];
            else
              raise_error(&p.gs->error, ERR_CAPACITY);
          }
          if (p.writeback == CSMV_WRITEBACK_SERVER) TXWriteBack<DEPTH>(ts, vs, ws);
          ms.tsl[lane] = ts;
        }
        base += __popc(s);
      }
      const uint32_t ncommit = base - C;
      __threadfence();
      __syncwarp();
      if (lane == 0) {
        if (p.writeback == CSMV_WRITEBACK_SERVER && ncommit) st_release_gpu(&p.gs->clock, base);
        st_release_gpu(&p.gs->turn, ((unsigned long long)base << 32) | (ticket + 1u));
        stat_add(sm.stat, ST_SECTIONS, 1);
      }
      done_of_me |= sec_of_me;
      if (p.writeback == CSMV_WRITEBACK_CLIENT && ncommit) {
        const uint32_t nw = __popc(__ballot_sync(0xFFFFFFFFu, lane < nc && sec_of_me != 0));
        if (lane == 0) {
          bid = sm.next_bid;
          sm.next_bid = (bid + 1) % kBatchDescs;
          sm.batch[bid].first_ts = C + 1;
          sm.batch[bid].last_ts = base;
          sm.batch[bid].remaining = nw;
        }
        bid = __shfl_sync(0xFFFFFFFFu, bid, 0);
      }
    }
    if (aborted_run) break;
    __syncwarp();
    if (lane < nc && ((ready >> lane) & 1u)) {
      MailSlot<MAXR, MAXW>& ms = sm.mail[lane];
      ms.ok = done_of_me;
      ms.bid = bid;
      st_release_cta(&ms.rep, seen);
    }
    if (lane == 0) {
      stat_add(sm.stat, ST_ABORT_READ_WRITE, stat_rw);
      stat_add(sm.stat, ST_ABORT_RECORD_AGE, stat_ra);
    }
  }
}

// ---------------------------------------------------------------------------------------------
// Serial lane: one warp runs a stream in stream order with the GPU to itself (no other commit
// kernel in flight), for transfers a scheduler predicts to conflict. A round's 32 transfers
// read the latest versions, then resolve their intra-round dependencies as one chain in lane
// order (each lane takes the values written by the nearest lower lane, as the chain mode of the
// commit kernel does), take consecutive timestamps in lane order and install their versions:
// the lowest lane writing an account installs every version of that account written in the
// round, in lane order, into its slots (victim = empty, else oldest), then stores them. No locks,
// no timestamp server, no validation: the lane is exclusive by construction, and every round
// commits. The timestamp order continues gs->ts_next and leaves the clock at the last one.
// ---------------------------------------------------------------------------------------------
template <int DEPTH, int MAXR>
__device__ __forceinline__ int32_t latest_of(const unsigned long long (&s)[DEPTH]) {
  uint32_t best = 0;
  int32_t v = 0;
  bool any = false;
#pragma unroll
  for (int d = 0; d < DEPTH; d++) {
    const uint32_t t = version_ts(s[d]);
    if (t != kEmptyTs && (!any || t > best)) {
      any = true;
      best = t;
      v = version_val(s[d]);
    }
  }
  return v;
}

constexpr int kLaneHash = 128;  // writer table of one serial-lane round (<= 64 accounts)

__device__ __forceinline__ uint32_t lane_hash(uint32_t a) { return (a * 0x9E3779B1u) >> 25; }

// Mask of the round's lanes writing account x (0 if none), from the shared-memory table.
__device__ __forceinline__ uint32_t writers_of(const uint32_t* hk, const uint32_t* hm, uint32_t x) {
  for (uint32_t h = lane_hash(x), probes = 0; probes < (uint32_t)kLaneHash; probes++) {
    const uint32_t k = hk[h];
    if (k == x) return hm[h];
    if (k == 0xFFFFFFFFu) return 0u;
    h = (h + 1u) & (kLaneHash - 1u);
  }
  return 0u;
}

// Slot of the want-th victim (empty first, else oldest; lowest index on ties) of DEPTH slots.
template <int DEPTH>
__device__ __forceinline__ int victim_rank_slot(const unsigned long long (&sl)[DEPTH], uint32_t want) {
  int slot = 0;
  if (want == 0) {  // the common case: the account's only (or first) writer of the round
    uint32_t best = version_ts(sl[0]) + 1u;
#pragma unroll
    for (int d = 1; d < DEPTH; d++) {
      const uint32_t k = version_ts(sl[d]) + 1u;
      if (k < best) {
        best = k;
        slot = d;
      }
    }
    return slot;
  }
#pragma unroll
  for (int d = 0; d < DEPTH; d++) {
    const uint32_t kd = version_ts(sl[d]) + 1u;
    uint32_t before = 0;
#pragma unroll
    for (int e = 0; e < DEPTH; e++) {
      const uint32_t ke = version_ts(sl[e]) + 1u;
      before += (ke < kd || (ke == kd && e < d)) ? 1u : 0u;
    }
    if (before == want) slot = d;
  }
  return slot;
}

// Shared memory of the serial lane. Round g's version slots are copied (cp.async, one round
// ahead) into stage[g & 1]; tables[g & 1] maps each account round g writes to the mask of its
// writer lanes and, after the round's installs, to its slots - round g+1 patches the slots it
// staged before round g's stores from there. 16-byte chunks of a lane's row are XOR-swizzled by
// lane so a quarter-warp's 16-byte reads hit distinct banks.
template <int DEPTH, int MAXR>
struct SerialSmem {
  unsigned long long stage[2][MAXR][32][DEPTH];
  unsigned long long ent[2][kLaneHash][DEPTH];
  uint32_t hk[2][kLaneHash], hm[2][kLaneHash];
};

template <int DEPTH, int MAXR>
__host__ __device__ constexpr size_t serial_smem_bytes() { return sizeof(SerialSmem<DEPTH, MAXR>); }

constexpr uint32_t kTomb = 0xFFFFFFFEu;  // table key of an account the round did not write

// Table slot of account x in table (hk) or -1.
__device__ __forceinline__ int table_slot(const uint32_t* hk, uint32_t x) {
  for (uint32_t h = lane_hash(x), probes = 0; probes < (uint32_t)kLaneHash; probes++) {
    const uint32_t k = hk[h];
    if (k == x) return (int)h;
    if (k == 0xFFFFFFFFu) return -1;
    h = (h + 1u) & (kLaneHash - 1u);
  }
  return -1;
}

template <int DEPTH, int MAXR>
__global__ void __launch_bounds__(32, 1) bank_serial_kernel(BankParams p) {
  extern __shared__ __align__(16) unsigned char serial_smem_raw[];
  SerialSmem<DEPTH, MAXR>& S = *reinterpret_cast<SerialSmem<DEPTH, MAXR>*>(serial_smem_raw);
  constexpr uint32_t kCh = DEPTH / 2, kSw = (kCh - 1u) < 3u ? (kCh - 1u) : 3u;
  const uint32_t lane = lane_id();
  const VersionStore vs{p.slots, p.n_items};
  const uint32_t base0 = ld_acquire_gpu(&p.gs->ts_next);  // == clock: nothing in flight
  uint32_t base = base0;
  unsigned long long n_upd = 0, n_nowrite = 0, n_ro = 0;
  const uint32_t R = p.n_rounds;

  auto load_opoff = [&](uint32_t r, uint32_t& op, uint32_t& off) {
    op = 0u;
    off = 0u;
    if (r < R) {
      op = p.op[r * 32u + lane];
      off = p.off[r * 32u + lane];
    }
  };
  auto load_addr = [&](uint32_t r, uint32_t op, uint32_t off, uint32_t (&a)[MAXR]) {
    const uint32_t nr = CSMV_OP_NREADS(op);
    const bool upd = r < R && CSMV_OP_KIND(op) != CSMV_KIND_READONLY;
#pragma unroll
    for (int k = 0; k < MAXR; k++) a[k] = (upd && k < (int)nr) ? p.addr[off + k] : 0u;
  };
  // copies of round r's slots into stage[buf] (transfers only; out-of-range ids are skipped here
  // and reported when the round is processed); one commit group per round, empty or not
  auto stage_round = [&](uint32_t r, uint32_t op, const uint32_t (&a)[MAXR], int buf) {
    if (r < R && CSMV_OP_KIND(op) != CSMV_KIND_READONLY) {
      const uint32_t nr = CSMV_OP_NREADS(op);
#pragma unroll
      for (int k = 0; k < MAXR; k++) {
        if (k >= (int)nr || a[k] >= p.n_items) continue;
        const unsigned long long* item = vs.slots + (size_t)a[k] * DEPTH;
#pragma unroll
        for (uint32_t c = 0; c < kCh; c++)
          cp_async16(&S.stage[buf][k][lane][(c ^ (lane & kSw)) * 2u], item + c * 2u);
      }
    }
    cp_async_commit();
  };
  auto staged = [&](int buf, int k, unsigned long long (&sl)[DEPTH]) {
#pragma unroll
    for (uint32_t c = 0; c < kCh; c++) {
      const unsigned long long* q = &S.stage[buf][k][lane][(c ^ (lane & kSw)) * 2u];
      sl[2 * c] = q[0];
      sl[2 * c + 1] = q[1];
    }
  };

  // pipeline: round g's addresses and staged slots are ready when g starts; round g+1's
  // addresses too; round g+2's op / offset
  uint32_t op_c, off_c, op_1, off_1, op_2, off_2, a_c[MAXR], a_1[MAXR];
  load_opoff(0, op_c, off_c);
  load_opoff(1, op_1, off_1);
  load_opoff(2, op_2, off_2);
  load_addr(0, op_c, off_c, a_c);
  load_addr(1, op_1, off_1, a_1);
  for (uint32_t i = lane; i < (uint32_t)kLaneHash; i += 32) S.hk[1][i] = 0xFFFFFFFFu;  // "round -1"
  stage_round(0, op_c, a_c, 0);
  __syncwarp();

  for (uint32_t g = 0; g < R; g++) {
    const int cb = (int)(g & 1u), pb = cb ^ 1;
    const uint32_t t = g * 32u + lane;
    // ahead: round g+1's slots, round g+2's addresses, round g+3's op / offset
    stage_round(g + 1, op_1, a_1, pb);
    uint32_t a_2[MAXR], op_3, off_3;
    load_addr(g + 2, op_2, off_2, a_2);
    load_opoff(g + 3, op_3, off_3);

    const uint32_t op = op_c, off = off_c;
    const uint32_t kind = CSMV_OP_KIND(op), nr = CSMV_OP_NREADS(op);
    const bool ro = __all_sync(0xFFFFFFFFu, kind == CSMV_KIND_READONLY);
    bool bad = (ro != (kind == CSMV_KIND_READONLY)) || (!ro && (nr < 2 || nr > (uint32_t)MAXR));
    if (!ro) {
#pragma unroll
      for (int k = 0; k < MAXR; k++) bad |= (k < (int)nr) && a_c[k] >= p.n_items;
    } else {
#pragma unroll 8
      for (uint32_t k = 0; k < nr; k++) bad |= p.addr[off + k] >= p.n_items;
    }
    if (__any_sync(0xFFFFFFFFu, bad)) {
      if (lane == 0) raise_error(&p.gs->error, ERR_DATA);
      break;
    }
    cp_async_wait_group<1>();  // round g's copies (round g+1's may still be in flight)
    __syncwarp();
    if (ro) {  // read-only: the state after every earlier transaction of the stream
      uint32_t sum = 0;
      for (uint32_t k0 = 0; k0 < nr; k0 += 8) {
        int32_t v8[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
          v8[j] = 0;
          if (k0 + j < nr) {
            unsigned long long sl[DEPTH];
            const unsigned long long* item = vs.slots + (size_t)p.addr[off + k0 + j] * DEPTH;
#pragma unroll
            for (int d = 0; d < DEPTH; d += 2) ld_relaxed_gpu_v2(item + d, sl[d], sl[d + 1]);
            v8[j] = latest_of<DEPTH, MAXR>(sl);
          }
        }
#pragma unroll
        for (int j = 0; j < 8; j++) sum += (uint32_t)v8[j];
      }
      if (p.log) {
        p.outcome[t] = base | kSnapFlag;
        p.result[t] = (int32_t)sum;
      }
      if (p.txn_aborts) p.txn_aborts[t] = 0u;
      n_ro += 32;
      for (uint32_t i = lane; i < (uint32_t)kLaneHash; i += 32) S.hk[cb][i] = 0xFFFFFFFFu;
    } else {
      uint32_t* hk = S.hk[cb];
      uint32_t* hm = S.hm[cb];
      const uint32_t* hk_prev = S.hk[pb];
      const uint32_t b1 = a_c[1] != a_c[0] ? a_c[1] : 0xFFFFFFFFu;
      for (uint32_t i = lane; i < (uint32_t)kLaneHash; i += 32) {
        hk[i] = 0xFFFFFFFFu;
        hm[i] = 0u;
      }
      __syncwarp();
      // the round's writers: account -> lane mask (a transfer with a0 == a1 writes it once)
      int hs[2] = {-1, -1};
#pragma unroll
      for (int w = 0; w < 2; w++) {
        const uint32_t x = w ? b1 : a_c[0];
        if (x == 0xFFFFFFFFu) continue;
        for (uint32_t h = lane_hash(x), probes = 0; probes < (uint32_t)kLaneHash; probes++) {
          const uint32_t prev = atomicCAS(&hk[h], 0xFFFFFFFFu, x);
          if (prev == 0xFFFFFFFFu || prev == x) {
            atomicOr(&hm[h], 1u << lane);
            hs[w] = (int)h;
            break;
          }
          h = (h + 1u) & (kLaneHash - 1u);
        }
      }
      // my slots as round g found them: staged, or patched from round g-1's installs
      int32_t v[MAXR];
      unsigned long long ed[2][DEPTH];
#pragma unroll
      for (int k = 0; k < MAXR; k++) {
        v[k] = 0;
        if (k >= (int)nr) continue;
        unsigned long long sl[DEPTH];
        const int e = table_slot(hk_prev, a_c[k]);
        if (e >= 0) {
#pragma unroll
          for (int d = 0; d < DEPTH; d++) sl[d] = S.ent[pb][e][d];
        } else {
          staged(cb, k, sl);
        }
        v[k] = latest_of<DEPTH, MAXR>(sl);
        if (k < 2)
#pragma unroll
          for (int d = 0; d < DEPTH; d++) ed[k][d] = sl[d];
      }
      __syncwarp();
      // lower lanes that may write what I read; writers of each of my written accounts
      uint32_t dep = 0;
#pragma unroll
      for (int k = 0; k < MAXR; k++)
        if (k < (int)nr) dep |= writers_of(hk, hm, a_c[k]);
      dep &= lanemask_lt();
      const uint32_t pot0 = hs[0] >= 0 ? hm[hs[0]] : 0u;
      const uint32_t pot1 = hs[1] >= 0 ? hm[hs[1]] : 0u;
      // forward the writes of each source lane, in lane order
      const ModMagic mm(CSMV_OP_AMOD(op));
      for (uint32_t m = __reduce_or_sync(0xFFFFFFFFu, dep); m; m &= m - 1) {
        const uint32_t i = __ffs(m) - 1;
        int32_t w0, w1;
        const bool hw = transfer_writes<MAXR>(op, nr, v, mm, w0, w1);
        const bool hwi = __shfl_sync(0xFFFFFFFFu, hw, i);
        const uint32_t x0 = __shfl_sync(0xFFFFFFFFu, a_c[0], i), x1 = __shfl_sync(0xFFFFFFFFu, a_c[1], i);
        const int32_t y0 = __shfl_sync(0xFFFFFFFFu, w0, i), y1 = __shfl_sync(0xFFFFFFFFu, w1, i);
        if (lane > i && hwi) {
#pragma unroll
          for (int k = 0; k < MAXR; k++) {
            if (k >= (int)nr) continue;
            if (a_c[k] == x1)
              v[k] = y1;
            else if (a_c[k] == x0)
              v[k] = y0;
          }
        }
      }
      int32_t w0, w1;
      const bool has_w = transfer_writes<MAXR>(op, nr, v, mm, w0, w1);
      const uint32_t wm = __ballot_sync(0xFFFFFFFFu, has_w);
      const uint32_t rank = __popc(wm & lanemask_lt());
      const uint32_t my_ts = base + rank + 1u;
      // installs: a version newer than every kept one replaces the victim (empty, else oldest),
      // so the round's n writers of an account fill its slots in the victim order of the slots
      // as the round found them - writer r (lane order) takes order[r % DEPTH] - and only the
      // last DEPTH of them survive; the last one also stamps the commit word (stamp = last
      // writer, unlocked), through which the stamp protocol reads the latest version. The
      // account's table entry receives the same slots for the next round.
      uint32_t same[2], total[2], r[2];
#pragma unroll
      for (int k = 0; k < 2; k++) {
        const uint32_t potk = k ? pot1 : pot0;
        same[k] = potk & wm;
        total[k] = __popc(same[k]);
        r[k] = __popc(same[k] & lanemask_lt());
        if (has_w && hs[k] >= 0 && r[k] == 0)  // the first writer copies the round-start slots
#pragma unroll
          for (int d = 0; d < DEPTH; d++) S.ent[cb][hs[k]][d] = ed[k][d];
        // an account none of its would-be writers wrote (funds short) holds no entry for the
        // next round: its key becomes a tombstone that lookups step over
        if (hs[k] >= 0 && same[k] == 0u && (potk & lanemask_lt()) == 0u) S.hk[cb][hs[k]] = kTomb;
      }
      __syncwarp();
      if (has_w) {
#pragma unroll
        for (int k = 0; k < 2; k++) {
          if (hs[k] < 0 || r[k] + DEPTH < total[k]) continue;
          const int slot = victim_rank_slot<DEPTH>(ed[k], r[k] % DEPTH);
          const int32_t val = (k == 0 && b1 != 0xFFFFFFFFu) ? w0 : w1;
          const unsigned long long ver = pack_version(my_ts, val);
          S.ent[cb][hs[k]][slot] = ver;
          st_relaxed_gpu(vs.slots + (size_t)a_c[k] * DEPTH + slot, ver);
          if (r[k] + 1u == total[k]) st_relaxed_gpu(&p.cw[a_c[k]], (unsigned long long)my_ts);
        }
      }
      if (p.log) {
        if (has_w) {
          const uint32_t li = my_ts - 1u - p.log_base;
          if (li < p.log_cap)
            p.log_txn[li] = t;
          else
            raise_error(&p.gs->error, ERR_CAPACITY);
          p.outcome[t] = my_ts;
        } else {
          p.outcome[t] = (base + rank) | kSnapFlag;  // serialised after the lower writers
        }
        p.result[t] = 0;
      }
      if (p.txn_aborts) p.txn_aborts[t] = 0u;
      n_upd += __popc(wm);
      n_nowrite += 32u - __popc(wm);
      base += __popc(wm);
    }
    __syncwarp();  // this round's versions, table and stage reads before the next round
    op_c = op_1;
    off_c = off_1;
    op_1 = op_2;
    off_1 = off_2;
    op_2 = op_3;
    off_2 = off_3;
#pragma unroll
    for (int k = 0; k < MAXR; k++) {
      a_c[k] = a_1[k];
      a_1[k] = a_2[k];
    }
  }
  cp_async_wait_all();
  // completion-bitmap words whose timestamps this lane passed over without setting bits: clear
  // them as the clock advance of the commit kernel would, before a later lap reuses them
  if (base > base0) {
    const uint32_t w_lo = (base0 + 1u) >> 5, w_end = (base + 1u) >> 5;  // words [w_lo, w_end)
    const uint32_t cnt = min(w_end > w_lo ? w_end - w_lo : 0u, p.done_mask + 1u);
    for (uint32_t i = lane; i < cnt; i += 32) st_relaxed_gpu(&p.done[(w_lo + i) & p.done_mask], 0u);
  }
  __threadfence();
  if (lane == 0) {
    st_relaxed_gpu(&p.gs->ts_next, base);
    st_release_gpu(&p.gs->clock, base);
    atomicAdd(&p.stats[ST_COMMIT_UPDATE], n_upd);
    atomicAdd(&p.stats[ST_COMMIT_NOWRITE], n_nowrite);
    atomicAdd(&p.stats[ST_COMMIT_RO], n_ro);
    atomicAdd(&p.stats[ST_SECTIONS], (unsigned long long)p.n_rounds);
    atomicAdd(&p.stats[ST_ROUNDS], (unsigned long long)p.n_rounds);
  }
}

template <int DEPTH, int MAXR, int MAXW>
__global__ void __launch_bounds__(512, 1) bank_kernel(BankParams p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CtaShared<MAXR, MAXW>& sm = *reinterpret_cast<CtaShared<MAXR, MAXW>*>(smem_raw);
  const uint32_t warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    sm.done_warps = 0;
    sm.next_bid = 0;
  }
  for (uint32_t i = threadIdx.x; i < ST_COUNT; i += blockDim.x) sm.stat[i] = 0;
  for (uint32_t i = threadIdx.x; i < p.nc; i += blockDim.x) {
    sm.mail[i].req = 0;
    sm.mail[i].rep = 0;
  }
  __syncthreads();
  if (warp == 0) {
    if (p.validate == CSMV_VALIDATE_STAMP)
      server_warp_stamp(p.nc, p.batch, p.gs, sm);
    else
      server_warp_ring<DEPTH, MAXR, MAXW>(p, sm);
  } else {
    GroupScratch* gx = reinterpret_cast<GroupScratch*>(
        smem_raw + group_scratch_offset(cta_shared_bytes<MAXR, MAXW>(p.nc)));
    client_warp<DEPTH, MAXR, MAXW>(p, sm, warp - 1, sm.mail[warp - 1], &sm.done_warps,
                                   gx + (warp - 1));
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < ST_COUNT; i += blockDim.x)
    if (sm.stat[i]) atomicAdd(&p.stats[i], sm.stat[i]);
}

// The thread-block-cluster form (one commit server for several blocks; the reference has no
// cluster code): the client warps of every CTA of a cluster post to the commit-server warp of
// the cluster's leader CTA, through mailboxes in the leader's shared memory reached over
// distributed shared memory. Stamp protocol only.
template <int DEPTH, int MAXR, int MAXW>
__global__ void __launch_bounds__(512, 1) bank_cluster_kernel(BankParams p) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CtaShared<MAXR, MAXW>& sm = *reinterpret_cast<CtaShared<MAXR, MAXW>*>(smem_raw);
  const uint32_t warp = threadIdx.x >> 5, rank = cluster.block_rank(), cs = cluster.num_blocks();
  const uint32_t nct = p.nc * cs;  // mailboxes of the cluster (<= 32)
  if (threadIdx.x == 0) {
    sm.done_warps = 0;
    sm.next_bid = 0;
  }
  for (uint32_t i = threadIdx.x; i < ST_COUNT; i += blockDim.x) sm.stat[i] = 0;
  for (uint32_t i = threadIdx.x; i < nct; i += blockDim.x) {
    sm.mail[i].req = 0;
    sm.mail[i].rep = 0;
  }
  cluster.sync();  // the leader's mailboxes are set before any client posts
  CtaShared<MAXR, MAXW>* lead = cluster.map_shared_rank(&sm, 0);
  if (warp == 0) {
    if (rank == 0) server_warp_stamp<CtaShared<MAXR, MAXW>, true>(nct, p.batch, p.gs, sm);
  } else {
    GroupScratch* gx = reinterpret_cast<GroupScratch*>(
        smem_raw + group_scratch_offset(cta_shared_bytes<MAXR, MAXW>(nct)));
    client_warp<DEPTH, MAXR, MAXW, true>(p, sm, warp - 1, lead->mail[rank * p.nc + warp - 1],
                                         &lead->done_warps, gx + (warp - 1));
  }
  cluster.sync();  // no CTA leaves while its mailboxes in the leader may still be touched
  for (uint32_t i = threadIdx.x; i < ST_COUNT; i += blockDim.x)
    if (sm.stat[i]) atomicAdd(&p.stats[i], sm.stat[i]);
}

}  // namespace csmv
