// memcd_kernel.cuh - transactional set-associative cache (the reference's memcachedGPU driver,
// memcachedGPU/memcdSH.cu:237-448) on the stamp commit protocol (sm_103a).
//
// Reference: four versioned arrays (key, val, ts, state) of one word each per way; a SET reads
// key/state/ts of every way with TXRead, picks the way holding the key (valid) or else the one
// with the smallest LRU timestamp, and writes all four items; a GET reads key/state of each way
// read-only and the value of the first match. Every transaction goes through the single
// commit-server block.
//
// Here an entry (set, way) holds kMemcdDepth versions; version j is
//   tag  (8 bytes): ts << 32 | valid << 31 | 31-bit key hash   - one single-copy-atomic word
//   rec  (64 bytes): {lru, 0, 0, 0}, 16-byte key, 32-byte value
// A writer (holding the entry's lock) empties the victim's tag, fences, writes the record,
// fences and publishes the new tag; a reader re-reads the tag after the record, so a record is
// used only if its tag did not move (a sequence-lock). The tags of a set's 8 ways sit in one
// 128-byte line: a GET at snapshot S loads them in one access, picks per way the newest version
// <= S, and reads only the records whose valid hash matches, in way order (first full key match
// wins, as the reference breaks at the first match). A SET reads each way's latest committed
// version (by its commit word), chooses the slot by the reference's rule, locks only that entry,
// takes a commit timestamp from the CTA's server, validates the eight stamps and installs the
// new version. Rounds of 32 requests are warp-uniform GETs or SETs (memcdSH.cu:333-339).
#pragma once
#include <cstdint>

#include "bank_kernel.cuh"

namespace csmv {

constexpr int kWays = 8;
constexpr int kMemcdDepth = 2;
constexpr uint32_t kValidBit = 0x80000000u;

struct MemcdParams {
  const uint32_t* kind;  // [n] 0 = GET, 1 = SET
  const uint4* key;      // [n]
  const uint4* val;      // [2n]
  uint32_t n_rounds;
  uint32_t tick;         // LRU timestamp a SET writes (the reference's curr_clock)
  uint32_t n_sets;
  unsigned long long* tag;  // [entry][kMemcdDepth]
  uint4* rec;               // [entry][kMemcdDepth][4]
  unsigned long long* cw;   // [entry] commit words
  uint32_t* done;
  uint32_t done_mask;
  GlobalSync* gs;
  uint32_t* found;       // [n]
  uint4* val_out;        // [2n]
  uint32_t* log_txn;
  uint32_t* outcome;
  uint32_t log, log_base, log_cap;
  unsigned long long* stats;
  uint32_t nc, batch, spin_log2;
};

struct MemcdMail {
  uint32_t req, rep, snap, cand, base, pad[3];
};

struct MemcdShared {
  uint32_t done_warps, pad[3];
  unsigned long long stat[ST_COUNT];
  MemcdMail mail[kMaxClientWarps];
};

// Set of a 16-byte key (the reference takes its one-word key modulo nbSets,
// memcdSH.cu:79-82; the four words are mixed first) and the 31-bit hash kept in the tag.
__host__ __device__ __forceinline__ uint32_t memcd_mix(uint32_t k0, uint32_t k1, uint32_t k2,
                                                       uint32_t k3) {
  uint32_t h = k0 * 0x9E3779B1u ^ k1 * 0x85EBCA6Bu ^ k2 * 0xC2B2AE35u ^ k3 * 0x27D4EB2Fu;
  return h ^ (h >> 16);
}
__host__ __device__ __forceinline__ uint32_t memcd_set_of(uint32_t h, uint32_t n_sets) {
  return h % n_sets;
}
__host__ __device__ __forceinline__ uint32_t memcd_tag_hash(uint32_t h) {
  return (h * 0x2C1B3C6Du) & 0x7FFFFFFFu;
}

__device__ __forceinline__ bool key_eq(uint4 a, uint4 b) {
  return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w;
}
__device__ __forceinline__ uint4 ld_relaxed_gpu_v4(const uint4* p) {
  uint4 v;
  asm volatile("ld.relaxed.gpu.global.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p)
               : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_gpu_v4(uint4* p, uint4 v) {
  asm volatile("st.relaxed.gpu.global.v4.u32 [%0], {%1, %2, %3, %4};" ::"l"(p), "r"(v.x),
               "r"(v.y), "r"(v.z), "r"(v.w)
               : "memory");
}
__device__ __forceinline__ uint32_t tag_ts(unsigned long long t) { return (uint32_t)(t >> 32); }

// One round of 32 requests (request r on this lane), run until every request has committed.
// Returns false when the warp must stop (device error raised).
__device__ bool memcd_round(const MemcdParams& p, MemcdShared& sm, MemcdMail& ms, uint32_t me,
                            uint32_t r, uint32_t& seq, uint32_t tick) {
  constexpr int D = kMemcdDepth;
  const uint32_t lane = lane_id();
  bool failed = false;
  {
    const uint32_t kind = p.kind[r];
    const bool is_set = __all_sync(0xFFFFFFFFu, kind == 1u);
    if (__any_sync(0xFFFFFFFFu, (kind == 1u) != is_set || kind > 1u)) {  // mixed round
      if (lane == 0) raise_error(&p.gs->error, ERR_DATA);
      return false;
    }
    const uint4 key = p.key[r];
    const uint32_t hmix = memcd_mix(key.x, key.y, key.z, key.w);
    const uint32_t e0 = memcd_set_of(hmix, p.n_sets) * kWays;
    const uint32_t th = memcd_tag_hash(hmix) | kValidBit;
    uint4 nv0 = make_uint4(0, 0, 0, 0), nv1 = nv0;
    if (is_set) {
      nv0 = p.val[2 * r];
      nv1 = p.val[2 * r + 1];
    }
    uint32_t pending = 0xFFFFFFFFu, attempts = 0, lock_fails = 0;
    while (pending) {
      if (lane == 0) atomicAdd(&sm.stat[ST_ROUNDS], 1ull);
      if (++attempts > (1u << 20)) {
        if (lane == 0) raise_error(&p.gs->error, ERR_LIVELOCK);
        failed = true;
        break;
      }
      if (lock_fails) {
        const uint32_t h = (me * 0x9E3779B1u) ^ (attempts * 0x85EBCA6Bu);
        __nanosleep((h >> 16) & ((64u << lock_fails) - 1u));
      }
      const bool mine = (pending >> lane) & 1u;
      uint32_t snap = 0;
      if (lane == 0) snap = ld_acquire_gpu(&p.gs->clock);
      snap = __shfl_sync(0xFFFFFFFFu, snap, 0);
      // the set's tag words: 8 ways x kMemcdDepth versions, one 128-byte line
      unsigned long long tg[kWays * D];
      if (mine) {
#pragma unroll
        for (int i = 0; i < kWays * D; i += 2)
          ld_relaxed_gpu_v2(p.tag + (size_t)e0 * D + i, tg[i], tg[i + 1]);
      }

      if (!is_set) {
        // GET: the latest committed version of each way, read through its commit word and
        // re-checked afterwards (a double collect), serialised at the largest stamp read. The
        // stamp's version is never a writer's victim (that is the older slot), so its record
        // stays put while the stamp does. Locks: a holder with a timestamp above the snapshot
        // commits after it and is ignored; one below it, or one still without a timestamp when
        // the GET looks, may commit inside the snapshot, so the GET waits (bounded) or retries.
        bool found = false, aged = false;
        uint32_t smax = 0;
        uint4 o0 = make_uint4(0, 0, 0, 0), o1 = o0;
        if (mine) {
          unsigned long long w1[kWays];
#pragma unroll
          for (int wy = 0; wy < kWays; wy++) w1[wy] = ld_relaxed_gpu(&p.cw[e0 + wy]);
#pragma unroll
          for (int wy = 0; wy < kWays; wy++) {
            // a holder still without a timestamp is waited for (bounded); so, briefly, is one
            // with a timestamp (a SET about to install: waiting for it costs less than the
            // retry its timestamp below the snapshot would force)
            for (uint32_t it = 0; it < 512u; it++) {
              const uint32_t own = (uint32_t)(w1[wy] >> 32);
              if (own == 0u || ((own & kPendingFlag) && it >= 32u)) break;
              __nanosleep(64);
              w1[wy] = ld_relaxed_gpu(&p.cw[e0 + wy]);
            }
          }
          fence_acq_rel_gpu();  // versions after the stamps
          unsigned long long tg2[kWays * D];
#pragma unroll
          for (int i = 0; i < kWays * D; i += 2)
            ld_relaxed_gpu_v2(p.tag + (size_t)e0 * D + i, tg2[i], tg2[i + 1]);
          int pick[kWays];
          unsigned long long ptag[kWays];
#pragma unroll
          for (int wy = 0; wy < kWays; wy++) {
            const uint32_t st = (uint32_t)w1[wy], own = (uint32_t)(w1[wy] >> 32);
            if (own != 0u && !(own & kPendingFlag)) aged = true;  // still no timestamp: retry
            smax = max(smax, st);
            int j = -1;
            unsigned long long t0 = 0;
#pragma unroll
            for (int q = 0; q < D; q++)
              if (tag_ts(tg2[wy * D + q]) == st) {
                j = q;
                t0 = tg2[wy * D + q];
              }
            pick[wy] = j;
            ptag[wy] = t0;
            aged |= j < 0;
          }
#pragma unroll
          for (int wy = 0; wy < kWays; wy++) {
            const uint32_t own = (uint32_t)(w1[wy] >> 32);
            if ((own & kPendingFlag) && (own & ~kPendingFlag) < smax) aged = true;
          }
#pragma unroll
          for (int wy = 0; wy < kWays; wy++) {
            const unsigned long long t0 = ptag[wy];
            // skip: decided, or not valid, or another key's hash
            if (aged || found || (uint32_t)t0 != th) continue;
            const size_t v = (size_t)(e0 + wy) * D + pick[wy];
            const uint4 kk = ld_relaxed_gpu_v4(p.rec + v * 4 + 1);
            if (key_eq(kk, key)) {
              found = true;
              o0 = ld_relaxed_gpu_v4(p.rec + v * 4 + 2);
              o1 = ld_relaxed_gpu_v4(p.rec + v * 4 + 3);
            }
          }
          fence_acq_rel_gpu();
#pragma unroll
          for (int wy = 0; wy < kWays; wy++) {  // the second collect
            const unsigned long long w2 = ld_relaxed_gpu(&p.cw[e0 + wy]);
            const uint32_t own = (uint32_t)(w2 >> 32);
            if ((uint32_t)w2 != (uint32_t)w1[wy]) aged = true;
            if ((own & kPendingFlag) && (own & ~kPendingFlag) < smax) aged = true;
            // a holder without a timestamp that locked after the first collect draws its
            // timestamp after every stamp read here: it lands above the snapshot
          }
        }
        const bool done = mine && !aged;
        if (done) {
          p.found[r] = found ? 1u : 0u;
          p.val_out[2 * r] = o0;
          p.val_out[2 * r + 1] = o1;
          // every commit up to the clock read before the first collect was visible to it, so
          // the state read is also the state at that clock when it is the later of the two
          if (p.log) p.outcome[r] = max(smax, snap) | kSnapFlag;
        }
        const uint32_t dm = __ballot_sync(0xFFFFFFFFu, done);
        const uint32_t am = __ballot_sync(0xFFFFFFFFu, mine && aged);
        if (lane == 0) {
          stat_add(sm.stat, ST_COMMIT_RO, __popc(dm));
          stat_add(sm.stat, ST_ABORT_DATA_AGE, __popc(am));
        }
        pending &= ~dm;
        continue;
      }

      // SET: each way's latest committed version (the one whose ts is the way's stamp); the
      // slot by the reference's rule: the way holding the key (valid), else the smallest LRU
      // timestamp, first on ties (memcdSH.cu:365-387)
      uint32_t stw[kWays];
      bool aborted = false;
      int slot = -1;
      uint32_t slot_lru = 0;
      bool matched = false;
#pragma unroll
      for (int wy = 0; wy < kWays; wy++) stw[wy] = 0;
      if (mine) {
        unsigned long long wordv[kWays];
#pragma unroll
        for (int wy = 0; wy < kWays; wy++) wordv[wy] = ld_relaxed_gpu(&p.cw[e0 + wy]);
        fence_acq_rel_gpu();  // the record loads stay behind the tag loads (sequence lock)
        int sj[kWays];
        unsigned long long s0[kWays];
        uint32_t lru[kWays];
        bool km[kWays];
#pragma unroll
        for (int wy = 0; wy < kWays; wy++) {
          const uint32_t st = (uint32_t)wordv[wy];
          stw[wy] = st;
          int j = -1;
          unsigned long long t0 = 0;
#pragma unroll
          for (int q = 0; q < D; q++)
            if (tag_ts(tg[wy * D + q]) == st) {
              j = q;
              t0 = tg[wy * D + q];
            }
          sj[wy] = j;
          s0[wy] = t0;
          lru[wy] = 0;
          km[wy] = false;
          if (j < 0) {  // the stamp's version not seen yet (fetched concurrently): retry
            aborted = true;
            continue;
          }
          const size_t v = (size_t)(e0 + wy) * D + j;
          const uint4 hd = ld_relaxed_gpu_v4(p.rec + v * 4);
          const uint4 kk = ld_relaxed_gpu_v4(p.rec + v * 4 + 1);
          lru[wy] = hd.x;
          km[wy] = ((uint32_t)t0 & kValidBit) && key_eq(kk, key);
        }
        fence_acq_rel_gpu();
        unsigned long long tg2[kWays * D];
#pragma unroll
        for (int i = 0; i < kWays * D; i += 2)
          ld_relaxed_gpu_v2(p.tag + (size_t)e0 * D + i, tg2[i], tg2[i + 1]);
#pragma unroll
        for (int wy = 0; wy < kWays; wy++) {
#pragma unroll
          for (int q = 0; q < D; q++)
            if (q == sj[wy] && tg2[wy * D + q] != s0[wy]) aborted = true;  // record moved
          if (!matched) {
            if (km[wy]) {
              slot = wy;
              matched = true;
            } else if (slot < 0 || lru[wy] < slot_lru) {
              slot = wy;
              slot_lru = lru[wy];
            }
          }
        }
      }
      const uint32_t target = e0 + (uint32_t)(slot < 0 ? 0 : slot);
      // intra-warp: lane order over (reads: the 8 entries of the set, write: the slot)
      ReadSet<kWays> rs;
      WriteSet<1> ws;
      bool cand_me = mine && !aborted;
      if (cand_me) {
        rs.n = kWays;
#pragma unroll
        for (int wy = 0; wy < kWays; wy++) rs.addr[wy] = e0 + wy;
        ws.n = 1;
        ws.addr[0] = target;
      }
      uint32_t cand = __ballot_sync(0xFFFFFFFFu, cand_me);
      const uint32_t overlap = TXWriteOverlap(ws, cand_me);
      const bool attempt = cand_me && (overlap & cand) == 0;
      const bool got = attempt && atomicCAS(owner_word(p.cw, target), 0u, me) == 0u;
      const uint32_t locked = __ballot_sync(0xFFFFFFFFu, got);
      const uint32_t pass = TXPreValidation(rs, ws, got);
      if (got && !((pass >> lane) & 1u)) st_relaxed_gpu(owner_word(p.cw, target), 0u);
      const uint32_t agm = __ballot_sync(0xFFFFFFFFu, mine && aborted);
      if (lane == 0) {
        stat_add(sm.stat, ST_ABORT_DATA_AGE, __popc(agm));
        stat_add(sm.stat, ST_ABORT_WRITE_WRITE, __popc(cand & ~locked));
        stat_add(sm.stat, ST_ABORT_PREVALID, __popc(locked & ~pass));
      }
      lock_fails = __ballot_sync(0xFFFFFFFFu, attempt && !got) ? min(lock_fails + 1, 6u) : 0u;
      cand = pass;
      cand_me = (cand >> lane) & 1u;
      if (cand == 0) continue;
      // commit timestamps from the CTA's server
      seq++;
      __syncwarp();
      if (lane == 0) {
        ms.snap = snap;
        ms.cand = cand;
        st_release_cta(&ms.req, seq);
      }
      bool ok_wait = true;
      if (lane == 0)
        ok_wait = bounded_wait([&] { return ld_acquire_cta(&ms.rep) == seq; }, &p.gs->error,
                               ERR_WAIT_REPLY, p.spin_log2);
      ok_wait = __shfl_sync(0xFFFFFFFFu, ok_wait, 0);
      if (!ok_wait) {
        failed = true;
        break;
      }
      (void)ld_acquire_cta(&ms.rep);
      const uint32_t base = ms.base;
      const uint32_t my_ts = base + 1 + __popc(cand & lanemask_lt());
      fence_acq_rel_gpu();
      if (cand_me) st_relaxed_gpu(owner_word(p.cw, target), kPendingFlag | my_ts);
      bool valid = cand_me;
      if (cand_me) {
        unsigned long long wd[kWays];
#pragma unroll
        for (int wy = 0; wy < kWays; wy++) wd[wy] = ld_relaxed_gpu(&p.cw[e0 + wy]);
#pragma unroll
        for (int wy = 0; wy < kWays; wy++) {
          if (!valid) continue;
          // a lock of an earlier or not yet numbered holder: wait (bounded) for its outcome;
          // a later holder is ordered after this SET and is ignored
          bool settled = false;
          for (uint32_t it = 0; it < 2048; it++) {
            const uint32_t own = (uint32_t)(wd[wy] >> 32);
            if (own == 0u || own == me ||
                ((own & kPendingFlag) && (own & ~kPendingFlag) >= my_ts)) {
              settled = true;
              break;
            }
            __nanosleep(32);
            wd[wy] = ld_relaxed_gpu(&p.cw[e0 + wy]);
          }
          valid = settled && (uint32_t)wd[wy] == stw[wy];
        }
      }
      const uint32_t okm = __ballot_sync(0xFFFFFFFFu, valid);
      if (lane == 0) stat_add(sm.stat, ST_ABORT_READ_WRITE, __popc(cand & ~okm));
      if (p.log && cand_me) {
        const uint32_t li = my_ts - 1 - p.log_base;
        if (li < p.log_cap)
          p.log_txn[li] = valid ? r : kHole;
        else
          raise_error(&p.gs->error, ERR_CAPACITY);
      }
      if (valid) {  // install: an empty version first, else the oldest (we hold the lock)
        const size_t v0 = (size_t)target * D;
        int vic = 0;
        uint32_t vkey = 0xFFFFFFFFu;
#pragma unroll
        for (int j = 0; j < D; j++) {
          const uint32_t k = tag_ts(ld_relaxed_gpu(p.tag + v0 + j)) + 1u;
          if (j == 0 || k < vkey) {
            vkey = k;
            vic = j;
          }
        }
        const size_t v = v0 + vic;
        st_relaxed_gpu(p.tag + v, (unsigned long long)kEmptyTs << 32);  // readers: moving
        __threadfence();
        st_relaxed_gpu_v4(p.rec + v * 4, make_uint4(tick, 0u, 0u, 0u));
        st_relaxed_gpu_v4(p.rec + v * 4 + 1, key);
        st_relaxed_gpu_v4(p.rec + v * 4 + 2, nv0);
        st_relaxed_gpu_v4(p.rec + v * 4 + 3, nv1);
        __threadfence();
        st_relaxed_gpu(p.tag + v, ((unsigned long long)my_ts << 32) | th);
        if (p.log) p.outcome[r] = my_ts;
        p.found[r] = 0u;
        p.val_out[2 * r] = make_uint4(0, 0, 0, 0);
        p.val_out[2 * r + 1] = make_uint4(0, 0, 0, 0);
      }
      __threadfence();  // with the relaxed store below, the release of the stamp
      if (cand_me) {
        if (valid)
          st_relaxed_gpu(&p.cw[target], (unsigned long long)my_ts);
        else
          st_relaxed_gpu(owner_word(p.cw, target), 0u);
      }
      __syncwarp();
      if (lane == 0) {
        complete_range(p.done, p.done_mask, p.gs, base + 1, base + __popc(cand));
        stat_add(sm.stat, ST_COMMIT_UPDATE, __popc(okm));
      }
      pending &= ~okm;
      uint32_t err = 0;
      if (lane == 0) err = ld_relaxed_gpu(&p.gs->error);
      if (__shfl_sync(0xFFFFFFFFu, err, 0) != 0) {
        failed = true;
        break;
      }
    }
  }
  return !failed;
}

__device__ void memcd_client(const MemcdParams& p, MemcdShared& sm, uint32_t w) {
  MemcdMail& ms = sm.mail[w];
  const uint32_t lane = lane_id();
  const uint32_t me = blockIdx.x * p.nc + w + 1;
  uint32_t seq = 0;
  for (;;) {
    uint32_t g = 0;
    if (lane == 0) g = atomicAdd(&p.gs->round_next, 1u);
    g = __shfl_sync(0xFFFFFFFFu, g, 0);
    if (g >= p.n_rounds) break;
    if (!memcd_round(p, sm, ms, me, g * 32u + lane, seq, p.tick)) break;
  }
  __syncwarp();
  if (lane == 0) atomicAdd(&sm.done_warps, 1u);
}

__global__ void __launch_bounds__(512, 1) memcd_kernel(MemcdParams p) {
  __shared__ MemcdShared sm;
  const uint32_t warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) sm.done_warps = 0;
  for (uint32_t i = threadIdx.x; i < ST_COUNT; i += blockDim.x) sm.stat[i] = 0;
  for (uint32_t i = threadIdx.x; i < p.nc; i += blockDim.x) {
    sm.mail[i].req = 0;
    sm.mail[i].rep = 0;
  }
  __syncthreads();
  if (warp == 0)
    server_warp_stamp(p.nc, p.batch, p.gs, sm);
  else
    memcd_client(p, sm, warp - 1);
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < ST_COUNT; i += blockDim.x)
    if (sm.stat[i]) atomicAdd(&p.stats[i], sm.stat[i]);
}

// ---------------------------------------------------------------------------------------------
// Serving: a persistent kernel that admits request batches as the host publishes them.
//
// Requests live in a ring ("arena") of pinned, mapped host memory that the kernel reads and
// writes in place (coherent over the C2C link of a Grace-Blackwell node): request i of a batch
// that starts at arena index f is request (f + i) mod arena size. The host publishes a batch by
// filling its descriptor and then bumping ctl->submitted (release). ONE warp (the first client
// warp of CTA 0) is the admitter: it alone polls the host's control words, turns newly
// published batches into rounds of 32 requests appended to the device round queue, and releases
// the queue tail; it runs no rounds. Every other client warp takes a ticket (the next round
// index, one atomic add) and polls the queue tail in device memory until its round exists, then
// runs it with the cache's commit protocol, so rounds of different batches overlap on the device
// and idle warps put no traffic on the host link (and little on the queue's line: a warp polls
// less often the farther its ticket is from the tail). After a round, the warp makes its results
// visible to the host and counts the round off its batch; the batch's last round stamps done_ns
// and sets done (release). Once ctl->stop is set and every published batch is admitted, or when
// the host has published nothing and every round is done for idle_ns (error ERR_WAIT_REQUEST),
// the admitter raises dev->quit; a warp leaves when quit is set and its ticket is past the tail.
// ---------------------------------------------------------------------------------------------
constexpr uint32_t kServeSlots = 1024;  // batch descriptors in flight at most

struct ServeHostCtl {     // mapped host memory
  uint32_t submitted;     // host: batches published
  uint32_t stop;          // host: finish what is published, then return
  uint32_t error;         // device: first device error of the session (0 = none)
  uint32_t pad[13];
};

struct ServeBatchDesc {   // mapped host memory, one per in-flight batch (slot = batch % kServeSlots)
  uint32_t first, n_req, tick, seq;
  unsigned long long admit_ns, done_ns;  // device global timer
  uint32_t done, sets, pad[6];
};

struct alignas(128) ServeDev {  // device memory
  alignas(128) uint32_t admitted;     // batches turned into rounds
  alignas(128) uint32_t q_head;       // round tickets taken
  alignas(128) uint32_t q_tail;       // rounds appended
  alignas(128) uint32_t rounds_done;  // rounds completed
  alignas(128) uint32_t quit;         // no round will be appended any more
};

struct ServeParams {
  ServeHostCtl* ctl;
  ServeBatchDesc* desc;
  ServeDev* dev;
  uint2* rq;             // [q_mask + 1] {first request index, batch slot}
  uint32_t q_mask;
  uint32_t arena_mask;
  uint32_t* remaining;   // [kServeSlots] rounds left per batch
  uint32_t* tick;        // [kServeSlots] LRU tick per batch
  unsigned long long idle_ns;
  uint32_t serial;       // 1: one batch on the device at a time
};

// The admitter's loop, warp-collective: the only reader of the host's control words.
__device__ void serve_admitter(const MemcdParams& p, const ServeParams& s) {
  const uint32_t lane = lane_id();
  uint32_t adm = 0, qt = 0, last_sub = 0;
  unsigned long long idle_since = globaltimer_ns();
  for (;;) {
    uint32_t sub = 0, stop = 0, err = 0, done = 0;
    if (lane == 0) {
      sub = ld_acquire_sys(&s.ctl->submitted);
      stop = ld_acquire_sys(&s.ctl->stop);
      err = ld_relaxed_gpu(&p.gs->error);
      done = ld_relaxed_gpu(&s.dev->rounds_done);
    }
    sub = __shfl_sync(0xFFFFFFFFu, sub, 0);
    stop = __shfl_sync(0xFFFFFFFFu, stop, 0);
    err = __shfl_sync(0xFFFFFFFFu, err, 0);
    done = __shfl_sync(0xFFFFFFFFu, done, 0);
    if (err) {
      if (lane == 0) st_release_sys(&s.ctl->error, err);  // the host sees it without waiting
      break;
    }
    // one batch at a time (s.serial): the next batch's rounds are appended once every round
    // appended so far is done, so a batch runs alone on the device, as a synchronous call would
    const uint32_t admit_to = (s.serial && done != qt) ? adm : (s.serial ? min(sub, adm + 1u) : sub);
    const bool fresh = adm < admit_to;
    for (uint32_t guard = 0; adm < admit_to && guard < kServeSlots; guard++, adm++) {
      const uint32_t slot = adm % kServeSlots;
      uint32_t first = 0, n = 0, tk = 0;
      if (lane == 0) {
        const volatile ServeBatchDesc* d = s.desc + slot;
        first = d->first;
        n = d->n_req;
        tk = d->tick;
      }
      first = __shfl_sync(0xFFFFFFFFu, first, 0);
      n = __shfl_sync(0xFFFFFFFFu, n, 0);
      tk = __shfl_sync(0xFFFFFFFFu, tk, 0);
      const uint32_t rounds = n / 32u;
      for (uint32_t i = lane; i < rounds; i += 32)
        s.rq[(qt + i) & s.q_mask] = make_uint2((first + 32u * i) & s.arena_mask, slot);
      if (lane == 0) {
        s.remaining[slot] = rounds;
        s.tick[slot] = tk;
        s.desc[slot].admit_ns = globaltimer_ns();
      }
      qt += rounds;
    }
    __syncwarp();
    if (fresh && lane == 0) {
      st_relaxed_gpu(&s.dev->admitted, adm);
      __threadfence();
      st_release_gpu(&s.dev->q_tail, qt);  // rounds, counts and ticks before the tail
    }
    const unsigned long long now = globaltimer_ns();
    if (sub != last_sub || done != qt) {  // the host published, or rounds are running: not idle
      last_sub = sub;
      idle_since = now;
    }
    if (stop && adm == sub) break;  // (serial: adm reaches sub only after the last admission)
    if (now - idle_since > s.idle_ns) {
      if (lane == 0) {
        raise_error(&p.gs->error, ERR_WAIT_REQUEST);
        st_release_sys(&s.ctl->error, ERR_WAIT_REQUEST);
      }
      break;
    }
    if (!fresh) __nanosleep(256);
  }
  if (lane == 0) st_release_gpu(&s.dev->quit, 1u);
}

__device__ void serve_client(const MemcdParams& p, const ServeParams& s, MemcdShared& sm,
                             uint32_t w) {
  MemcdMail& ms = sm.mail[w];
  const uint32_t lane = lane_id();
  const uint32_t me = blockIdx.x * p.nc + w + 1;
  uint32_t seq = 0;
  if (blockIdx.x == 0 && w == 0) {
    serve_admitter(p, s);
  } else {
    for (;;) {
      uint32_t state = 0u, first = 0u, slot = 0u;  // 1: a round, 2: leave
      if (lane == 0) {
        const uint32_t ticket = atomicAdd(&s.dev->q_head, 1u);
        for (;;) {
          const uint32_t tail = ld_acquire_gpu(&s.dev->q_tail);
          if (ticket < tail) {
            const uint2 e = s.rq[ticket & s.q_mask];
            first = e.x;
            slot = e.y;
            state = 1u;
            break;
          }
          if (ld_acquire_gpu(&s.dev->quit) && ticket >= ld_acquire_gpu(&s.dev->q_tail)) {
            state = 2u;  // nothing more will be appended
            break;
          }
          if (ld_relaxed_gpu(&p.gs->error)) {
            state = 2u;
            break;
          }
          // the farther back a ticket is, the more rounds must be appended before it: poll
          // less often, so idle warps do not crowd the queue's L2 line
          __nanosleep(min(64u + 32u * (ticket - tail), 8192u));
        }
      }
      state = __shfl_sync(0xFFFFFFFFu, state, 0);
      if (state == 2u) break;
      first = __shfl_sync(0xFFFFFFFFu, first, 0);
      slot = __shfl_sync(0xFFFFFFFFu, slot, 0);
      uint32_t tk = 0;
      if (lane == 0) tk = ld_relaxed_gpu(&s.tick[slot]);
      tk = __shfl_sync(0xFFFFFFFFu, tk, 0);
      if (!memcd_round(p, sm, ms, me, (first + lane) & s.arena_mask, seq, tk)) {
        if (lane == 0) st_release_sys(&s.ctl->error, max(1u, ld_relaxed_gpu(&p.gs->error)));
        break;
      }
      __syncwarp();
      if (lane == 0) {
        __threadfence_system();  // this round's results reach the host before its batch completes
        if (atomicSub(&s.remaining[slot], 1u) == 1u) {
          s.desc[slot].done_ns = globaltimer_ns();
          __threadfence_system();
          st_release_sys(&s.desc[slot].done, 1u);
        }
        atomicAdd(&s.dev->rounds_done, 1u);
      }
    }
  }
  __syncwarp();
  if (lane == 0) atomicAdd(&sm.done_warps, 1u);
}

__global__ void __launch_bounds__(512, 1) memcd_serve_kernel(MemcdParams p, ServeParams s) {
  __shared__ MemcdShared sm;
  const uint32_t warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) sm.done_warps = 0;
  for (uint32_t i = threadIdx.x; i < ST_COUNT; i += blockDim.x) sm.stat[i] = 0;
  for (uint32_t i = threadIdx.x; i < p.nc; i += blockDim.x) {
    sm.mail[i].req = 0;
    sm.mail[i].rep = 0;
  }
  __syncthreads();
  if (warp == 0)
    server_warp_stamp(p.nc, p.batch, p.gs, sm);
  else
    serve_client(p, s, sm, warp - 1);
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < ST_COUNT; i += blockDim.x)
    if (sm.stat[i]) atomicAdd(&p.stats[i], sm.stat[i]);
}

}  // namespace csmv
