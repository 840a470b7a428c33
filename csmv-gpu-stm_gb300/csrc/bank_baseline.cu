// bank_baseline.cu - the reference's naive baseline STM as a comparison arm over the bank
// handle (csmv_bank_run_baseline_device).
//
// The reference's baseline bank (bank/baseline: "a naive implementation ... based on JVSTM")
// has no commit server: every transaction reads at its snapshot with the version rule
// (bank/baseline/API.cu:3-59), validates its read set against the commit records written since
// its snapshot (TXValidate, API.cu:83-140) and commits inside one global critical section, the
// CAS on the record ring's write head (TXAddToRecordNaive, API.cu:228-316): it appends its
// record, writes its versions back and moves the global clock. This restatement keeps that
// algorithm - snapshot reads, validation against records, one commit section for the whole GPU
// - with the section taken once per warp instead of once per thread, in ticket order: the
// warp's transactions that pass validation commit in lane order inside it, a lane that reads
// what a lower lane of the section writes is aborted like a record conflict, and the clock
// moves once per section.
//
// State: the handle's version slots, commit words (kept as stamps, so stamp-protocol runs carry
// on from a baseline run), record ring {ts, n_writes, w0, w1} and log. The commit order
// continues the handle's (ts_next and clock move together), so runs of the engine and of this
// arm interleave on one bank and replay as one log.
#include <algorithm>
#include <chrono>

#include "bank_internal.h"

namespace csmv {
namespace {

template <int DEPTH, int MAXR>
__global__ void __launch_bounds__(512, 1) baseline_kernel(BankParams p) {
  constexpr uint32_t FULL = 0xFFFFFFFFu;
  __shared__ unsigned long long stat[ST_COUNT];
  for (uint32_t i = threadIdx.x; i < ST_COUNT; i += blockDim.x) stat[i] = 0;
  __syncthreads();
  const uint32_t lane = lane_id();
  const VersionStore vs{p.slots, p.n_items};
  const uint32_t me = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  bool failed = false;
  while (!failed) {
    uint32_t g = 0;
    if (lane == 0) g = atomicAdd(&p.gs->round_next, 1u);
    g = __shfl_sync(FULL, g, 0);
    if (g >= p.n_rounds) break;
    const uint32_t t = g * 32u + lane;
    const uint32_t op = p.op[t], kind = CSMV_OP_KIND(op), nr = CSMV_OP_NREADS(op), off = p.off[t];
    const bool ro = __all_sync(FULL, kind == CSMV_KIND_READONLY);  // warp-uniform by format
    bool bad = (ro != (kind == CSMV_KIND_READONLY)) || (!ro && (nr < 2 || nr > (uint32_t)MAXR));
    uint32_t a[MAXR];
#pragma unroll
    for (int k = 0; k < MAXR; k++) {
      a[k] = (!ro && !bad && k < (int)nr) ? p.addr[off + k] : 0u;
      bad |= a[k] >= p.n_items;
    }
    if (ro)
      for (uint32_t k = 0; k < nr; k++) bad |= p.addr[off + k] >= p.n_items;
    if (bad) raise_error(&p.gs->error, ERR_DATA);
    if (__any_sync(FULL, bad)) break;

    uint32_t pending = FULL, attempts = 0;
    while (pending) {
      if (++attempts > (1u << 20)) {  // no round may retry forever: report and leave
        if (lane == 0) raise_error(&p.gs->error, ERR_LIVELOCK);
        failed = true;
        break;
      }
      if (lane == 0) stat_add(stat, ST_ROUNDS, 1u);
      if (attempts > 1u) {  // randomized, growing pause before a retry
        const uint32_t h = (me * 0x9E3779B1u) ^ (attempts * 0x85EBCA6Bu);
        __nanosleep((h >> 16) & ((64u << min(attempts, 6u)) - 1u));
      }
      const bool mine = (pending >> lane) & 1u;
      uint32_t snap = 0;
      if (lane == 0) snap = ld_acquire_gpu(&p.gs->clock);
      snap = __shfl_sync(FULL, snap, 0);
      bool aborted = false;

      if (ro) {  // read-only: the snapshot's values, no validation (bank/baseline/API.cu:42-59)
        uint32_t s = 0;
        if (mine)
          for (uint32_t k = 0; k < nr; k++)
            s += (uint32_t)TXReadOnly<DEPTH>(vs, p.addr[off + k], snap, &aborted);
        const bool done = mine && !aborted;
        if (done && p.log) {
          p.outcome[t] = snap | kSnapFlag;
          p.result[t] = (int32_t)s;
        }
        const uint32_t dm = __ballot_sync(FULL, done), am = __ballot_sync(FULL, mine && aborted);
        if (lane == 0) {
          stat_add(stat, ST_COMMIT_RO, __popc(dm));
          stat_add(stat, ST_ABORT_DATA_AGE, __popc(am));
        }
        pending &= ~dm;
        continue;
      }

      // a transfer: its reads at the snapshot, then its writes
      int32_t v[MAXR];
#pragma unroll
      for (int k = 0; k < MAXR; k++)
        v[k] = (mine && k < (int)nr) ? TXReadOnly<DEPTH>(vs, a[k], snap, &aborted) : 0;
      int32_t w0 = 0, w1 = 0;
      const bool moved = transfer_writes<MAXR>(op, nr, v, w0, w1);
      bool cand = mine && !aborted;
      const uint32_t agem = __ballot_sync(FULL, mine && aborted);
      if (lane == 0) stat_add(stat, ST_ABORT_DATA_AGE, __popc(agem));
      if (!__any_sync(FULL, cand)) continue;

      // validation against the records committed after the snapshot (a record that a later lap
      // of the ring overwrote means the snapshot is too old to check: the reference's
      // record-age abort). As in the reference (TXAddToRecordNaive), the records are checked
      // while the warp waits for the section and only the ones added meanwhile inside it, so the
      // section itself stays short.
      bool age = false, rw = false;
      uint32_t checked = snap;
      auto scan = [&](uint32_t hi) {  // records (checked, hi]
        if (cand && !age && !rw && hi > checked) {
          if (hi - snap > p.ring_mask) {
            age = true;
          } else {
            for (uint32_t ts = checked + 1u; ts <= hi && !age && !rw; ts += 4u) {
              uint4 r[4];
#pragma unroll
              for (uint32_t q = 0; q < 4u; q++)  // four records in flight
                r[q] = ts + q <= hi ? __ldcg(&p.ring[(ts + q) & p.ring_mask]) : make_uint4(ts + q, 0u, 0u, 0u);
#pragma unroll
              for (uint32_t q = 0; q < 4u; q++) {
                if (r[q].x != ts + q) age = true;
#pragma unroll
                for (int k = 0; k < MAXR; k++)
                  if (k < (int)nr && ((r[q].y >= 1u && r[q].z == a[k]) || (r[q].y >= 2u && r[q].w == a[k])))
                    rw = true;
              }
            }
          }
        }
        checked = hi;
      };
      // the global commit section (the reference's CAS on the record ring's write head), entered
      // in ticket order: with hundreds of warps racing for one word, CAS winners are the warps
      // nearest its L2 slice and a far warp can starve
      uint32_t ticket = 0;
      if (lane == 0) ticket = atomicAdd(&p.gs->section, 1u);
      bool got = false;
      const uint64_t limit = 1ull << p.spin_log2;
      for (uint64_t it = 0; it < limit; it++) {
        uint32_t turn = 0, hi = 0, err = 0;
        if (lane == 0) {
          turn = ld_acquire_gpu(&p.gs->section_serving) == ticket;
          hi = ld_acquire_gpu(&p.gs->ts_next);  // records up to it are written
          if ((it & 63u) == 63u) err = ld_relaxed_gpu(&p.gs->error);
        }
        turn = __shfl_sync(FULL, turn, 0);
        hi = __shfl_sync(FULL, hi, 0);
        __syncwarp();  // the records up to hi are read after lane 0's acquire of ts_next
        scan(hi);
        if (turn) {
          got = true;
          break;
        }
        if (__shfl_sync(FULL, err, 0) != 0u) break;
        __nanosleep(64);
      }
      if (!got) {
        if (lane == 0) raise_error(&p.gs->error, ERR_WAIT_TURN);
        failed = true;
        break;
      }
      __syncwarp();  // every lane's loads and stores below follow lane 0's acquire of the turn
      uint32_t head = 0;
      if (lane == 0) head = ld_relaxed_gpu(&p.gs->ts_next);
      head = __shfl_sync(FULL, head, 0);
      scan(head);
      cand = cand && !age && !rw;
      // the section's lanes commit in lane order: a lane that reads an account a lower lane of
      // the section writes read it before that commit, so it aborts as for a record
      for (uint32_t j = 0; j < 31u; j++) {
        const uint32_t cm = __ballot_sync(FULL, cand && moved);
        if (!((cm >> j) & 1u)) continue;
        const uint32_t x0 = __shfl_sync(FULL, a[0], j), x1 = __shfl_sync(FULL, a[1], j);
        if (cand && lane > j) {
#pragma unroll
          for (int k = 0; k < MAXR; k++)
            if (k < (int)nr && (a[k] == x0 || a[k] == x1)) {
              cand = false;
              rw = true;
            }
        }
      }
      const uint32_t vm = __ballot_sync(FULL, cand), wm = __ballot_sync(FULL, cand && moved);
      const uint32_t n = __popc(vm);
      const uint32_t my_ts = head + 1u + __popc(vm & lanemask_lt());
      if (cand) {
        // write-back: the section's committing lanes write disjoint accounts (a writer also
        // reads what it writes, so a second writer of an account was aborted above)
        if (moved) {
          SlotEditor<DEPTH> ed;
          ed.load(p.slots + (size_t)a[1] * DEPTH);
          ed.insert(my_ts, w1);  // a transfer writes a1 last (a0 == a1 keeps the credit)
          ed.store(p.slots + (size_t)a[1] * DEPTH);
          st_relaxed_gpu(&p.cw[a[1]], (unsigned long long)my_ts);
          if (a[0] != a[1]) {
            ed.load(p.slots + (size_t)a[0] * DEPTH);
            ed.insert(my_ts, w0);
            ed.store(p.slots + (size_t)a[0] * DEPTH);
            st_relaxed_gpu(&p.cw[a[0]], (unsigned long long)my_ts);
          }
        }
        p.ring[my_ts & p.ring_mask] =
            moved ? make_uint4(my_ts, a[0] != a[1] ? 2u : 1u, a[1], a[0]) : make_uint4(my_ts, 0u, 0u, 0u);
        if (p.log) {
          const uint32_t li = my_ts - 1u - p.log_base;
          if (li < p.log_cap)
            p.log_txn[li] = t;
          else
            raise_error(&p.gs->error, ERR_CAPACITY);
          p.outcome[t] = my_ts;
          p.result[t] = 0;
        }
      }
      fence_acq_rel_gpu();  // versions, records and stamps before the clock that exposes them
      __syncwarp();
      const uint32_t agm = __ballot_sync(FULL, age), rwm = __ballot_sync(FULL, rw);
      if (lane == 0) {
        if (n) {
          st_relaxed_gpu(&p.gs->ts_next, head + n);
          st_release_gpu(&p.gs->clock, head + n);
        }
        st_release_gpu(&p.gs->section_serving, ticket + 1u);
        stat_add(stat, ST_COMMIT_UPDATE, __popc(wm));
        stat_add(stat, ST_COMMIT_NOWRITE, __popc(vm & ~wm));
        stat_add(stat, ST_ABORT_RECORD_AGE, __popc(agm));
        stat_add(stat, ST_ABORT_READ_WRITE, __popc(rwm));
        stat_add(stat, ST_SECTIONS, 1u);
      }
      pending &= ~vm;
      uint32_t err = 0;
      if (lane == 0) err = ld_relaxed_gpu(&p.gs->error);
      if (__shfl_sync(FULL, err, 0) != 0u) {
        failed = true;
        break;
      }
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < ST_COUNT; i += blockDim.x)
    if (stat[i]) atomicAdd(&p.stats[i], stat[i]);
}

using BaselineFn = void (*)(BankParams);

template <int MAXR>
BaselineFn pick_baseline_r(uint32_t depth) {
  switch (depth) {
    case 2: return baseline_kernel<2, MAXR>;
    case 4: return baseline_kernel<4, MAXR>;
    case 8: return baseline_kernel<8, MAXR>;
    case 16: return baseline_kernel<16, MAXR>;
    default: return nullptr;
  }
}

}  // namespace
}  // namespace csmv

using namespace csmv;

extern "C" csmv_status csmv_bank_run_baseline_device(csmv_bank_t* h, const csmv_bank_stream* s,
                                                     csmv_stats* out) {
  if (!h) return CSMV_ERR_INVALID_ARG;
  if (!h->loaded) {
    set_error("csmv_bank_load must come first");
    return CSMV_ERR_STATE;
  }
  csmv_status st = check_stream(h, s);
  if (st != CSMV_OK) return st;
  if (s->split_round || s->lock_last || s->lane_start || s->backoff) {
    set_error("the baseline arm runs the stream as one queue: no deferred queue, lanes, heat "
              "classes or backoff");
    return CSMV_ERR_INVALID_ARG;
  }
  if (h->cfg.validate != CSMV_VALIDATE_STAMP) {
    set_error("the baseline arm continues the stamp protocol's commit order only");
    return CSMV_ERR_INVALID_ARG;
  }
  const uint32_t max_reads = h->cfg.max_reads == 4 ? 4u : 8u;
  const BaselineFn fn = max_reads == 4 ? pick_baseline_r<4>(h->cfg.version_depth)
                                       : pick_baseline_r<8>(h->cfg.version_depth);
  if (!fn) {
    set_error("version_depth %u has no baseline kernel", h->cfg.version_depth);
    return CSMV_ERR_INVALID_ARG;
  }
  CSMV_CUDA(cudaSetDevice(h->cfg.device));
  auto t0 = std::chrono::steady_clock::now();
  BankParams p = bank_params(h, s->op, s->off, s->addr, s->n_txn, nullptr);
  p.grp = nullptr;
  h->last_grouped = false;
  CSMV_CUDA(cudaMemsetAsync(&h->gs->section, 0, 4, h->stream));
  CSMV_CUDA(cudaMemsetAsync(&h->gs->section_serving, 0, 4, h->stream));
  const uint32_t base0 = h->last_final_ts;
  st = bank_begin_run(h);
  if (st != CSMV_OK) return st;
  fn<<<h->ctas, h->cfg.client_warps * 32u, 0, h->stream>>>(p);
  CSMV_CUDA(cudaGetLastError());
  st = bank_end_run(h, s->n_txn, out);
  if (st == CSMV_OK && h->last_final_ts > base0) {
    // completion-bitmap words whose timestamps this run passed over without setting bits are
    // cleared, as the engine's clock advance would, before a later lap of the bitmap reuses them
    const uint32_t w_lo = (base0 + 1u) >> 5, w_end = (h->last_final_ts + 1u) >> 5;
    const uint32_t cnt = w_end > w_lo ? std::min(w_end - w_lo, kDoneWords) : 0u;
    const uint32_t start = w_lo & (kDoneWords - 1u), first = std::min(cnt, kDoneWords - start);
    if (first) CSMV_CUDA(cudaMemsetAsync(h->done + start, 0, (size_t)first * 4, h->stream));
    if (cnt > first) CSMV_CUDA(cudaMemsetAsync(h->done, 0, (size_t)(cnt - first) * 4, h->stream));
    CSMV_CUDA(cudaStreamSynchronize(h->stream));
  }
  if (out)
    out->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return st;
}
