/*
 * csmv_oracle.c - CPU oracle for the CSMV commit path. TEST INFRASTRUCTURE ONLY: nothing in
 * the product links or runs this file; tests/, __graft_entry__.smoke() and bench.py's CPU legs
 * load it through ctypes as the checker and the CPU baseline.
 *
 * Each function cites the reference file:line (DMRNunes/csmv-gpu-stm) whose rule it restates.
 */
#define _GNU_SOURCE
#include "csmv_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ======================================================================================
 * RNG
 * ==================================================================================== */

/* RAND_R_FNC of bank/csmv_sh/API.cuh:37-53: three LCG steps, 11+10+10 bits. */
uint64_t orc_rand_r(uint64_t* state) {
  uint64_t next = *state;
  uint64_t result;
  next = next * 1103515245ull + 12345ull;
  result = (next / 65536ull) % 2048ull;
  next = next * 1103515245ull + 12345ull;
  result <<= 10;
  result ^= (next / 65536ull) % 1024ull;
  next = next * 1103515245ull + 12345ull;
  result <<= 10;
  result ^= (next / 65536ull) % 1024ull;
  *state = next;
  return result;
}

/* splitmix64 finalizer; the stream generator's counter hash (no reference counterpart: the
 * reference draws addresses from a per-thread LCG whose state depends on retries). */
uint64_t orc_h64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

static uint64_t rnd64(uint64_t seed, uint64_t a, uint64_t b) {
  return orc_h64(orc_h64(seed + 0xD6E8FEB86659FD93ull * a) ^ b);
}

uint32_t orc_rnd32(uint64_t seed, uint64_t a, uint64_t b) {
  return (uint32_t)(rnd64(seed, a, b) >> 32);
}

static uint32_t below(uint32_t r, uint32_t n) { return (uint32_t)(((uint64_t)r * n) >> 32); }

/* ======================================================================================
 * Zipf by rejection-inversion (W. Hormann, G. Derflinger, "Rejection-inversion to generate
 * variates from monotone discrete distributions", ACM TOMACS 6(3), 1996) - the method the
 * reference's key generator cites (memcachedGPU/keyGenAndCacheStore.cpp:8-12).
 * ==================================================================================== */
typedef struct {
  double s, n, hx1, hn, sh;
} zipf_t;

static double zf_h1(double x) { /* log1p(x)/x */
  return fabs(x) > 1e-8 ? log1p(x) / x : 1.0 - x * (0.5 - x * (1.0 / 3.0 - 0.25 * x));
}
static double zf_h2(double x) { /* expm1(x)/x */
  return fabs(x) > 1e-8 ? expm1(x) / x : 1.0 + x * 0.5 * (1.0 + x * (1.0 / 3.0) * (1.0 + 0.25 * x));
}
static double zf_H(const zipf_t* z, double x) {
  double lx = log(x);
  return zf_h2((1.0 - z->s) * lx) * lx;
}
static double zf_h(const zipf_t* z, double x) { return exp(-z->s * log(x)); }
static double zf_Hinv(const zipf_t* z, double x) {
  double t = x * (1.0 - z->s);
  if (t < -1.0) t = -1.0;
  return exp(zf_h1(t) * x);
}
static void zf_init(zipf_t* z, double s, uint32_t n) {
  z->s = s;
  z->n = (double)n;
  z->hx1 = zf_H(z, 1.5) - 1.0;
  z->hn = zf_H(z, z->n + 0.5);
  z->sh = 2.0 - zf_Hinv(z, zf_H(z, 2.5) - zf_h(z, 2.0));
}
/* rank in [1, n] */
static uint32_t zf_sample(const zipf_t* z, uint64_t seed, uint64_t i, uint64_t c) {
  for (uint32_t it = 0; it < 256; it++) {
    double u01 = (double)(rnd64(seed, i, 0x10000ull + (c << 8) + it) >> 11) * 0x1p-53;
    double u = z->hn + u01 * (z->hx1 - z->hn);
    double x = zf_Hinv(z, u);
    double k = floor(x + 0.5);
    if (k < 1.0) k = 1.0;
    if (k > z->n) k = z->n;
    if (k - x <= z->sh || u >= zf_H(z, k + 0.5) - zf_h(z, k)) return (uint32_t)k;
  }
  return 1;
}

/* ======================================================================================
 * Bank stream generator (restatement of the product generator; see include/csmv.h for the
 * format). Round g is read-only with probability pr_read_pct, warp-uniform as in
 * bank/csmv_sh/exe.cu:134-139.
 * ==================================================================================== */
typedef struct {
  const orc_bank_workload* w;
  zipf_t z;
  uint32_t hot_n;
} gen_t;

static uint32_t draw_account(const gen_t* g, uint64_t i, uint64_t c) {
  const orc_bank_workload* w = g->w;
  uint32_t n = w->n_accounts;
  if (w->dist == 1) return zf_sample(&g->z, w->seed, i, c) - 1u;
  if (w->dist == 2) {
    uint64_t epoch = w->shift_every ? i / w->shift_every : 0;
    uint32_t base = below(orc_rnd32(w->seed, (2ull << 40) + epoch, 0), n);
    uint32_t r1 = orc_rnd32(w->seed, i, 0x100ull + 2 * c);
    uint32_t r2 = orc_rnd32(w->seed, i, 0x101ull + 2 * c);
    double thr = w->hot_prob * 4294967296.0;
    if ((double)r1 < thr) return (uint32_t)(((uint64_t)base + below(r2, g->hot_n)) % n);
    return below(r2, n);
  }
  return below(orc_rnd32(w->seed, i, 0x100ull + 2 * c), n);
}

int orc_bank_stream_size(const orc_bank_workload* w, uint64_t* n_addr) {
  if (!w || !n_addr || w->n_txn % 32 || w->n_accounts == 0) return 1;
  uint64_t total = 0;
  for (uint32_t g = 0; g < w->n_txn / 32; g++) {
    int ro = below(orc_rnd32(w->seed, (1ull << 40) + g, 0), 100) < w->pr_read_pct;
    total += 32ull * (ro ? w->ro_reads : w->up_reads);
  }
  *n_addr = total;
  return 0;
}

int orc_bank_generate(const orc_bank_workload* w, uint32_t* op, uint32_t* off, uint32_t* addr) {
  if (!w || w->n_txn % 32 || w->n_accounts == 0 || w->up_reads < 2 || w->up_reads > 32 ||
      w->up_reads > w->n_accounts || w->ro_reads < 1 || w->ro_reads > 32 || w->amt_lo < 1 ||
      w->amt_hi < w->amt_lo || w->amt_hi > 4095)
    return 1;
  gen_t g;
  g.w = w;
  if (w->dist == 1) zf_init(&g.z, w->zipf_theta, w->n_accounts);
  g.hot_n = (uint32_t)(w->hot_frac * (double)w->n_accounts);
  if (g.hot_n < 1) g.hot_n = 1;
  uint64_t pos = 0;
  for (uint32_t r = 0; r < w->n_txn / 32; r++) {
    int ro = below(orc_rnd32(w->seed, (1ull << 40) + r, 0), 100) < w->pr_read_pct;
    for (uint32_t lane = 0; lane < 32; lane++) {
      uint64_t i = (uint64_t)r * 32 + lane;
      off[i] = (uint32_t)pos;
      if (ro) {
        op[i] = 0u | (w->ro_reads << 2) | (1u << 8) | (1u << 20);
        for (uint32_t k = 0; k < w->ro_reads; k++) addr[pos++] = draw_account(&g, i, k * 64);
      } else {
        uint32_t amt0 = w->amt_lo + below(orc_rnd32(w->seed, i, 1), w->amt_hi - w->amt_lo + 1);
        op[i] = (w->kind & 3u) | (w->up_reads << 2) | (amt0 << 8) | (w->amt_hi << 20);
        for (uint32_t k = 0; k < w->up_reads; k++) {
          uint32_t a = 0;
          int ok = 0;
          for (uint32_t att = 0; att < 64 && !ok; att++) {
            a = draw_account(&g, i, k * 64 + att);
            ok = 1;
            for (uint32_t j = 0; j < k; j++)
              if (addr[pos - k + j] == a) ok = 0;
          }
          while (!ok) { /* tiny account counts only: next unused id */
            a = (a + 1) % w->n_accounts;
            ok = 1;
            for (uint32_t j = 0; j < k; j++)
              if (addr[pos - k + j] == a) ok = 0;
          }
          addr[pos++] = a;
        }
      }
    }
  }
  return 0;
}

/* ======================================================================================
 * Version lists
 * ==================================================================================== */

/* TXRead / TXReadOnly rule of bank/csmv_sh/API.cu:20-40 (and 47-66): abort (DataAge) when the
 * snapshot is older than the oldest kept version, else scan from head back to tail for the
 * first version with ts <= snapshot. Returns 0 with *out set, or 1 on abort. */
int orc_ref_read(uint16_t head, uint16_t tail, const uint32_t* version, const int32_t* value,
                 int maxv, uint32_t ts, int32_t* out) {
  if (ts < version[tail]) return 1;
  for (int i = head;; i = (i - 1 + maxv) % maxv) {
    if (version[i] <= ts) {
      *out = value[i];
      return 0;
    }
    if (i == tail) break;
  }
  return 1;
}

/* TXWriteBack rotation of bank/csmv_sh/API.cu:157-174: drop the tail when the ring is full,
 * write version/value at head+1, advance head. */
void orc_ref_writeback(uint16_t* head, uint16_t* tail, uint32_t* version, int32_t* value,
                       int maxv, uint32_t ts, int32_t v) {
  int nh = (*head + 1) % maxv;
  if (nh == *tail) *tail = (uint16_t)((*tail + 1) % maxv);
  version[nh] = ts;
  value[nh] = v;
  *head = (uint16_t)nh;
}

/* Packed layout: the newest version with ts <= snapshot is the largest such ts among the
 * slots; no such slot means the reference's DataAge abort. */
int orc_packed_read(const uint64_t* slots, int depth, uint32_t ts, int32_t* out) {
  int best = -1;
  uint32_t bts = 0;
  for (int d = 0; d < depth; d++) {
    uint32_t t = (uint32_t)(slots[d] >> 32);
    if (t == 0xFFFFFFFFu || t > ts) continue;
    if (best < 0 || t > bts) {
      best = d;
      bts = t;
    }
  }
  if (best < 0) return 1;
  *out = (int32_t)(uint32_t)slots[best];
  return 0;
}

/* Victim for a new version: first empty slot, else the oldest (smallest ts) - the slot the
 * reference's tail advance frees. Ties cannot happen (timestamps of one item are unique). */
int orc_packed_victim(const uint64_t* slots, int depth) {
  int v = 0;
  uint32_t key = (uint32_t)(slots[0] >> 32) + 1u; /* empty (0xFFFFFFFF) -> 0 */
  for (int d = 1; d < depth; d++) {
    uint32_t k = (uint32_t)(slots[d] >> 32) + 1u;
    if (k < key) {
      key = k;
      v = d;
    }
  }
  return v;
}

void orc_packed_writeback(uint64_t* slots, int depth, uint32_t ts, int32_t v) {
  int d = orc_packed_victim(slots, depth);
  slots[d] = ((uint64_t)ts << 32) | (uint32_t)v;
}

/* ======================================================================================
 * Pre-validation: TXPreValidation of batchedAtrInsert/csmv_sh/API.cu:94-191.
 * conflict bit i of lane l: a lower lane i writes an address lane l read. Resolution: a lane
 * with no conflicts commits; a lane conflicting with a committed lane aborts; a conflict with
 * an aborted lane is dropped. Conflicts point only to lower lanes, so resolving lanes in
 * increasing order reaches the same fixpoint as the reference's shuffle rounds.
 * ==================================================================================== */
uint32_t orc_prevalidate(const uint32_t* rs, const uint32_t* n_rs, int rs_stride,
                         const uint32_t* ws, const uint32_t* n_ws, int ws_stride,
                         uint32_t active, uint32_t* conflict) {
  uint32_t cf[32];
  for (int l = 0; l < 32; l++) {
    cf[l] = 0;
    if (!((active >> l) & 1)) continue;
    for (int i = l - 1; i >= 0; i--) {
      if (!((active >> i) & 1)) continue;
      for (uint32_t j = 0; j < n_ws[i]; j++)
        for (uint32_t k = 0; k < n_rs[l]; k++)
          if (rs[l * rs_stride + k] == ws[i * ws_stride + j]) cf[l] |= 1u << i;
    }
  }
  uint32_t commit = 0;
  for (int l = 0; l < 32; l++) {
    if (conflict) conflict[l] = cf[l];
    if (!((active >> l) & 1)) continue;
    if ((cf[l] & commit) == 0) commit |= 1u << l;
  }
  return commit;
}

/* ======================================================================================
 * Record-ring validation
 * ==================================================================================== */

static int rs_hit(const orc_record* r, const uint32_t* rs, int nrs) {
  for (uint32_t j = 0; j < r->n_writes; j++)
    for (int k = 0; k < nrs; k++)
      if (rs[k] == r->ws[j]) return 1;
  return 0;
}

/* TXValidate of bank/csmv_sh/API.cu:88-144: skip stale tail records, RecordAge when the
 * oldest kept record is newer than the snapshot, then scan hp back to oldhp while records
 * are newer than the snapshot. */
int orc_ref_validate(const orc_record* recs, int ring, int hp, int tp, int oldhp, int ts,
                     const uint32_t* rs, int nrs) {
  int aux;
  while ((aux = (int)recs[tp].txn) > (int)recs[hp].txn) tp = (tp + 1) % ring;
  if (aux > ts) return ORC_ABORT_RECORD_AGE;
  for (int i = hp; i != oldhp; i = (i - 1 + ring) % ring) {
    if ((int)recs[i].txn <= ts) break;
    if (rs_hit(&recs[i], rs, nrs)) return ORC_ABORT_READ_WRITE;
  }
  return ORC_VALID;
}

/* TXValidate of batchedAtrInsert/csmv_sh/API.cu:193-228: RecordAge when the tail record is
 * newer than the snapshot or the scan reaches the tail. */
int orc_batched_validate(const orc_record* recs, int ring, int hp, int tp, int oldhp, int ts,
                         const uint32_t* rs, int nrs) {
  if ((int)recs[tp].txn > ts) return ORC_ABORT_RECORD_AGE;
  for (int i = hp; i != oldhp; i = (i - 1 + ring) % ring) {
    if ((int)recs[i].txn <= ts) break;
    if (i == tp) return ORC_ABORT_RECORD_AGE;
    if (rs_hit(&recs[i], rs, nrs)) return ORC_ABORT_READ_WRITE;
  }
  return ORC_VALID;
}

/* Collaborative TXValidate of collabValidation/csmv_sh/API.cu:193-266. For each lane's
 * transaction the warp scans ring slots (anchor, hp] with anchor = ts % ring, lane-strided;
 * a write-set hit is a ReadWrite abort, an overwritten anchor (record newer than ts) is the
 * "spurious" RecordAge abort. A tail record newer than ts aborts first (RecordAge). */
void orc_collab_validate(const orc_record* recs, int ring, int hp, int tp, const int* ts,
                         const uint32_t* rs, const uint32_t* n_rs, int rs_stride, int* out) {
  for (int lane = 0; lane < 32; lane++) {
    out[lane] = ORC_VALID;
    int t = ts[lane];
    if (t < 0) continue;
    if ((int)recs[tp].txn > t) {
      out[lane] = ORC_ABORT_RECORD_AGE;
      continue;
    }
    int anchor = t % ring;
    int conflict = 0, spurious = 0;
    for (int ml = 0; ml < 32; ml++) { /* every lane's share of the scan */
      int span = hp >= anchor ? hp - ml - anchor : hp + ring - ml - anchor;
      int iters = span > 0 ? (span + 31) / 32 : 0;
      for (int i = ((hp - ml) % ring + ring) % ring; iters > 0; i = ((i - 32) % ring + ring) % ring, iters--) {
        if (rs_hit(&recs[i], rs + lane * rs_stride, (int)n_rs[lane])) conflict = 1;
        if ((int)recs[anchor].txn > t) spurious = 1;
      }
    }
    if (conflict)
      out[lane] = ORC_ABORT_READ_WRITE;
    else if (spurious)
      out[lane] = ORC_ABORT_RECORD_AGE;
  }
}

/* Batched commit timestamps of batchedAtrInsert/csmv_sh/API.cu:296-377: the warp reserves
 * popc(ballot) slots with one CAS; lane l gets prev + popc(ballot & lanemask_lt(l)) + 1. */
void orc_batched_ts(uint32_t ballot, uint32_t prev_ts, uint32_t* ts_out) {
  for (int l = 0; l < 32; l++) {
    if (!((ballot >> l) & 1)) {
      ts_out[l] = 0;
      continue;
    }
    uint32_t lt = l ? (ballot & ((1u << l) - 1u)) : 0u;
    ts_out[l] = prev_ts + (uint32_t)__builtin_popcount(lt) + 1u;
  }
}

/* GB300 engine rule: a transaction with snapshot snap validated when the newest commit is
 * `frontier` conflicts iff a commit with ts in (snap, frontier] wrote an address it read; in
 * ring mode it also aborts (RecordAge) when the ring of `ring` records no longer reaches
 * snap+1, i.e. snap + ring <= frontier - the reference's "oldest record newer than ts" rule. */
int orc_window_validate(const orc_record* by_ts, uint32_t snap, uint32_t frontier,
                        uint32_t ring, const uint32_t* rs, int nrs, int ring_mode) {
  if (ring_mode && (uint64_t)snap + ring <= frontier) return ORC_ABORT_RECORD_AGE;
  for (uint32_t t = snap + 1; t <= frontier; t++)
    if (rs_hit(&by_ts[t - 1], rs, nrs)) return ORC_ABORT_READ_WRITE;
  return ORC_VALID;
}

/* ======================================================================================
 * memcached SET slot choice, memcachedGPU/memcdSH.cu:365-387 (bit test of state & INVALID
 * is always false because INVALID == 0, so the "empty slot" branch takes any older slot).
 * ==================================================================================== */
int orc_memcd_set_slot(const int32_t* keys, const int32_t* states, const int32_t* ages,
                       int ways, int32_t key) {
  int slot = -1, slot_age = -1, slot_state = -1;
  for (int j = 0; j < ways; j++) {
    if (keys[j] == key && (states[j] & 1)) return j;
    if (slot == -1 || (!(slot_state & 0) && ages[j] < slot_age)) {
      slot = j;
      slot_state = states[j];
      slot_age = ages[j];
    }
  }
  return slot;
}

/* ======================================================================================
 * Bank semantics, replay checker, deterministic model, CPU baselines
 * ==================================================================================== */

int orc_bank_exec(uint32_t op, const uint32_t* addrs, const int32_t* vals, uint32_t* waddr,
                  int32_t* wval, int32_t* result) {
  uint32_t kind = op & 3u, nr = (op >> 2) & 63u;
  if (kind == 0) {
    uint32_t s = 0;
    for (uint32_t k = 0; k < nr; k++) s += (uint32_t)vals[k];
    *result = (int32_t)s;
    return 0;
  }
  uint32_t amt0 = (op >> 8) & 4095u, amod = (op >> 20) & 4095u;
  uint32_t acc = amt0 - 1u;
  for (uint32_t k = 2; k < nr; k++) acc += (uint32_t)vals[k];
  uint32_t amt = 1u + acc % amod;
  *result = 0;
  if (kind == 1 && !(vals[0] >= (int32_t)amt)) return 0;
  waddr[0] = addrs[0];
  wval[0] = (int32_t)((uint32_t)vals[0] - amt);
  waddr[1] = addrs[1];
  wval[1] = (int32_t)((uint32_t)vals[1] + amt);
  return 2;
}

#define SNAP_FLAG 0x80000000u

static int fail(char* msg, int len, const char* fmt, ...) __attribute__((format(printf, 3, 4)));
#include <stdarg.h>
static int fail(char* msg, int len, const char* fmt, ...) {
  if (msg && len > 0) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, (size_t)len, fmt, ap);
    va_end(ap);
  }
  return 1;
}

static void init_slots(uint64_t* slots, uint32_t n, int depth, const int32_t* init) {
  for (uint32_t i = 0; i < n; i++) {
    slots[(uint64_t)i * depth] = (uint32_t)init[i]; /* ts 0 */
    for (int d = 1; d < depth; d++) slots[(uint64_t)i * depth + d] = 0xFFFFFFFFull << 32;
  }
}

static int check_snapshot_txn(uint32_t t, const uint32_t* op, const uint32_t* off,
                              const uint32_t* addr, const int32_t* vals, const int32_t* result,
                              char* msg, int len) {
  int32_t v[64], r = 0, wv[2];
  uint32_t wa[2];
  uint32_t nr = (op[t] >> 2) & 63u;
  for (uint32_t k = 0; k < nr; k++) v[k] = vals[addr[off[t] + k]];
  int nw = orc_bank_exec(op[t], addr + off[t], v, wa, wv, &r);
  if ((op[t] & 3u) == 0) {
    if (result && result[t] != r)
      return fail(msg, len, "txn %u: read-only result %d, snapshot state gives %d", t,
                  result[t], r);
    return 0;
  }
  if (nw != 0)
    return fail(msg, len, "txn %u: committed without writes but snapshot state has funds", t);
  return 0;
}

int orc_bank_check(uint32_t n_txn, const uint32_t* op, const uint32_t* off, const uint32_t* addr,
                   uint32_t n_accounts, const int32_t* init, int depth, uint32_t final_ts,
                   const uint32_t* log_txn, const uint32_t* outcome, const int32_t* result,
                   const uint64_t* final_slots, char* msg, int msg_len) {
  return orc_bank_check_groups(n_txn, op, off, addr, n_accounts, init, depth, final_ts, log_txn,
                               outcome, result, NULL, final_slots, msg, msg_len);
}

#define GROUP_END(g, ts) (!(g) || (((g)[((ts)-1u) >> 5] >> (((ts)-1u) & 31u)) & 1u))
#define ORC_GROUP_MAX 4096

/* Installs of one commit group: each account's last write of the group, as one version. The
 * engine's group commit installs exactly these (the versions in between are never visible). */
static void flush_group(uint64_t* slots, int depth, uint32_t* ga, uint32_t* gts, int32_t* gv,
                        int* gn) {
  for (int i = *gn - 1; i >= 0; i--) {
    int later = 0;
    for (int j = i + 1; j < *gn && !later; j++) later = ga[j] == ga[i];
    if (!later) orc_packed_writeback(slots + (uint64_t)ga[i] * depth, depth, gts[i], gv[i]);
  }
  *gn = 0;
}

int orc_bank_check_groups(uint32_t n_txn, const uint32_t* op, const uint32_t* off,
                          const uint32_t* addr, uint32_t n_accounts, const int32_t* init,
                          int depth, uint32_t final_ts, const uint32_t* log_txn,
                          const uint32_t* outcome, const int32_t* result,
                          const uint32_t* group_end, const uint64_t* final_slots, char* msg,
                          int msg_len) {
  int rc = 0, gn = 0;
  uint8_t* seen = calloc(n_txn ? n_txn : 1, 1);
  int32_t* vals = malloc(sizeof(int32_t) * (n_accounts ? n_accounts : 1));
  uint64_t* slots = malloc(sizeof(uint64_t) * (size_t)n_accounts * depth + 8);
  uint32_t* bucket_head = malloc(sizeof(uint32_t) * ((size_t)final_ts + 1));
  uint32_t* next = malloc(sizeof(uint32_t) * (n_txn ? n_txn : 1));
  uint32_t* ga = malloc(sizeof(uint32_t) * ORC_GROUP_MAX);
  uint32_t* gts = malloc(sizeof(uint32_t) * ORC_GROUP_MAX);
  int32_t* gv = malloc(sizeof(int32_t) * ORC_GROUP_MAX);
  if (!seen || !vals || !slots || !bucket_head || !next || !ga || !gts || !gv) {
    rc = fail(msg, msg_len, "oracle out of memory");
    goto out;
  }
  /* 1. the log names distinct transfers; outcomes agree with it. 0xFFFFFFFF is a hole: a
   * timestamp handed to a transaction that then failed validation (no commit). */
  for (uint32_t ts = 1; ts <= final_ts; ts++) {
    uint32_t t = log_txn[ts - 1];
    if (t == 0xFFFFFFFFu) continue;
    if (t >= n_txn) {
      rc = fail(msg, msg_len, "ts %u: txn id %u out of range", ts, t);
      goto out;
    }
    if ((op[t] & 3u) == 0) {
      rc = fail(msg, msg_len, "ts %u: read-only txn %u in the commit log", ts, t);
      goto out;
    }
    if (seen[t]) {
      rc = fail(msg, msg_len, "ts %u: txn %u committed twice", ts, t);
      goto out;
    }
    if (outcome[t] != ts) {
      rc = fail(msg, msg_len, "ts %u: txn %u outcome says %u", ts, t, outcome[t]);
      goto out;
    }
    seen[t] = 1;
  }
  for (uint32_t b = 0; b <= final_ts; b++) bucket_head[b] = 0xFFFFFFFFu;
  for (uint32_t t = 0; t < n_txn; t++) {
    if (seen[t]) continue;
    if (!(outcome[t] & SNAP_FLAG)) {
      rc = fail(msg, msg_len, "txn %u: outcome %u is neither a logged commit nor a snapshot",
                t, outcome[t]);
      goto out;
    }
    uint32_t s = outcome[t] & ~SNAP_FLAG;
    if (s > final_ts) {
      rc = fail(msg, msg_len, "txn %u: snapshot %u beyond final ts %u", t, s, final_ts);
      goto out;
    }
    next[t] = bucket_head[s];
    bucket_head[s] = t;
  }
  /* 2. serial replay in commit-ts order, checking snapshot transactions at their ts */
  for (uint32_t i = 0; i < n_accounts; i++) vals[i] = init[i];
  init_slots(slots, n_accounts, depth, init);
  for (uint32_t ts = 0; ts <= final_ts; ts++) {
    if (ts > 0 && log_txn[ts - 1] != 0xFFFFFFFFu) {
      uint32_t t = log_txn[ts - 1];
      int32_t v[64], r, wv[2];
      uint32_t wa[2];
      uint32_t nr = (op[t] >> 2) & 63u;
      for (uint32_t k = 0; k < nr; k++) v[k] = vals[addr[off[t] + k]];
      /* a logged commit may have no writes: a chained transfer that lacked funds at its
       * place in the order; the final-state comparison catches a wrong decision either way */
      int nw = orc_bank_exec(op[t], addr + off[t], v, wa, wv, &r);
      for (int k = 0; k < nw; k++) {
        vals[wa[k]] = wv[k];
        if (gn == ORC_GROUP_MAX) {
          rc = fail(msg, msg_len, "ts %u: commit group holds more than %d writes", ts,
                    ORC_GROUP_MAX);
          goto out;
        }
        ga[gn] = wa[k];
        gts[gn] = ts;
        gv[gn] = wv[k];
        gn++;
      }
    }
    if (ts > 0 && GROUP_END(group_end, ts)) flush_group(slots, depth, ga, gts, gv, &gn);
    if (ts > 0 && !GROUP_END(group_end, ts) && bucket_head[ts] != 0xFFFFFFFFu) {
      rc = fail(msg, msg_len, "txn %u: snapshot %u falls inside a commit group", bucket_head[ts],
                ts);
      goto out;
    }
    for (uint32_t t = bucket_head[ts]; t != 0xFFFFFFFFu; t = next[t])
      if ((rc = check_snapshot_txn(t, op, off, addr, vals, result, msg, msg_len))) goto out;
  }
  if (gn) {
    rc = fail(msg, msg_len, "the last commit group does not end at the final ts %u", final_ts);
    goto out;
  }
  /* 3. invariant and final version state */
  {
    int64_t s0 = 0, s1 = 0;
    for (uint32_t i = 0; i < n_accounts; i++) {
      s0 += init[i];
      s1 += vals[i];
    }
    if (s0 != s1) {
      rc = fail(msg, msg_len, "total balance %lld != initial %lld", (long long)s1,
                (long long)s0);
      goto out;
    }
  }
  if (final_slots) {
    for (uint64_t i = 0; i < (uint64_t)n_accounts * depth; i++)
      if (final_slots[i] != slots[i]) {
        rc = fail(msg, msg_len,
                  "account %llu slot %llu: device (ts %u, %d) vs replay (ts %u, %d)",
                  (unsigned long long)(i / depth), (unsigned long long)(i % depth),
                  (uint32_t)(final_slots[i] >> 32), (int32_t)(uint32_t)final_slots[i],
                  (uint32_t)(slots[i] >> 32), (int32_t)(uint32_t)slots[i]);
        goto out;
      }
  }
out:
  free(seen);
  free(vals);
  free(slots);
  free(bucket_head);
  free(next);
  free(ga);
  free(gts);
  free(gv);
  return rc;
}

static uint32_t newest_ts(const uint64_t* slots, int depth) {
  uint32_t m = 0;
  for (int d = 0; d < depth; d++) {
    uint32_t t = (uint32_t)(slots[d] >> 32);
    if (t != 0xFFFFFFFFu && t > m) m = t;
  }
  return m;
}

/* Read-only outcome of a transfer that wrote nothing: the ring protocol serialises it at its
 * snapshot, the stamp protocol (it reads latest versions) at the newest stamp it read. */
static uint32_t nowrite_snap(uint32_t t, const uint32_t* op, const uint32_t* off,
                             const uint32_t* addr, const uint64_t* slots, int depth, int locks,
                             uint32_t snap) {
  if (!locks || (op[t] & 3u) == 0) return snap;
  uint32_t m = 0, nr = (op[t] >> 2) & 63u;
  for (uint32_t k = 0; k < nr; k++) {
    uint32_t x = newest_ts(slots + (uint64_t)addr[off[t] + k] * depth, depth);
    if (x > m) m = x;
  }
  return m;
}

/* Deterministic model of the engine with one client warp: rounds run in order; every
 * attempt snapshots the current clock, executes, drops no-write transfers as snapshot
 * commits, pre-validates (or lets the server resolve lane order), and commits the surviving
 * lanes with consecutive timestamps in lane order. Failed lanes retry the same transaction. */
int orc_bank_sim_1warp(uint32_t n_txn, const uint32_t* op, const uint32_t* off,
                       const uint32_t* addr, uint32_t n_accounts, const int32_t* init,
                       int depth, int prevalidate, int locks, uint64_t* slots, uint32_t* log_txn,
                       uint32_t* outcome, int32_t* result, orc_sim_stats* st) {
  memset(st, 0, sizeof(*st));
  init_slots(slots, n_accounts, depth, init);
  uint32_t clock = 0;
  uint32_t rs[32][32], nrs[32], ws[32][2], nws[32];
  int32_t wv[32][2];
  for (uint32_t g = 0; g < n_txn / 32; g++) {
    uint32_t pending = 0xFFFFFFFFu;
    while (pending) {
      st->rounds++;
      uint32_t snap = clock, cand = 0;
      if (prevalidate == 3 && (op[g * 32] & 3u) != 0) {
        /* group commit: with one warp every lock is free and every read current, so the round's
         * pending transfers take consecutive timestamps in lane order and run as a chain; each
         * written account gets one version, its last writer's */
        uint32_t ga[64], gts[64];
        int32_t gv[64];
        int gn = 0;
        for (int l = 0; l < 32; l++) {
          if (!((pending >> l) & 1)) continue;
          uint32_t t = g * 32 + l, nr = (op[t] >> 2) & 63;
          int32_t v[64], r = 0, wv2[2];
          uint32_t wa2[2];
          for (uint32_t k = 0; k < nr; k++) {
            uint32_t x = addr[off[t] + k];
            int found = -1;
            for (int j = gn - 1; j >= 0; j--)
              if (ga[j] == x) {
                found = j;
                break;
              }
            if (found >= 0) {
              v[k] = gv[found];
            } else if (orc_packed_read(slots + (uint64_t)x * depth, depth, 0xFFFFFFFEu, &v[k])) {
              return 1;
            }
          }
          uint32_t ts = ++clock;
          int nw = orc_bank_exec(op[t], addr + off[t], v, wa2, wv2, &r);
          for (int k = 0; k < nw; k++) {
            ga[gn] = wa2[k];
            gts[gn] = ts;
            gv[gn] = wv2[k];
            gn++;
          }
          log_txn[ts - 1] = t;
          outcome[t] = ts;
          result[t] = 0;
          if (nw > 0)
            st->commits_update++;
          else
            st->commits_nowrite++;
        }
        flush_group(slots, depth, ga, gts, gv, &gn);
        pending = 0;
        continue;
      }
      if (prevalidate == 2) { /* intra-warp chaining: the round runs serially in lane order */
        int32_t* round_val = (int32_t*)malloc(sizeof(int32_t) * 32 * 64);
        uint32_t round_addr[32 * 2];
        int n_w = 0;
        uint32_t links = 0;
        uint32_t ws_a[32][2];
        int32_t ws_v[32][2];
        int has[32];
        for (int l = 0; l < 32; l++) {
          has[l] = 0;
          if (!((pending >> l) & 1)) continue;
          uint32_t t = g * 32 + l, nr = (op[t] >> 2) & 63;
          int32_t v[64], r = 0;
          int fwd = 0;
          for (uint32_t k = 0; k < nr; k++) {
            uint32_t x = addr[off[t] + k];
            int found = -1;
            for (int j = n_w - 1; j >= 0; j--)
              if (round_addr[j] == x) {
                found = j;
                break;
              }
            if (found >= 0) {
              v[k] = round_val[found];
              fwd = 1;
            } else if (orc_packed_read(slots + (uint64_t)x * depth, depth, snap, &v[k])) {
              free(round_val);
              return 1;
            }
          }
          int nw = orc_bank_exec(op[t], addr + off[t], v, ws_a[l], ws_v[l], &r);
          for (int k = 0; k < nw; k++) {
            round_addr[n_w] = ws_a[l][k];
            round_val[n_w] = ws_v[l][k];
            n_w++;
          }
          has[l] = nw > 0;
          (void)fwd;
          if ((op[t] & 3u) != 0) { /* every transfer is a link, also one that writes nothing */
            links |= 1u << l;
          } else {
            outcome[t] = nowrite_snap(t, op, off, addr, slots, depth, locks, snap) | SNAP_FLAG;
            result[t] = r;
            if ((op[t] & 3u) == 0)
              st->commits_readonly++;
            else
              st->commits_nowrite++;
          }
        }
        /* the chain's links take consecutive timestamps; each written account gets one
         * version, its last link's (the chain is published to the clock as one range) */
        uint32_t ga[64], gts[64];
        int32_t gv[64];
        int gn = 0;
        for (int l = 0; l < 32; l++) {
          if (!((links >> l) & 1)) continue;
          uint32_t t = g * 32 + l, ts = ++clock;
          log_txn[ts - 1] = t;
          outcome[t] = ts;
          result[t] = 0;
          if (has[l]) {
            for (int k = 0; k < 2; k++) {
              ga[gn] = ws_a[l][k];
              gts[gn] = ts;
              gv[gn] = ws_v[l][k];
              gn++;
            }
            st->commits_update++;
          } else {
            st->commits_nowrite++;
          }
        }
        flush_group(slots, depth, ga, gts, gv, &gn);
        free(round_val);
        pending = 0;
        continue;
      }
      for (int l = 0; l < 32; l++) {
        nrs[l] = nws[l] = 0;
        if (!((pending >> l) & 1)) continue;
        uint32_t t = g * 32 + l, nr = (op[t] >> 2) & 63u;
        int32_t v[64], r = 0;
        for (uint32_t k = 0; k < nr; k++) {
          if (orc_packed_read(slots + (uint64_t)addr[off[t] + k] * depth, depth, snap, &v[k]))
            return 1; /* cannot happen with one warp */
          rs[l][k] = addr[off[t] + k];
        }
        nrs[l] = nr;
        int nw = orc_bank_exec(op[t], addr + off[t], v, ws[l], wv[l], &r);
        if (nw == 0) {
          outcome[t] = nowrite_snap(t, op, off, addr, slots, depth, locks, snap) | SNAP_FLAG;
          result[t] = r;
          if ((op[t] & 3u) == 0)
            st->commits_readonly++;
          else
            st->commits_nowrite++;
          pending &= ~(1u << l);
          continue;
        }
        nws[l] = (uint32_t)nw;
        cand |= 1u << l;
      }
      if (!cand) continue;
      uint32_t locked = cand;
      if (locks) { /* only the lowest candidate writing an address takes its lock */
        for (int l = 0; l < 32; l++) {
          if (!((cand >> l) & 1)) continue;
          for (int i = 0; i < l; i++) {
            if (!((cand >> i) & 1)) continue;
            for (uint32_t x = 0; x < nws[l]; x++)
              for (uint32_t y = 0; y < nws[i]; y++)
                if (ws[l][x] == ws[i][y]) locked &= ~(1u << l);
          }
        }
        st->aborts_write_write += (uint64_t)__builtin_popcount(cand & ~locked);
      }
      uint32_t pass = orc_prevalidate(&rs[0][0], nrs, 32, &ws[0][0], nws, 2, locked, NULL);
      if (prevalidate)
        st->aborts_prevalid += (uint64_t)__builtin_popcount(locked & ~pass);
      else
        st->aborts_read_write += (uint64_t)__builtin_popcount(locked & ~pass);
      for (int l = 0; l < 32; l++) {
        if (!((pass >> l) & 1)) continue;
        uint32_t t = g * 32 + l, ts = ++clock;
        log_txn[ts - 1] = t;
        outcome[t] = ts;
        result[t] = 0;
        for (uint32_t k = 0; k < nws[l]; k++)
          orc_packed_writeback(slots + (uint64_t)ws[l][k] * depth, depth, ts, wv[l][k]);
        st->commits_update++;
      }
      pending &= ~pass;
    }
  }
  st->final_ts = clock;
  return 0;
}

static uint64_t now_ns(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (uint64_t)t.tv_sec * 1000000000ull + (uint64_t)t.tv_nsec;
}

static void exec_in_place(uint32_t t, const uint32_t* op, const uint32_t* off,
                          const uint32_t* addr, int32_t* vals) {
  int32_t v[64], r, wv[2];
  uint32_t wa[2];
  uint32_t nr = (op[t] >> 2) & 63u;
  for (uint32_t k = 0; k < nr; k++) v[k] = vals[addr[off[t] + k]];
  int nw = orc_bank_exec(op[t], addr + off[t], v, wa, wv, &r);
  for (int k = 0; k < nw; k++) vals[wa[k]] = wv[k];
}

/* Single-thread serial execution in stream order. */
int orc_bank_serial(uint32_t n_txn, const uint32_t* op, const uint32_t* off,
                    const uint32_t* addr, uint32_t n_accounts, int32_t* vals, uint64_t* ns) {
  (void)n_accounts;
  uint64_t t0 = now_ns();
  for (uint32_t t = 0; t < n_txn; t++) exec_in_place(t, op, off, addr, vals);
  *ns = now_ns() - t0;
  return 0;
}

/* Host-threaded lock-based execution: each transaction takes the striped spinlocks of its
 * accounts in ascending stripe order, executes, releases. */
#define ORC_STRIPES (1u << 16)
typedef struct {
  const uint32_t *op, *off, *addr;
  int32_t* vals;
  uint32_t n_txn;
  volatile uint32_t* next;
  uint8_t* locks;
} lk_arg;

static void* lk_worker(void* p) {
  lk_arg* a = (lk_arg*)p;
  uint32_t stripes[64];
  for (;;) {
    uint32_t base = __atomic_fetch_add(a->next, 64u, __ATOMIC_RELAXED);
    if (base >= a->n_txn) break;
    uint32_t end = base + 64 < a->n_txn ? base + 64 : a->n_txn;
    for (uint32_t t = base; t < end; t++) {
      uint32_t nr = (a->op[t] >> 2) & 63u, ns = 0;
      for (uint32_t k = 0; k < nr; k++) {
        uint32_t s = a->addr[a->off[t] + k] & (ORC_STRIPES - 1);
        uint32_t j = ns;
        while (j > 0 && stripes[j - 1] > s) {
          stripes[j] = stripes[j - 1];
          j--;
        }
        if (j > 0 && stripes[j - 1] == s) { /* duplicate: undo shift */
          for (uint32_t q = j; q < ns; q++) stripes[q] = stripes[q + 1];
          continue;
        }
        stripes[j] = s;
        ns++;
      }
      for (uint32_t k = 0; k < ns; k++)
        while (__atomic_exchange_n(&a->locks[stripes[k]], 1, __ATOMIC_ACQUIRE))
          while (__atomic_load_n(&a->locks[stripes[k]], __ATOMIC_RELAXED)) {
          }
      exec_in_place(t, a->op, a->off, a->addr, a->vals);
      for (uint32_t k = 0; k < ns; k++) __atomic_store_n(&a->locks[stripes[k]], 0, __ATOMIC_RELEASE);
    }
  }
  return NULL;
}

int orc_bank_locked(uint32_t n_txn, const uint32_t* op, const uint32_t* off,
                    const uint32_t* addr, uint32_t n_accounts, int32_t* vals, int nthreads,
                    uint64_t* ns) {
  (void)n_accounts;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 512) nthreads = 512;
  uint8_t* locks = calloc(ORC_STRIPES, 1);
  pthread_t th[512];
  volatile uint32_t next = 0;
  lk_arg a = {op, off, addr, vals, n_txn, &next, locks};
  uint64_t t0 = now_ns();
  for (int i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, lk_worker, &a);
  for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
  *ns = now_ns() - t0;
  free(locks);
  return 0;
}

/* ======================================================================================
 * Transactional cache: serial semantics, replay checker, CPU baseline
 *
 * Entry e = set*8 + way holds 2 versions; version v = e*2 + j has a tag
 * (ts << 32 | valid << 31 | 31-bit key hash, empty = ts 0xFFFFFFFF) and a 16-word record
 * {lru, 0, 0, 0, key[4], value[8]}. The state of an entry is its newest version (largest ts).
 * SET slot rule: orc_memcd_set_slot (memcdSH.cu:365-387) over the ways' newest versions.
 * ==================================================================================== */
#define MC_WAYS 8
#define MC_D 2

uint32_t orc_memcd_mix(const uint32_t* k) {
  uint32_t h = k[0] * 0x9E3779B1u ^ k[1] * 0x85EBCA6Bu ^ k[2] * 0xC2B2AE35u ^ k[3] * 0x27D4EB2Fu;
  return h ^ (h >> 16);
}
static uint32_t mc_tag_hash(uint32_t h) { return (h * 0x2C1B3C6Du) & 0x7FFFFFFFu; }

void orc_memcd_init_table(uint32_t n_sets, uint64_t* tags, uint32_t* recs) {
  size_t nv = (size_t)n_sets * MC_WAYS * MC_D;
  for (size_t v = 0; v < nv; v++) tags[v] = (v % MC_D == 0) ? 0ull : (0xFFFFFFFFull << 32);
  memset(recs, 0, nv * 16 * sizeof(uint32_t));
}

static int mc_newest(const uint64_t* tags, size_t e) {
  int best = -1;
  uint32_t bts = 0;
  for (int j = 0; j < MC_D; j++) {
    uint32_t t = (uint32_t)(tags[e * MC_D + j] >> 32);
    if (t == 0xFFFFFFFFu) continue;
    if (best < 0 || t > bts) {
      best = j;
      bts = t;
    }
  }
  return best;
}

/* GET at the table's current state: 1 on a hit (value copied to out[8]). */
static int mc_get(uint32_t n_sets, const uint64_t* tags, const uint32_t* recs, const uint32_t* key,
                  uint32_t* out) {
  size_t e0 = (size_t)(orc_memcd_mix(key) % n_sets) * MC_WAYS;
  for (int w = 0; w < MC_WAYS; w++) {
    int j = mc_newest(tags, e0 + w);
    if (j < 0) continue;
    size_t v = (e0 + w) * MC_D + j;
    const uint32_t* r = recs + v * 16;
    if ((tags[v] & 0x80000000ull) && !memcmp(r + 4, key, 16)) {
      memcpy(out, r + 8, 32);
      return 1;
    }
  }
  memset(out, 0, 32);
  return 0;
}

/* SET with commit timestamp ts: slot by the reference rule, new version into the victim. */
static void mc_set(uint32_t n_sets, uint64_t* tags, uint32_t* recs, const uint32_t* key,
                   const uint32_t* val, uint32_t tick, uint32_t ts) {
  uint32_t h = orc_memcd_mix(key);
  size_t e0 = (size_t)(h % n_sets) * MC_WAYS;
  int32_t match[MC_WAYS], state[MC_WAYS], age[MC_WAYS];
  for (int w = 0; w < MC_WAYS; w++) {
    int j = mc_newest(tags, e0 + w);
    size_t v = (e0 + w) * MC_D + (j < 0 ? 0 : j);
    const uint32_t* r = recs + v * 16;
    state[w] = (j >= 0 && (tags[v] & 0x80000000ull)) ? 1 : 0;
    match[w] = (j >= 0 && !memcmp(r + 4, key, 16)) ? 1 : 0;
    age[w] = (int32_t)r[0];
  }
  int slot = orc_memcd_set_slot(match, state, age, MC_WAYS, 1);
  size_t e = e0 + slot;
  int vic = 0;
  uint32_t vkey = (uint32_t)(tags[e * MC_D] >> 32) + 1u;
  for (int j = 1; j < MC_D; j++) {
    uint32_t k = (uint32_t)(tags[e * MC_D + j] >> 32) + 1u;
    if (k < vkey) {
      vkey = k;
      vic = j;
    }
  }
  size_t v = e * MC_D + vic;
  tags[v] = ((uint64_t)ts << 32) | 0x80000000ull | mc_tag_hash(h);
  uint32_t* r = recs + v * 16;
  r[0] = tick;
  r[1] = r[2] = r[3] = 0;
  memcpy(r + 4, key, 16);
  memcpy(r + 8, val, 32);
}

void orc_memcd_serial(uint32_t n_req, const uint32_t* kind, const uint32_t* key,
                      const uint32_t* val, uint32_t tick, uint32_t n_sets, uint32_t base_ts,
                      uint64_t* tags, uint32_t* recs, uint32_t* found, uint32_t* val_out,
                      uint32_t* log_txn, uint32_t* outcome, uint32_t* n_log) {
  uint32_t ts = base_ts;
  for (uint32_t i = 0; i < n_req; i++) {
    if (kind[i] == 1u) {
      ts++;
      mc_set(n_sets, tags, recs, key + 4 * (size_t)i, val + 8 * (size_t)i, tick, ts);
      if (found) found[i] = 0;
      if (val_out) memset(val_out + 8 * (size_t)i, 0, 32);
      if (log_txn) log_txn[ts - base_ts - 1] = i;
      if (outcome) outcome[i] = ts;
    } else {
      uint32_t tmp[8];
      uint32_t f = (uint32_t)mc_get(n_sets, tags, recs, key + 4 * (size_t)i, tmp);
      if (found) found[i] = f;
      if (val_out) memcpy(val_out + 8 * (size_t)i, tmp, 32);
      if (outcome) outcome[i] = ts | SNAP_FLAG;
    }
  }
  if (n_log) *n_log = ts - base_ts;
}

int orc_memcd_check(uint32_t n_req, const uint32_t* kind, const uint32_t* key,
                    const uint32_t* val, uint32_t tick, uint32_t n_sets, const uint64_t* tags0,
                    const uint32_t* recs0, uint32_t base_ts, uint32_t n_log,
                    const uint32_t* log_txn, const uint32_t* outcome, const uint32_t* found,
                    const uint32_t* val_out, const uint64_t* tags, const uint32_t* recs,
                    char* msg, int msg_len) {
  int rc = 0;
  size_t nv = (size_t)n_sets * MC_WAYS * MC_D;
  uint64_t* mt = malloc(nv * 8);
  uint32_t* mr = malloc(nv * 64);
  uint8_t* seen = calloc(n_req ? n_req : 1, 1);
  uint32_t* head = malloc(sizeof(uint32_t) * ((size_t)n_log + 1));
  uint32_t* next = malloc(sizeof(uint32_t) * (n_req ? n_req : 1));
  if (!mt || !mr || !seen || !head || !next) {
    rc = fail(msg, msg_len, "oracle out of memory");
    goto out;
  }
  if (tags0) {
    memcpy(mt, tags0, nv * 8);
    memcpy(mr, recs0, nv * 64);
  } else {
    orc_memcd_init_table(n_sets, mt, mr);
  }
  /* 1. the log names distinct SETs with matching outcomes; every SET committed once */
  for (uint32_t k = 0; k < n_log; k++) {
    uint32_t r = log_txn[k], ts = base_ts + k + 1;
    if (r == 0xFFFFFFFFu) continue;
    if (r >= n_req || kind[r] != 1u) {
      rc = fail(msg, msg_len, "ts %u: request %u is not a SET of this batch", ts, r);
      goto out;
    }
    if (seen[r]) {
      rc = fail(msg, msg_len, "ts %u: request %u committed twice", ts, r);
      goto out;
    }
    if (outcome[r] != ts) {
      rc = fail(msg, msg_len, "ts %u: request %u outcome says %u", ts, r, outcome[r]);
      goto out;
    }
    seen[r] = 1;
  }
  /* 2. GETs bucketed by snapshot */
  for (uint32_t b = 0; b <= n_log; b++) head[b] = 0xFFFFFFFFu;
  for (uint32_t r = 0; r < n_req; r++) {
    if (kind[r] == 1u) {
      if (!seen[r]) {
        rc = fail(msg, msg_len, "SET %u never committed", r);
        goto out;
      }
      continue;
    }
    if (!(outcome[r] & SNAP_FLAG)) {
      rc = fail(msg, msg_len, "GET %u has no snapshot (outcome %u)", r, outcome[r]);
      goto out;
    }
    uint32_t snap = outcome[r] & ~SNAP_FLAG;
    if (snap < base_ts || snap > base_ts + n_log) {
      rc = fail(msg, msg_len, "GET %u: snapshot %u outside [%u, %u]", r, snap, base_ts,
                base_ts + n_log);
      goto out;
    }
    next[r] = head[snap - base_ts];
    head[snap - base_ts] = r;
  }
  /* 3. replay in ts order; GETs at snapshot s see every SET with ts <= s */
  for (uint32_t k = 0; k <= n_log; k++) {
    for (uint32_t r = head[k]; r != 0xFFFFFFFFu; r = next[r]) {
      uint32_t want[8];
      uint32_t f = (uint32_t)mc_get(n_sets, mt, mr, key + 4 * (size_t)r, want);
      if (found[r] != f || memcmp(val_out + 8 * (size_t)r, want, 32)) {
        rc = fail(msg, msg_len, "GET %u at snapshot %u: device found=%u val0=%u, replay found=%u val0=%u",
                  r, base_ts + k, found[r], val_out[8 * (size_t)r], f, want[0]);
        goto out;
      }
    }
    if (k == n_log) break;
    uint32_t r = log_txn[k];
    if (r == 0xFFFFFFFFu) continue;
    mc_set(n_sets, mt, mr, key + 4 * (size_t)r, val + 8 * (size_t)r, tick, base_ts + k + 1);
    if (found[r] != 0u) {
      rc = fail(msg, msg_len, "SET %u reports found=%u", r, found[r]);
      goto out;
    }
  }
  /* 4. the version store is bit-exact */
  for (size_t v = 0; v < nv; v++) {
    if (tags[v] != mt[v] || memcmp(recs + 16 * v, mr + 16 * v, 64)) {
      rc = fail(msg, msg_len, "version %zu (set %zu way %zu slot %zu): device tag %016llx lru %u "
                "key0 %u, replay tag %016llx lru %u key0 %u", v, v / (MC_WAYS * MC_D),
                (v / MC_D) % MC_WAYS, v % MC_D, (unsigned long long)tags[v], recs[16 * v],
                recs[16 * v + 4], (unsigned long long)mt[v], mr[16 * v], mr[16 * v + 4]);
      goto out;
    }
  }
out:
  free(mt);
  free(mr);
  free(seen);
  free(head);
  free(next);
  return rc;
}

int orc_memcd_serial_time(uint32_t n_req, const uint32_t* kind, const uint32_t* key,
                          const uint32_t* val, uint32_t tick, uint32_t n_sets, uint64_t* tags,
                          uint32_t* recs, uint32_t* found, uint32_t* val_out, uint64_t* ns) {
  struct timespec a, b;
  clock_gettime(CLOCK_MONOTONIC, &a);
  orc_memcd_serial(n_req, kind, key, val, tick, n_sets, 0, tags, recs, found, val_out, NULL, NULL,
                   NULL);
  clock_gettime(CLOCK_MONOTONIC, &b);
  *ns = (uint64_t)(b.tv_sec - a.tv_sec) * 1000000000ull + (uint64_t)(b.tv_nsec - a.tv_nsec);
  return 0;
}
