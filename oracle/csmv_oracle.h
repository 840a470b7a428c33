/*
 * csmv_oracle.h - CPU oracle for the CSMV commit path. TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs may load
 * this library; the product (csmv-gpu-stm_gb300/) never links, imports or runs it.
 *
 * Every function restates one piece of the reference algorithm (paths relative to the
 * DMRNunes/csmv-gpu-stm project root) in plain C so the CUDA path can be checked against it:
 *   - orc_rand_r            RAND_R_FNC LCG, bank/csmv_sh/API.cuh:37-53
 *   - orc_ref_read          TXRead/TXReadOnly version-list rule, bank/csmv_sh/API.cu:5-67
 *   - orc_ref_writeback     TXWriteBack version rotation, bank/csmv_sh/API.cu:147-190
 *   - orc_packed_*          the same rules on the GB300 packed (ts|value) slot layout
 *   - orc_prevalidate       TXPreValidation, csmv_optimizations/batchedAtrInsert/csmv_sh/API.cu:94-191
 *   - orc_ref_validate      TXValidate (plain), bank/csmv_sh/API.cu:88-144
 *   - orc_batched_validate  TXValidate (batched), batchedAtrInsert/csmv_sh/API.cu:193-228
 *   - orc_collab_validate   TXValidate (collaborative), collabValidation/csmv_sh/API.cu:193-266
 *   - orc_batched_ts        commit-ts offsets, batchedAtrInsert/csmv_sh/API.cu:296-377
 *   - orc_memcd_set_slot    SET slot choice, memcachedGPU/memcdSH.cu:365-387
 *   - orc_memcd_serial      serial GET/SET semantics of the cache, memcdSH.cu:343-440
 *   - orc_memcd_check       replay of a cache batch's commit log (exactness oracle)
 *   - orc_bank_check        serial replay of a commit log in commit-ts order (exactness oracle)
 *   - orc_bank_check_groups the same for group commits (one installed version per account and
 *                           group, no snapshot inside a group)
 *   - orc_bank_sim_1warp    deterministic model of one client warp + one server
 *   - orc_bank_serial / orc_bank_locked   CPU baselines (single thread / striped locks)
 *
 * Parity pin: the restatements of the read rule, write-back, plain and batched validation and
 * pre-validation are checked against the reference's own functions compiled for the host
 * (oracle/ref_build.sh -> oracle/_ref/libcsmv_ref.so) and against the golden vectors in
 * tests/golden/ that the same build generated.
 */
#ifndef CSMV_ORACLE_H_
#define CSMV_ORACLE_H_
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- RNG ---------------------------------------------------------------------------- */
uint64_t orc_rand_r(uint64_t* state);
uint64_t orc_h64(uint64_t x);
uint32_t orc_rnd32(uint64_t seed, uint64_t a, uint64_t b);

/* ---- workload (same field order as csmv_bank_workload in include/csmv.h) ------------- */
typedef struct orc_bank_workload {
  uint64_t seed;
  uint32_t n_accounts, n_txn, pr_read_pct, ro_reads, up_reads, kind, amt_lo, amt_hi, dist;
  double zipf_theta, hot_frac, hot_prob;
  uint32_t shift_every;
} orc_bank_workload;

int orc_bank_stream_size(const orc_bank_workload* w, uint64_t* n_addr);
int orc_bank_generate(const orc_bank_workload* w, uint32_t* op, uint32_t* off, uint32_t* addr);

/* ---- version-list rules ------------------------------------------------------------- */
/* reference layout: head/tail indices into version[]/value[] of length maxv */
int orc_ref_read(uint16_t head, uint16_t tail, const uint32_t* version, const int32_t* value,
                 int maxv, uint32_t ts, int32_t* out);
void orc_ref_writeback(uint16_t* head, uint16_t* tail, uint32_t* version, int32_t* value,
                       int maxv, uint32_t ts, int32_t v);
/* packed layout: slots[d] = ts<<32 | value, empty = ts 0xFFFFFFFF */
int orc_packed_read(const uint64_t* slots, int depth, uint32_t ts, int32_t* out);
int orc_packed_victim(const uint64_t* slots, int depth);
void orc_packed_writeback(uint64_t* slots, int depth, uint32_t ts, int32_t v);

/* ---- pre-validation ------------------------------------------------------------------ */
/* rs: 32 lanes x rs_stride addresses (n_rs[l] used); ws likewise. Returns the commit mask;
 * conflict[l] receives lane l's conflict bits (lower lanes whose writes it read). Lanes not
 * in `active` neither commit nor cause conflicts. */
uint32_t orc_prevalidate(const uint32_t* rs, const uint32_t* n_rs, int rs_stride,
                         const uint32_t* ws, const uint32_t* n_ws, int ws_stride,
                         uint32_t active, uint32_t* conflict);

/* ---- record ring validation --------------------------------------------------------- */
typedef struct orc_record {
  uint32_t txn;      /* transactionNumber */
  uint32_t n_writes;
  uint32_t ws[4];
} orc_record;

enum { ORC_VALID = 0, ORC_ABORT_RECORD_AGE = 1, ORC_ABORT_READ_WRITE = 2 };

int orc_ref_validate(const orc_record* recs, int ring, int hp, int tp, int oldhp, int ts,
                     const uint32_t* rs, int nrs);
int orc_batched_validate(const orc_record* recs, int ring, int hp, int tp, int oldhp, int ts,
                         const uint32_t* rs, int nrs);
/* collaborative validation of 32 lanes: ts[l] < 0 means the lane does not validate;
 * out[l] = ORC_* verdict (lanes with ts < 0 report ORC_VALID but are not candidates). */
void orc_collab_validate(const orc_record* recs, int ring, int hp, int tp, const int* ts,
                         const uint32_t* rs, const uint32_t* n_rs, int rs_stride, int* out);
/* ts for passing lanes: prev_ts + popc(ballot & lanemask_lt) + 1, 0 for failed lanes */
void orc_batched_ts(uint32_t ballot, uint32_t prev_ts, uint32_t* ts_out);

/* GB300 engine rule: window validation of a snapshot against every committed transaction
 * with ts in (snap, frontier]; RecordAge when the ring (size ring) no longer reaches snap. */
int orc_window_validate(const orc_record* by_ts /* index ts-1 */, uint32_t snap,
                        uint32_t frontier, uint32_t ring, const uint32_t* rs, int nrs,
                        int ring_mode);

/* ---- memcached slot choice ---------------------------------------------------------- */
int orc_memcd_set_slot(const int32_t* keys, const int32_t* states, const int32_t* ages,
                       int ways, int32_t key);

/* ---- transactional cache (8 ways, 2 versions per entry; layout in include/csmv.h) ------ */
uint32_t orc_memcd_mix(const uint32_t* key4);
void orc_memcd_init_table(uint32_t n_sets, uint64_t* tags, uint32_t* recs);
/* Executes requests in order (SET i gets the next timestamp after base_ts); any of found,
 * val_out, log_txn, outcome, n_log may be NULL. */
void orc_memcd_serial(uint32_t n_req, const uint32_t* kind, const uint32_t* key,
                      const uint32_t* val, uint32_t tick, uint32_t n_sets, uint32_t base_ts,
                      uint64_t* tags, uint32_t* recs, uint32_t* found, uint32_t* val_out,
                      uint32_t* log_txn, uint32_t* outcome, uint32_t* n_log);
/* Replays the batch's SETs in commit-ts order from the table before the batch (tags0/recs0,
 * NULL = empty), checks every GET against the state at its snapshot and the final version
 * store bit for bit. 0 = ok, else a message in msg. */
int orc_memcd_check(uint32_t n_req, const uint32_t* kind, const uint32_t* key,
                    const uint32_t* val, uint32_t tick, uint32_t n_sets, const uint64_t* tags0,
                    const uint32_t* recs0, uint32_t base_ts, uint32_t n_log,
                    const uint32_t* log_txn, const uint32_t* outcome, const uint32_t* found,
                    const uint32_t* val_out, const uint64_t* tags, const uint32_t* recs,
                    char* msg, int msg_len);
/* CPU baseline: serial execution, elapsed nanoseconds in *ns. */
int orc_memcd_serial_time(uint32_t n_req, const uint32_t* kind, const uint32_t* key,
                          const uint32_t* val, uint32_t tick, uint32_t n_sets, uint64_t* tags,
                          uint32_t* recs, uint32_t* found, uint32_t* val_out, uint64_t* ns);

/* ---- bank execution semantics -------------------------------------------------------- */
/* Execute one transaction against `vals`; returns number of writes (0/2) and fills
 * waddr/wval, or the read-only result in *result. */
int orc_bank_exec(uint32_t op, const uint32_t* addrs, const int32_t* vals_in,
                  uint32_t* waddr, int32_t* wval, int32_t* result);

/* Replay checker. Returns 0 on success, else an error code with a message in msg. */
int orc_bank_check(uint32_t n_txn, const uint32_t* op, const uint32_t* off, const uint32_t* addr,
                   uint32_t n_accounts, const int32_t* init, int depth, uint32_t final_ts,
                   const uint32_t* log_txn, const uint32_t* outcome, const int32_t* result,
                   const uint64_t* final_slots, char* msg, int msg_len);

/* The same with commit groups: group_end is a bitmap over timestamps 1..final_ts (bit ts-1 set
 * when ts ends a group; NULL = every timestamp ends its own). A group's writes install one
 * version per account - its last write - and no snapshot may fall inside a group. */
int orc_bank_check_groups(uint32_t n_txn, const uint32_t* op, const uint32_t* off,
                          const uint32_t* addr, uint32_t n_accounts, const int32_t* init,
                          int depth, uint32_t final_ts, const uint32_t* log_txn,
                          const uint32_t* outcome, const int32_t* result,
                          const uint32_t* group_end, const uint64_t* final_slots, char* msg,
                          int msg_len);

/* Deterministic model of the GB300 engine with one client warp and one server. */
typedef struct orc_sim_stats {
  uint64_t commits_update, commits_readonly, commits_nowrite, aborts_prevalid,
      aborts_read_write, rounds, aborts_write_write;
  uint32_t final_ts;
} orc_sim_stats;
/* locks = 1 models the stamp protocol's intra-warp rule (a lane whose write set overlaps a lower
 * candidate's does not lock; lane order is then resolved among the locked lanes), locks = 0 the
 * ring protocol (lane order among all candidates). */
int orc_bank_sim_1warp(uint32_t n_txn, const uint32_t* op, const uint32_t* off,
                       const uint32_t* addr, uint32_t n_accounts, const int32_t* init,
                       int depth, int prevalidate, int locks, uint64_t* slots_out,
                       uint32_t* log_txn, uint32_t* outcome, int32_t* result, orc_sim_stats* st);

/* CPU baselines: executes the stream, returns elapsed nanoseconds in *ns. */
int orc_bank_serial(uint32_t n_txn, const uint32_t* op, const uint32_t* off,
                    const uint32_t* addr, uint32_t n_accounts, int32_t* vals, uint64_t* ns);
int orc_bank_locked(uint32_t n_txn, const uint32_t* op, const uint32_t* off,
                    const uint32_t* addr, uint32_t n_accounts, int32_t* vals, int nthreads,
                    uint64_t* ns);

#ifdef __cplusplus
}
#endif
#endif
