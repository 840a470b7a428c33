/*
 * csmv.h - C ABI of the GB300 CSMV (client/server multi-versioned STM) commit path.
 *
 * The original project (DMRNunes/csmv-gpu-stm) has no library boundary: its "API" is the
 * header-compiled device functions (TXBegin/TXRead/TXWrite/TXAddToRecord/TXWriteBack, see
 * csmv_tx.cuh) plus per-driver host helpers TXInit/TXEnd and the bank/memcached command lines.
 * Each entry point below replaces one of those host-side pieces; the comment names the
 * reference code it stands in for (paths are relative to the reference project root).
 *
 * Conventions
 *  - Every function returns a csmv_status (0 = CSMV_OK) and never aborts the process
 *    (the reference's CUDA_CHECK_ERROR dereferences NULL on purpose, bank/csmv_sh/API.cuh:27-35).
 *  - Pointers named host_* are host memory; dev_* are device pointers owned by the caller.
 *  - One handle drives one GPU; handles are not thread-safe.
 */
#ifndef CSMV_H_
#define CSMV_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CSMV_ABI_VERSION 3 /* 2: csmv_bank_config.flow_warps, CSMV_ERR_IO, lanes and trace files;
                              3: group commit (prevalidate 3), csmv_bank_stream.backoff,
                              csmv_bank_read_groups, scheduler grouping and backoff fields */

typedef enum csmv_status {
  CSMV_OK = 0,
  CSMV_ERR_INVALID_ARG = 1,  /* a size, pointer or option is out of range                 */
  CSMV_ERR_CUDA = 2,         /* a CUDA runtime call failed (csmv_last_error has the text)   */
  CSMV_ERR_OOM = 3,          /* device or host allocation failed                            */
  CSMV_ERR_TIMEOUT = 4,      /* a bounded device wait ran out; the kernel returned early     */
  CSMV_ERR_CAPACITY = 5,     /* commit log / result buffers too small for the run           */
  CSMV_ERR_NO_DEVICE = 6,    /* no CUDA device, or the device is not sm_103                  */
  CSMV_ERR_STATE = 7,        /* call order violated (e.g. run before load)                  */
  CSMV_ERR_IO = 8            /* a file could not be opened, read or written, or is not a valid
                                stream / commit-log file (magic, version, size, checksum)     */
} csmv_status;

/* ------------------------------------------------------------------------------------------
 * Transaction stream format (bank)
 *
 * A stream holds n_txn transactions, n_txn a multiple of 32: transaction i runs on lane i%32
 * of the client warp that picked round i/32. A round is warp-uniform in kind, exactly as the
 * reference decides read-only vs update per warp (bank/csmv_sh/exe.cu:134-139).
 *
 *   op[i]   bits 0-1  kind:  0 = read-only sum of nreads accounts
 *                            1 = transfer if sufficient funds (skip -> commits with no writes)
 *                            2 = transfer unconditionally (the reference's -1/+1 transfer,
 *                                bank/csmv_sh/exe.cu:191-200)
 *           bits 2-7  nreads (1..32; transfers need >= 2)
 *           bits 8-19 amt0   (1..4095)
 *           bits 20-31 amod  (1..4095)
 *   off[i]  index of the first address of transaction i in addr[]
 *   addr[]  account ids; addr[off[i] + k], k < nreads
 *
 * Transfer semantics (v[k] = value read from addr[off[i]+k]):
 *   amt = 1 + ((amt0 - 1) + sum_{k>=2} (uint32)v[k]) % amod      (uint32 arithmetic)
 *   kind 1: if v[0] >= amt: write a0 = v[0]-amt, a1 = v[1]+amt;  else no writes
 *   kind 2: always write a0 = v[0]-amt, a1 = v[1]+amt
 * Read-only: result = (int32)(sum_k (uint32)v[k]).
 * ------------------------------------------------------------------------------------------ */
#define CSMV_OP_KIND(op) ((op)&3u)
#define CSMV_OP_NREADS(op) (((op) >> 2) & 63u)
#define CSMV_OP_AMT0(op) (((op) >> 8) & 4095u)
#define CSMV_OP_AMOD(op) (((op) >> 20) & 4095u)
#define CSMV_MAKE_OP(kind, nreads, amt0, amod)                                          \
  ((uint32_t)(kind) | ((uint32_t)(nreads) << 2) | ((uint32_t)(amt0) << 8) |             \
   ((uint32_t)(amod) << 20))

enum { CSMV_KIND_READONLY = 0, CSMV_KIND_TRANSFER = 1, CSMV_KIND_TRANSFER_ALWAYS = 2 };

typedef struct csmv_bank_stream {
  uint32_t n_txn;
  const uint32_t* op;   /* [n_txn]  */
  const uint32_t* off;  /* [n_txn]  */
  const uint32_t* addr; /* [n_addr] */
  uint64_t n_addr;
  /* Optional, zero = unused. */
  uint32_t* txn_aborts;    /* out [n_txn]: failed attempts of each transaction (same memory
                              kind as op: host for csmv_bank_run, device for _run_device)    */
  uint32_t split_round;    /* > 0: rounds [split_round, n_txn/32) form a deferred queue that
                              only the first deferred_warps client warps of the grid serve, so
                              at most that many of its rounds run at once (a scheduler's
                              likely-conflicting transactions); they serve the main queue
                              [0, split_round) once it is empty                              */
  uint32_t deferred_warps;
  const uint32_t* backoff; /* optional [n_txn] (same memory kind as op): before a round retries,
                              its warp pauses a random time below the largest backoff[i] (ns)
                              of its uncommitted transactions (a scheduler's backoff; the
                              reference retries at once, bank/csmv_sh/exe.cu:142-269)      */
  uint32_t* txn_waits;     /* optional out [n_txn] (same memory kind as op): 1 when the
                              transaction's commit group found one of its write locks held by
                              another warp and waited for it (group commit), else 0 - a
                              conflict the engine resolved by waiting instead of aborting   */
  const uint8_t* lock_last; /* optional [n_accounts of the bank] (same memory kind as op; group
                              commit only): heat class of each account, 0 = none. Group commit
                              takes the locks of classed accounts after all others, by class
                              and account (the hottest last); a group that cannot take every
                              lock at once queues, holding nothing, for its hottest account and
                              takes its other locks at the head of that queue, so a hot lock is
                              held only while its group commits (a scheduler's hot accounts) */
  const uint32_t* lane_start; /* optional [deferred_warps + 1] (same memory kind as op), with
                              split_round: the deferred queue is cut into deferred_warps lanes,
                              lane i = rounds [lane_start[i], lane_start[i+1]) (absolute round
                              indices, split_round <= lane_start[0] <= ... <= n_txn/32), each
                              served in order by the one warp of global index i, which then
                              joins the main queue: a hot account's rounds on one warp hold its
                              lock back to back, with no hand-off between warps              */
} csmv_bank_stream;

/* Account-choice distributions for the workload generator. */
enum {
  CSMV_DIST_UNIFORM = 0,
  CSMV_DIST_ZIPF = 1,    /* Zipf(theta) by rejection-inversion (Hormann & Derflinger 1996)  */
  CSMV_DIST_HOTSPOT = 2  /* hot_frac of the accounts get hot_prob of the draws; the hot
                            window moves to a new random place every shift_every txns       */
};

typedef struct csmv_bank_workload {
  uint64_t seed;
  uint32_t n_accounts;
  uint32_t n_txn;          /* multiple of 32 */
  uint32_t pr_read_pct;    /* % of rounds that are read-only (0..100)               */
  uint32_t ro_reads;       /* accounts summed by a read-only transaction             */
  uint32_t up_reads;       /* accounts read by a transfer (>= 2)                     */
  uint32_t kind;           /* CSMV_KIND_TRANSFER or CSMV_KIND_TRANSFER_ALWAYS        */
  uint32_t amt_lo, amt_hi; /* transfer amount range (amt0 drawn uniformly)           */
  uint32_t dist;           /* CSMV_DIST_*                                            */
  double zipf_theta;
  double hot_frac, hot_prob;
  uint32_t shift_every;
} csmv_bank_workload;

/* Generate a stream on the host into caller buffers (sizes from csmv_bank_stream_size). */
csmv_status csmv_bank_stream_size(const csmv_bank_workload* w, uint64_t* n_addr);
csmv_status csmv_bank_generate(const csmv_bank_workload* w, uint32_t* host_op,
                               uint32_t* host_off, uint32_t* host_addr);

/* ------------------------------------------------------------------------------------------
 * Bank engine
 * ------------------------------------------------------------------------------------------ */

/* How a server validates a read set. */
enum {
  CSMV_VALIDATE_STAMP = 0,     /* per-item commit timestamp (latest writer) - the "ts" form   */
  CSMV_VALIDATE_RING = 1,      /* scan of the commit-record ring, lanes strided over records and
                                  probing a shared-memory hash of the batch's read sets (the
                                  collaborative scan, collabValidation/csmv_sh/API.cu:193-266) */
  CSMV_VALIDATE_RING_LANE = 2  /* each lane scans the ring for its own transaction
                                  (plain TXValidate, bank/csmv_sh/API.cu:88-144)              */
};

/* Where write-back happens (csmv_optimizations/clientWriteback moves it to the server). */
enum { CSMV_WRITEBACK_CLIENT = 0, CSMV_WRITEBACK_SERVER = 1 };

/* What one commit section covers. */
enum {
  CSMV_BATCH_LANE = 0,  /* one transaction per section (plain TXAddToRecord, API.cu:193-272)  */
  CSMV_BATCH_WARP = 1,  /* one client warp per section (batchedAtrInsert TXAddToRecord)        */
  CSMV_BATCH_CTA = 2,   /* every pending client warp of the CTA in one section                 */
  CSMV_BATCH_CLUSTER = 3 /* client warps of a thread-block cluster post to the server warp of
                            the cluster's leader CTA through distributed shared memory (one
                            server for several blocks; no counterpart in the reference);
                            stamp protocol, client_warps x cluster_size <= 32, ctas a
                            multiple of cluster_size                                           */
};

typedef struct csmv_bank_config {
  uint32_t n_accounts;
  int32_t init_value;          /* every account starts at this balance                        */
  uint32_t version_depth;      /* versions kept per account, 2..16                            */
  uint32_t ring_size;          /* commit-record ring entries, power of two, >= 64             */
  uint32_t client_warps;       /* client warps per CTA (1..15)                                */
  uint32_t ctas;               /* CTAs; 0 = as many as fit co-resident on the GPU             */
  uint32_t cluster_size;       /* CTAs per cluster for CSMV_BATCH_CLUSTER (2, 4 or 8)          */
  uint32_t validate;           /* CSMV_VALIDATE_*                                             */
  uint32_t writeback;          /* CSMV_WRITEBACK_*                                            */
  uint32_t batch;              /* CSMV_BATCH_*                                                */
  uint32_t prevalidate;        /* 0 = none; 1 = intra-warp pre-validation (batchedAtrInsert,
                                  API.cu:94-191); 2 = intra-warp chaining (stamp protocol);
                                  3 = group commit (stamp protocol): a warp's round locks every
                                  account it may write once, waiting in one total order (the
                                  stream's heat classes last, first-come first-served queues),
                                  reads them under the locks, draws the round's timestamps from
                                  its server, validates every read of an account it does not
                                  lock, runs the transfers that pass as a chain in lane order
                                  and installs ONE version per account (the last writer's); the
                                  clock passes a group's timestamps at once, so no snapshot
                                  sees its intermediate states                                 */
  uint32_t log_commits;        /* 1 = keep the per-ts commit log and per-txn outcomes         */
  uint32_t max_txn;            /* largest stream a run may carry (sizes the logs)             */
  uint32_t spin_limit_log2;    /* bounded waits give up after 2^this polls (default 24)       */
  int32_t device;
  uint32_t flow_warps;         /* warps of the dataflow lane's execution CTA, 1..16 (0 = 8)    */
  uint32_t max_reads;          /* reads of a transfer the commit kernel holds: 0 or 8 = up to 8;
                                  4 = up to 4 (a leaner kernel; a transfer with more reads is
                                  malformed, CSMV_ERR_INVALID_ARG). Read-only transactions may
                                  read up to 32 accounts either way                            */
  uint32_t group_grace;        /* group commit: polls (about 0.1 us each) a hot queue's head
                                  keeps trying its other locks after taking its hottest one,
                                  before the lanes whose locks are still held sit the attempt
                                  out (default 4)                                              */
  uint32_t group_read_wait;    /* group commit: polls (about 0.5 us each) a lane makes for an
                                  earlier group's lock on an account it only reads before it
                                  gives up and its transaction is retried (default 8; 0 = wait
                                  up to 4096 polls). Short waits keep a hot lock's holds short */
} csmv_bank_config;

void csmv_bank_config_default(csmv_bank_config* cfg);

typedef struct csmv_stats {
  uint64_t commits_update;     /* transfers that committed with writes                        */
  uint64_t commits_readonly;   /* read-only transactions                                       */
  uint64_t commits_nowrite;    /* transfers skipped for insufficient funds (commit, no writes) */
  uint64_t aborts_data_age;    /* a needed version was already evicted (API.cu:20-24)          */
  uint64_t aborts_record_age;  /* commit ring no longer covers the snapshot (API.cu:93-100)    */
  uint64_t aborts_read_write;  /* read item written by a later committed transaction          */
  uint64_t aborts_prevalid;    /* lost to a lower lane / earlier batch member (API.cu:94-191)  */
  uint64_t aborts_write_write; /* write lock held by another warp (stamp protocol)             */
  uint64_t sections;           /* commit sections entered (global order steps)                */
  uint64_t rounds;             /* warp rounds executed, retries included                      */
  uint32_t final_ts;           /* last timestamp handed out (commits and holes)                */
  uint32_t error;              /* device error word (0 = none); see csmv_last_error           */
  double kernel_ms;            /* device time of the run, CUDA events on the engine stream    */
  double total_ms;             /* host wall time of the call                                   */
} csmv_stats;

typedef struct csmv_bank_t csmv_bank_t;

/* Replaces TXInit (bank/csmv_sh/API.cu:293-333) and create_gbc/init_gbc
 * (sync_lib/one_phase_server.h:13-42, sync_lib/msg_aux.h:39-92): allocates the versioned
 * accounts, record ring, mailboxes and logs on the device. */
csmv_status csmv_bank_create(const csmv_bank_config* cfg, csmv_bank_t** out);

/* Replaces the initial-value part of TXInit: head version of every account gets
 * host_values[i] (or cfg->init_value when host_values is NULL), timestamp 0. */
csmv_status csmv_bank_load(csmv_bank_t* h, const int32_t* host_values);

/* Runs a whole stream from HOST buffers: copies it in, runs the persistent commit kernel
 * (replaces parent_kernel/server_kernel/client_kernel, bank/csmv_sh/exe.cu:89-338) until every
 * transaction has committed, and copies the statistics back. */
csmv_status csmv_bank_run(csmv_bank_t* h, const csmv_bank_stream* host_stream,
                          csmv_stats* out);

/* Same, with the stream already resident in device memory (dev pointers). */
csmv_status csmv_bank_run_device(csmv_bank_t* h, const csmv_bank_stream* dev_stream,
                                 csmv_stats* out);

/* Serial lane (no counterpart in the reference): one warp runs the device-resident stream in
 * stream order with the GPU to itself - a round's 32 transfers resolve their dependencies as a
 * chain in lane order and commit together, with no locks, timestamp server or validation -
 * continuing the commit order of the handle (stamp protocol only). Meant for transactions a
 * scheduler predicts to conflict; no other run of the handle may be in flight. Every
 * transaction commits; read-only ones see the state after all earlier ones. */
csmv_status csmv_bank_run_serial_device(csmv_bank_t* h, const csmv_bank_stream* dev_stream,
                                        csmv_stats* out);

/* Dataflow lane (no counterpart in the reference): the same contract and the same end state as
 * csmv_bank_run_serial_device - timestamps, version slots, commit words, log, outcomes and
 * results are identical - but every transaction whose inputs are known runs at once. Each read
 * is matched to the last earlier write of its account in the stream by a device radix sort;
 * one CTA then runs the transactions, each as soon as its producers have published, and the
 * commit (timestamps, log, version installs) is written in parallel. Limits per call: 2^25
 * transactions, 2^26 accesses (CSMV_ERR_CAPACITY). A malformed transaction (bad size, account
 * or mixed round) fails the call with nothing applied (CSMV_ERR_INVALID_ARG). Device scratch
 * of about 28 B per access and 40 B per transaction is kept by the handle after the first
 * call. */
csmv_status csmv_bank_run_flow_device(csmv_bank_t* h, const csmv_bank_stream* dev_stream,
                                      csmv_stats* out);

/* csmv_bank_run_baseline_device - the reference's naive baseline STM (bank/baseline, JVSTM
 * style; TXRead / TXValidate / TXAddToRecordNaive at bank/baseline/API.cu:3-140, 228-316) as a
 * comparison arm on the same bank: no commit server; every transaction reads at its snapshot,
 * validates against the commit records written since, and commits inside one global critical
 * section, taken here once per warp (the warp's passing transactions commit in lane order).
 * Same device stream, state, log, outcomes and results as csmv_bank_run_device (stamp protocol
 * handles only; no deferred queue, lanes, heat classes or backoff), so its runs replay in the
 * oracle and interleave with the engine's on one bank. Grid: the handle's CTAs x client warps. */
csmv_status csmv_bank_run_baseline_device(csmv_bank_t* h, const csmv_bank_stream* dev_stream,
                                          csmv_stats* out);

/* ------------------------------------------------------------------------------------------
 * On-disk streams and commit logs, so CPU and GPU runs replay identical inputs and a run's
 * commit order can be kept (the reference stores raw arrays without a header,
 * memcachedGPU/keyGenAndCacheStore.cpp:151-182). Little-endian files with a header (magic,
 * version, sizes) and an FNV-1a checksum of the payload; a mismatch returns CSMV_ERR_IO.
 * All buffers are host memory.
 * ---------------------------------------------------------------------------------------- */
csmv_status csmv_stream_save(const char* path, const csmv_bank_stream* host_stream);
csmv_status csmv_stream_info(const char* path, uint32_t* n_txn, uint64_t* n_addr);
/* CSMV_ERR_CAPACITY when the file holds more than the caps. */
csmv_status csmv_stream_load(const char* path, uint32_t* host_op, uint32_t* host_off,
                             uint32_t* host_addr, uint32_t n_txn_cap, uint64_t n_addr_cap);
/* A run's commit log as csmv_bank_read_log returns it: log_txn[k] = transaction of timestamp
 * base_ts + k + 1 (0xFFFFFFFF = hole), outcome and result per transaction. */
csmv_status csmv_log_save(const char* path, uint32_t base_ts, const uint32_t* host_log_txn,
                          uint32_t n_log, const uint32_t* host_outcome,
                          const int32_t* host_result, uint32_t n_txn);
csmv_status csmv_log_info(const char* path, uint32_t* n_txn, uint32_t* n_log, uint32_t* base_ts);
csmv_status csmv_log_load(const char* path, uint32_t* host_log_txn, uint32_t n_log_cap,
                          uint32_t* host_outcome, int32_t* host_result, uint32_t n_txn_cap);

/* Replaces TXEnd (bank/csmv_sh/API.cu:335-359): latest value of every account. */
csmv_status csmv_bank_read_values(csmv_bank_t* h, int32_t* host_values);

/* Raw version slots: n_accounts*version_depth words, (uint64)ts << 32 | (uint32)value, an
 * empty slot has ts 0xFFFFFFFF. */
csmv_status csmv_bank_read_versions(csmv_bank_t* h, uint64_t* host_slots);

/* Commit log of the last run (needs log_commits): host_log_txn[k] = transaction id that
 * committed with timestamp base+k+1 (base = final ts of the previous run), for every timestamp
 * the run used; 0xFFFFFFFF marks a timestamp whose transaction failed validation after taking
 * it (stamp protocol). host_outcome[i] for every transaction i:
 * commit ts for a transfer with writes, else (snapshot | 0x80000000) for read-only/no-write;
 * host_result[i] = read-only sum (0 otherwise). Any pointer may be NULL. */
csmv_status csmv_bank_read_log(csmv_bank_t* h, uint32_t* host_log_txn, uint32_t n_log,
                               uint32_t* host_outcome, int32_t* host_result, uint32_t n_txn);

/* Commit groups of the last run (needs log_commits): bit k of host_bits (word k / 32, bit k % 32)
 * is set when timestamp base + k + 1 ends a commit group - the timestamps of one group commit
 * (prevalidate 3), whose writes installed one version per account. Runs of other modes and
 * lanes install every write, and every timestamp ends its own group (all bits set). n_log as
 * csmv_bank_read_log; host_bits holds (n_log + 31) / 32 words. */
csmv_status csmv_bank_read_groups(csmv_bank_t* h, uint32_t* host_bits, uint32_t n_log);

/* SM count, CTAs and threads per CTA of the commit kernel, and device bytes the handle holds. */
csmv_status csmv_bank_device_info(csmv_bank_t* h, int* n_sms, int* ctas, int* threads_per_cta,
                                  size_t* device_bytes);

void csmv_bank_destroy(csmv_bank_t* h);

/* Bank run that allocates no device memory. No counterpart in the reference: it exists for
 * callers that cannot call cudaMalloc - a host that gives the library a fixed memory budget and
 * forbids allocation after start-up, or a process whose device memory belongs to another
 * allocator. It runs the default engine (stamp validation, CTA batches, client write-back,
 * pre-validation, 4 versions per account) with its scratch - version store, commit words,
 * completion bitmap, commit log - in one fixed device array of about 4.8 MiB, which every GPU
 * that loads the library holds until the process exits. Limits: n_accounts <= 65536 and
 * n_txn <= 65536 per call (larger sizes return CSMV_ERR_CAPACITY), and at most
 * CSMV_NOALLOC_MAX_TIMESTAMPS commit timestamps per call - a transaction that fails validation
 * after drawing a timestamp uses one too, so a very contended stream can run out; the kernel
 * then stops and the call returns CSMV_ERR_CAPACITY with a message naming that limit.
 * stream_desc is a HOST struct whose op, off and addr arrays (and txn_aborts / backoff, when
 * set) are in device memory; split_round, deferred_warps and txn_waits must be 0. The other
 * pointers are device memory owned by the caller: dev_init_values[n_accounts] in;
 * dev_values[n_accounts] (latest value of each account), dev_outcome[n_txn] and dev_result[n_txn]
 * (as csmv_bank_read_log) out. cuda_stream is a cudaStream_t (NULL = the legacy default stream);
 * the call returns after the stream has finished the run, with the caller's current device
 * restored; out->kernel_ms is 0 (no events are created), out->total_ms is the host wall time.
 * Calls share the array and keep nothing between them, so calls that overlap on the GPU race:
 * serialise them. The first call on a device looks up the array's device address and caches
 * it; make that first call before any stream capture, and make no call on a device after a
 * cudaDeviceReset of it (the reset voids the cached address). */
#define CSMV_NOALLOC_MAX_ACCOUNTS 65536
#define CSMV_NOALLOC_MAX_TXN 65536
#define CSMV_NOALLOC_MAX_TIMESTAMPS (8 * CSMV_NOALLOC_MAX_TXN)
csmv_status csmv_bank_run_noalloc(int32_t device, void* cuda_stream, uint32_t n_accounts,
                                  const int32_t* dev_init_values,
                                  const csmv_bank_stream* stream_desc, uint32_t client_warps,
                                  uint32_t ctas, int32_t* dev_values, uint32_t* dev_outcome,
                                  int32_t* dev_result, csmv_stats* out);

/* ------------------------------------------------------------------------------------------
 * Transactional cache (memcachedGPU/memcdSH.cu)
 *
 * An 8-way set-associative table of n_sets sets. An entry holds a 16-byte key (4 uint32
 * words), a 32-byte value (8 words), a valid flag and an LRU timestamp, each SET a
 * transaction over its set as in the reference (memcdSH.cu:343-398): it reads the 8 ways, takes
 * the way that holds the key (valid), else the way with the smallest LRU timestamp (first on
 * ties), and writes key, value, LRU = the batch's tick and valid. A GET reads the set at a
 * snapshot and returns the value of the valid way holding the key (memcdSH.cu:400-440).
 * Two versions of each entry are kept.
 *
 * Request batch: n_req requests, a multiple of 32; requests [32r, 32r+32) are all GETs or all
 * SETs (the reference decides GET vs SET per warp, memcdSH.cu:333-339).
 *   kind[i]            CSMV_MEMCD_GET or CSMV_MEMCD_SET
 *   key[4i .. 4i+3]    key words
 *   val[8i .. 8i+7]    value words (SET; ignored for GET)
 *   found[i]           out: GET 1 = hit, 0 = miss; SET 0
 *   val_out[8i ..]     out: GET hit value, else zeros
 *   tick               LRU timestamp the batch's SETs write: the reference's curr_clock, which
 *                      its host loop sets to 1 and increments after every batch (memcdSH.cu:573,648)
 * The key's set is h % n_sets (the reference's one-word key % nbSets, memcdSH.cu:80-83, over
 * four words) with h = k0*0x9E3779B1 ^ k1*0x85EBCA6B ^ k2*0xC2B2AE35 ^ k3*0x27D4EB2F (uint32),
 * h ^= h >> 16. Device batches need 16-byte aligned key, val and val_out.
 * ------------------------------------------------------------------------------------------ */
enum { CSMV_MEMCD_GET = 0, CSMV_MEMCD_SET = 1 };
#define CSMV_MEMCD_WAYS 8
#define CSMV_MEMCD_KEY_WORDS 4
#define CSMV_MEMCD_VAL_WORDS 8

typedef struct csmv_memcd_batch {
  uint32_t n_req;
  uint32_t tick;
  const uint32_t* kind;   /* [n_req]     */
  const uint32_t* key;    /* [n_req * 4] */
  const uint32_t* val;    /* [n_req * 8] */
  uint32_t* found;        /* [n_req]     */
  uint32_t* val_out;      /* [n_req * 8] */
} csmv_memcd_batch;

typedef struct csmv_memcd_workload {
  uint64_t seed;
  uint32_t n_keys;     /* key population; request keys are drawn from ids 0..n_keys-1        */
  uint32_t n_req;      /* multiple of 32                                                     */
  uint32_t get_pct;    /* % of rounds that are GETs (0..100)                                  */
  uint32_t dist;       /* CSMV_DIST_UNIFORM or CSMV_DIST_ZIPF (over key ids)                  */
  double zipf_theta;
} csmv_memcd_workload;

/* Requests of a seeded workload into caller buffers (kind [n_req], key [4 n_req],
 * val [8 n_req]). Key id k has words {k, h(k,1), h(k,2), h(k,3)}; replaces the reference's
 * host key generation (memcdSH.cu:590-600, 624-634). */
csmv_status csmv_memcd_generate(const csmv_memcd_workload* w, uint32_t* host_kind,
                                uint32_t* host_key, uint32_t* host_val);

typedef struct csmv_memcd_config {
  uint32_t n_sets;           /* sets (2^20 for the 8 M-entry cache)                            */
  uint32_t n_ways;           /* must be 8                                                       */
  uint32_t version_depth;    /* versions per entry, must be 2                                   */
  uint32_t client_warps;     /* client warps per CTA (1..15)                                    */
  uint32_t ctas;             /* CTAs; 0 = as many as fit co-resident                            */
  uint32_t batch;            /* CSMV_BATCH_WARP or CSMV_BATCH_CTA                               */
  uint32_t log_commits;      /* 1 = keep the per-ts commit log and per-request outcomes        */
  uint32_t max_req;          /* largest batch a run may carry                                  */
  uint32_t spin_limit_log2;  /* bounded waits give up after 2^this polls                        */
  int32_t device;
} csmv_memcd_config;

typedef struct csmv_memcd_t csmv_memcd_t;

void csmv_memcd_config_default(csmv_memcd_config* cfg);

/* Replaces the cache allocation of memcdSH's main (memcdSH.cu:557-566), create_gbc and TXInit. */
csmv_status csmv_memcd_create(const csmv_memcd_config* cfg, csmv_memcd_t** out);

/* Empties the table (every entry invalid, LRU 0, memcdSH.cu:567-574) and restarts the commit
 * order at timestamp 0. */
csmv_status csmv_memcd_clear(csmv_memcd_t* h);

/* Runs one batch from HOST buffers (copies in, runs the commit kernel, copies results out):
 * one iteration of the reference's batch loop (memcdSH.cu:622-651). */
csmv_status csmv_memcd_run(csmv_memcd_t* h, const csmv_memcd_batch* host_batch, csmv_stats* out);

/* Same with every batch pointer in device memory. */
csmv_status csmv_memcd_run_device(csmv_memcd_t* h, const csmv_memcd_batch* dev_batch,
                                  csmv_stats* out);

/* Raw version store: host_tags[v] = ts << 32 | valid << 31 | key hash (empty: ts 0xFFFFFFFF),
 * host_recs[16 v ..] = {lru, 0, 0, 0, key[4], value[8]}, v = (set*8 + way)*2 + version.
 * Either pointer may be NULL. */
csmv_status csmv_memcd_read_table(csmv_memcd_t* h, uint64_t* host_tags, uint32_t* host_recs);

/* Commit log of the last run: host_log_txn[k] = request that committed a SET with timestamp
 * *base_ts + k + 1 (0xFFFFFFFF: a timestamp whose SET failed validation);
 * host_outcome[i] = commit ts of a SET, (snapshot | 0x80000000) of a GET. */
csmv_status csmv_memcd_read_log(csmv_memcd_t* h, uint32_t* host_log_txn, uint32_t n_log,
                                uint32_t* host_outcome, uint32_t n_req, uint32_t* base_ts);

csmv_status csmv_memcd_device_info(csmv_memcd_t* h, int* n_sms, int* ctas, int* threads_per_cta,
                                   size_t* device_bytes);
void csmv_memcd_destroy(csmv_memcd_t* h);

/* ------------------------------------------------------------------------------------------
 * Serving loop for the cache (replaces the reference's host batch loop, memcdSH.cu:622-651,
 * which launches one kernel per batch and waits for it). The table stays on the device; one
 * persistent kernel, replayed from a CUDA graph captured at create, serves a session. Request
 * batches of any size (multiple of 32) are copied into a ring of pinned, mapped host memory and
 * published; the kernel admits them as they arrive, so batches that arrive while others run are
 * served alongside them. A batch is admitted only while the ring has room for it, the SETs in
 * flight stay within max_inflight_sets and fewer than 1024 batches are in flight; otherwise
 * csmv_serve_submit returns CSMV_ERR_CAPACITY and the caller retries after completions. Each
 * batch gets a device completion stamp; results are read with csmv_serve_poll.
 * ------------------------------------------------------------------------------------------ */
typedef struct csmv_serve_config {
  uint32_t n_sets;             /* cache sets (8 ways, 2 versions per entry)                     */
  uint32_t client_warps;       /* client warps per CTA (1..15)                                  */
  uint32_t ctas;               /* 0 = as many as fit co-resident                                */
  uint32_t arena_requests;     /* request ring size, power of two (1024..2^24)                  */
  uint32_t max_inflight_sets;  /* SET requests in flight at most (admission)                    */
  uint32_t idle_timeout_ms;    /* the kernel returns (error) after this long without work       */
  int32_t device;
  uint32_t log_cap;            /* > 0: each session logs its commits (commit ts -> arena index
                                  of the request, for its first log_cap timestamps) and every
                                  request's outcome, for a replay by a checker; 0 = off       */
  uint32_t serial_batches;     /* 1 (default): one batch on the device at a time (the next
                                  batch's rounds are admitted when every earlier round is done);
                                  0: batches overlap (more throughput at full load, longer tail
                                  latency below it)                                            */
} csmv_serve_config;
typedef struct csmv_serve_t csmv_serve_t;
void csmv_serve_config_default(csmv_serve_config* cfg);
/* Allocates the table (empty), the ring and the descriptors, and captures the session graph. */
csmv_status csmv_serve_create(const csmv_serve_config* cfg, csmv_serve_t** out);
/* Launches a session (one replay of the captured graph); the table carries over sessions. */
csmv_status csmv_serve_start(csmv_serve_t* s);
/* Publishes a batch (host pointers: kind, key, val, tick; found / val_out are not used here);
 * *batch_id numbers batches from 0 within the session. */
csmv_status csmv_serve_submit(csmv_serve_t* s, const csmv_memcd_batch* host_batch,
                              uint64_t* batch_id);
/* *done = 1 once the batch completed; its results are then copied to host_found [n] and
 * host_val_out [8 n] (either may be NULL) and *device_ns = admission -> completion (device).
 * A batch polled done is collected: its ring slots are reused by later batches (in admission
 * order), after which a poll still reports done but returns no results. Batches that are never
 * collected keep their slots, so admission stalls until they are polled. */
csmv_status csmv_serve_poll(csmv_serve_t* s, uint64_t batch_id, uint32_t* done,
                            uint32_t* host_found, uint32_t* host_val_out, uint64_t* device_ns);
/* As csmv_serve_poll, also copying each request's outcome to host_outcome [n] (log_cap > 0):
 * the commit timestamp of a SET, the snapshot | 2^31 of a GET. */
csmv_status csmv_serve_poll_logged(csmv_serve_t* s, uint64_t batch_id, uint32_t* done,
                                   uint32_t* host_found, uint32_t* host_val_out,
                                   uint32_t* host_outcome, uint64_t* device_ns);
/* After csmv_serve_stop (log_cap > 0): host_log_txn[k] = arena index of the request that
 * committed with timestamp *base_ts + k + 1 (0xFFFFFFFF: a hole), for the *n_used timestamps of
 * the session (CSMV_ERR_CAPACITY when n_log is smaller). */
csmv_status csmv_serve_read_log(csmv_serve_t* s, uint32_t* host_log_txn, uint32_t n_log,
                                uint32_t* n_used, uint32_t* base_ts);
/* Ends the session once every published batch is served; statistics of the session. */
csmv_status csmv_serve_stop(csmv_serve_t* s, csmv_stats* out);
/* Version store between sessions (layout as csmv_memcd_read_table). */
csmv_status csmv_serve_read_table(csmv_serve_t* s, uint64_t* host_tags, uint32_t* host_recs);
void csmv_serve_destroy(csmv_serve_t* s);

/* ------------------------------------------------------------------------------------------
 * Conflict predictor network (no counterpart in the reference; the learned scheduler below
 * uses it). 64 input features -> 128 -> 128 -> 1, ReLU, ReLU, sigmoid = probability that a
 * transaction aborts. Weights are kept in bf16 for the kernels (rounded from fp32 master
 * copies), arithmetic accumulates in fp32; training minimises the mean binary cross-entropy
 * with Adam. Parameter block (fp32, CSMV_MLP_PARAMS floats):
 *   W1 [64][128] | b1 [128] | W2 [128][128] | b2 [128] | w3 [128] | b3 [1] | 3 zeros
 * Features are bf16 [n][64]; labels fp32 [n] in {0, 1}. Device pointers are dev_*.
 * ------------------------------------------------------------------------------------------ */
#define CSMV_MLP_IN 64
#define CSMV_MLP_HIDDEN 128
#define CSMV_MLP_PARAMS 24964
typedef struct csmv_mlp_t csmv_mlp_t;
csmv_status csmv_mlp_create(int32_t device, uint64_t seed, csmv_mlp_t** out);
csmv_status csmv_mlp_set_params(csmv_mlp_t* m, const float* host_params); /* resets Adam */
csmv_status csmv_mlp_get_params(csmv_mlp_t* m, float* host_params);
/* dev_p[i] = predicted abort probability of sample i */
csmv_status csmv_mlp_forward(csmv_mlp_t* m, uint32_t n, const uint16_t* dev_x, float* dev_p);
/* Adds the gradient of the mean loss over the n samples to the handle's accumulator;
 * *host_loss (optional) = that mean loss. */
csmv_status csmv_mlp_grad(csmv_mlp_t* m, uint32_t n, const uint16_t* dev_x, const float* dev_y,
                          float* host_loss);
csmv_status csmv_mlp_get_grads(csmv_mlp_t* m, float* host_grads);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) from the accumulated gradient, then clears it. */
csmv_status csmv_mlp_adam_step(csmv_mlp_t* m, float lr);
void csmv_mlp_destroy(csmv_mlp_t* m);

/* ------------------------------------------------------------------------------------------
 * Learned conflict scheduler (no counterpart in the reference). It reorders and groups a chunk
 * of a bank stream before the unchanged commit engine runs it - every transaction is still
 * validated by the engine, so results stay exact:
 *  1. probe: the first probe_rounds_pct % of the chunk's rounds run in stream order, with
 *     per-transaction abort counts and lock waits; their transfers label the network's
 *     training data (aborted or waited for a lock: a conflict) and refresh per-range abort
 *     rates; train_steps Adam steps follow;
 *  2. plan: the network scores the remaining transfers from 64 features (hashed access counts
 *     of the accounts in the chunk, recent abort rates of their ranges); a transfer scoring
 *     above threshold is keyed by its more frequent written account, and the k-th of c
 *     transfers with one key is placed at (k + u)/c of the chunk (u a hash in [0, 1)), the
 *     others at u; read-only rounds are interleaved evenly; transfers scoring above
 *     defer_threshold go to the engine's deferred queue (deferred_warps warps). The planned
 *     rounds run as one engine call.
 * Streams are device-resident (csmv_bank_run_device); the bank needs max_txn >= chunk size.
 * ------------------------------------------------------------------------------------------ */
typedef struct csmv_sched_config {
  uint32_t n_accounts;        /* accounts of the bank (range bins of the abort-rate features) */
  uint32_t max_txn;           /* largest chunk, multiple of 32                                */
  uint32_t probe_rounds_pct;  /* % of each chunk's rounds run in stream order to label data   */
  uint32_t probe_every;       /* probe (and train on) one chunk in this many (>= 1)           */
  uint32_t train_steps;       /* Adam steps per chunk on the probe slice                      */
  float lr;                   /* Adam learning rate                                           */
  float threshold;            /* predicted abort probability above which a transfer is spaced */
  float defer_threshold;      /* above this it is deferred (> 1 = never)                      */
  uint32_t deferred_warps;    /* warps serving the deferred queue                             */
  uint32_t serial_lane;       /* deferred transfers run after the rest: 1 on the serial lane,
                                 2 on the dataflow lane (csmv_bank_run_flow_device)           */
  uint64_t seed;
  int32_t device;
  uint32_t plan;              /* 0 = spread flagged transfers by key (above); 1 = group them:
                                 flagged transfers are sorted by the two hottest accounts they
                                 touch (sketch count >= hot_count), so a round's 32 transfers
                                 share their hot accounts and the engine's group commit
                                 (prevalidate 3) locks each once for all of them; each hot
                                 account's rounds are spread evenly over the plan, the other
                                 transfers keep stream order in rounds of their own            */
  uint32_t hot_count;         /* plan 1: accesses in the chunk that make an account hot
                                 (0 = the chunk's transfers / 16384, at least 2)               */
  uint32_t score;             /* 0 = the network's predicted probability flags transfers;
                                 1 = the raw sketch-count score (the transfer's largest access
                                 count / the chunk's largest), no network - the ablation      */
  uint32_t backoff_ns;        /* per-transaction retry backoff: score x backoff_ns for scores
                                 >= 1/4, else 0 (0 = no backoff array)                          */
  uint32_t hot_last;          /* plan 1 on a group-commit bank: 1 (default) passes the plan's
                                 hot accounts to the engine as heat classes (the stream's
                                 lock_last, 1 + 4 log2(count / hot_count) capped at 255), so
                                 they are locked last and queued for; 0 = plain account order */
  uint32_t key_written;       /* plan 1: 1 (default) = a transfer's group key ranks the hot
                                 accounts it writes above those it only reads (rounds share the
                                 locks they take); 0 = the hottest accounts touched           */
  uint32_t hot_lanes;         /* plan 1 on a group-commit bank: up to this many (<= 64) of the
                                 hottest accounts, each filling at least 1/64 of the plan's
                                 transfer rounds, get a lane: their rounds run last, in order,
                                 on one warp each (the stream's lane_start), so a hot account's
                                 lock passes between no warps; 0 (default) = no lanes        */
} csmv_sched_config;

typedef struct csmv_sched_report {
  csmv_stats probe;           /* engine statistics of the probe run                          */
  csmv_stats planned;         /* ... of the planned run                                      */
  csmv_stats serial;          /* ... and of the serial- or dataflow-lane run               */
  float loss;                 /* mean cross-entropy on the probe slice before this chunk's steps */
  uint32_t n_probe, n_planned, n_flagged, n_deferred_rounds, n_serial;
  double train_ms, plan_ms;   /* device time of training / of features, inference and planning */
} csmv_sched_report;

typedef struct csmv_sched_t csmv_sched_t;
void csmv_sched_config_default(csmv_sched_config* cfg);
csmv_status csmv_sched_create(const csmv_sched_config* cfg, csmv_sched_t** out);
/* Both steps on one chunk (dev_stream: device pointers). */
csmv_status csmv_sched_run(csmv_sched_t* s, csmv_bank_t* bank, const csmv_bank_stream* dev_stream,
                           csmv_sched_report* out);
/* The steps separately (same chunk, in this order), so a caller can read the engine's commit
 * log after each run: probe; plan and run the concurrent part; run the serial part (a no-op
 * unless serial_lane is set and the plan deferred transfers). */
csmv_status csmv_sched_probe(csmv_sched_t* s, csmv_bank_t* bank,
                             const csmv_bank_stream* dev_stream, csmv_sched_report* out);
csmv_status csmv_sched_plan_run(csmv_sched_t* s, csmv_bank_t* bank,
                                const csmv_bank_stream* dev_stream, csmv_sched_report* out);
csmv_status csmv_sched_serial_run(csmv_sched_t* s, csmv_bank_t* bank,
                                  const csmv_bank_stream* dev_stream, csmv_sched_report* out);
/* Last plan: host_perm[i] = chunk index of the transaction the planned runs executed as their
 * i-th (n >= chunk size - 32 * probe_rounds): the concurrent part is perm[0, 32 * split_round)
 * when the serial lane took the rest (split_round = 0: one concurrent run of everything). */
csmv_status csmv_sched_read_plan(csmv_sched_t* s, uint32_t* host_perm, uint32_t n,
                                 uint32_t* probe_rounds, uint32_t* split_round);
/* The scheduler's network (owned by the scheduler). */
csmv_mlp_t* csmv_sched_mlp(csmv_sched_t* s);
void csmv_sched_destroy(csmv_sched_t* s);

/* ------------------------------------------------------------------------------------------
 * Autotuner (no counterpart in the reference, whose launch shape is fixed on the command line):
 * measures the engine on a sample of the caller's stream over client warps per CTA (1, 2, 4,
 * 8: the block size and the number of mailboxes per commit-server warp), CTAs per SM (1, 2),
 * versions per account (4, 8), and - for the stamp protocol - the commit method (prevalidate
 * 1: per transaction with pre-validation; 3: group commit) and, when every transfer of the
 * sample reads at most four accounts, the kernels specialised for it (max_reads 4, else 0);
 * the rest of *base is fixed. Every candidate runs once from host_init (NULL:
 * base->init_value), the best quarter `repeats` more times, and the fastest median wins.
 * out->best is *base with the winning shape and method.
 * ------------------------------------------------------------------------------------------ */
#define CSMV_TUNE_MAX_TRIALS 64
typedef struct csmv_tune_trial {
  uint32_t client_warps, ctas, version_depth, runs;
  int32_t status;             /* csmv_status of the candidate (e.g. does not fit)           */
  double tx_per_s;            /* committed tx/s of the sample (median over runs)            */
  double abort_rate;
  uint32_t prevalidate, max_reads;  /* the candidate's commit method and read specialisation */
} csmv_tune_trial;
typedef struct csmv_tune_result {
  csmv_bank_config best;
  uint32_t n_trials;
  csmv_tune_trial trials[CSMV_TUNE_MAX_TRIALS];
} csmv_tune_result;
csmv_status csmv_bank_autotune(const csmv_bank_config* base, const csmv_bank_stream* host_sample,
                               const int32_t* host_init, uint32_t repeats, csmv_tune_result* out);

/* The cache's autotuner: client warps per CTA (1, 2, 4, 8) x CTAs per SM (1, 2), the rest of
 * *base fixed (max_req at least the sample's size, logging off). Each candidate is a fresh
 * cache: host_fill (optional) runs first untimed, then host_sample once; the best quarter runs
 * the sample `repeats` more times and the fastest median kernel time wins. Trials report
 * requests/s in tx_per_s and version_depth 2. out->best is *base with the winning shape. */
typedef struct csmv_memcd_tune_result {
  csmv_memcd_config best;
  uint32_t n_trials;
  csmv_tune_trial trials[CSMV_TUNE_MAX_TRIALS];
} csmv_memcd_tune_result;
csmv_status csmv_memcd_autotune(const csmv_memcd_config* base, const csmv_memcd_batch* host_fill,
                                const csmv_memcd_batch* host_sample, uint32_t repeats,
                                csmv_memcd_tune_result* out);

/* ------------------------------------------------------------------------------------------
 * L2 atomic rates of the device (no counterpart in the reference): the bounds of the commit
 * path, which runs on L2 atomics and on chains of dependent L2 round trips (a contended lock
 * passes between warps through a few of them). Measured by the library's own kernels with CUDA
 * events: returning atomicAdds of a full grid on one word, and on pseudo-random words of a
 * 64 MB (L2-resident) buffer; and the latency of one dependent 64-bit CAS (one thread, a chain
 * of CASes on one word). Allocates and frees a 64 MB buffer.
 * ------------------------------------------------------------------------------------------ */
typedef struct csmv_atomic_rates {
  double same_word_per_s;  /* returning atomics per second on a single word                  */
  double spread_per_s;     /* returning atomics per second spread over L2                    */
  double cas_chain_ns;     /* latency of one dependent CAS (one L2 round trip)               */
  double kernel_ms;        /* device time of the measurement                                 */
} csmv_atomic_rates;
csmv_status csmv_measure_atomics(int32_t device, csmv_atomic_rates* out);

/* Page-locked host buffers for staging streams (the e2e path copies from pinned memory).
 * Replaces CUDA_DUAL_ALLOC's cudaMallocHost half (memcachedGPU/cuda_util.h:50-60). */
csmv_status csmv_pinned_alloc(size_t bytes, void** out);
void csmv_pinned_free(void* p);

/* Text of the last error on this thread (static storage). */
const char* csmv_last_error(void);
const char* csmv_status_str(csmv_status s);
int csmv_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* CSMV_H_ */
