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

#define CSMV_ABI_VERSION 1

typedef enum csmv_status {
  CSMV_OK = 0,
  CSMV_ERR_INVALID_ARG = 1,  /* a size, pointer or option is out of range                 */
  CSMV_ERR_CUDA = 2,         /* a CUDA runtime call failed (csmv_last_error has the text)   */
  CSMV_ERR_OOM = 3,          /* device or host allocation failed                            */
  CSMV_ERR_TIMEOUT = 4,      /* a bounded device wait ran out; the kernel returned early     */
  CSMV_ERR_CAPACITY = 5,     /* commit log / result buffers too small for the run           */
  CSMV_ERR_NO_DEVICE = 6,    /* no CUDA device, or the device is not sm_103                  */
  CSMV_ERR_STATE = 7         /* call order violated (e.g. run before load)                  */
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
  CSMV_BATCH_CLUSTER = 3 /* client warps of a thread-block cluster post to one server warp
                            through distributed shared memory                                  */
};

typedef struct csmv_bank_config {
  uint32_t n_accounts;
  int32_t init_value;          /* every account starts at this balance                        */
  uint32_t version_depth;      /* versions kept per account, 2..16                            */
  uint32_t ring_size;          /* commit-record ring entries, power of two, >= 64             */
  uint32_t client_warps;       /* client warps per CTA (1..31)                                */
  uint32_t ctas;               /* CTAs; 0 = as many as fit co-resident on the GPU             */
  uint32_t cluster_size;       /* CTAs per cluster for CSMV_BATCH_CLUSTER (2..8)               */
  uint32_t validate;           /* CSMV_VALIDATE_*                                             */
  uint32_t writeback;          /* CSMV_WRITEBACK_*                                            */
  uint32_t batch;              /* CSMV_BATCH_*                                                */
  uint32_t prevalidate;        /* 1 = intra-warp pre-validation (batchedAtrInsert)             */
  uint32_t log_commits;        /* 1 = keep the per-ts commit log and per-txn outcomes         */
  uint32_t max_txn;            /* largest stream a run may carry (sizes the logs)             */
  uint32_t spin_limit_log2;    /* bounded waits give up after 2^this polls (default 26)       */
  int32_t device;
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

/* Device pointers of the engine's stream-input buffers (capacity max_txn / n_addr_cap) so a
 * caller can stage input itself and call csmv_bank_run_device. */
csmv_status csmv_bank_device_info(csmv_bank_t* h, int* n_sms, int* ctas, int* threads_per_cta,
                                  size_t* device_bytes);

void csmv_bank_destroy(csmv_bank_t* h);

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
