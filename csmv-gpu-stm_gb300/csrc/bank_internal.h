// bank_internal.h - the bank handle and the run helpers shared by the bank engine's translation
// units (bank_engine.cu: create / load / concurrent and serial runs; bank_flow.cu: the dataflow
// lane). Not part of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include "bank_kernel.cuh"
#include "common.h"

namespace csmv {

constexpr uint32_t kDoneWords = 1u << 16;  // 2^21 timestamps in flight at most
using KernelFn = void (*)(BankParams);

// kernels for transfers of at most four reads (bank_engine_r4.cu)
KernelFn pick_kernel_r4(uint32_t depth);
KernelFn pick_cluster_r4(uint32_t depth);
size_t cta_shared_bytes_r4(uint32_t n_mail);

struct FlowScratch;                                        // bank_flow.cu
void flow_scratch_free(FlowScratch* f);                    // frees the dataflow lane's buffers
csmv_status flow_scratch_reset(FlowScratch* f, cudaStream_t s);  // zeroes its per-account counts

}  // namespace csmv

struct csmv_bank_t {
  csmv_bank_config cfg{};
  int n_sms = 0, ctas = 0, threads = 0;
  size_t smem = 0, device_bytes = 0;
  csmv::KernelFn kernel = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  unsigned long long* slots = nullptr;
  unsigned long long* cw = nullptr;
  uint4* ring = nullptr;
  uint32_t* done = nullptr;
  uint32_t log_cap = 0;
  csmv::GlobalSync* gs = nullptr;
  uint32_t* log_txn = nullptr;
  uint32_t* outcome = nullptr;
  int32_t* result = nullptr;
  unsigned long long* stats = nullptr;
  uint32_t* d_op = nullptr;
  uint32_t* d_off = nullptr;
  uint32_t* d_addr = nullptr;
  uint32_t* d_aborts = nullptr;
  uint32_t* d_backoff = nullptr;  // host-buffer runs: the stream's backoff array, copied in
  uint32_t* d_waits = nullptr;    // host-buffer runs: per-transaction lock waits, copied out
  uint8_t* d_lock_last = nullptr; // host-buffer runs: the stream's heat classes, copied in
  uint32_t* d_lanes = nullptr;    // host-buffer runs: the stream's lanes of the deferred queue
  uint32_t* grp = nullptr;        // group-end bitmap of the last run (log_commits)
  uint32_t* tk = nullptr;         // group commit: per account {next ticket, ticket served}
  uint32_t grp_words = 0;
  bool last_grouped = false;      // the last run was a group-commit run of the engine
  uint64_t addr_cap = 0;
  bool loaded = false;
  uint32_t last_final_ts = 0, last_n_txn = 0, run_base_ts = 0;
  csmv::FlowScratch* flow = nullptr;  // dataflow lane buffers, made on its first run
};

namespace csmv {

// Checks a stream against the handle (sizes, split round).
csmv_status check_stream(const csmv_bank_t* h, const csmv_bank_stream* s);
// Kernel parameters of a run of n_txn transactions over the handle's state.
BankParams bank_params(const csmv_bank_t* h, const uint32_t* op, const uint32_t* off,
                       const uint32_t* addr, uint32_t n_txn, uint32_t* txn_aborts);
// Resets the run cursors, error word and statistics, and records the start event.
csmv_status bank_begin_run(csmv_bank_t* h);
// Records the end event, waits for the stream, reads statistics and the commit cursor into
// *out and advances the handle's log window; maps a device error to a status.
csmv_status bank_end_run(csmv_bank_t* h, uint32_t n_txn, csmv_stats* out);

}  // namespace csmv
