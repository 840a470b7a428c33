// refapi_test.cu - a bank client written in the reference's style against include/csmv_ref_api.cuh
// (the reference's device API signatures on this project's version store), part of the
// device-test library. The client loop follows the reference's structure
// (csmv_optimizations/batchedAtrInsert/csmv_sh/exe.cu:128-269): per warp, a round that is
// read-only or update as a whole; per attempt TXBegin, the reads (TXRead / TXReadOnly), the
// writes (TXWrite), then for update rounds TXPreValidation, TXAddToRecord and TXWriteBack called
// by the whole warp, and a retry while any lane of the warp still has to commit
// (do { ... } while (vote_ballot(retry))). Its transactions come from a stream (include/csmv.h
// format) instead of an in-kernel random generator, and every commit is logged (commit
// timestamp -> transaction), so a run replays exactly in the CPU oracle. The commit decisions are
// the API's; nothing here validates, locks or orders anything by itself.
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../../include/csmv.h"
#include "../../../include/csmv_ref_api.cuh"

namespace {

constexpr uint32_t kFull = 0xFFFFFFFFu;
constexpr uint32_t kSnap = 0x80000000u;

__global__ void ref_style_bank_client(VertionedDataItem* data, readSet* rs, writeSet* ws,
                                      TMmetadata* meta, TXRecord* records, Statistics* stats,
                                      time_rate* times, const uint32_t* op, const uint32_t* off,
                                      const uint32_t* addr, uint32_t n_rounds,
                                      uint32_t* round_cursor, uint32_t* log_txn,
                                      uint32_t log_cap, uint32_t* outcome, int32_t* result,
                                      uint32_t* failures) {
  const uint tid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint lane = threadIdx.x & 31u;
  for (;;) {
    uint g = 0;
    if (lane == 0) g = atomicAdd(round_cursor, 1u);
    g = __shfl_sync(kFull, g, 0);
    if (g >= n_rounds) break;  // warp-uniform
    const uint t = g * 32u + lane;
    const uint o = op[t], kind = CSMV_OP_KIND(o), nr = CSMV_OP_NREADS(o);
    const bool read_only = __shfl_sync(kFull, kind, 0) == CSMV_KIND_READONLY;  // per warp
    bool retry = true;
    uint32_t attempts = 0;
    do {
      const uint timestamp = TXBegin(tid, ws, rs);
      bool isAborted = false;
      int v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      if (read_only) {
        uint32_t sum = 0;
        for (uint k = 0; k < nr && retry && !isAborted; k++)
          sum += (uint32_t)TXReadOnly(data, (int)addr[off[t] + k], timestamp, rs, ws, tid, &isAborted);
        if (retry && !isAborted) {  // a read-only transaction commits at its snapshot
          outcome[t] = timestamp | kSnap;
          result[t] = (int32_t)sum;
          atomicAdd(&stats->nbCommits, 1);
          retry = false;
        } else if (retry) {
          atomicAdd(&stats->nbAbortsDataAge, 1);
        }
      } else {
        for (uint k = 0; k < nr && k < 8 && retry && !isAborted; k++)
          v[k] = TXRead(data, (int)addr[off[t] + k], timestamp, rs, ws, tid, &isAborted);
        bool writes = false;
        if (retry && !isAborted) {  // the transfer of include/csmv.h
          uint32_t acc = CSMV_OP_AMT0(o) - 1u;
          for (uint k = 2; k < nr && k < 8; k++) acc += (uint32_t)v[k];
          const uint32_t amt = 1u + acc % CSMV_OP_AMOD(o);
          if (kind == CSMV_KIND_TRANSFER_ALWAYS || v[0] >= (int32_t)amt) {
            TXWrite(data, (int)((uint32_t)v[0] - amt), (int)addr[off[t]], ws, tid);
            TXWrite(data, (int)((uint32_t)v[1] + amt), (int)addr[off[t] + 1], ws, tid);
            writes = true;
          } else {  // funds short: it commits without writes, at its snapshot
            outcome[t] = timestamp | kSnap;
            result[t] = 0;
            atomicAdd(&stats->nbCommits, 1);
            retry = false;
          }
        }
        if (retry && isAborted) atomicAdd(&stats->nbAbortsDataAge, 1);
        // commit process, called by the whole warp
        const bool pre = TXPreValidation(tid, rs, ws);
        const bool live = retry && writes && !isAborted && pre;
        if (retry && writes && !isAborted && !pre) atomicAdd(&stats->nbAbortsPreValid, 1);
        const int ts = TXAddToRecord(meta, records, rs, ws, stats, times,
                                     live ? (int)timestamp : -1, (int)tid);
        TXWriteBack(ts, data, ws[tid]);
        if (ts > 0) {
          if ((uint32_t)ts - 1u < log_cap)
            log_txn[ts - 1] = t;
          else
            atomicExch(failures, 1u);
          outcome[t] = (uint32_t)ts;
          result[t] = 0;
          retry = false;
        }
      }
      if (++attempts > (1u << 16)) {  // a round that never commits is reported, not retried forever
        if (lane == 0) atomicExch(failures, 2u);
        break;
      }
    } while (__ballot_sync(kFull, retry) != 0u);
  }
}

template <class T>
T* dev_copy(const T* host, size_t n) {
  T* d = nullptr;
  if (cudaMalloc(&d, n * sizeof(T) + 16) != cudaSuccess) return nullptr;
  if (host) cudaMemcpy(d, host, n * sizeof(T), cudaMemcpyHostToDevice);
  return d;
}

}  // namespace

extern "C" {

// Runs a stream through the reference-style client on blocks x threads threads (a multiple of 32,
// all co-resident); host buffers in and out. slots_out: n_accounts x CSMV_REF_DEPTH packed
// versions; log_out[ts-1] = transaction of commit ts; *final_ts = the clock after the run.
// Returns 0, or 1 (CUDA error), 2 (a wait of the API ran out), 3 (log too small), 4 (a round
// never committed).
int csmv_devtest_refapi_bank(const uint32_t* op, const uint32_t* off, const uint32_t* addr,
                             uint32_t n_txn, uint64_t n_addr, uint32_t n_accounts,
                             const int32_t* init, uint32_t blocks, uint32_t threads,
                             uint64_t* slots_out, uint32_t* log_out, uint32_t log_cap,
                             uint32_t* outcome_out, int32_t* result_out, uint32_t* final_ts) {
  std::vector<VertionedDataItem> items(n_accounts);
  for (uint32_t i = 0; i < n_accounts; i++) items[i] = csmv_ref_init_item(init[i]);
  const uint32_t n_threads = blocks * threads;
  VertionedDataItem* d_data = dev_copy(items.data(), n_accounts);
  readSet* d_rs = dev_copy<readSet>(nullptr, n_threads);
  writeSet* d_ws = dev_copy<writeSet>(nullptr, n_threads);
  TMmetadata* d_meta = dev_copy<TMmetadata>(nullptr, 1);
  TXRecord* d_rec = dev_copy<TXRecord>(nullptr, CSMV_REF_RECORDS);
  Statistics* d_stats = dev_copy<Statistics>(nullptr, 1);
  time_rate* d_times = dev_copy<time_rate>(nullptr, n_threads);
  uint32_t* d_op = dev_copy(op, n_txn);
  uint32_t* d_off = dev_copy(off, n_txn);
  uint32_t* d_addr = dev_copy(addr, n_addr);
  uint32_t* d_cur = dev_copy<uint32_t>(nullptr, 2);
  uint32_t* d_log = dev_copy<uint32_t>(nullptr, log_cap);
  uint32_t* d_out = dev_copy<uint32_t>(nullptr, n_txn);
  int32_t* d_res = dev_copy<int32_t>(nullptr, n_txn);
  int rc = 0;
  if (!d_data || !d_rs || !d_ws || !d_meta || !d_rec || !d_stats || !d_times || !d_op || !d_off ||
      !d_addr || !d_cur || !d_log || !d_out || !d_res) {
    rc = 1;
  } else {
    cudaMemset(d_rs, 0, (size_t)n_threads * sizeof(readSet));
    cudaMemset(d_ws, 0, (size_t)n_threads * sizeof(writeSet));
    cudaMemset(d_meta, 0, sizeof(TMmetadata));
    cudaMemset(d_rec, 0, (size_t)CSMV_REF_RECORDS * sizeof(TXRecord));
    cudaMemset(d_stats, 0, sizeof(Statistics));
    cudaMemset(d_cur, 0, 8);
    cudaMemset(d_log, 0xFF, (size_t)log_cap * 4);
    const uint32_t zero = 0;
    cudaMemcpyToSymbol(csmv_ref_clock, &zero, 4);
    cudaMemcpyToSymbol(csmv_ref_error, &zero, 4);
    ref_style_bank_client<<<blocks, threads>>>(d_data, d_rs, d_ws, d_meta, d_rec, d_stats, d_times,
                                               d_op, d_off, d_addr, n_txn / 32, d_cur, d_log,
                                               log_cap, d_out, d_res, d_cur + 1);
    if (cudaDeviceSynchronize() != cudaSuccess) rc = 1;
    uint32_t fails = 0, err = 0;
    cudaMemcpy(&fails, d_cur + 1, 4, cudaMemcpyDeviceToHost);
    cudaMemcpyFromSymbol(&err, csmv_ref_error, 4);
    cudaMemcpyFromSymbol(final_ts, csmv_ref_clock, 4);
    if (!rc && err) rc = 2;
    if (!rc && fails == 1) rc = 3;
    if (!rc && fails == 2) rc = 4;
    cudaMemcpy(slots_out, d_data, (size_t)n_accounts * sizeof(VertionedDataItem),
               cudaMemcpyDeviceToHost);
    cudaMemcpy(log_out, d_log, (size_t)log_cap * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(outcome_out, d_out, (size_t)n_txn * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(result_out, d_res, (size_t)n_txn * 4, cudaMemcpyDeviceToHost);
  }
  void* bufs[] = {d_data, d_rs, d_ws, d_meta, d_rec, d_stats, d_times, d_op,
                  d_off,  d_addr, d_cur, d_log, d_out, d_res};
  for (void* b : bufs) cudaFree(b);
  return rc;
}

int csmv_devtest_refapi_depth(void) { return CSMV_REF_DEPTH; }

}  // extern "C"
