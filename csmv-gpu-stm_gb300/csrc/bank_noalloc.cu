// bank_noalloc.cu - a bank run that allocates no device memory (csmv_bank_run_noalloc).
//
// The engine behind csmv_bank_create allocates its version store, commit words, completion
// bitmap and commit log with cudaMalloc when a handle is made. Some callers cannot allow that:
// a host that hands the library a fixed memory budget and forbids allocation after start-up, a
// process whose device memory is owned by another allocator (a framework's caching pool), or a
// latency-critical loop where an allocation could block or fail. For them this entry point runs
// the same commit kernel (stamp protocol, CTA-batched timestamps, client write-back,
// pre-validation, version depth 4) with all of its scratch in the file-scope device array
// below. The caller passes only inputs and outputs, all in device memory.
//
// Limits: at most CSMV_NOALLOC_MAX_ACCOUNTS accounts and CSMV_NOALLOC_MAX_TXN transactions per
// call, and at most kLogCap = 8 x CSMV_NOALLOC_MAX_TXN commit timestamps (a transaction that
// fails validation after drawing a timestamp uses one too); past that the kernel stops and the
// call returns CSMV_ERR_CAPACITY. The array is kNoAllocScratchBytes (about 4.8 MiB) and every GPU
// that loads the library holds it until the process exits. Calls share the array, so two calls
// that overlap on the GPU (on different streams, or from different host threads) race and
// corrupt each other's results: serialise them. The first call on a device looks up the
// array's device address (a host-side reference to a __device__ array is not a device address)
// and sets the kernel's shared-memory limit, and caches both; make that first call before any
// stream capture. A cudaDeviceReset unloads the module and voids the cache: a process that
// resets a device must not call this entry point on it afterwards. The caller's current device
// is restored before the call returns.
#include <chrono>
#include <cstring>
#include <mutex>

#include "bank_kernel.cuh"
#include "common.h"

using namespace csmv;

namespace {

constexpr int kDepth = 4, kMaxR = 8, kMaxW = 2;
constexpr uint32_t kDoneWords = 1u << 14;  // 2^19 timestamps in flight
constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kSlotsOff = 0;
constexpr size_t kCwOff = kSlotsOff + align256((size_t)CSMV_NOALLOC_MAX_ACCOUNTS * kDepth * 8);
constexpr size_t kDoneOff = kCwOff + align256((size_t)CSMV_NOALLOC_MAX_ACCOUNTS * 8);
constexpr size_t kLogOff = kDoneOff + align256((size_t)kDoneWords * 4);
constexpr uint32_t kLogCap = 8u * CSMV_NOALLOC_MAX_TXN;  // timestamps incl. failed validations
constexpr size_t kSyncOff = kLogOff + align256((size_t)kLogCap * 4);
constexpr size_t kStatsOff = kSyncOff + align256(sizeof(GlobalSync));
constexpr size_t kNoAllocScratchBytes = kStatsOff + align256(ST_COUNT * 8);

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
struct DeviceSetup {
  bool ready = false;
  unsigned char* scratch = nullptr;  // device address of g_noalloc_scratch on this device
  int n_sms = 0;
};
DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_mu;

auto kKernel = bank_kernel<kDepth, kMaxR, kMaxW>;

csmv_status setup_device(int device, DeviceSetup** out) {
  std::lock_guard<std::mutex> lock(g_setup_mu);
  DeviceSetup& s = g_setup[device];
  if (!s.ready) {
    int n_sms = 0;
    csmv_status st = check_device(device, &n_sms);
    if (st != CSMV_OK) return st;
    CSMV_CUDA(cudaSetDevice(device));
    void* p = nullptr;
    CSMV_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    CSMV_CUDA(cudaFuncSetAttribute((const void*)kKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)cta_shared_bytes<kMaxR, kMaxW>(kMaxClientWarps)));
    s.scratch = static_cast<unsigned char*>(p);
    s.n_sms = n_sms;
    s.ready = true;
  }
  *out = &s;
  return CSMV_OK;
}

// Version store from the caller's initial values: value at ts 0, the other slots empty.
__global__ void noalloc_init_slots(unsigned long long* slots, const int32_t* init, uint32_t n) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n * kDepth; i += gridDim.x * blockDim.x)
    slots[i] = (i % kDepth == 0) ? (unsigned long long)(uint32_t)init[i / kDepth]
                                 : ((unsigned long long)kEmptyTs << 32);
}

// Latest value of every account (the version with the largest timestamp).
__global__ void noalloc_final_values(const unsigned long long* slots, int32_t* values, uint32_t n) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    uint32_t best = 0;
    int32_t v = 0;
    bool any = false;
    for (int d = 0; d < kDepth; d++) {
      const unsigned long long s = slots[(size_t)i * kDepth + d];
      const uint32_t ts = version_ts(s);
      if (ts != kEmptyTs && (!any || ts > best)) {
        any = true;
        best = ts;
        v = version_val(s);
      }
    }
    values[i] = v;
  }
}

// Restores the caller's current device when the call returns.
struct DeviceRestore {
  int prev = -1;
  DeviceRestore() {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
  }
  ~DeviceRestore() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

csmv_status run_noalloc(int32_t device, void* cuda_stream, uint32_t n_accounts,
                        const int32_t* dev_init_values, const csmv_bank_stream* stream_desc,
                        uint32_t client_warps, uint32_t ctas, int32_t* dev_values,
                        uint32_t* dev_outcome, int32_t* dev_result, csmv_stats* out);

}  // namespace

extern "C" csmv_status csmv_bank_run_noalloc(int32_t device, void* cuda_stream,
                                             uint32_t n_accounts, const int32_t* dev_init_values,
                                             const csmv_bank_stream* stream_desc,
                                             uint32_t client_warps, uint32_t ctas,
                                             int32_t* dev_values, uint32_t* dev_outcome,
                                             int32_t* dev_result, csmv_stats* out) {
  DeviceRestore restore;
  return run_noalloc(device, cuda_stream, n_accounts, dev_init_values, stream_desc, client_warps,
                     ctas, dev_values, dev_outcome, dev_result, out);
}

namespace {

csmv_status run_noalloc(int32_t device, void* cuda_stream, uint32_t n_accounts,
                        const int32_t* dev_init_values, const csmv_bank_stream* stream_desc,
                        uint32_t client_warps, uint32_t ctas, int32_t* dev_values,
                        uint32_t* dev_outcome, int32_t* dev_result, csmv_stats* out) {
  auto bad = [](const char* why) {
    set_error("csmv_bank_run_noalloc: %s", why);
    return CSMV_ERR_INVALID_ARG;
  };
  const csmv_bank_stream* dev_stream = stream_desc;  // a host struct holding device arrays
  if (device < 0 || device >= kMaxDevices) return bad("device out of range");
  if (!dev_init_values || !dev_stream || !dev_values || !dev_outcome || !dev_result)
    return bad("null pointer");
  if (!dev_stream->op || !dev_stream->off || !dev_stream->addr) return bad("null stream array");
  if (dev_stream->split_round || dev_stream->deferred_warps)
    return bad("the deferred queue (split_round, deferred_warps) is not available here");
  if (dev_stream->txn_waits) return bad("txn_waits is not produced here (no group commit)");
  if (dev_stream->lock_last) return bad("lock_last orders group commit's locks (no group commit here)");
  if (dev_stream->lane_start) return bad("the deferred queue (lane_start) is not available here");
  if (n_accounts < 2) return bad("n_accounts < 2");
  if (n_accounts > CSMV_NOALLOC_MAX_ACCOUNTS) {
    set_error("csmv_bank_run_noalloc: %u accounts exceed the fixed scratch limit of %u", n_accounts,
              (unsigned)CSMV_NOALLOC_MAX_ACCOUNTS);
    return CSMV_ERR_CAPACITY;
  }
  if (dev_stream->n_txn == 0 || dev_stream->n_txn % 32) return bad("n_txn must be a positive multiple of 32");
  if (dev_stream->n_txn > CSMV_NOALLOC_MAX_TXN) {
    set_error("csmv_bank_run_noalloc: %u transactions exceed the fixed scratch limit of %u",
              dev_stream->n_txn, (unsigned)CSMV_NOALLOC_MAX_TXN);
    return CSMV_ERR_CAPACITY;
  }
  if (client_warps < 1 || client_warps > (uint32_t)kMaxClientWarps) return bad("client_warps must be 1..15");
  DeviceSetup* ds = nullptr;
  csmv_status st = setup_device(device, &ds);
  if (st != CSMV_OK) return st;
  CSMV_CUDA(cudaSetDevice(device));
  cudaStream_t stream = static_cast<cudaStream_t>(cuda_stream);
  const int threads = (int)(client_warps + 1) * 32;
  const size_t smem = cta_shared_bytes<kMaxR, kMaxW>(client_warps);
  int per_sm = 0;
  CSMV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kKernel, threads, smem));
  const int max_ctas = per_sm * ds->n_sms;
  const int grid = ctas ? (int)ctas : max_ctas;
  if (grid < 1 || grid > max_ctas) {
    set_error("csmv_bank_run_noalloc: %d CTAs requested, %d can be co-resident", grid, max_ctas);
    return CSMV_ERR_INVALID_ARG;
  }
  auto t0 = std::chrono::steady_clock::now();
  unsigned char* base = ds->scratch;
  auto* slots = reinterpret_cast<unsigned long long*>(base + kSlotsOff);
  auto* cw = reinterpret_cast<unsigned long long*>(base + kCwOff);
  auto* done = reinterpret_cast<uint32_t*>(base + kDoneOff);
  auto* log_txn = reinterpret_cast<uint32_t*>(base + kLogOff);
  auto* gs = reinterpret_cast<GlobalSync*>(base + kSyncOff);
  auto* stats = reinterpret_cast<unsigned long long*>(base + kStatsOff);
  // the array keeps the previous call's contents: everything the kernel expects at zero is
  // cleared here, and the version store is rebuilt from the caller's initial values
  CSMV_CUDA(cudaMemsetAsync(cw, 0, (size_t)n_accounts * 8, stream));
  CSMV_CUDA(cudaMemsetAsync(done, 0, (size_t)kDoneWords * 4, stream));
  CSMV_CUDA(cudaMemsetAsync(gs, 0, sizeof(GlobalSync), stream));
  CSMV_CUDA(cudaMemsetAsync(stats, 0, ST_COUNT * 8, stream));
  noalloc_init_slots<<<ds->n_sms * 2, 256, 0, stream>>>(slots, dev_init_values, n_accounts);
  CSMV_CUDA(cudaGetLastError());
  BankParams p{};
  p.op = dev_stream->op;
  p.off = dev_stream->off;
  p.addr = dev_stream->addr;
  p.n_rounds = dev_stream->n_txn / 32;
  p.n_items = n_accounts;
  p.slots = slots;
  p.cw = cw;
  p.ring = nullptr;  // the stamp protocol keeps no record ring
  p.ring_mask = 0;
  p.done = done;
  p.done_mask = kDoneWords - 1;
  p.gs = gs;
  p.log_txn = log_txn;
  p.outcome = dev_outcome;
  p.result = dev_result;
  p.stats = stats;
  p.log = 1;
  p.log_base = 0;
  p.log_cap = kLogCap;
  p.nc = client_warps;
  p.validate = CSMV_VALIDATE_STAMP;
  p.writeback = CSMV_WRITEBACK_CLIENT;
  p.batch = CSMV_BATCH_CTA;
  p.prevalidate = 1;
  p.spin_log2 = 24;
  p.txn_aborts = dev_stream->txn_aborts;  // device memory, like op
  p.backoff = dev_stream->backoff;
  void* args[] = {&p};
  CSMV_CUDA(cudaLaunchCooperativeKernel((const void*)kKernel, dim3(grid), dim3(threads), args, smem,
                                        stream));
  noalloc_final_values<<<ds->n_sms * 2, 256, 0, stream>>>(slots, dev_values, n_accounts);
  CSMV_CUDA(cudaGetLastError());
  unsigned long long h_stats[ST_COUNT];
  GlobalSync h_gs;
  CSMV_CUDA(cudaMemcpyAsync(h_stats, stats, sizeof(h_stats), cudaMemcpyDeviceToHost, stream));
  CSMV_CUDA(cudaMemcpyAsync(&h_gs, gs, sizeof(h_gs), cudaMemcpyDeviceToHost, stream));
  CSMV_CUDA(cudaStreamSynchronize(stream));
  if (out) {
    std::memset(out, 0, sizeof(*out));
    out->commits_update = h_stats[ST_COMMIT_UPDATE];
    out->commits_readonly = h_stats[ST_COMMIT_RO];
    out->commits_nowrite = h_stats[ST_COMMIT_NOWRITE];
    out->aborts_data_age = h_stats[ST_ABORT_DATA_AGE];
    out->aborts_read_write = h_stats[ST_ABORT_READ_WRITE];
    out->aborts_prevalid = h_stats[ST_ABORT_PREVALID];
    out->aborts_write_write = h_stats[ST_ABORT_WRITE_WRITE];
    out->sections = h_stats[ST_SECTIONS];
    out->rounds = h_stats[ST_ROUNDS];
    out->final_ts = h_gs.ts_next;
    out->error = h_gs.error;
    out->total_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  if (h_gs.error == ERR_CAPACITY) {
    set_error("csmv_bank_run_noalloc: the run used more than the fixed scratch's %u commit "
              "timestamps (aborted attempts draw timestamps too)",
              kLogCap);
    return CSMV_ERR_CAPACITY;
  }
  if (h_gs.error) {
    set_error("csmv_bank_run_noalloc: device error %u", h_gs.error);
    return h_gs.error == ERR_DATA ? CSMV_ERR_INVALID_ARG : CSMV_ERR_TIMEOUT;
  }
  return CSMV_OK;
}

}  // namespace
