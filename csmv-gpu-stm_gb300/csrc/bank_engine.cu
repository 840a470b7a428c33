// bank_engine.cu - C-ABI host side of the bank commit engine (include/csmv.h).
//
// Data layout in HBM (all item-major, allocated once per handle):
//   slots  n_accounts * depth * 8 B   packed (ts << 32 | value) versions; depth 4 = one sector
//   cw     n_accounts * 8 B           commit word: stamp (ts of the last committed writer) and
//                                      write-lock owner, one 8-byte word per account
//   ring   ring_size * 16 B           commit records {ts, n_writes, w0, w1}
//   done   256 KB                     completion bitmap, one bit per commit timestamp
//   logs   8*max_txn*4 + max_txn*8 B  log_txn[ts-1] (holes included), outcome[txn], result[txn]
//   sync   6 x 128 B lines            turn / ticket / clock / ts cursor / round cursor / error
#include <chrono>
#include <cstring>
#include <vector>

#include "bank_internal.h"

using namespace csmv;

namespace {
constexpr int kMaxR = 8;
constexpr int kMaxW = 2;

KernelFn pick_kernel(uint32_t depth) {
  switch (depth) {
    case 2: return bank_kernel<2, kMaxR, kMaxW>;
    case 4: return bank_kernel<4, kMaxR, kMaxW>;
    case 8: return bank_kernel<8, kMaxR, kMaxW>;
    case 16: return bank_kernel<16, kMaxR, kMaxW>;
    default: return nullptr;
  }
}

KernelFn pick_cluster(uint32_t depth) {
  switch (depth) {
    case 2: return bank_cluster_kernel<2, kMaxR, kMaxW>;
    case 4: return bank_cluster_kernel<4, kMaxR, kMaxW>;
    case 8: return bank_cluster_kernel<8, kMaxR, kMaxW>;
    case 16: return bank_cluster_kernel<16, kMaxR, kMaxW>;
    default: return nullptr;
  }
}

size_t serial_smem(uint32_t depth) {
  switch (depth) {
    case 2: return serial_smem_bytes<2, kMaxR>();
    case 4: return serial_smem_bytes<4, kMaxR>();
    case 8: return serial_smem_bytes<8, kMaxR>();
    case 16: return serial_smem_bytes<16, kMaxR>();
    default: return 0;
  }
}

KernelFn pick_serial(uint32_t depth) {
  switch (depth) {
    case 2: return bank_serial_kernel<2, kMaxR>;
    case 4: return bank_serial_kernel<4, kMaxR>;
    case 8: return bank_serial_kernel<8, kMaxR>;
    case 16: return bank_serial_kernel<16, kMaxR>;
    default: return nullptr;
  }
}
}  // namespace

extern "C" void csmv_bank_config_default(csmv_bank_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->n_accounts = 4096;
  c->init_value = 1000;
  c->version_depth = 4;
  c->ring_size = 1u << 16;
  c->client_warps = 15;
  c->ctas = 0;
  c->cluster_size = 2;
  c->validate = CSMV_VALIDATE_STAMP;
  c->writeback = CSMV_WRITEBACK_CLIENT;
  c->batch = CSMV_BATCH_CTA;
  c->prevalidate = 1;
  c->log_commits = 1;
  c->max_txn = 1u << 20;
  c->spin_limit_log2 = 24;
  c->device = 0;
  c->group_grace = 4;
  c->group_read_wait = 8;
}

static csmv_status validate_config(const csmv_bank_config* c) {
  auto bad = [](const char* why) {
    set_error("invalid bank config: %s", why);
    return CSMV_ERR_INVALID_ARG;
  };
  if (!c) return bad("null");
  if (c->n_accounts < 2) return bad("n_accounts < 2");
  if (c->n_accounts >= 0x80000000u) return bad("n_accounts >= 2^31");
  if (!pick_kernel(c->version_depth)) return bad("version_depth must be 2, 4, 8 or 16");
  if (c->ring_size < 64 || (c->ring_size & (c->ring_size - 1))) return bad("ring_size");
  if (c->client_warps < 1 || c->client_warps > (uint32_t)kMaxClientWarps) return bad("client_warps");
  if (c->validate > CSMV_VALIDATE_RING_LANE) return bad("validate");
  if (c->writeback > CSMV_WRITEBACK_SERVER) return bad("writeback");
  if (c->batch > CSMV_BATCH_CLUSTER) return bad("batch");
  if (c->batch == CSMV_BATCH_CLUSTER) {
    if (c->validate != CSMV_VALIDATE_STAMP) return bad("cluster batching runs the stamp protocol");
    if (c->cluster_size != 2 && c->cluster_size != 4 && c->cluster_size != 8)
      return bad("cluster_size must be 2, 4 or 8");
    if (c->client_warps * c->cluster_size > 32)
      return bad("client_warps x cluster_size must be <= 32 (one server lane per mailbox)");
  }
  if (c->prevalidate > 3) return bad("prevalidate must be 0, 1, 2 or 3");
  if (c->prevalidate >= 2 && c->validate != CSMV_VALIDATE_STAMP)
    return bad("intra-warp chaining and group commit run the stamp protocol");
  if (c->validate != CSMV_VALIDATE_STAMP && c->batch == CSMV_BATCH_LANE &&
      c->writeback != CSMV_WRITEBACK_SERVER)
    return bad("per-transaction sections need server write-back");
  if (c->max_txn == 0 || c->max_txn % 32) return bad("max_txn must be a positive multiple of 32");
  if (c->spin_limit_log2 < 10 || c->spin_limit_log2 > 30) return bad("spin_limit_log2");
  if (c->flow_warps > 16) return bad("flow_warps must be 0 (default) or 1..16");
  if (c->max_reads != 0 && c->max_reads != 4 && c->max_reads != 8)
    return bad("max_reads must be 0 (8), 4 or 8");
  return CSMV_OK;
}

static void free_all(csmv_bank_t* h) {
  cudaFree(h->slots);
  cudaFree(h->cw);
  cudaFree(h->ring);
  cudaFree(h->done);
  cudaFree(h->gs);
  cudaFree(h->log_txn);
  cudaFree(h->outcome);
  cudaFree(h->result);
  cudaFree(h->stats);
  cudaFree(h->d_op);
  cudaFree(h->d_off);
  cudaFree(h->d_addr);
  cudaFree(h->d_aborts);
  cudaFree(h->d_backoff);
  cudaFree(h->d_waits);
  cudaFree(h->d_lock_last);
  cudaFree(h->d_lanes);
  cudaFree(h->grp);
  cudaFree(h->tk);
  flow_scratch_free(h->flow);
  h->flow = nullptr;
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->stream) cudaStreamDestroy(h->stream);
}

extern "C" csmv_status csmv_bank_create(const csmv_bank_config* cfg, csmv_bank_t** out) {
  if (!out) return CSMV_ERR_INVALID_ARG;
  *out = nullptr;
  csmv_status st = validate_config(cfg);
  if (st != CSMV_OK) return st;
  int n_sms = 0;
  if ((st = check_device(cfg->device, &n_sms)) != CSMV_OK) return st;
  CSMV_CUDA(cudaSetDevice(cfg->device));
  int coop = 0;
  CSMV_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, cfg->device));
  if (!coop) {
    set_error("device does not support cooperative launch");
    return CSMV_ERR_NO_DEVICE;
  }
  csmv_bank_t* h = new csmv_bank_t;
  h->cfg = *cfg;
  h->n_sms = n_sms;
  const bool cluster = cfg->batch == CSMV_BATCH_CLUSTER;
  const bool r4 = cfg->max_reads == 4;
  if (r4)
    h->kernel = cluster ? pick_cluster_r4(cfg->version_depth) : pick_kernel_r4(cfg->version_depth);
  else
    h->kernel = cluster ? pick_cluster(cfg->version_depth) : pick_kernel(cfg->version_depth);
  h->threads = (int)(cfg->client_warps + 1) * 32;
  // cluster form: every CTA reserves the cluster's mailboxes; the leader's are used
  const uint32_t n_mail = cfg->client_warps * (cluster ? cfg->cluster_size : 1u);
  h->smem = r4 ? cta_shared_bytes_r4(n_mail) : cta_shared_bytes<kMaxR, kMaxW>(n_mail);
  if (cfg->prevalidate == 3)  // one group-commit table per client warp of the CTA
    h->smem = group_scratch_offset(h->smem) + cfg->client_warps * sizeof(GroupScratch);
  auto fail = [&](csmv_status s) {
    free_all(h);
    delete h;
    return s;
  };
  if ((st = cuda_status(cudaFuncSetAttribute((const void*)h->kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)h->smem),
                        "cudaFuncSetAttribute")) != CSMV_OK ||
      (st = cuda_status(cudaFuncSetAttribute((const void*)pick_serial(cfg->version_depth),
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)serial_smem(cfg->version_depth)),
                        "cudaFuncSetAttribute")) != CSMV_OK)
    return fail(st);
  int max_ctas = 0;
  if (cluster) {
    cudaLaunchConfig_t lc = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cfg->cluster_size;
    at[0].val.clusterDim.y = at[0].val.clusterDim.z = 1;
    lc.gridDim = dim3(cfg->cluster_size * (uint32_t)n_sms);
    lc.blockDim = dim3(h->threads);
    lc.dynamicSmemBytes = h->smem;
    lc.attrs = at;
    lc.numAttrs = 1;
    int clusters = 0;
    if ((st = cuda_status(cudaOccupancyMaxActiveClusters(&clusters, (const void*)h->kernel, &lc),
                          "cluster occupancy")) != CSMV_OK)
      return fail(st);
    max_ctas = clusters * (int)cfg->cluster_size;
    if (cfg->ctas && cfg->ctas % cfg->cluster_size) {
      set_error("ctas must be a multiple of cluster_size");
      return fail(CSMV_ERR_INVALID_ARG);
    }
  } else {
    int per_sm = 0;
    if ((st = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, h->kernel,
                                                                         h->threads, h->smem),
                          "occupancy")) != CSMV_OK)
      return fail(st);
    max_ctas = per_sm * n_sms;
  }
  if (max_ctas <= 0) {
    set_error("kernel does not fit on an SM (threads %d, smem %zu)", h->threads, h->smem);
    return fail(CSMV_ERR_INVALID_ARG);
  }
  h->ctas = cfg->ctas ? (int)cfg->ctas : max_ctas;
  if (h->ctas > max_ctas) {
    set_error("%d CTAs requested, only %d can be co-resident", h->ctas, max_ctas);
    return fail(CSMV_ERR_INVALID_ARG);
  }
  const size_t n = cfg->n_accounts, D = cfg->version_depth;
  h->log_cap = cfg->log_commits ? (cfg->max_txn > 0x1FFFFFFFu ? 0xFFFFFFFFu : cfg->max_txn * 8u) : 1u;
  struct {
    void** p;
    size_t bytes;
  } allocs[] = {
      {(void**)&h->slots, n * D * 8},       {(void**)&h->cw, n * 8},
      {(void**)&h->ring, (size_t)cfg->ring_size * 16}, {(void**)&h->gs, sizeof(GlobalSync)},
      {(void**)&h->done, (size_t)kDoneWords * 4},
      {(void**)&h->log_txn, (size_t)h->log_cap * 4}, {(void**)&h->outcome, (size_t)cfg->max_txn * 4},
      {(void**)&h->result, (size_t)cfg->max_txn * 4},  {(void**)&h->stats, ST_COUNT * 8},
      {(void**)&h->d_op, (size_t)cfg->max_txn * 4},    {(void**)&h->d_off, (size_t)cfg->max_txn * 4},
      {(void**)&h->d_aborts, (size_t)cfg->max_txn * 4},
      {(void**)&h->d_backoff, (size_t)cfg->max_txn * 4},
      {(void**)&h->d_waits, (size_t)cfg->max_txn * 4},
      {(void**)&h->grp, (size_t)((h->log_cap + 31u) / 32u) * 4},
      {(void**)&h->tk, n * 8},
  };
  h->grp_words = (h->log_cap + 31u) / 32u;
  for (auto& a : allocs) {
    if ((st = cuda_status(cudaMalloc(a.p, a.bytes), "cudaMalloc")) != CSMV_OK) return fail(st);
    h->device_bytes += a.bytes;
  }
  if ((st = cuda_status(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "stream")) != CSMV_OK ||
      (st = cuda_status(cudaEventCreate(&h->ev0), "event")) != CSMV_OK ||
      (st = cuda_status(cudaEventCreate(&h->ev1), "event")) != CSMV_OK)
    return fail(st);
  *out = h;
  return CSMV_OK;
}

extern "C" csmv_status csmv_bank_load(csmv_bank_t* h, const int32_t* host_values) {
  if (!h) return CSMV_ERR_INVALID_ARG;
  CSMV_CUDA(cudaSetDevice(h->cfg.device));
  const size_t n = h->cfg.n_accounts, D = h->cfg.version_depth;
  std::vector<unsigned long long> slots(n * D, 0xFFFFFFFFull << 32);
  for (size_t i = 0; i < n; i++)
    slots[i * D] = (uint32_t)(host_values ? host_values[i] : h->cfg.init_value);  // ts 0
  CSMV_CUDA(cudaMemcpyAsync(h->slots, slots.data(), n * D * 8, cudaMemcpyHostToDevice, h->stream));
  CSMV_CUDA(cudaMemsetAsync(h->cw, 0, n * 8, h->stream));
  CSMV_CUDA(cudaMemsetAsync(h->ring, 0, (size_t)h->cfg.ring_size * 16, h->stream));
  CSMV_CUDA(cudaMemsetAsync(h->done, 0, (size_t)kDoneWords * 4, h->stream));
  CSMV_CUDA(cudaMemsetAsync(h->gs, 0, sizeof(GlobalSync), h->stream));
  if (h->flow) {
    csmv_status st = flow_scratch_reset(h->flow, h->stream);
    if (st != CSMV_OK) return st;
  }
  CSMV_CUDA(cudaStreamSynchronize(h->stream));
  h->loaded = true;
  h->last_final_ts = 0;
  h->last_n_txn = 0;
  return CSMV_OK;
}

csmv_status csmv::check_stream(const csmv_bank_t* h, const csmv_bank_stream* s) {
  if (!s || !s->op || !s->off || !s->addr || s->n_txn == 0 || s->n_txn % 32) {
    set_error("stream: n_txn must be a positive multiple of 32 with op/off/addr set");
    return CSMV_ERR_INVALID_ARG;
  }
  if (s->n_txn > h->cfg.max_txn) {
    set_error("stream of %u transactions exceeds max_txn %u", s->n_txn, h->cfg.max_txn);
    return CSMV_ERR_CAPACITY;
  }
  if (s->split_round > s->n_txn / 32 || (s->split_round && s->deferred_warps == 0)) {
    set_error("stream: split_round must be <= n_txn/32, with deferred_warps > 0");
    return CSMV_ERR_INVALID_ARG;
  }
  if (s->lane_start && !s->split_round) {
    set_error("stream: lane_start cuts the deferred queue; it needs split_round");
    return CSMV_ERR_INVALID_ARG;
  }
  if (s->lock_last && !(h->cfg.prevalidate == 3 && h->cfg.validate == CSMV_VALIDATE_STAMP)) {
    set_error("stream: lock_last orders the locks of group commit (prevalidate 3, stamp protocol)");
    return CSMV_ERR_INVALID_ARG;
  }
  return CSMV_OK;
}

bool csmv::bank_group_commit(const csmv_bank_t* h, uint32_t* n_accounts) {
  *n_accounts = h->cfg.n_accounts;
  return h->cfg.prevalidate == 3 && h->cfg.validate == CSMV_VALIDATE_STAMP;
}

BankParams csmv::bank_params(const csmv_bank_t* h, const uint32_t* op, const uint32_t* off,
                             const uint32_t* addr, uint32_t n_txn, uint32_t* txn_aborts) {
  const csmv_bank_config& c = h->cfg;
  BankParams p{};
  p.op = op;
  p.off = off;
  p.addr = addr;
  p.n_rounds = n_txn / 32;
  p.n_items = c.n_accounts;
  p.grace = c.group_grace;
  p.read_wait = c.group_read_wait;
  p.slots = h->slots;
  p.cw = h->cw;
  p.ring = h->ring;
  p.ring_mask = c.ring_size - 1;
  p.done = h->done;
  p.done_mask = kDoneWords - 1;
  p.gs = h->gs;
  p.log_txn = h->log_txn;
  p.outcome = h->outcome;
  p.result = h->result;
  p.stats = h->stats;
  p.log = c.log_commits;
  p.log_base = h->last_final_ts;
  p.log_cap = h->log_cap;
  p.nc = c.client_warps;
  p.validate = c.validate;
  p.writeback = c.writeback;
  p.batch = c.batch;
  p.prevalidate = c.prevalidate;
  p.spin_log2 = c.spin_limit_log2;
  p.txn_aborts = txn_aborts;
  p.grp = (c.log_commits && c.prevalidate >= 2 && c.validate == CSMV_VALIDATE_STAMP) ? h->grp : nullptr;
  p.tk = h->tk;
  return p;
}

csmv_status csmv::bank_begin_run(csmv_bank_t* h) {
  // the commit order carries on from the previous run: only the cursors and error reset
  CSMV_CUDA(cudaMemsetAsync(&h->gs->round_next, 0, 4, h->stream));
  CSMV_CUDA(cudaMemsetAsync(&h->gs->round_deferred, 0, 4, h->stream));
  CSMV_CUDA(cudaMemsetAsync(&h->gs->error, 0, 4, h->stream));
  CSMV_CUDA(cudaMemsetAsync(h->stats, 0, ST_COUNT * 8, h->stream));
  CSMV_CUDA(cudaEventRecord(h->ev0, h->stream));
  return CSMV_OK;
}

csmv_status csmv::bank_end_run(csmv_bank_t* h, uint32_t n_txn, csmv_stats* out) {
  const csmv_bank_config& c = h->cfg;
  CSMV_CUDA(cudaEventRecord(h->ev1, h->stream));
  unsigned long long st[ST_COUNT];
  GlobalSync gs;
  CSMV_CUDA(cudaMemcpyAsync(st, h->stats, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
  CSMV_CUDA(cudaMemcpyAsync(&gs, h->gs, sizeof(gs), cudaMemcpyDeviceToHost, h->stream));
  CSMV_CUDA(cudaStreamSynchronize(h->stream));
  float ms = 0;
  CSMV_CUDA(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
  const uint32_t final_ts = c.validate == CSMV_VALIDATE_STAMP ? gs.ts_next : (uint32_t)(gs.turn >> 32);
  h->last_n_txn = n_txn;
  h->run_base_ts = h->last_final_ts;
  h->last_final_ts = final_ts;
  if (out) {
    out->commits_update = st[ST_COMMIT_UPDATE];
    out->commits_readonly = st[ST_COMMIT_RO];
    out->commits_nowrite = st[ST_COMMIT_NOWRITE];
    out->aborts_data_age = st[ST_ABORT_DATA_AGE];
    out->aborts_record_age = st[ST_ABORT_RECORD_AGE];
    out->aborts_read_write = st[ST_ABORT_READ_WRITE];
    out->aborts_prevalid = st[ST_ABORT_PREVALID];
    out->aborts_write_write = st[ST_ABORT_WRITE_WRITE];
    out->sections = st[ST_SECTIONS];
    out->rounds = st[ST_ROUNDS];
    out->final_ts = final_ts;
    out->error = gs.error;
    out->kernel_ms = ms;
  }
  if (gs.error) {
    if (gs.error == ERR_CAPACITY) {
      set_error("device error 5: the run used more timestamps than the commit log holds "
                "(8 x max_txn; aborted attempts take timestamps too)");
      return CSMV_ERR_CAPACITY;
    }
    set_error("device error %u (1 turn, 2 clock, 3 reply, 4 request, 5 capacity, 6 data, "
              "7 livelock, 8 dataflow wait)",
              gs.error);
    return gs.error == ERR_DATA ? CSMV_ERR_INVALID_ARG : CSMV_ERR_TIMEOUT;
  }
  return CSMV_OK;
}

static csmv_status launch(csmv_bank_t* h, const uint32_t* op, const uint32_t* off,
                          const uint32_t* addr, uint32_t n_txn, uint32_t* txn_aborts,
                          uint32_t split_round, uint32_t deferred_warps, const uint32_t* backoff,
                          uint32_t* txn_waits, const uint8_t* lock_last, csmv_stats* out,
                          bool serial = false, const uint32_t* lane_start = nullptr) {
  const csmv_bank_config& c = h->cfg;
  BankParams p = bank_params(h, op, off, addr, n_txn, txn_aborts);
  p.split_round = split_round;
  p.deferred_warps = deferred_warps;
  p.lane_start = split_round ? lane_start : nullptr;
  p.backoff = backoff;
  p.lock_last = serial ? nullptr : lock_last;
  p.txn_waits = txn_waits;
  if (txn_waits && (serial || c.prevalidate != 3))  // only group commit waits on locks
    CSMV_CUDA(cudaMemsetAsync(txn_waits, 0, (size_t)n_txn * 4, h->stream));
  if (serial) p.grp = nullptr;
  if (p.grp) CSMV_CUDA(cudaMemsetAsync(h->grp, 0, (size_t)h->grp_words * 4, h->stream));
  if (!serial && c.prevalidate == 3)  // empty lock queues (a failed run may have left tickets)
    CSMV_CUDA(cudaMemsetAsync(h->tk, 0, (size_t)c.n_accounts * 8, h->stream));
  h->last_grouped = p.grp != nullptr;
  csmv_status bst = bank_begin_run(h);
  if (bst != CSMV_OK) return bst;
  void* args[] = {&p};
  if (serial) {
    pick_serial(c.version_depth)<<<1, 32, serial_smem(c.version_depth), h->stream>>>(p);
    CSMV_CUDA(cudaGetLastError());
  } else if (c.batch == CSMV_BATCH_CLUSTER) {
    // clusters of cluster_size CTAs; the grid never exceeds the co-resident clusters
    cudaLaunchConfig_t lc = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = c.cluster_size;
    at[0].val.clusterDim.y = at[0].val.clusterDim.z = 1;
    lc.gridDim = dim3(h->ctas);
    lc.blockDim = dim3(h->threads);
    lc.dynamicSmemBytes = h->smem;
    lc.stream = h->stream;
    lc.attrs = at;
    lc.numAttrs = 1;
    CSMV_CUDA(cudaLaunchKernelExC(&lc, (const void*)h->kernel, args));
  } else {
    CSMV_CUDA(cudaLaunchCooperativeKernel((const void*)h->kernel, dim3(h->ctas), dim3(h->threads),
                                          args, h->smem, h->stream));
  }
  return bank_end_run(h, n_txn, out);
}

extern "C" csmv_status csmv_bank_run_device(csmv_bank_t* h, const csmv_bank_stream* s,
                                            csmv_stats* out) {
  if (!h) return CSMV_ERR_INVALID_ARG;
  if (!h->loaded) {
    set_error("csmv_bank_load must come first");
    return CSMV_ERR_STATE;
  }
  csmv_status st = check_stream(h, s);
  if (st != CSMV_OK) return st;
  CSMV_CUDA(cudaSetDevice(h->cfg.device));
  auto t0 = std::chrono::steady_clock::now();
  st = launch(h, s->op, s->off, s->addr, s->n_txn, s->txn_aborts, s->split_round,
              s->deferred_warps, s->backoff, s->txn_waits, s->lock_last, out, false, s->lane_start);
  if (out)
    out->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return st;
}

extern "C" csmv_status csmv_bank_run_serial_device(csmv_bank_t* h, const csmv_bank_stream* s,
                                                   csmv_stats* out) {
  if (!h) return CSMV_ERR_INVALID_ARG;
  if (!h->loaded) {
    set_error("csmv_bank_load must come first");
    return CSMV_ERR_STATE;
  }
  csmv_status st = check_stream(h, s);
  if (st != CSMV_OK) return st;
  if (h->cfg.validate != CSMV_VALIDATE_STAMP) {
    set_error("the serial lane continues the stamp protocol's commit order only");
    return CSMV_ERR_INVALID_ARG;
  }
  CSMV_CUDA(cudaSetDevice(h->cfg.device));
  auto t0 = std::chrono::steady_clock::now();
  st = launch(h, s->op, s->off, s->addr, s->n_txn, s->txn_aborts, 0, 0, nullptr, s->txn_waits,
              nullptr, out, true);
  if (out)
    out->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return st;
}

extern "C" csmv_status csmv_bank_run(csmv_bank_t* h, const csmv_bank_stream* s, csmv_stats* out) {
  if (!h) return CSMV_ERR_INVALID_ARG;
  if (!h->loaded) {
    set_error("csmv_bank_load must come first");
    return CSMV_ERR_STATE;
  }
  csmv_status st = check_stream(h, s);
  if (st != CSMV_OK) return st;
  CSMV_CUDA(cudaSetDevice(h->cfg.device));
  auto t0 = std::chrono::steady_clock::now();
  if (s->n_addr > h->addr_cap) {
    cudaFree(h->d_addr);
    h->d_addr = nullptr;
    h->addr_cap = 0;
    CSMV_CUDA(cudaMalloc(&h->d_addr, s->n_addr * 4));
    h->addr_cap = s->n_addr;
  }
  CSMV_CUDA(cudaMemcpyAsync(h->d_op, s->op, (size_t)s->n_txn * 4, cudaMemcpyHostToDevice, h->stream));
  CSMV_CUDA(cudaMemcpyAsync(h->d_off, s->off, (size_t)s->n_txn * 4, cudaMemcpyHostToDevice, h->stream));
  CSMV_CUDA(cudaMemcpyAsync(h->d_addr, s->addr, s->n_addr * 4, cudaMemcpyHostToDevice, h->stream));
  if (s->backoff)
    CSMV_CUDA(cudaMemcpyAsync(h->d_backoff, s->backoff, (size_t)s->n_txn * 4,
                              cudaMemcpyHostToDevice, h->stream));
  if (s->lane_start) {  // host lanes: checked here, then copied
    const uint32_t nr = s->n_txn / 32;
    bool ok = s->deferred_warps <= 4096u && s->lane_start[0] >= s->split_round;
    for (uint32_t i = 0; ok && i < s->deferred_warps; i++)
      ok = s->lane_start[i] <= s->lane_start[i + 1] && s->lane_start[i + 1] <= nr;
    if (!ok) {
      set_error("stream: lane_start must rise from split_round to at most n_txn/32");
      return CSMV_ERR_INVALID_ARG;
    }
    cudaFree(h->d_lanes);
    h->d_lanes = nullptr;
    CSMV_CUDA(cudaMalloc(&h->d_lanes, (size_t)(s->deferred_warps + 1) * 4));
    CSMV_CUDA(cudaMemcpyAsync(h->d_lanes, s->lane_start, (size_t)(s->deferred_warps + 1) * 4,
                              cudaMemcpyHostToDevice, h->stream));
  }
  if (s->lock_last) {
    if (!h->d_lock_last) CSMV_CUDA(cudaMalloc(&h->d_lock_last, h->cfg.n_accounts));
    CSMV_CUDA(cudaMemcpyAsync(h->d_lock_last, s->lock_last, h->cfg.n_accounts,
                              cudaMemcpyHostToDevice, h->stream));
  }
  st = launch(h, h->d_op, h->d_off, h->d_addr, s->n_txn, s->txn_aborts ? h->d_aborts : nullptr,
              s->split_round, s->deferred_warps, s->backoff ? h->d_backoff : nullptr,
              s->txn_waits ? h->d_waits : nullptr, s->lock_last ? h->d_lock_last : nullptr, out,
              false, s->lane_start ? h->d_lanes : nullptr);
  if (st == CSMV_OK && (s->txn_aborts || s->txn_waits)) {
    if (s->txn_aborts)
      CSMV_CUDA(cudaMemcpyAsync(s->txn_aborts, h->d_aborts, (size_t)s->n_txn * 4,
                                cudaMemcpyDeviceToHost, h->stream));
    if (s->txn_waits)
      CSMV_CUDA(cudaMemcpyAsync(s->txn_waits, h->d_waits, (size_t)s->n_txn * 4,
                                cudaMemcpyDeviceToHost, h->stream));
    CSMV_CUDA(cudaStreamSynchronize(h->stream));
  }
  if (out)
    out->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return st;
}

extern "C" csmv_status csmv_bank_read_versions(csmv_bank_t* h, uint64_t* host_slots) {
  if (!h || !host_slots) return CSMV_ERR_INVALID_ARG;
  CSMV_CUDA(cudaSetDevice(h->cfg.device));
  CSMV_CUDA(cudaMemcpy(host_slots, h->slots, (size_t)h->cfg.n_accounts * h->cfg.version_depth * 8,
                       cudaMemcpyDeviceToHost));
  return CSMV_OK;
}

extern "C" csmv_status csmv_bank_read_values(csmv_bank_t* h, int32_t* host_values) {
  if (!h || !host_values) return CSMV_ERR_INVALID_ARG;
  const size_t n = h->cfg.n_accounts, D = h->cfg.version_depth;
  std::vector<uint64_t> slots(n * D);
  csmv_status st = csmv_bank_read_versions(h, slots.data());
  if (st != CSMV_OK) return st;
  for (size_t i = 0; i < n; i++) {  // newest version = largest ts (the reference's head)
    uint32_t best_ts = 0;
    int32_t v = 0;
    bool any = false;
    for (size_t d = 0; d < D; d++) {
      const uint64_t s = slots[i * D + d];
      const uint32_t ts = (uint32_t)(s >> 32);
      if (ts == 0xFFFFFFFFu) continue;
      if (!any || ts > best_ts) {
        any = true;
        best_ts = ts;
        v = (int32_t)(uint32_t)s;
      }
    }
    host_values[i] = v;
  }
  return CSMV_OK;
}

extern "C" csmv_status csmv_bank_read_log(csmv_bank_t* h, uint32_t* host_log_txn, uint32_t n_log,
                                          uint32_t* host_outcome, int32_t* host_result,
                                          uint32_t n_txn) {
  if (!h) return CSMV_ERR_INVALID_ARG;
  if (!h->cfg.log_commits) {
    set_error("handle was created with log_commits = 0");
    return CSMV_ERR_STATE;
  }
  CSMV_CUDA(cudaSetDevice(h->cfg.device));
  const uint32_t commits = h->last_final_ts - h->run_base_ts;  // timestamps, holes included
  if (host_log_txn) {
    if (n_log < commits) {
      set_error("log buffer holds %u entries, run used %u timestamps", n_log, commits);
      return CSMV_ERR_CAPACITY;
    }
    // entry k holds the transaction that committed with ts = run_base_ts + k + 1
    CSMV_CUDA(cudaMemcpy(host_log_txn, h->log_txn, (size_t)commits * 4,
                         cudaMemcpyDeviceToHost));
  }
  if (n_txn > h->last_n_txn) n_txn = h->last_n_txn;
  if (host_outcome) CSMV_CUDA(cudaMemcpy(host_outcome, h->outcome, (size_t)n_txn * 4, cudaMemcpyDeviceToHost));
  if (host_result) CSMV_CUDA(cudaMemcpy(host_result, h->result, (size_t)n_txn * 4, cudaMemcpyDeviceToHost));
  return CSMV_OK;
}

extern "C" csmv_status csmv_bank_read_groups(csmv_bank_t* h, uint32_t* host_bits, uint32_t n_log) {
  if (!h || !host_bits) return CSMV_ERR_INVALID_ARG;
  if (!h->cfg.log_commits) {
    set_error("handle was created with log_commits = 0");
    return CSMV_ERR_STATE;
  }
  const uint32_t used = h->last_final_ts - h->run_base_ts;
  if (n_log < used) {
    set_error("group buffer covers %u timestamps, run used %u", n_log, used);
    return CSMV_ERR_CAPACITY;
  }
  const uint32_t words = (used + 31u) / 32u;
  if (!h->last_grouped) {  // every timestamp is its own group
    for (uint32_t i = 0; i < (n_log + 31u) / 32u; i++) host_bits[i] = 0xFFFFFFFFu;
    return CSMV_OK;
  }
  CSMV_CUDA(cudaSetDevice(h->cfg.device));
  if (words) CSMV_CUDA(cudaMemcpy(host_bits, h->grp, (size_t)words * 4, cudaMemcpyDeviceToHost));
  for (uint32_t i = words; i < (n_log + 31u) / 32u; i++) host_bits[i] = 0u;
  return CSMV_OK;
}

extern "C" csmv_status csmv_bank_device_info(csmv_bank_t* h, int* n_sms, int* ctas,
                                             int* threads_per_cta, size_t* device_bytes) {
  if (!h) return CSMV_ERR_INVALID_ARG;
  if (n_sms) *n_sms = h->n_sms;
  if (ctas) *ctas = h->ctas;
  if (threads_per_cta) *threads_per_cta = h->threads;
  if (device_bytes) *device_bytes = h->device_bytes + h->addr_cap * 4;
  return CSMV_OK;
}

extern "C" void csmv_bank_destroy(csmv_bank_t* h) {
  if (!h) return;
  cudaSetDevice(h->cfg.device);
  free_all(h);
  delete h;
}

// ---------------------------------------------------------------------------------------------
// Autotuner: picks the engine's launch shape for a workload by measurement. Candidates: client
// warps per CTA 1, 2, 4, 8 (block size; each client warp owns one mailbox of its CTA's server),
// CTAs per SM (1 or 2, as co-residency allows) and versions per account (4, 8). Every candidate
// runs the caller's sample once from the same initial state; the best quarter runs `repeats`
// more times and the fastest median wins (successive halving).
// ---------------------------------------------------------------------------------------------
#include <algorithm>

namespace {
struct Trial {
  csmv_bank_config cfg;
  double best_ms = 1e30;
  std::vector<double> ms;
  double abort_rate = 0;
  csmv_status st = CSMV_OK;
};

csmv_status tune_run(const csmv_bank_config& cfg, const csmv_bank_stream* s, const int32_t* init,
                     uint32_t times, Trial& t) {
  csmv_bank_t* h = nullptr;
  csmv_status st = csmv_bank_create(&cfg, &h);
  if (st != CSMV_OK) return st;
  for (uint32_t i = 0; i < times && st == CSMV_OK; i++) {
    if ((st = csmv_bank_load(h, init)) != CSMV_OK) break;
    csmv_stats out;
    if ((st = csmv_bank_run(h, s, &out)) != CSMV_OK) break;
    t.ms.push_back(out.kernel_ms);
    const double c = (double)(out.commits_update + out.commits_readonly + out.commits_nowrite);
    const double a = (double)(out.aborts_data_age + out.aborts_record_age + out.aborts_read_write +
                              out.aborts_prevalid + out.aborts_write_write);
    t.abort_rate = a / std::max(1.0, a + c);
  }
  csmv_bank_destroy(h);
  return st;
}
}  // namespace

extern "C" csmv_status csmv_bank_autotune(const csmv_bank_config* base,
                                          const csmv_bank_stream* host_sample,
                                          const int32_t* host_init, uint32_t repeats,
                                          csmv_tune_result* out) {
  if (!base || !host_sample || !out || repeats == 0) return CSMV_ERR_INVALID_ARG;
  std::memset(out, 0, sizeof(*out));
  int n_sms = 0;
  csmv_status st = check_device(base->device, &n_sms);
  if (st != CSMV_OK) return st;
  // commit methods and read specialisations worth trying on this sample
  std::vector<uint32_t> methods{base->prevalidate}, reads{base->max_reads};
  if (base->validate == CSMV_VALIDATE_STAMP) methods = {1u, 3u};
  if (host_sample->op) {
    uint32_t widest = 0;
    for (uint32_t i = 0; i < host_sample->n_txn; i++) {
      const uint32_t o = host_sample->op[i];
      if (CSMV_OP_KIND(o) != CSMV_KIND_READONLY) widest = std::max(widest, CSMV_OP_NREADS(o));
    }
    if (widest <= 4u) reads = {0u, 4u};
  }
  std::vector<Trial> trials;
  for (uint32_t method : methods)
    for (uint32_t mr : reads)
      for (uint32_t depth : {4u, 8u})
        for (uint32_t cw : {1u, 2u, 4u, 8u})
          for (uint32_t per_sm : {1u, 2u}) {
            Trial t;
            t.cfg = *base;
            t.cfg.prevalidate = method;
            t.cfg.max_reads = mr;
            t.cfg.version_depth = depth;
            t.cfg.client_warps = cw;
            t.cfg.ctas = per_sm * (uint32_t)n_sms;
            t.cfg.max_txn = std::max(base->max_txn, host_sample->n_txn);
            t.cfg.log_commits = 0;
            trials.push_back(t);
          }
  for (auto& t : trials) {
    t.st = tune_run(t.cfg, host_sample, host_init, 1, t);
    if (t.st == CSMV_OK) t.best_ms = t.ms.back();
  }
  std::vector<size_t> order(trials.size());
  for (size_t i = 0; i < order.size(); i++) order[i] = i;
  std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return trials[a].best_ms < trials[b].best_ms; });
  const size_t keep = std::max<size_t>(1, trials.size() / 4);
  for (size_t r = 0; r < keep; r++) {
    Trial& t = trials[order[r]];
    if (t.st != CSMV_OK) continue;
    t.st = tune_run(t.cfg, host_sample, host_init, repeats, t);
    std::vector<double> m = t.ms;
    std::sort(m.begin(), m.end());
    t.best_ms = m[m.size() / 2];  // median over every run
  }
  size_t best = order[0];
  for (size_t r = 0; r < keep; r++)
    if (trials[order[r]].st == CSMV_OK && trials[order[r]].best_ms < trials[best].best_ms) best = order[r];
  if (trials[best].st != CSMV_OK) {
    set_error("autotune: no candidate ran (%s)", csmv_status_str(trials[best].st));
    return trials[best].st;
  }
  out->best = trials[best].cfg;
  out->best.log_commits = base->log_commits;
  out->best.max_txn = base->max_txn;
  out->n_trials = (uint32_t)std::min<size_t>(trials.size(), CSMV_TUNE_MAX_TRIALS);
  for (uint32_t i = 0; i < out->n_trials; i++) {
    const Trial& t = trials[i];
    csmv_tune_trial& o = out->trials[i];
    o.client_warps = t.cfg.client_warps;
    o.ctas = t.cfg.ctas;
    o.version_depth = t.cfg.version_depth;
    o.runs = (uint32_t)t.ms.size();
    o.status = (int32_t)t.st;
    o.tx_per_s = t.st == CSMV_OK ? host_sample->n_txn / (t.best_ms * 1e-3) : 0.0;
    o.abort_rate = t.abort_rate;
    o.prevalidate = t.cfg.prevalidate;
    o.max_reads = t.cfg.max_reads;
  }
  return CSMV_OK;
}
