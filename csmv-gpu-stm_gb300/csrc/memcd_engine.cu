// memcd_engine.cu - C-ABI host side of the transactional cache (include/csmv.h, memcached part).
//
// Data layout in HBM (entry = set * 8 + way, allocated once per handle):
//   tag   entries * 2 * 8 B    version tags: ts << 32 | valid << 31 | 31-bit key hash; the 16
//                              tags of a set are one 128-byte line
//   rec   entries * 2 * 64 B   version records {lru, 0, 0, 0 | key[4] | value[8]}
//   cw    entries * 8 B        commit word: stamp (ts of the last committed SET) and lock owner
//   done  256 KB               completion bitmap, one bit per commit timestamp
//   logs  8*max_req*4 + max_req*4 B   log_txn[ts-1] (holes included), outcome[req]
//   io    max_req * (4 + 16 + 32 + 4 + 32) B   request / response staging for host-buffer runs
#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>

#include "common.h"
#include "memcd_kernel.cuh"

using namespace csmv;

namespace {
constexpr uint32_t kDoneWords = 1u << 16;
}

struct csmv_memcd_t {
  csmv_memcd_config cfg{};
  int n_sms = 0, ctas = 0, threads = 0;
  size_t device_bytes = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  unsigned long long* tag = nullptr;
  uint4* rec = nullptr;
  unsigned long long* cw = nullptr;
  uint32_t* done = nullptr;
  GlobalSync* gs = nullptr;
  uint32_t log_cap = 0;
  uint32_t* log_txn = nullptr;
  uint32_t* outcome = nullptr;
  unsigned long long* stats = nullptr;
  uint32_t* d_kind = nullptr;
  uint4* d_key = nullptr;
  uint4* d_val = nullptr;
  uint32_t* d_found = nullptr;
  uint4* d_out = nullptr;
  bool loaded = false;
  uint32_t last_final_ts = 0, last_n_req = 0, run_base_ts = 0;
};

extern "C" void csmv_memcd_config_default(csmv_memcd_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->n_sets = 1u << 20;
  c->n_ways = kWays;
  c->version_depth = kMemcdDepth;
  c->client_warps = 4;
  c->ctas = 0;
  c->batch = CSMV_BATCH_CTA;
  c->log_commits = 1;
  c->max_req = 1u << 16;
  c->spin_limit_log2 = 24;
  c->device = 0;
}

static csmv_status validate_config(const csmv_memcd_config* c) {
  auto bad = [](const char* why) {
    set_error("invalid memcd config: %s", why);
    return CSMV_ERR_INVALID_ARG;
  };
  if (!c) return bad("null");
  if (c->n_sets < 1 || c->n_sets > (1u << 26)) return bad("n_sets must be 1..2^26");
  if (c->n_ways != (uint32_t)kWays) return bad("n_ways must be 8");
  if (c->version_depth != (uint32_t)kMemcdDepth) return bad("version_depth must be 2");
  if (c->client_warps < 1 || c->client_warps > (uint32_t)kMaxClientWarps) return bad("client_warps");
  if (c->batch != CSMV_BATCH_WARP && c->batch != CSMV_BATCH_CTA) return bad("batch (warp or cta)");
  if (c->max_req == 0 || c->max_req % 32) return bad("max_req must be a positive multiple of 32");
  if (c->spin_limit_log2 < 10 || c->spin_limit_log2 > 30) return bad("spin_limit_log2");
  return CSMV_OK;
}

static void free_all(csmv_memcd_t* h) {
  cudaFree(h->tag);
  cudaFree(h->rec);
  cudaFree(h->cw);
  cudaFree(h->done);
  cudaFree(h->gs);
  cudaFree(h->log_txn);
  cudaFree(h->outcome);
  cudaFree(h->stats);
  cudaFree(h->d_kind);
  cudaFree(h->d_key);
  cudaFree(h->d_val);
  cudaFree(h->d_found);
  cudaFree(h->d_out);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->stream) cudaStreamDestroy(h->stream);
}

extern "C" csmv_status csmv_memcd_create(const csmv_memcd_config* cfg, csmv_memcd_t** out) {
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
  csmv_memcd_t* h = new csmv_memcd_t;
  h->cfg = *cfg;
  h->n_sms = n_sms;
  h->threads = (int)(cfg->client_warps + 1) * 32;
  auto fail = [&](csmv_status s) {
    free_all(h);
    delete h;
    return s;
  };
  int per_sm = 0;
  if ((st = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, memcd_kernel,
                                                                       h->threads, 0),
                        "occupancy")) != CSMV_OK)
    return fail(st);
  const int max_ctas = per_sm * n_sms;
  if (max_ctas <= 0) {
    set_error("kernel does not fit on an SM (threads %d)", h->threads);
    return fail(CSMV_ERR_INVALID_ARG);
  }
  h->ctas = cfg->ctas ? (int)cfg->ctas : max_ctas;
  if (h->ctas > max_ctas) {
    set_error("%d CTAs requested, only %d can be co-resident", h->ctas, max_ctas);
    return fail(CSMV_ERR_INVALID_ARG);
  }
  const size_t ent = (size_t)cfg->n_sets * kWays, D = kMemcdDepth, R = cfg->max_req;
  h->log_cap = cfg->log_commits ? (cfg->max_req > 0x1FFFFFFFu ? 0xFFFFFFFFu : cfg->max_req * 8u) : 1u;
  struct {
    void** p;
    size_t bytes;
  } allocs[] = {
      {(void**)&h->tag, ent * D * 8},        {(void**)&h->rec, ent * D * 64},
      {(void**)&h->cw, ent * 8},             {(void**)&h->gs, sizeof(GlobalSync)},
      {(void**)&h->done, (size_t)kDoneWords * 4},
      {(void**)&h->log_txn, (size_t)h->log_cap * 4}, {(void**)&h->outcome, R * 4},
      {(void**)&h->stats, ST_COUNT * 8},     {(void**)&h->d_kind, R * 4},
      {(void**)&h->d_key, R * 16},           {(void**)&h->d_val, R * 32},
      {(void**)&h->d_found, R * 4},          {(void**)&h->d_out, R * 32},
  };
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

// Initial table: every entry holds one invalid version with ts 0 (the reference's state array
// zeroed with head_ptr 1, memcdSH.cu:562-574); the other version slots are empty.
__global__ void memcd_clear_kernel(unsigned long long* tag, size_t n_tags) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_tags; i += stride)
    tag[i] = (i % kMemcdDepth == 0) ? 0ull : ((unsigned long long)kEmptyTs << 32);
}

extern "C" csmv_status csmv_memcd_clear(csmv_memcd_t* h) {
  if (!h) return CSMV_ERR_INVALID_ARG;
  CSMV_CUDA(cudaSetDevice(h->cfg.device));
  const size_t ent = (size_t)h->cfg.n_sets * kWays;
  memcd_clear_kernel<<<h->n_sms * 4, 256, 0, h->stream>>>(h->tag, ent * kMemcdDepth);
  CSMV_CUDA(cudaGetLastError());
  CSMV_CUDA(cudaMemsetAsync(h->rec, 0, ent * kMemcdDepth * 64, h->stream));
  CSMV_CUDA(cudaMemsetAsync(h->cw, 0, ent * 8, h->stream));
  CSMV_CUDA(cudaMemsetAsync(h->done, 0, (size_t)kDoneWords * 4, h->stream));
  CSMV_CUDA(cudaMemsetAsync(h->gs, 0, sizeof(GlobalSync), h->stream));
  CSMV_CUDA(cudaStreamSynchronize(h->stream));
  h->loaded = true;
  h->last_final_ts = h->run_base_ts = h->last_n_req = 0;
  return CSMV_OK;
}

static csmv_status check_batch(const csmv_memcd_t* h, const csmv_memcd_batch* b) {
  if (!b || !b->kind || !b->key || !b->val || !b->found || !b->val_out || b->n_req == 0 ||
      b->n_req % 32) {
    set_error("batch: n_req must be a positive multiple of 32 with every pointer set");
    return CSMV_ERR_INVALID_ARG;
  }
  if (b->n_req > h->cfg.max_req) {
    set_error("batch of %u requests exceeds max_req %u", b->n_req, h->cfg.max_req);
    return CSMV_ERR_CAPACITY;
  }
  return CSMV_OK;
}

static csmv_status launch(csmv_memcd_t* h, const uint32_t* kind, const uint4* key, const uint4* val,
                          uint32_t* found, uint4* val_out, uint32_t n_req, uint32_t tick,
                          csmv_stats* out) {
  const csmv_memcd_config& c = h->cfg;
  MemcdParams p{};
  p.kind = kind;
  p.key = key;
  p.val = val;
  p.n_rounds = n_req / 32;
  p.tick = tick;
  p.n_sets = c.n_sets;
  p.tag = h->tag;
  p.rec = h->rec;
  p.cw = h->cw;
  p.done = h->done;
  p.done_mask = kDoneWords - 1;
  p.gs = h->gs;
  p.found = found;
  p.val_out = val_out;
  p.log_txn = h->log_txn;
  p.outcome = h->outcome;
  p.log = c.log_commits;
  p.log_base = h->last_final_ts;
  p.log_cap = h->log_cap;
  p.stats = h->stats;
  p.nc = c.client_warps;
  p.batch = c.batch;
  p.spin_log2 = c.spin_limit_log2;
  CSMV_CUDA(cudaMemsetAsync(&h->gs->round_next, 0, 4, h->stream));
  CSMV_CUDA(cudaMemsetAsync(&h->gs->error, 0, 4, h->stream));
  CSMV_CUDA(cudaMemsetAsync(h->stats, 0, ST_COUNT * 8, h->stream));
  void* args[] = {&p};
  CSMV_CUDA(cudaEventRecord(h->ev0, h->stream));
  CSMV_CUDA(cudaLaunchCooperativeKernel((const void*)memcd_kernel, dim3(h->ctas), dim3(h->threads),
                                        args, 0, h->stream));
  CSMV_CUDA(cudaEventRecord(h->ev1, h->stream));
  unsigned long long st[ST_COUNT];
  GlobalSync gs;
  CSMV_CUDA(cudaMemcpyAsync(st, h->stats, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
  CSMV_CUDA(cudaMemcpyAsync(&gs, h->gs, sizeof(gs), cudaMemcpyDeviceToHost, h->stream));
  CSMV_CUDA(cudaStreamSynchronize(h->stream));
  float ms = 0;
  CSMV_CUDA(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
  h->last_n_req = n_req;
  h->run_base_ts = h->last_final_ts;
  h->last_final_ts = gs.ts_next;
  if (out) {
    std::memset(out, 0, sizeof(*out));
    out->commits_update = st[ST_COMMIT_UPDATE];
    out->commits_readonly = st[ST_COMMIT_RO];
    out->aborts_data_age = st[ST_ABORT_DATA_AGE];
    out->aborts_read_write = st[ST_ABORT_READ_WRITE];
    out->aborts_prevalid = st[ST_ABORT_PREVALID];
    out->aborts_write_write = st[ST_ABORT_WRITE_WRITE];
    out->sections = st[ST_SECTIONS];
    out->rounds = st[ST_ROUNDS];
    out->final_ts = gs.ts_next;
    out->error = gs.error;
    out->kernel_ms = ms;
  }
  if (gs.error) {
    set_error("device error %u (3 reply, 5 capacity, 6 mixed GET/SET round, 7 livelock)", gs.error);
    return gs.error == ERR_DATA ? CSMV_ERR_INVALID_ARG : CSMV_ERR_TIMEOUT;
  }
  return CSMV_OK;
}

static csmv_status ready(csmv_memcd_t* h) {
  if (!h) return CSMV_ERR_INVALID_ARG;
  if (!h->loaded) {
    set_error("csmv_memcd_clear must come first");
    return CSMV_ERR_STATE;
  }
  return CSMV_OK;
}

extern "C" csmv_status csmv_memcd_run_device(csmv_memcd_t* h, const csmv_memcd_batch* b,
                                             csmv_stats* out) {
  csmv_status st = ready(h);
  if (st != CSMV_OK || (st = check_batch(h, b)) != CSMV_OK) return st;
  if (((uintptr_t)b->key | (uintptr_t)b->val | (uintptr_t)b->val_out) & 15u) {
    set_error("device batch: key, val and val_out must be 16-byte aligned");
    return CSMV_ERR_INVALID_ARG;
  }
  CSMV_CUDA(cudaSetDevice(h->cfg.device));
  auto t0 = std::chrono::steady_clock::now();
  st = launch(h, b->kind, (const uint4*)b->key, (const uint4*)b->val, b->found, (uint4*)b->val_out,
              b->n_req, b->tick, out);
  if (out)
    out->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return st;
}

extern "C" csmv_status csmv_memcd_run(csmv_memcd_t* h, const csmv_memcd_batch* b, csmv_stats* out) {
  csmv_status st = ready(h);
  if (st != CSMV_OK || (st = check_batch(h, b)) != CSMV_OK) return st;
  CSMV_CUDA(cudaSetDevice(h->cfg.device));
  auto t0 = std::chrono::steady_clock::now();
  const size_t n = b->n_req;
  CSMV_CUDA(cudaMemcpyAsync(h->d_kind, b->kind, n * 4, cudaMemcpyHostToDevice, h->stream));
  CSMV_CUDA(cudaMemcpyAsync(h->d_key, b->key, n * 16, cudaMemcpyHostToDevice, h->stream));
  CSMV_CUDA(cudaMemcpyAsync(h->d_val, b->val, n * 32, cudaMemcpyHostToDevice, h->stream));
  st = launch(h, h->d_kind, h->d_key, h->d_val, h->d_found, h->d_out, b->n_req, b->tick, out);
  if (st == CSMV_OK) {
    CSMV_CUDA(cudaMemcpyAsync(b->found, h->d_found, n * 4, cudaMemcpyDeviceToHost, h->stream));
    CSMV_CUDA(cudaMemcpyAsync(b->val_out, h->d_out, n * 32, cudaMemcpyDeviceToHost, h->stream));
    CSMV_CUDA(cudaStreamSynchronize(h->stream));
  }
  if (out)
    out->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return st;
}

// The cache's autotuner: each candidate shape on a fresh cache, fill untimed, the sample timed
// by its kernel time; successive halving as in the bank's tuner.
extern "C" csmv_status csmv_memcd_autotune(const csmv_memcd_config* base,
                                           const csmv_memcd_batch* host_fill,
                                           const csmv_memcd_batch* host_sample, uint32_t repeats,
                                           csmv_memcd_tune_result* out) {
  if (!base || !host_sample || !out || repeats == 0) return CSMV_ERR_INVALID_ARG;
  std::memset(out, 0, sizeof(*out));
  int n_sms = 0;
  csmv_status st = check_device(base->device, &n_sms);
  if (st != CSMV_OK) return st;
  struct Cand {
    csmv_memcd_config cfg;
    std::vector<double> ms;
    double med = 1e30, abort_rate = 0;
    csmv_status st = CSMV_OK;
  };
  std::vector<Cand> cands;
  for (uint32_t cw : {1u, 2u, 4u, 8u})
    for (uint32_t per_sm : {1u, 2u}) {
      Cand c;
      c.cfg = *base;
      c.cfg.client_warps = cw;
      c.cfg.ctas = per_sm * (uint32_t)n_sms;
      c.cfg.log_commits = 0;
      c.cfg.max_req = std::max(base->max_req, std::max(host_sample->n_req,
                                                        host_fill ? host_fill->n_req : 0u));
      cands.push_back(c);
    }
  const size_t n = host_sample->n_req;
  std::vector<uint32_t> found(n);
  std::vector<uint32_t> vout(n * 8);
  auto run = [&](Cand& c, uint32_t times) {
    csmv_memcd_t* h = nullptr;
    csmv_status s = csmv_memcd_create(&c.cfg, &h);
    if (s != CSMV_OK) return s;
    s = csmv_memcd_clear(h);
    if (s == CSMV_OK && host_fill) {
      csmv_memcd_batch f = *host_fill;
      std::vector<uint32_t> ff(f.n_req), fv((size_t)f.n_req * 8);
      f.found = ff.data();
      f.val_out = fv.data();
      s = csmv_memcd_run(h, &f, nullptr);
    }
    for (uint32_t i = 0; i < times && s == CSMV_OK; i++) {
      csmv_memcd_batch b = *host_sample;
      b.found = found.data();
      b.val_out = vout.data();
      csmv_stats o;
      if ((s = csmv_memcd_run(h, &b, &o)) != CSMV_OK) break;
      c.ms.push_back(o.kernel_ms);
      const double cm = (double)(o.commits_update + o.commits_readonly);
      const double ab = (double)(o.aborts_data_age + o.aborts_read_write + o.aborts_prevalid +
                                 o.aborts_write_write);
      c.abort_rate = ab / std::max(1.0, ab + cm);
    }
    csmv_memcd_destroy(h);
    return s;
  };
  for (auto& c : cands) {
    c.st = run(c, 1);
    if (c.st == CSMV_OK) c.med = c.ms.back();
  }
  std::vector<size_t> order(cands.size());
  for (size_t i = 0; i < order.size(); i++) order[i] = i;
  std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return cands[a].med < cands[b].med; });
  const size_t keep = std::max<size_t>(1, cands.size() / 4);
  for (size_t r = 0; r < keep; r++) {
    Cand& c = cands[order[r]];
    if (c.st != CSMV_OK) continue;
    c.st = run(c, repeats);
    std::vector<double> m = c.ms;
    std::sort(m.begin(), m.end());
    c.med = m[m.size() / 2];
  }
  size_t best = order[0];
  for (size_t r = 0; r < keep; r++)
    if (cands[order[r]].st == CSMV_OK && cands[order[r]].med < cands[best].med) best = order[r];
  if (cands[best].st != CSMV_OK) {
    set_error("memcd autotune: no candidate ran (%s)", csmv_status_str(cands[best].st));
    return cands[best].st;
  }
  out->best = cands[best].cfg;
  out->best.log_commits = base->log_commits;
  out->best.max_req = base->max_req;
  out->n_trials = (uint32_t)cands.size();
  for (uint32_t i = 0; i < out->n_trials; i++) {
    const Cand& c = cands[i];
    csmv_tune_trial& o = out->trials[i];
    o.client_warps = c.cfg.client_warps;
    o.ctas = c.cfg.ctas;
    o.version_depth = kMemcdDepth;
    o.runs = (uint32_t)c.ms.size();
    o.status = (int32_t)c.st;
    o.tx_per_s = c.st == CSMV_OK ? (double)n / (c.med * 1e-3) : 0.0;
    o.abort_rate = c.abort_rate;
  }
  return CSMV_OK;
}

extern "C" csmv_status csmv_memcd_read_table(csmv_memcd_t* h, uint64_t* host_tags,
                                             uint32_t* host_recs) {
  csmv_status st = ready(h);
  if (st != CSMV_OK) return st;
  CSMV_CUDA(cudaSetDevice(h->cfg.device));
  const size_t nv = (size_t)h->cfg.n_sets * kWays * kMemcdDepth;
  if (host_tags) CSMV_CUDA(cudaMemcpy(host_tags, h->tag, nv * 8, cudaMemcpyDeviceToHost));
  if (host_recs) CSMV_CUDA(cudaMemcpy(host_recs, h->rec, nv * 64, cudaMemcpyDeviceToHost));
  return CSMV_OK;
}

extern "C" csmv_status csmv_memcd_read_log(csmv_memcd_t* h, uint32_t* host_log_txn, uint32_t n_log,
                                           uint32_t* host_outcome, uint32_t n_req,
                                           uint32_t* base_ts) {
  csmv_status st = ready(h);
  if (st != CSMV_OK) return st;
  if (!h->cfg.log_commits) {
    set_error("handle was created with log_commits = 0");
    return CSMV_ERR_STATE;
  }
  CSMV_CUDA(cudaSetDevice(h->cfg.device));
  const uint32_t used = h->last_final_ts - h->run_base_ts;
  if (base_ts) *base_ts = h->run_base_ts;
  if (host_log_txn) {
    if (n_log < used) {
      set_error("log buffer holds %u entries, run used %u timestamps", n_log, used);
      return CSMV_ERR_CAPACITY;
    }
    CSMV_CUDA(cudaMemcpy(host_log_txn, h->log_txn, (size_t)used * 4, cudaMemcpyDeviceToHost));
  }
  if (n_req > h->last_n_req) n_req = h->last_n_req;
  if (host_outcome)
    CSMV_CUDA(cudaMemcpy(host_outcome, h->outcome, (size_t)n_req * 4, cudaMemcpyDeviceToHost));
  return CSMV_OK;
}

extern "C" csmv_status csmv_memcd_device_info(csmv_memcd_t* h, int* n_sms, int* ctas,
                                              int* threads_per_cta, size_t* device_bytes) {
  if (!h) return CSMV_ERR_INVALID_ARG;
  if (n_sms) *n_sms = h->n_sms;
  if (ctas) *ctas = h->ctas;
  if (threads_per_cta) *threads_per_cta = h->threads;
  if (device_bytes) *device_bytes = h->device_bytes;
  return CSMV_OK;
}

extern "C" void csmv_memcd_destroy(csmv_memcd_t* h) {
  if (!h) return;
  cudaSetDevice(h->cfg.device);
  free_all(h);
  delete h;
}

// =============================================================================================
// Serving loop (csmv_serve_*): the table on the device, a persistent kernel replayed from a
// captured CUDA graph, request batches admitted from a pinned, mapped host ring as room frees up.
//
// Host-side admission: a batch of n requests is admitted when the arena has n free request
// slots (slots free when the batches holding them complete, in admission order), when it keeps
// the SETs in flight within max_inflight_sets (every SET installs a version; bounding them
// bounds how fast versions a GET still needs can be overwritten) and when fewer than 1024
// batches are in flight.
// =============================================================================================
#include <atomic>

struct csmv_serve_t {
  csmv_serve_config cfg{};
  int n_sms = 0, ctas = 0, threads = 0;
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  // table
  unsigned long long* tag = nullptr;
  uint4* rec = nullptr;
  unsigned long long* cw = nullptr;
  uint32_t* done = nullptr;
  GlobalSync* gs = nullptr;
  unsigned long long* stats = nullptr;
  uint32_t* dummy_log = nullptr;  // log/outcome pointers of the params (logging is off)
  // serving state (device)
  ServeDev* dev = nullptr;
  uint2* rq = nullptr;
  uint32_t* remaining = nullptr;
  uint32_t* tick = nullptr;
  // mapped host memory
  ServeHostCtl* ctl = nullptr;
  ServeBatchDesc* desc = nullptr;
  uint32_t *h_kind = nullptr, *h_key = nullptr, *h_val = nullptr, *h_found = nullptr,
           *h_out = nullptr, *h_outcome = nullptr;
  // commit log (log_cap > 0): the kernel's parameters are updated per session (its base ts)
  uint32_t* log_txn = nullptr;
  cudaGraphNode_t knode = nullptr;
  MemcdParams kp{};
  ServeParams ksp{};
  uint32_t base_ts = 0, end_ts = 0;
  // host bookkeeping
  bool running = false;
  uint64_t submitted = 0, retired = 0, arena_head = 0, arena_tail = 0, inflight_sets = 0;
  bool collected[kServeSlots] = {};  // polled done: its slots may be reused
};

extern "C" void csmv_serve_config_default(csmv_serve_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->n_sets = 1u << 20;
  c->client_warps = 4;
  c->ctas = 0;
  c->arena_requests = 1u << 18;
  c->max_inflight_sets = 1u << 15;
  c->idle_timeout_ms = 10000;
  c->device = 0;
  c->serial_batches = 1;
}

static void serve_free(csmv_serve_t* h) {
  if (h->exec) cudaGraphExecDestroy(h->exec);
  if (h->graph) cudaGraphDestroy(h->graph);
  void* dptr[] = {h->tag, h->rec, h->cw, h->done, h->gs, h->stats, h->dummy_log,
                  h->dev, h->rq, h->remaining, h->tick, h->log_txn};
  for (void* p : dptr) cudaFree(p);
  void* hptr[] = {h->ctl, h->desc, h->h_kind, h->h_key, h->h_val, h->h_found, h->h_out,
                  h->h_outcome};
  for (void* p : hptr)
    if (p) cudaFreeHost(p);
  if (h->stream) cudaStreamDestroy(h->stream);
}

template <class T>
static T* dev_ptr_of(T* host) {
  void* d = nullptr;
  if (cudaHostGetDevicePointer(&d, host, 0) != cudaSuccess) return nullptr;
  return static_cast<T*>(d);
}

extern "C" csmv_status csmv_serve_create(const csmv_serve_config* cfg, csmv_serve_t** out) {
  if (!out || !cfg) return CSMV_ERR_INVALID_ARG;
  *out = nullptr;
  const uint32_t A = cfg->arena_requests;
  if (cfg->n_sets < 1 || cfg->n_sets > (1u << 26) || cfg->client_warps < 1 ||
      cfg->client_warps > (uint32_t)kMaxClientWarps || A < 1024 || (A & (A - 1)) ||
      A > (1u << 24) || cfg->max_inflight_sets == 0 || cfg->idle_timeout_ms == 0) {
    set_error("invalid serve config (arena_requests: power of two 1024..2^24)");
    return CSMV_ERR_INVALID_ARG;
  }
  int n_sms = 0;
  csmv_status st = check_device(cfg->device, &n_sms);
  if (st != CSMV_OK) return st;
  CSMV_CUDA(cudaSetDevice(cfg->device));
  csmv_serve_t* h = new csmv_serve_t;
  h->cfg = *cfg;
  h->n_sms = n_sms;
  h->threads = (int)(cfg->client_warps + 1) * 32;
  auto fail = [&](csmv_status s) {
    serve_free(h);
    delete h;
    return s;
  };
  int per_sm = 0;
  if ((st = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, memcd_serve_kernel,
                                                                       h->threads, 0),
                        "occupancy")) != CSMV_OK)
    return fail(st);
  const int max_ctas = per_sm * n_sms;
  h->ctas = cfg->ctas ? (int)cfg->ctas : max_ctas;
  if (h->ctas < 1 || h->ctas > max_ctas) {
    set_error("%d CTAs requested, %d can be co-resident", h->ctas, max_ctas);
    return fail(CSMV_ERR_INVALID_ARG);
  }
  const size_t ent = (size_t)cfg->n_sets * kWays, D = kMemcdDepth;
  const uint32_t qcap = A / 32;  // rounds of a full arena
  struct {
    void** p;
    size_t bytes;
  } dallocs[] = {
      {(void**)&h->tag, ent * D * 8}, {(void**)&h->rec, ent * D * 64}, {(void**)&h->cw, ent * 8},
      {(void**)&h->done, (size_t)kDoneWords * 4}, {(void**)&h->gs, sizeof(GlobalSync)},
      {(void**)&h->stats, ST_COUNT * 8}, {(void**)&h->dummy_log, 64},
      {(void**)&h->dev, sizeof(ServeDev)}, {(void**)&h->rq, (size_t)qcap * 8},
      {(void**)&h->remaining, kServeSlots * 4}, {(void**)&h->tick, kServeSlots * 4},
  };
  for (auto& a : dallocs)
    if ((st = cuda_status(cudaMalloc(a.p, a.bytes), "cudaMalloc")) != CSMV_OK) return fail(st);
  struct {
    void** p;
    size_t bytes;
  } hallocs[] = {
      {(void**)&h->ctl, sizeof(ServeHostCtl)}, {(void**)&h->desc, kServeSlots * sizeof(ServeBatchDesc)},
      {(void**)&h->h_kind, (size_t)A * 4}, {(void**)&h->h_key, (size_t)A * 16},
      {(void**)&h->h_val, (size_t)A * 32}, {(void**)&h->h_found, (size_t)A * 4},
      {(void**)&h->h_out, (size_t)A * 32},
  };
  for (auto& a : hallocs)
    if ((st = cuda_status(cudaHostAlloc(a.p, a.bytes, cudaHostAllocMapped), "cudaHostAlloc")) != CSMV_OK)
      return fail(st);
  if (cfg->log_cap) {
    if ((st = cuda_status(cudaMalloc(&h->log_txn, (size_t)cfg->log_cap * 4), "cudaMalloc")) != CSMV_OK ||
        (st = cuda_status(cudaHostAlloc(&h->h_outcome, (size_t)A * 4, cudaHostAllocMapped),
                          "cudaHostAlloc")) != CSMV_OK)
      return fail(st);
  }
  std::memset(h->ctl, 0, sizeof(ServeHostCtl));
  std::memset(h->desc, 0, kServeSlots * sizeof(ServeBatchDesc));
  if ((st = cuda_status(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "stream")) != CSMV_OK)
    return fail(st);
  // empty table (memcdSH.cu:567-574), commit order at 0
  memcd_clear_kernel<<<n_sms * 4, 256, 0, h->stream>>>(h->tag, ent * D);
  if ((st = cuda_status(cudaGetLastError(), "clear")) != CSMV_OK ||
      (st = cuda_status(cudaMemsetAsync(h->rec, 0, ent * D * 64, h->stream), "memset")) != CSMV_OK ||
      (st = cuda_status(cudaMemsetAsync(h->cw, 0, ent * 8, h->stream), "memset")) != CSMV_OK ||
      (st = cuda_status(cudaMemsetAsync(h->done, 0, (size_t)kDoneWords * 4, h->stream), "memset")) != CSMV_OK ||
      (st = cuda_status(cudaMemsetAsync(h->gs, 0, sizeof(GlobalSync), h->stream), "memset")) != CSMV_OK ||
      (st = cuda_status(cudaStreamSynchronize(h->stream), "sync")) != CSMV_OK)
    return fail(st);
  // the session graph: reset the serving cursors and statistics, run the persistent kernel
  MemcdParams p{};
  p.kind = dev_ptr_of(h->h_kind);
  p.key = reinterpret_cast<const uint4*>(dev_ptr_of(h->h_key));
  p.val = reinterpret_cast<const uint4*>(dev_ptr_of(h->h_val));
  p.found = dev_ptr_of(h->h_found);
  p.val_out = reinterpret_cast<uint4*>(dev_ptr_of(h->h_out));
  ServeParams sp{};
  sp.ctl = dev_ptr_of(h->ctl);
  sp.desc = dev_ptr_of(h->desc);
  if (!p.kind || !p.key || !p.val || !p.found || !p.val_out || !sp.ctl || !sp.desc) {
    set_error("cudaHostGetDevicePointer failed");
    return fail(CSMV_ERR_CUDA);
  }
  p.n_rounds = 0;
  p.tick = 1;
  p.n_sets = cfg->n_sets;
  p.tag = h->tag;
  p.rec = h->rec;
  p.cw = h->cw;
  p.done = h->done;
  p.done_mask = kDoneWords - 1;
  p.gs = h->gs;
  p.log_txn = h->dummy_log;
  p.outcome = h->dummy_log;
  p.log = 0;
  p.log_base = 0;
  p.log_cap = 1;
  if (cfg->log_cap) {  // the base timestamp is set per session (csmv_serve_start)
    p.log_txn = h->log_txn;
    p.outcome = dev_ptr_of(h->h_outcome);
    p.log = 1;
    p.log_cap = cfg->log_cap;
    if (!p.outcome) {
      set_error("cudaHostGetDevicePointer failed");
      return fail(CSMV_ERR_CUDA);
    }
  }
  p.stats = h->stats;
  p.nc = cfg->client_warps;
  p.batch = CSMV_BATCH_CTA;
  p.spin_log2 = 24;
  sp.dev = h->dev;
  sp.rq = h->rq;
  sp.q_mask = qcap - 1;
  sp.arena_mask = A - 1;
  sp.remaining = h->remaining;
  sp.tick = h->tick;
  sp.idle_ns = (unsigned long long)cfg->idle_timeout_ms * 1000000ull;
  sp.serial = cfg->serial_batches ? 1u : 0u;
  cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) e = cudaMemsetAsync(h->dev, 0, sizeof(ServeDev), h->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(&h->gs->round_next, 0, 4, h->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(&h->gs->error, 0, 4, h->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(h->stats, 0, ST_COUNT * 8, h->stream);
  if (e == cudaSuccess) {
    memcd_serve_kernel<<<h->ctas, h->threads, 0, h->stream>>>(p, sp);
    e = cudaGetLastError();
  }
  cudaGraph_t g = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(h->stream, &g);
  if (e == cudaSuccess) e = e2;
  h->graph = g;
  if ((st = cuda_status(e, "capture of the serving graph")) != CSMV_OK) return fail(st);
  if ((st = cuda_status(cudaGraphInstantiate(&h->exec, h->graph, 0), "cudaGraphInstantiate")) != CSMV_OK)
    return fail(st);
  h->kp = p;
  h->ksp = sp;
  if (cfg->log_cap) {  // the kernel node, whose parameters each session updates
    cudaGraphNode_t nodes[8];
    size_t n_nodes = 8;
    if ((st = cuda_status(cudaGraphGetNodes(h->graph, nodes, &n_nodes), "cudaGraphGetNodes")) != CSMV_OK)
      return fail(st);
    for (size_t i = 0; i < n_nodes; i++) {
      cudaGraphNodeType ty;
      if (cudaGraphNodeGetType(nodes[i], &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel)
        h->knode = nodes[i];
    }
    if (!h->knode) {
      set_error("serving graph without a kernel node");
      return fail(CSMV_ERR_CUDA);
    }
  }
  *out = h;
  return CSMV_OK;
}

extern "C" csmv_status csmv_serve_start(csmv_serve_t* h) {
  if (!h) return CSMV_ERR_INVALID_ARG;
  if (h->running) {
    set_error("serving session already running");
    return CSMV_ERR_STATE;
  }
  CSMV_CUDA(cudaSetDevice(h->cfg.device));
  std::memset(h->ctl, 0, sizeof(ServeHostCtl));
  std::memset(h->desc, 0, kServeSlots * sizeof(ServeBatchDesc));
  std::atomic_thread_fence(std::memory_order_seq_cst);
  h->submitted = h->retired = h->arena_head = h->arena_tail = h->inflight_sets = 0;
  if (h->cfg.log_cap) {  // this session's log starts after the last timestamp drawn so far
    GlobalSync gs;
    CSMV_CUDA(cudaMemcpy(&gs, h->gs, sizeof(gs), cudaMemcpyDeviceToHost));
    h->base_ts = h->end_ts = gs.ts_next;
    CSMV_CUDA(cudaMemset(h->log_txn, 0xFF, (size_t)h->cfg.log_cap * 4));
    h->kp.log_base = h->base_ts;
    void* args[] = {&h->kp, &h->ksp};
    cudaKernelNodeParams kn{};
    kn.func = (void*)memcd_serve_kernel;
    kn.gridDim = dim3(h->ctas);
    kn.blockDim = dim3(h->threads);
    kn.sharedMemBytes = 0;
    kn.kernelParams = args;
    CSMV_CUDA(cudaGraphExecKernelNodeSetParams(h->exec, h->knode, &kn));
  }
  CSMV_CUDA(cudaGraphLaunch(h->exec, h->stream));
  h->running = true;
  return CSMV_OK;
}

static bool batch_done(const csmv_serve_t* h, uint64_t b) {
  const volatile uint32_t* d = &h->desc[b % kServeSlots].done;
  const bool done = *d != 0u;
  std::atomic_thread_fence(std::memory_order_acquire);
  return done;
}

// Retire collected batches in admission order (frees arena slots and the SET budget).
static void serve_retire(csmv_serve_t* h) {
  while (h->retired < h->submitted && h->collected[h->retired % kServeSlots]) {
    const ServeBatchDesc& d = h->desc[h->retired % kServeSlots];
    h->arena_tail += d.n_req;
    h->inflight_sets -= d.sets;
    h->retired++;
  }
}

extern "C" csmv_status csmv_serve_submit(csmv_serve_t* h, const csmv_memcd_batch* b,
                                         uint64_t* batch_id) {
  if (!h || !b || !b->kind || !b->key || !b->val || b->n_req == 0 || b->n_req % 32) {
    set_error("serve submit: n_req must be a positive multiple of 32 with kind/key/val set");
    return CSMV_ERR_INVALID_ARG;
  }
  if (!h->running) {
    set_error("serve submit: no session running");
    return CSMV_ERR_STATE;
  }
  if (const uint32_t err = *reinterpret_cast<volatile uint32_t*>(&h->ctl->error)) {
    set_error("serving kernel stopped with device error %u", err);
    return CSMV_ERR_TIMEOUT;
  }
  const uint32_t A = h->cfg.arena_requests, n = b->n_req;
  if (n > A) {
    set_error("batch of %u requests exceeds the arena (%u)", n, A);
    return CSMV_ERR_INVALID_ARG;
  }
  uint32_t sets = 0;
  for (uint32_t i = 0; i < n; i++) sets += b->kind[i] == CSMV_MEMCD_SET;
  serve_retire(h);
  if (h->arena_head + n - h->arena_tail > A || h->inflight_sets + sets > h->cfg.max_inflight_sets ||
      h->submitted - h->retired >= kServeSlots) {
    set_error("serve submit: no room (arena slots, SET budget or descriptors); retry later");
    return CSMV_ERR_CAPACITY;
  }
  const uint32_t first = (uint32_t)(h->arena_head & (A - 1));
  const uint32_t n1 = std::min(n, A - first), n2 = n - n1;
  std::memcpy(h->h_kind + first, b->kind, (size_t)n1 * 4);
  std::memcpy(h->h_key + (size_t)first * 4, b->key, (size_t)n1 * 16);
  std::memcpy(h->h_val + (size_t)first * 8, b->val, (size_t)n1 * 32);
  if (n2) {
    std::memcpy(h->h_kind, b->kind + n1, (size_t)n2 * 4);
    std::memcpy(h->h_key, b->key + (size_t)n1 * 4, (size_t)n2 * 16);
    std::memcpy(h->h_val, b->val + (size_t)n1 * 8, (size_t)n2 * 32);
  }
  ServeBatchDesc& d = h->desc[h->submitted % kServeSlots];
  h->collected[h->submitted % kServeSlots] = false;
  d.first = first;
  d.n_req = n;
  d.tick = b->tick;
  d.seq = (uint32_t)h->submitted;
  d.sets = sets;
  d.admit_ns = d.done_ns = 0;
  d.done = 0;
  std::atomic_thread_fence(std::memory_order_seq_cst);  // requests and descriptor, then publish
  *reinterpret_cast<volatile uint32_t*>(&h->ctl->submitted) = (uint32_t)(h->submitted + 1);
  if (batch_id) *batch_id = h->submitted;
  h->submitted++;
  h->arena_head += n;
  h->inflight_sets += sets;
  return CSMV_OK;
}

extern "C" csmv_status csmv_serve_poll(csmv_serve_t* h, uint64_t batch_id, uint32_t* done,
                                       uint32_t* host_found, uint32_t* host_val_out,
                                       uint64_t* device_ns) {
  return csmv_serve_poll_logged(h, batch_id, done, host_found, host_val_out, nullptr, device_ns);
}

extern "C" csmv_status csmv_serve_poll_logged(csmv_serve_t* h, uint64_t batch_id, uint32_t* done,
                                              uint32_t* host_found, uint32_t* host_val_out,
                                              uint32_t* host_outcome, uint64_t* device_ns) {
  if (!h || !done) return CSMV_ERR_INVALID_ARG;
  if (host_outcome && !h->cfg.log_cap) {
    set_error("outcomes are kept only with log_cap > 0");
    return CSMV_ERR_STATE;
  }
  *done = 0;
  if (batch_id >= h->submitted) {
    set_error("batch %llu not submitted", (unsigned long long)batch_id);
    return CSMV_ERR_INVALID_ARG;
  }
  if (batch_id < h->retired) {  // collected earlier and its slots reused: done, no results
    *done = 1;
    return CSMV_OK;
  }
  if (!batch_done(h, batch_id)) {
    const uint32_t err = *reinterpret_cast<volatile uint32_t*>(&h->ctl->error);
    if (err) {  // the session stopped on a device error: this batch will not complete
      set_error("serving kernel stopped with device error %u", err);
      return CSMV_ERR_TIMEOUT;
    }
    return CSMV_OK;
  }
  h->collected[batch_id % kServeSlots] = true;
  const ServeBatchDesc& d = h->desc[batch_id % kServeSlots];
  const uint32_t A = h->cfg.arena_requests, n = d.n_req, first = d.first;
  const uint32_t n1 = std::min(n, A - first), n2 = n - n1;
  if (host_found) {
    std::memcpy(host_found, h->h_found + first, (size_t)n1 * 4);
    if (n2) std::memcpy(host_found + n1, h->h_found, (size_t)n2 * 4);
  }
  if (host_val_out) {
    std::memcpy(host_val_out, h->h_out + (size_t)first * 8, (size_t)n1 * 32);
    if (n2) std::memcpy(host_val_out + (size_t)n1 * 8, h->h_out, (size_t)n2 * 32);
  }
  if (host_outcome) {
    std::memcpy(host_outcome, h->h_outcome + first, (size_t)n1 * 4);
    if (n2) std::memcpy(host_outcome + n1, h->h_outcome, (size_t)n2 * 4);
  }
  if (device_ns) *device_ns = d.done_ns > d.admit_ns ? d.done_ns - d.admit_ns : 0;
  *done = 1;
  return CSMV_OK;
}

extern "C" csmv_status csmv_serve_stop(csmv_serve_t* h, csmv_stats* out) {
  if (!h) return CSMV_ERR_INVALID_ARG;
  if (!h->running) {
    set_error("no serving session running");
    return CSMV_ERR_STATE;
  }
  CSMV_CUDA(cudaSetDevice(h->cfg.device));
  std::atomic_thread_fence(std::memory_order_seq_cst);
  *reinterpret_cast<volatile uint32_t*>(&h->ctl->stop) = 1u;
  cudaError_t e = cudaStreamSynchronize(h->stream);
  h->running = false;
  CSMV_CUDA(e);
  unsigned long long st[ST_COUNT];
  GlobalSync gs;
  CSMV_CUDA(cudaMemcpy(st, h->stats, sizeof(st), cudaMemcpyDeviceToHost));
  CSMV_CUDA(cudaMemcpy(&gs, h->gs, sizeof(gs), cudaMemcpyDeviceToHost));
  serve_retire(h);
  h->end_ts = gs.ts_next;
  if (out) {
    std::memset(out, 0, sizeof(*out));
    out->commits_update = st[ST_COMMIT_UPDATE];
    out->commits_readonly = st[ST_COMMIT_RO];
    out->aborts_data_age = st[ST_ABORT_DATA_AGE];
    out->aborts_read_write = st[ST_ABORT_READ_WRITE];
    out->aborts_prevalid = st[ST_ABORT_PREVALID];
    out->aborts_write_write = st[ST_ABORT_WRITE_WRITE];
    out->sections = st[ST_SECTIONS];
    out->rounds = st[ST_ROUNDS];
    out->final_ts = gs.ts_next;
    out->error = gs.error;
  }
  if (gs.error) {
    set_error("serving kernel ended with device error %u (4: idle timeout)", gs.error);
    return CSMV_ERR_TIMEOUT;
  }
  return CSMV_OK;
}

extern "C" csmv_status csmv_serve_read_log(csmv_serve_t* h, uint32_t* host_log_txn, uint32_t n_log,
                                           uint32_t* n_used, uint32_t* base_ts) {
  if (!h) return CSMV_ERR_INVALID_ARG;
  if (!h->cfg.log_cap) {
    set_error("serving handle was created with log_cap = 0");
    return CSMV_ERR_STATE;
  }
  if (h->running) {
    set_error("stop the serving session first");
    return CSMV_ERR_STATE;
  }
  CSMV_CUDA(cudaSetDevice(h->cfg.device));
  const uint32_t used = h->end_ts - h->base_ts;
  if (n_used) *n_used = used;
  if (base_ts) *base_ts = h->base_ts;
  if (used > h->cfg.log_cap) {
    set_error("the session drew %u timestamps, the log holds %u", used, h->cfg.log_cap);
    return CSMV_ERR_CAPACITY;
  }
  if (host_log_txn) {
    if (n_log < used) {
      set_error("log buffer holds %u entries, the session used %u timestamps", n_log, used);
      return CSMV_ERR_CAPACITY;
    }
    CSMV_CUDA(cudaMemcpy(host_log_txn, h->log_txn, (size_t)used * 4, cudaMemcpyDeviceToHost));
  }
  return CSMV_OK;
}

extern "C" csmv_status csmv_serve_read_table(csmv_serve_t* h, uint64_t* host_tags,
                                             uint32_t* host_recs) {
  if (!h) return CSMV_ERR_INVALID_ARG;
  if (h->running) {
    set_error("stop the serving session first");
    return CSMV_ERR_STATE;
  }
  CSMV_CUDA(cudaSetDevice(h->cfg.device));
  const size_t nv = (size_t)h->cfg.n_sets * kWays * kMemcdDepth;
  if (host_tags) CSMV_CUDA(cudaMemcpy(host_tags, h->tag, nv * 8, cudaMemcpyDeviceToHost));
  if (host_recs) CSMV_CUDA(cudaMemcpy(host_recs, h->rec, nv * 64, cudaMemcpyDeviceToHost));
  return CSMV_OK;
}

extern "C" void csmv_serve_destroy(csmv_serve_t* h) {
  if (!h) return;
  cudaSetDevice(h->cfg.device);
  if (h->running) {
    *reinterpret_cast<volatile uint32_t*>(&h->ctl->stop) = 1u;
    cudaStreamSynchronize(h->stream);
  }
  serve_free(h);
  delete h;
}
