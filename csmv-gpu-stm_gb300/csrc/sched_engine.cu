// sched_engine.cu - the learned conflict scheduler (include/csmv.h, csmv_sched_*).
//
// It changes only the ORDER in which a chunk's transactions reach the unchanged commit engine
// (and, optionally, which ones wait in the engine's deferred queue): every transaction still
// runs through csmv_bank_run_device and is validated there, so results stay exactly those of a
// serial execution in commit order.
//
// Per chunk: (1) probe - the first probe_rounds_pct % of the rounds run in stream order with
// per-transaction abort counts; those transfers (features, aborted?) train the network for
// train_steps Adam steps, and their per-bin abort rates refresh the recent-abort features;
// (2) plan - the network scores the rest, flagged transfers are spread out by key
// (sched_kernels.cuh), and the planned stream runs.
#include <algorithm>
#include <chrono>
#include <cstring>

#include "common.h"
#include "sched_kernels.cuh"

using namespace csmv;

// network launchers (mlp_engine.cu)
csmv_status csmv_mlp_launch_forward(csmv_mlp_t* h, uint32_t n, const void* dev_x, float* dev_p,
                                    cudaStream_t stream);
csmv_status csmv_mlp_launch_grad(csmv_mlp_t* h, uint32_t n, const void* dev_x, const float* dev_y,
                                 cudaStream_t stream);
csmv_status csmv_mlp_launch_adam(csmv_mlp_t* h, float lr, cudaStream_t stream);
float* csmv_mlp_loss_ptr(csmv_mlp_t* h);

struct csmv_sched_t {
  csmv_sched_config cfg{};
  int n_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[4] = {};
  csmv_mlp_t* mlp = nullptr;
  uint32_t *sketch = nullptr, *key_count = nullptr, *key_rank = nullptr;
  uint4* x = nullptr;
  float *y = nullptr, *p = nullptr, *rates = nullptr;
  uint32_t* aborts = nullptr;
  unsigned long long* bin_stats = nullptr;
  uint32_t *key = nullptr, *bucket = nullptr, *bucket_count = nullptr, *bucket_start = nullptr,
           *bucket_fill = nullptr;
  uint32_t *order = nullptr, *perm = nullptr, *op2 = nullptr, *off2 = nullptr;
  uint32_t *ro_flag = nullptr, *ro_scan = nullptr, *ro_list = nullptr, *n_flagged = nullptr;
  uint32_t* waits = nullptr;  // probe: per-transaction lock waits of the engine
  // grouped plan (plan 1)
  uint32_t *hidx = nullptr, *key_start = nullptr, *tile_sum = nullptr, *tile_off = nullptr;
  uint32_t *rank = nullptr, *cold_pos = nullptr, *sorted = nullptr, *rbucket = nullptr;
  uint32_t *round_order = nullptr, *bo = nullptr, *bo2 = nullptr, *max_count = nullptr;
  uint8_t* lock_last = nullptr;  // heat classes of the bank's accounts (hot_last)
  uint32_t *lane_of = nullptr, *lane_count = nullptr, *lanes = nullptr;  // hot lanes (plan 1)
  uint32_t lock_last_n = 0;
  uint64_t chunks = 0;
  // the current chunk
  uint32_t n = 0, probe_rounds = 0, split_round = 0, planned = 0, serial_rounds = 0;
  bool probed = false;
};

extern "C" void csmv_sched_config_default(csmv_sched_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->n_accounts = 1u << 20;
  c->max_txn = 1u << 20;
  c->probe_rounds_pct = 5;
  c->probe_every = 1;
  c->train_steps = 2;
  c->lr = 3e-3f;
  c->threshold = 0.05f;
  c->defer_threshold = 2.0f;  // > 1: no deferral
  c->deferred_warps = 64;
  c->serial_lane = 0;
  c->seed = 1;
  c->device = 0;
  c->plan = 1;
  c->hot_count = 0;
  c->score = 0;
  c->backoff_ns = 2048;
  c->hot_last = 1;
  c->key_written = 1;
  c->hot_lanes = 0;
}

static void free_all(csmv_sched_t* s) {
  void* bufs[] = {s->sketch, s->key_count, s->key_rank, s->x, s->y, s->p, s->rates, s->aborts,
                  s->bin_stats, s->key, s->bucket, s->bucket_count, s->bucket_start,
                  s->bucket_fill, s->order, s->perm, s->op2, s->off2, s->ro_flag, s->ro_scan,
                  s->ro_list, s->n_flagged, s->waits, s->hidx, s->key_start, s->tile_sum,
                  s->tile_off, s->rank, s->cold_pos, s->sorted, s->rbucket, s->round_order,
                  s->bo, s->bo2, s->max_count, s->lock_last, s->lane_of, s->lane_count,
                  s->lanes};
  for (void* b : bufs) cudaFree(b);
  for (auto& e : s->ev)
    if (e) cudaEventDestroy(e);
  if (s->stream) cudaStreamDestroy(s->stream);
  if (s->mlp) csmv_mlp_destroy(s->mlp);
}

extern "C" csmv_status csmv_sched_create(const csmv_sched_config* cfg, csmv_sched_t** out) {
  if (!out || !cfg) return CSMV_ERR_INVALID_ARG;
  *out = nullptr;
  if (cfg->n_accounts < 2 || cfg->max_txn == 0 || cfg->max_txn % 32 || cfg->max_txn > (1u << 26) ||
      cfg->probe_rounds_pct > 100 || cfg->probe_every == 0 || !(cfg->lr > 0.f) ||
      cfg->deferred_warps == 0 || cfg->serial_lane > 2 || cfg->plan > 1 || cfg->score > 1) {
    set_error("invalid scheduler config");
    return CSMV_ERR_INVALID_ARG;
  }
  int n_sms = 0;
  csmv_status st = check_device(cfg->device, &n_sms);
  if (st != CSMV_OK) return st;
  CSMV_CUDA(cudaSetDevice(cfg->device));
  csmv_sched_t* s = new csmv_sched_t;
  s->cfg = *cfg;
  s->n_sms = n_sms;
  auto fail = [&](csmv_status e) {
    free_all(s);
    delete s;
    return e;
  };
  if ((st = csmv_mlp_create(cfg->device, cfg->seed, &s->mlp)) != CSMV_OK) return fail(st);
  const size_t n = cfg->max_txn, R = n / 32 + 2, SK = (size_t)1 << kSketchLog2;
  struct {
    void** p;
    size_t bytes;
  } allocs[] = {
      {(void**)&s->sketch, SK * 4},      {(void**)&s->key_count, SK * 4},
      {(void**)&s->key_rank, SK * 4},    {(void**)&s->x, n * 128},
      {(void**)&s->y, n * 4},            {(void**)&s->p, n * 4},
      {(void**)&s->rates, kRateBins * 4}, {(void**)&s->aborts, n * 4},
      {(void**)&s->bin_stats, kRateBins * 16}, {(void**)&s->key, n * 4},
      {(void**)&s->bucket, n * 4},       {(void**)&s->bucket_count, (R + kMaxLanes) * 4},
      {(void**)&s->bucket_start, (R + kMaxLanes) * 4}, {(void**)&s->bucket_fill, (R + kMaxLanes) * 4},
      {(void**)&s->lane_of, (size_t)kHotNone * 4}, {(void**)&s->lane_count, 4},
      {(void**)&s->lanes, (kMaxLanes + 1) * 4},
      {(void**)&s->order, n * 4},        {(void**)&s->perm, n * 4},
      {(void**)&s->op2, n * 4},          {(void**)&s->off2, n * 4},
      {(void**)&s->ro_flag, R * 4},      {(void**)&s->ro_scan, R * 4},
      {(void**)&s->ro_list, R * 4},      {(void**)&s->n_flagged, 4},
      {(void**)&s->waits, n * 4},
      {(void**)&s->hidx, (SK + 1) * 4},  {(void**)&s->key_start, (SK + 1) * 4},
      {(void**)&s->tile_sum, 65537 * 4}, {(void**)&s->tile_off, 65537 * 4},
      {(void**)&s->rank, n * 4},         {(void**)&s->cold_pos, (n + 1) * 4},
      {(void**)&s->sorted, n * 4},       {(void**)&s->rbucket, R * 4},
      {(void**)&s->round_order, R * 4},  {(void**)&s->bo, n * 4},
      {(void**)&s->bo2, n * 4},          {(void**)&s->max_count, 4},
  };
  for (auto& a : allocs)
    if ((st = cuda_status(cudaMalloc(a.p, a.bytes), "cudaMalloc")) != CSMV_OK) return fail(st);
  if ((st = cuda_status(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "stream")) != CSMV_OK)
    return fail(st);
  for (auto& e : s->ev)
    if ((st = cuda_status(cudaEventCreate(&e), "event")) != CSMV_OK) return fail(st);
  if ((st = cuda_status(cudaMemsetAsync(s->rates, 0, kRateBins * 4, s->stream), "memset")) != CSMV_OK ||
      (st = cuda_status(cudaMemsetAsync(s->bin_stats, 0, kRateBins * 16, s->stream), "memset")) != CSMV_OK ||
      (st = cuda_status(cudaStreamSynchronize(s->stream), "sync")) != CSMV_OK)
    return fail(st);
  *out = s;
  return CSMV_OK;
}

static csmv_status check_chunk(csmv_sched_t* s, const csmv_bank_stream* d) {
  if (!d || !d->op || !d->off || !d->addr || d->n_txn == 0 || d->n_txn % 32) {
    set_error("scheduler: chunk needs n_txn a positive multiple of 32 and op/off/addr");
    return CSMV_ERR_INVALID_ARG;
  }
  if (d->n_txn > s->cfg.max_txn) {
    set_error("scheduler: chunk of %u transactions exceeds max_txn %u", d->n_txn, s->cfg.max_txn);
    return CSMV_ERR_CAPACITY;
  }
  return CSMV_OK;
}

static uint32_t grid_for(const csmv_sched_t* s, uint32_t n) {
  const uint32_t g = (n + 255) / 256, cap = (uint32_t)s->n_sms * 8;
  return g == 0 ? 1 : (g < cap ? g : cap);
}

#define SCHED_LAUNCH_CHECK(what) CSMV_CUDA(cudaGetLastError())

// Exclusive scan of n counters into out[0..n] (out[n] = total), any n <= 2^28.
static csmv_status scan_multi(csmv_sched_t* s, const uint32_t* in, uint32_t n, uint32_t* out) {
  const uint32_t tiles = (n + kScanTile - 1u) / kScanTile;
  sched_scan_tiles_kernel<<<tiles ? tiles : 1u, 1024, 0, s->stream>>>(in, n, out, s->tile_sum);
  SCHED_LAUNCH_CHECK("scan tiles");
  sched_scan_kernel<<<1, 1024, 0, s->stream>>>(s->tile_sum, tiles, s->tile_off);
  SCHED_LAUNCH_CHECK("scan tile sums");
  sched_scan_add_kernel<<<grid_for(s, n + 1u), 256, 0, s->stream>>>(out, n, s->tile_off, tiles);
  SCHED_LAUNCH_CHECK("scan add");
  return CSMV_OK;
}

extern "C" csmv_status csmv_sched_probe(csmv_sched_t* s, csmv_bank_t* bank,
                                        const csmv_bank_stream* d, csmv_sched_report* rep) {
  if (!s || !bank) return CSMV_ERR_INVALID_ARG;
  csmv_status st = check_chunk(s, d);
  if (st != CSMV_OK) return st;
  CSMV_CUDA(cudaSetDevice(s->cfg.device));
  const uint32_t n = d->n_txn, R = n / 32;
  uint32_t P = (uint32_t)(((uint64_t)R * s->cfg.probe_rounds_pct + 99) / 100);
  if (P > R) P = R;
  if (s->chunks % s->cfg.probe_every) P = 0;  // this chunk is planned with the model as it is
  s->n = n;
  s->probe_rounds = P;
  s->probed = true;
  s->planned = 0;
  s->split_round = 0;
  s->serial_rounds = 0;
  if (rep) std::memset(rep, 0, sizeof(*rep));
  // hashed access counts of the whole chunk
  CSMV_CUDA(cudaMemsetAsync(s->sketch, 0, ((size_t)1 << kSketchLog2) * 4, s->stream));
  sched_count_kernel<<<grid_for(s, n), 256, 0, s->stream>>>(d->op, d->off, d->addr, n, s->sketch);
  SCHED_LAUNCH_CHECK("count");
  if (P == 0) return cuda_status(cudaStreamSynchronize(s->stream), "sync");
  const uint32_t np = P * 32;
  sched_features_kernel<<<grid_for(s, np), 256, 0, s->stream>>>(
      d->op, d->off, d->addr, 0, np, s->cfg.n_accounts, s->sketch, s->rates, s->x);
  SCHED_LAUNCH_CHECK("features");
  CSMV_CUDA(cudaStreamSynchronize(s->stream));
  // the probe slice in stream order, with per-transaction abort counts
  csmv_bank_stream ps = *d;
  ps.n_txn = np;
  ps.txn_aborts = s->aborts;
  ps.txn_waits = s->waits;
  ps.backoff = nullptr;
  ps.lock_last = nullptr;
  ps.lane_start = nullptr;
  ps.split_round = 0;
  ps.deferred_warps = 0;
  csmv_stats bst;
  st = csmv_bank_run_device(bank, &ps, &bst);
  if (rep) rep->probe = bst;
  if (st != CSMV_OK) return st;
  // labels, recent abort rates, training
  CSMV_CUDA(cudaEventRecord(s->ev[0], s->stream));
  sched_labels_kernel<<<grid_for(s, np), 256, 0, s->stream>>>(
      d->op, d->off, d->addr, np, s->cfg.n_accounts, s->aborts, s->waits, s->y, s->bin_stats);
  SCHED_LAUNCH_CHECK("labels");
  sched_rates_kernel<<<1, kRateBins, 0, s->stream>>>(s->bin_stats, s->rates);
  SCHED_LAUNCH_CHECK("rates");
  float loss = 0.f;
  for (uint32_t k = 0; k < s->cfg.train_steps; k++) {
    if ((st = csmv_mlp_launch_grad(s->mlp, np, s->x, s->y, s->stream)) != CSMV_OK) return st;
    if (k == 0) CSMV_CUDA(cudaMemcpyAsync(&loss, csmv_mlp_loss_ptr(s->mlp), 4, cudaMemcpyDeviceToHost, s->stream));
    if ((st = csmv_mlp_launch_adam(s->mlp, s->cfg.lr, s->stream)) != CSMV_OK) return st;
  }
  CSMV_CUDA(cudaEventRecord(s->ev[1], s->stream));
  CSMV_CUDA(cudaStreamSynchronize(s->stream));
  if (rep) {
    float ms = 0.f;
    CSMV_CUDA(cudaEventElapsedTime(&ms, s->ev[0], s->ev[1]));
    rep->train_ms = ms;
    rep->loss = s->cfg.train_steps ? loss / (float)np : 0.f;
    rep->n_probe = np;
  }
  return CSMV_OK;
}

extern "C" csmv_status csmv_sched_plan_run(csmv_sched_t* s, csmv_bank_t* bank,
                                           const csmv_bank_stream* d, csmv_sched_report* rep) {
  if (!s || !bank) return CSMV_ERR_INVALID_ARG;
  csmv_status st = check_chunk(s, d);
  if (st != CSMV_OK) return st;
  if (!s->probed || d->n_txn != s->n) {
    set_error("scheduler: csmv_sched_probe must come first, on the same chunk");
    return CSMV_ERR_STATE;
  }
  s->probed = false;
  CSMV_CUDA(cudaSetDevice(s->cfg.device));
  const uint32_t n = d->n_txn, R = n / 32, P = s->probe_rounds, t0 = P * 32, n1 = n - t0;
  if (n1 == 0) return CSMV_OK;
  const uint32_t Rp = R - P;  // planned rounds
  CSMV_CUDA(cudaEventRecord(s->ev[2], s->stream));
  sched_features_kernel<<<grid_for(s, n1), 256, 0, s->stream>>>(
      d->op, d->off, d->addr, t0, n, s->cfg.n_accounts, s->sketch, s->rates, s->x);
  SCHED_LAUNCH_CHECK("features");
  if ((st = csmv_mlp_launch_forward(s->mlp, n1, s->x + (size_t)t0 * 8, s->p, s->stream)) != CSMV_OK)
    return st;
  // read-only rounds of the planned part
  sched_ro_flags_kernel<<<grid_for(s, Rp), 256, 0, s->stream>>>(d->op, P, R, s->ro_flag);
  SCHED_LAUNCH_CHECK("ro_flags");
  sched_scan_kernel<<<1, 1024, 0, s->stream>>>(s->ro_flag, Rp, s->ro_scan);
  SCHED_LAUNCH_CHECK("scan");
  uint32_t r_ro = 0;
  CSMV_CUDA(cudaMemcpyAsync(&r_ro, s->ro_scan + Rp, 4, cudaMemcpyDeviceToHost, s->stream));
  CSMV_CUDA(cudaStreamSynchronize(s->stream));
  const uint32_t U = Rp - r_ro;  // transfer rounds
  uint32_t flagged = 0, deferred_rounds = 0;
  const uint32_t* run_op = d->op + t0;
  const uint32_t* run_off = d->off + t0;
  bool with_backoff = false, with_classes = false;
  uint32_t lanes_split = 0, lanes_n = 0;  // plan 1 with lanes: the laned rounds' split
  if (U > 0 && s->cfg.plan == 1) {
    // grouped plan: hot accounts, keys by the two hottest accounts touched, counting sort,
    // rounds of 32 consecutive sorted transfers spread by hot account
    const uint32_t SK = 1u << kSketchLog2;
    uint32_t hot = s->cfg.hot_count;
    if (!hot) hot = std::max(2u, (U * 32u) >> 14);
    const uint64_t seed = s->cfg.seed * 0x9E3779B97F4A7C15ull + s->chunks;
    sched_hot_flags_kernel<<<grid_for(s, SK), 256, 0, s->stream>>>(s->sketch, hot, s->key_rank);
    SCHED_LAUNCH_CHECK("hot flags");
    if ((st = scan_multi(s, s->key_rank, SK, s->hidx)) != CSMV_OK) return st;
    CSMV_CUDA(cudaMemsetAsync(s->key_count, 0, (size_t)SK * 4, s->stream));
    CSMV_CUDA(cudaMemsetAsync(s->n_flagged, 0, 4, s->stream));
    CSMV_CUDA(cudaMemsetAsync(s->max_count, 0, 4, s->stream));
    if (s->cfg.score == 1) {
      sched_max_kernel<<<grid_for(s, SK), 256, 0, s->stream>>>(s->sketch, SK, s->max_count);
      SCHED_LAUNCH_CHECK("max");
    }
    sched_group_keys_kernel<<<grid_for(s, n1), 256, 0, s->stream>>>(
        d->op, d->off, d->addr, t0, n, s->p, s->cfg.threshold, s->cfg.score, s->sketch,
        s->max_count, hot, s->hidx, s->key, s->rank, s->key_count, s->n_flagged, s->bo,
        s->cfg.backoff_ns, s->cfg.key_written);
    SCHED_LAUNCH_CHECK("group keys");
    if ((st = scan_multi(s, s->key_count, SK, s->key_start)) != CSMV_OK) return st;
    sched_cold_flags_kernel<<<grid_for(s, n1), 256, 0, s->stream>>>(n1, s->key, s->bucket);
    SCHED_LAUNCH_CHECK("cold flags");
    if ((st = scan_multi(s, s->bucket, n1, s->cold_pos)) != CSMV_OK) return st;
    sched_group_scatter_kernel<<<grid_for(s, n1), 256, 0, s->stream>>>(
        t0, n, s->key, s->rank, s->key_start, s->cold_pos, s->sorted);
    SCHED_LAUNCH_CHECK("group scatter");
    // lanes: the rounds of the hottest written accounts go to one warp each (hot_lanes)
    uint32_t bank_n = 0;
    const bool group = bank_group_commit(bank, &bank_n);
    const uint32_t K = group ? std::min(s->cfg.hot_lanes, kMaxLanes) : 0u;
    const uint32_t B = U + K;  // round buckets: U plan positions, then one per lane
    CSMV_CUDA(cudaMemsetAsync(s->bucket_count, 0, (size_t)(B + 1) * 4, s->stream));
    CSMV_CUDA(cudaMemsetAsync(s->bucket_fill, 0, (size_t)(B + 1) * 4, s->stream));
    if (K) {
      CSMV_CUDA(cudaMemsetAsync(s->lane_count, 0, 4, s->stream));
      sched_hot_lanes_kernel<<<grid_for(s, kHotNone), 256, 0, s->stream>>>(
          s->key_start, std::max(1u, U >> 6), K, s->lane_count, s->lane_of);
      SCHED_LAUNCH_CHECK("hot lanes");
    }
    sched_round_bucket_kernel<<<grid_for(s, U), 256, 0, s->stream>>>(
        t0, U, s->sorted, s->key, s->key_start, seed, K ? s->lane_of : nullptr, s->rbucket,
        s->bucket_count);
    SCHED_LAUNCH_CHECK("round buckets");
    if ((st = scan_multi(s, s->bucket_count, B, s->bucket_start)) != CSMV_OK) return st;
    sched_round_scatter_kernel<<<grid_for(s, U), 256, 0, s->stream>>>(
        U, s->rbucket, s->bucket_start, s->bucket_fill, s->round_order);
    SCHED_LAUNCH_CHECK("round scatter");
    sched_expand_rounds_kernel<<<grid_for(s, U * 32u), 256, 0, s->stream>>>(
        U, s->round_order, s->sorted, s->order);
    SCHED_LAUNCH_CHECK("expand");
    uint32_t laned = 0;  // rounds on lanes (the last ones of the plan)
    if (K) {
      uint32_t ends[2] = {0, 0};
      CSMV_CUDA(cudaMemcpyAsync(&ends[0], s->bucket_start + U, 4, cudaMemcpyDeviceToHost, s->stream));
      CSMV_CUDA(cudaMemcpyAsync(&ends[1], s->bucket_start + B, 4, cudaMemcpyDeviceToHost, s->stream));
      CSMV_CUDA(cudaStreamSynchronize(s->stream));
      laned = ends[1] - ends[0];
    }
    const uint32_t r_main = Rp - laned;
    sched_ro_list_kernel<<<grid_for(s, Rp), 256, 0, s->stream>>>(P, Rp, s->ro_flag, s->ro_scan,
                                                                s->ro_list);
    SCHED_LAUNCH_CHECK("ro_list");
    sched_emit_kernel<<<grid_for(s, n1), 256, 0, s->stream>>>(d->op, d->off, Rp, r_ro, r_main,
                                                             s->ro_list, s->order, s->perm,
                                                             s->op2, s->off2);
    SCHED_LAUNCH_CHECK("emit");
    if (laned) {
      sched_lane_start_kernel<<<1, 128, 0, s->stream>>>(U, K, r_main, s->bucket_start, s->lanes);
      SCHED_LAUNCH_CHECK("lane starts");
      lanes_split = r_main;
      lanes_n = K;
    }
    if (s->cfg.hot_last && group) {
      if (s->lock_last_n < bank_n) {
        cudaFree(s->lock_last);
        s->lock_last = nullptr;
        s->lock_last_n = 0;
        CSMV_CUDA(cudaMalloc(&s->lock_last, bank_n));
        s->lock_last_n = bank_n;
      }
      sched_lock_last_kernel<<<grid_for(s, bank_n), 256, 0, s->stream>>>(bank_n, s->sketch, hot,
                                                                         s->lock_last);
      SCHED_LAUNCH_CHECK("lock classes");
      with_classes = true;
    }
    if (s->cfg.backoff_ns) {
      sched_plan_backoff_kernel<<<grid_for(s, n1), 256, 0, s->stream>>>(n1, t0, s->perm, s->bo,
                                                                       s->bo2);
      SCHED_LAUNCH_CHECK("backoff");
      with_backoff = true;
    }
    CSMV_CUDA(cudaMemcpyAsync(&flagged, s->n_flagged, 4, cudaMemcpyDeviceToHost, s->stream));
    s->split_round = 0;
    run_op = s->op2;
    run_off = s->off2;
  } else if (U > 0) {
    const size_t SK = (size_t)1 << kSketchLog2;
    CSMV_CUDA(cudaMemsetAsync(s->key_count, 0, SK * 4, s->stream));
    CSMV_CUDA(cudaMemsetAsync(s->key_rank, 0, SK * 4, s->stream));
    CSMV_CUDA(cudaMemsetAsync(s->n_flagged, 0, 4, s->stream));
    sched_keys_kernel<<<grid_for(s, n1), 256, 0, s->stream>>>(
        d->op, d->off, d->addr, t0, n, s->p, s->cfg.threshold, s->sketch, s->key, s->key_count,
        s->n_flagged);
    SCHED_LAUNCH_CHECK("keys");
    CSMV_CUDA(cudaMemsetAsync(s->bucket_count, 0, (size_t)(U + 1) * 4, s->stream));
    CSMV_CUDA(cudaMemsetAsync(s->bucket_fill, 0, (size_t)(U + 1) * 4, s->stream));
    sched_bucket_kernel<<<grid_for(s, n1), 256, 0, s->stream>>>(
        d->op, t0, n, s->p, s->cfg.defer_threshold, s->key, s->key_count, s->key_rank, U,
        s->cfg.seed * 0x9E3779B97F4A7C15ull + s->chunks, s->bucket, s->bucket_count);
    SCHED_LAUNCH_CHECK("bucket");
    sched_scan_kernel<<<1, 1024, 0, s->stream>>>(s->bucket_count, U + 1, s->bucket_start);
    SCHED_LAUNCH_CHECK("scan");
    sched_scatter_kernel<<<grid_for(s, n1), 256, 0, s->stream>>>(t0, n, s->bucket, s->bucket_start,
                                                                s->bucket_fill, s->order);
    SCHED_LAUNCH_CHECK("scatter");
    uint32_t defer_start = 0;
    CSMV_CUDA(cudaMemcpyAsync(&defer_start, s->bucket_start + U, 4, cudaMemcpyDeviceToHost, s->stream));
    CSMV_CUDA(cudaMemcpyAsync(&flagged, s->n_flagged, 4, cudaMemcpyDeviceToHost, s->stream));
    CSMV_CUDA(cudaStreamSynchronize(s->stream));
    const uint32_t D = U * 32 - defer_start;  // deferred transfers
    deferred_rounds = (D + 31) / 32;
    const uint32_t r_main = r_ro + (U - deferred_rounds);
    sched_ro_list_kernel<<<grid_for(s, Rp), 256, 0, s->stream>>>(P, Rp, s->ro_flag, s->ro_scan,
                                                                s->ro_list);
    SCHED_LAUNCH_CHECK("ro_list");
    sched_emit_kernel<<<grid_for(s, n1), 256, 0, s->stream>>>(d->op, d->off, Rp, r_ro, r_main,
                                                             s->ro_list, s->order, s->perm,
                                                             s->op2, s->off2);
    SCHED_LAUNCH_CHECK("emit");
    s->split_round = deferred_rounds ? r_main : 0;
    run_op = s->op2;
    run_off = s->off2;
  } else {
    s->split_round = 0;  // only read-only rounds: nothing to reorder
  }
  CSMV_CUDA(cudaEventRecord(s->ev[3], s->stream));
  CSMV_CUDA(cudaStreamSynchronize(s->stream));
  s->planned = U > 0 ? n1 : 0;
  csmv_bank_stream rs = *d;
  rs.n_txn = n1;
  rs.op = run_op;
  rs.off = run_off;
  rs.txn_aborts = nullptr;
  rs.txn_waits = nullptr;
  rs.backoff = with_backoff ? s->bo2 : nullptr;
  rs.lock_last = with_classes ? s->lock_last : nullptr;
  rs.split_round = s->split_round;
  rs.deferred_warps = s->split_round ? s->cfg.deferred_warps : 0;
  rs.lane_start = nullptr;
  if (lanes_n) {
    rs.split_round = lanes_split;
    rs.deferred_warps = lanes_n;
    rs.lane_start = s->lanes;
  }
  if (s->cfg.serial_lane && s->split_round) {  // the deferred rounds wait for the serial lane
    s->serial_rounds = Rp - s->split_round;
    rs.n_txn = s->split_round * 32;
    rs.split_round = rs.deferred_warps = 0;
  }
  csmv_stats bst;
  std::memset(&bst, 0, sizeof(bst));
  if (rs.n_txn) st = csmv_bank_run_device(bank, &rs, &bst);
  s->chunks++;
  if (rep) {
    rep->planned = bst;
    float ms = 0.f;
    CSMV_CUDA(cudaEventElapsedTime(&ms, s->ev[2], s->ev[3]));
    rep->plan_ms = ms;
    rep->n_flagged = flagged;
    rep->n_deferred_rounds = deferred_rounds;
    rep->n_planned = n1;
  }
  return st;
}

extern "C" csmv_status csmv_sched_serial_run(csmv_sched_t* s, csmv_bank_t* bank,
                                             const csmv_bank_stream* d, csmv_sched_report* rep) {
  if (!s || !bank || !d) return CSMV_ERR_INVALID_ARG;
  if (rep) {
    std::memset(&rep->serial, 0, sizeof(rep->serial));
    rep->n_serial = 0;
  }
  if (!s->serial_rounds) return CSMV_OK;
  const uint32_t first = s->split_round * 32, n = s->serial_rounds * 32;
  s->serial_rounds = 0;
  csmv_bank_stream rs = *d;
  rs.n_txn = n;
  rs.op = s->op2 + first;
  rs.off = s->off2 + first;
  rs.txn_aborts = nullptr;
  rs.txn_waits = nullptr;
  rs.backoff = nullptr;
  rs.lock_last = nullptr;
  rs.lane_start = nullptr;
  rs.split_round = rs.deferred_warps = 0;
  csmv_stats bst;
  csmv_status st = s->cfg.serial_lane == 2 ? csmv_bank_run_flow_device(bank, &rs, &bst)
                                            : csmv_bank_run_serial_device(bank, &rs, &bst);
  if (rep) {
    rep->serial = bst;
    rep->n_serial = n;
  }
  return st;
}

extern "C" csmv_status csmv_sched_run(csmv_sched_t* s, csmv_bank_t* bank,
                                      const csmv_bank_stream* d, csmv_sched_report* rep) {
  csmv_sched_report a;
  csmv_status st = csmv_sched_probe(s, bank, d, &a);
  if (st != CSMV_OK) {
    if (rep) *rep = a;
    return st;
  }
  csmv_sched_report b, c;
  std::memset(&b, 0, sizeof(b));
  std::memset(&c, 0, sizeof(c));
  st = csmv_sched_plan_run(s, bank, d, &b);
  if (st == CSMV_OK) st = csmv_sched_serial_run(s, bank, d, &c);
  else std::memset(&c, 0, sizeof(c));
  if (rep) {
    *rep = a;
    rep->planned = b.planned;
    rep->serial = c.serial;
    rep->plan_ms = b.plan_ms;
    rep->n_flagged = b.n_flagged;
    rep->n_deferred_rounds = b.n_deferred_rounds;
    rep->n_planned = b.n_planned;
    rep->n_serial = c.n_serial;
  }
  return st;
}

extern "C" csmv_status csmv_sched_read_plan(csmv_sched_t* s, uint32_t* host_perm, uint32_t n,
                                            uint32_t* probe_rounds, uint32_t* split_round) {
  if (!s) return CSMV_ERR_INVALID_ARG;
  if (probe_rounds) *probe_rounds = s->probe_rounds;
  if (split_round) *split_round = s->split_round;
  if (host_perm) {
    const uint32_t n1 = s->n - s->probe_rounds * 32;
    if (n < n1) {
      set_error("plan buffer holds %u entries, the plan has %u", n, n1);
      return CSMV_ERR_CAPACITY;
    }
    CSMV_CUDA(cudaSetDevice(s->cfg.device));
    if (s->planned)
      CSMV_CUDA(cudaMemcpy(host_perm, s->perm, (size_t)n1 * 4, cudaMemcpyDeviceToHost));
    else
      for (uint32_t i = 0; i < n1; i++) host_perm[i] = s->probe_rounds * 32 + i;
  }
  return CSMV_OK;
}

extern "C" csmv_mlp_t* csmv_sched_mlp(csmv_sched_t* s) { return s ? s->mlp : nullptr; }

extern "C" void csmv_sched_destroy(csmv_sched_t* s) {
  if (!s) return;
  cudaSetDevice(s->cfg.device);
  free_all(s);
  delete s;
}
