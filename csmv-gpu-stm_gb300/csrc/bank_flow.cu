// bank_flow.cu - C-ABI host side of the dataflow lane (csmv_bank_run_flow_device).
//
// The lane runs a stream with the GPU to itself and leaves what the serial lane leaves: the same
// commit timestamps in stream order, versions in the same slots, commit words, log, outcomes and
// results (flow_kernels.cuh has the method). Its buffers are made on the first run and grown
// when a larger stream comes:
//   per transaction  eoff, wflag (4 B each, +1), out (16 B), tails (16 B)
//   per access       keys and values twice (16 B), wpos (4 B), src (8 B), radix counts
//   per account      cnt (4 B), zero between runs
#include <chrono>
#include <cstring>

#include "bank_internal.h"
#include "flow_kernels.cuh"

using namespace csmv;

namespace csmv {

struct FlowScratch {
  uint32_t txn_cap = 0, elem_cap = 0, items = 0, epoch = 0;
  uint32_t *eoff = nullptr, *wflag = nullptr, *cnt = nullptr, *n_tails = nullptr, *agg = nullptr;
  uint32_t *counts = nullptr, *wpos = nullptr, *key[2] = {nullptr, nullptr}, *val[2] = {nullptr, nullptr};
  unsigned long long *out = nullptr, *src = nullptr;
  uint2* tails = nullptr;
  uint32_t* host_total = nullptr;  // pinned: accesses, most reads of a transfer
};

void flow_scratch_free(FlowScratch* f) {
  if (!f) return;
  for (void* p : {(void*)f->eoff, (void*)f->wflag, (void*)f->cnt, (void*)f->n_tails, (void*)f->agg,
                  (void*)f->counts, (void*)f->wpos, (void*)f->key[0], (void*)f->key[1],
                  (void*)f->val[0], (void*)f->val[1], (void*)f->out, (void*)f->src, (void*)f->tails})
    cudaFree(p);
  cudaFreeHost(f->host_total);
  delete f;
}

csmv_status flow_scratch_reset(FlowScratch* f, cudaStream_t s) {
  if (f && f->cnt) CSMV_CUDA(cudaMemsetAsync(f->cnt, 0, (size_t)f->items * 4, s));
  return CSMV_OK;
}

}  // namespace csmv

namespace {

using FlowKernel = void (*)(FlowParams, const uint32_t*, const uint32_t*, const uint32_t*, uint32_t);
using InstallKernel = void (*)(FlowParams);

FlowKernel pick_src(uint32_t depth) {
  switch (depth) {
    case 2: return flow_src_kernel<2>;
    case 4: return flow_src_kernel<4>;
    case 8: return flow_src_kernel<8>;
    case 16: return flow_src_kernel<16>;
    default: return nullptr;
  }
}

InstallKernel pick_install(uint32_t depth) {
  switch (depth) {
    case 2: return flow_install_kernel<2>;
    case 4: return flow_install_kernel<4>;
    case 8: return flow_install_kernel<8>;
    case 16: return flow_install_kernel<16>;
    default: return nullptr;
  }
}

// Replaces *p by a fresh device array of n elements of T.
template <class T>
csmv_status grow(T** p, size_t n) {
  cudaFree(*p);
  *p = nullptr;
  return cuda_status(cudaMalloc((void**)p, n * sizeof(T)), "cudaMalloc (dataflow lane)");
}

csmv_status ensure_txn(csmv_bank_t* h, uint32_t n) {
  if (!h->flow) {
    h->flow = new FlowScratch;
    FlowScratch* f = h->flow;
    f->items = h->cfg.n_accounts;
    csmv_status st;
    if ((st = grow(&f->cnt, f->items)) != CSMV_OK || (st = grow(&f->n_tails, 2)) != CSMV_OK ||
        (st = grow(&f->agg, kScanMaxTiles + 1)) != CSMV_OK)
      return st;
    CSMV_CUDA(cudaMallocHost((void**)&f->host_total, 8));
    CSMV_CUDA(cudaFuncSetAttribute((const void*)flow_exec_kernel<4>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(FlowSmem)));
    CSMV_CUDA(cudaFuncSetAttribute((const void*)flow_exec_kernel<8>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(FlowSmem)));
    CSMV_CUDA(cudaMemsetAsync(f->cnt, 0, (size_t)f->items * 4, h->stream));
  }
  FlowScratch* f = h->flow;
  if (n <= f->txn_cap) return CSMV_OK;
  f->txn_cap = 0;
  csmv_status st;
  if ((st = grow(&f->eoff, (size_t)n + 1)) != CSMV_OK || (st = grow(&f->wflag, (size_t)n + 1)) != CSMV_OK ||
      (st = grow(&f->out, 2 * (size_t)n)) != CSMV_OK || (st = grow(&f->tails, 2 * (size_t)n)) != CSMV_OK)
    return st;
  CSMV_CUDA(cudaMemsetAsync(f->out, 0, 2 * (size_t)n * 8, h->stream));  // epoch 0: never current
  f->epoch = 0;
  f->txn_cap = n;
  return CSMV_OK;
}

csmv_status ensure_elem(FlowScratch* f, uint32_t e) {
  if (e <= f->elem_cap) return CSMV_OK;
  f->elem_cap = 0;
  const size_t tiles = (e + kRadixTile - 1) / kRadixTile;
  csmv_status st;
  if ((st = grow(&f->key[0], e)) != CSMV_OK || (st = grow(&f->key[1], e)) != CSMV_OK ||
      (st = grow(&f->val[0], e)) != CSMV_OK || (st = grow(&f->val[1], e)) != CSMV_OK ||
      (st = grow(&f->wpos, (size_t)e + 1)) != CSMV_OK || (st = grow(&f->src, e)) != CSMV_OK ||
      (st = grow(&f->counts, 256 * tiles + 1)) != CSMV_OK)
    return st;
  f->elem_cap = e;
  return CSMV_OK;
}

template <bool MAX>
csmv_status scan(uint32_t* data, uint32_t n, uint32_t* agg, cudaStream_t s) {
  if (n == 0) {
    CSMV_CUDA(cudaMemsetAsync(data, 0, 4, s));
    return CSMV_OK;
  }
  const uint32_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles > kScanMaxTiles) {
    set_error("dataflow lane: scan of %u words is over the limit", n);
    return CSMV_ERR_CAPACITY;
  }
  scan_reduce_kernel<MAX><<<tiles, kScanThreads, 0, s>>>(data, n, agg);
  scan_tiles_kernel<MAX><<<1, kScanThreads, 0, s>>>(agg, tiles, data + n);
  scan_apply_kernel<MAX><<<tiles, kScanThreads, 0, s>>>(data, n, agg);
  return cuda_status(cudaGetLastError(), "scan");
}

uint32_t grid_of(uint64_t n, uint32_t block) { return (uint32_t)((n + block - 1) / block); }

// Everything after the checks; the caller ends the run (statistics, status).
csmv_status flow_launch(csmv_bank_t* h, const csmv_bank_stream* s) {
  const uint32_t n = s->n_txn;
  FlowScratch* f = h->flow;
  cudaStream_t st = h->stream;
  FlowParams p{};
  p.b = bank_params(h, s->op, s->off, s->addr, n, s->txn_aborts);
  p.n_txn = n;
  p.eoff = f->eoff;
  p.out = f->out;
  p.wflag = f->wflag;
  p.cnt = f->cnt;
  p.tails = f->tails;
  p.n_tails = f->n_tails;
  CSMV_CUDA(cudaMemsetAsync(f->n_tails, 0, 8, st));  // tail count, most reads of a transfer
  flow_count_kernel<<<grid_of(n, 256), 256, 0, st>>>(p, 8u);
  CSMV_CUDA(cudaGetLastError());
  csmv_status rc = scan<false>(f->eoff, n, f->agg, st);
  if (rc != CSMV_OK) return rc;
  CSMV_CUDA(cudaMemcpyAsync(f->host_total, f->eoff + n, 4, cudaMemcpyDeviceToHost, st));
  CSMV_CUDA(cudaMemcpyAsync(f->host_total + 1, f->n_tails + 1, 4, cudaMemcpyDeviceToHost, st));
  CSMV_CUDA(cudaStreamSynchronize(st));
  const uint32_t E = *f->host_total;
  if (E > kFlowMaxElem) {
    set_error("dataflow lane: %u accesses in one call (at most %u)", E, kFlowMaxElem);
    return CSMV_ERR_CAPACITY;
  }
  if ((rc = ensure_elem(f, E > 0 ? E : 1)) != CSMV_OK) return rc;
  p.src = f->src;
  if (E > 0) {
    flow_elements_kernel<<<grid_of(n, 256), 256, 0, st>>>(p, f->key[0], f->val[0]);
    CSMV_CUDA(cudaGetLastError());
    // stable sort by account, 8 bits a pass over the bits an account id can have
    const uint32_t top = h->cfg.n_accounts - 1u;
    const uint32_t bits = top ? 32u - (uint32_t)__builtin_clz(top) : 1u;
    const uint32_t tiles = grid_of(E, kRadixTile);
    int cur = 0;
    for (uint32_t shift = 0; shift < bits; shift += 8) {
      flow_radix_hist_kernel<<<tiles, kRadixThreads, 0, st>>>(f->key[cur], E, shift, tiles, f->counts);
      CSMV_CUDA(cudaGetLastError());
      if ((rc = scan<false>(f->counts, 256u * tiles, f->agg, st)) != CSMV_OK) return rc;
      flow_radix_scatter_kernel<<<tiles, kRadixThreads, 0, st>>>(f->key[cur], f->val[cur], E, shift,
                                                                 tiles, f->counts, f->key[cur ^ 1],
                                                                 f->val[cur ^ 1]);
      CSMV_CUDA(cudaGetLastError());
      cur ^= 1;
    }
    flow_wpos_kernel<<<grid_of(E, 256), 256, 0, st>>>(f->val[cur], E, f->wpos);
    CSMV_CUDA(cudaGetLastError());
    if ((rc = scan<true>(f->wpos, E, f->agg, st)) != CSMV_OK) return rc;
    pick_src(h->cfg.version_depth)<<<grid_of(E, 256), 256, 0, st>>>(p, f->key[cur], f->val[cur],
                                                                   f->wpos, E);
    CSMV_CUDA(cudaGetLastError());
  }
  if (++f->epoch == 0) {  // after 2^32 runs: clear the output words, start over at epoch 1
    CSMV_CUDA(cudaMemsetAsync(f->out, 0, 2 * (size_t)f->txn_cap * 8, st));
    f->epoch = 1;
  }
  p.epoch = f->epoch;
  const uint32_t warps = h->cfg.flow_warps ? h->cfg.flow_warps : kFlowExecWarps;
  if (f->host_total[1] <= 4u)  // the most accounts a transfer of the stream reads
    flow_exec_kernel<4><<<1, 32 * warps, sizeof(FlowSmem), st>>>(p);
  else
    flow_exec_kernel<8><<<1, 32 * warps, sizeof(FlowSmem), st>>>(p);
  CSMV_CUDA(cudaGetLastError());
  if ((rc = scan<false>(f->wflag, n, f->agg, st)) != CSMV_OK) return rc;
  flow_finalize_kernel<<<grid_of(n, 256), 256, 0, st>>>(p);
  CSMV_CUDA(cudaGetLastError());
  pick_install(h->cfg.version_depth)<<<grid_of(2ull * n, 256), 256, 0, st>>>(p);
  CSMV_CUDA(cudaGetLastError());
  flow_end_kernel<<<1, 256, 0, st>>>(p);
  CSMV_CUDA(cudaGetLastError());
  return CSMV_OK;
}

}  // namespace

extern "C" csmv_status csmv_bank_run_flow_device(csmv_bank_t* h, const csmv_bank_stream* s,
                                                 csmv_stats* out) {
  if (!h) return CSMV_ERR_INVALID_ARG;
  if (!h->loaded) {
    set_error("csmv_bank_load must come first");
    return CSMV_ERR_STATE;
  }
  csmv_status st = check_stream(h, s);
  if (st != CSMV_OK) return st;
  if (h->cfg.validate != CSMV_VALIDATE_STAMP) {
    set_error("the dataflow lane continues the stamp protocol's commit order only");
    return CSMV_ERR_INVALID_ARG;
  }
  if (s->n_txn > kFlowMaxTxn) {
    set_error("dataflow lane: %u transactions in one call (at most %u)", s->n_txn, kFlowMaxTxn);
    return CSMV_ERR_CAPACITY;
  }
  CSMV_CUDA(cudaSetDevice(h->cfg.device));
  auto t0 = std::chrono::steady_clock::now();
  if ((st = ensure_txn(h, s->n_txn)) != CSMV_OK) return st;
  h->last_grouped = false;  // the lane installs every write
  if ((st = bank_begin_run(h)) != CSMV_OK) return st;
  csmv_status lst = flow_launch(h, s);
  st = bank_end_run(h, s->n_txn, out);  // waits for the stream whatever happened
  if (lst != CSMV_OK) st = lst;
  if (st != CSMV_OK) {
    // a failed run may leave per-account counts behind
    csmv_status rs = flow_scratch_reset(h->flow, h->stream);
    if (rs == CSMV_OK) cudaStreamSynchronize(h->stream);
  }
  if (out)
    out->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return st;
}
