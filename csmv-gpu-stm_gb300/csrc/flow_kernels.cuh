// flow_kernels.cuh - the dataflow lane (bank_flow.cu): a bank stream run with the GPU to itself,
// with the results, commit order and final state of running it in stream order (the serial lane,
// bank_serial_kernel), but with every transaction whose inputs are known in flight at once.
//
// Static analysis (all SMs):
//   count      elements per transaction - its reads, then its writes (one if both written
//              accounts are the same, else two); checks sizes and accounts (ERR_DATA: nothing
//              is applied)
//   scan       element offsets
//   elements   key = account, value = txn << 7 | code (read k: code k; write slot s: 64 + s)
//   sort       stable LSD radix sort by account, 8 bits per pass: per account, its accesses in
//              stream order
//   producers  an exclusive max-scan over the write positions gives every read the last earlier
//              write of its account (its producer, named txn * 2 + slot); a read without one
//              takes the account's latest committed version, looked up here
//   tails      the last write of each account, where its installs start
// Execution (one CTA, flow_exec_kernel): warp w runs the blocks of 32 consecutive transactions
//   w, w + 32, w + 64, ...; each lane polls its reads' producers' outputs until all have
//   arrived, runs its transfer and publishes the value of each account it writes - new, or
//   unchanged when the funds were short - to a shared-memory ring (the chain hand-offs) and to
//   global memory. A transaction waits only on earlier ones and the earliest unfinished one has
//   all its inputs, so the lane always makes progress; the polls are bounded all the same
//   (ERR_WAIT_FLOW).
// Commit (all SMs):
//   ranks      exclusive scan of the has-write flags: the writers take consecutive timestamps in
//              stream order, as in the serial lane
//   finalize   outcome, commit log and result of every transaction
//   install    per written account, from its tail back along the producer chain: the last
//              `depth` actual writes go to the slots the serial lane gives them (writer r of the
//              run takes the (r mod depth)-th victim of the slots as the run found them: empty
//              first, else oldest) and the last one stamps the commit word
//   end        clock and timestamp cursor, statistics, completion-bitmap words passed over
#pragma once
#include "bank_kernel.cuh"

namespace csmv {

constexpr uint32_t kFlowWrite = 64;                      // element codes >= 64 are writes
constexpr uint32_t kFlowMaxTxn = 1u << 25;               // element values pack txn << 7 | code
constexpr uint32_t kFlowMaxElem = 1u << 26;              // accesses per call
constexpr unsigned long long kFlowValue = 1ull << 63;    // src word: a value, no producer
constexpr uint32_t kFlowExecThreads = 512;   // the execution CTA at most (16 warps)
constexpr uint32_t kFlowExecWarps = 8;       // ... and by default

struct FlowParams {
  BankParams b;              // stream, version store, commit words, log, sync words, statistics
  uint32_t n_txn;
  uint32_t* eoff;            // [n_txn + 1] element counts, scanned to element offsets
  unsigned long long* src;   // [n_elem] per read: producer (txn * 2 + slot), or kFlowValue | value
  unsigned long long* out;   // [2 n_txn] output words: epoch << 32 | value
  uint32_t* wflag;           // [n_txn + 1] has-write flags, scanned to writer ranks
  uint32_t* cnt;             // [n_items] actual writes per account in this run (zero between runs)
  uint2* tails;              // [2 n_txn] (account, producer code of its last write)
  uint32_t* n_tails;         // [2]: tails written; the most accounts a transfer reads
  uint32_t epoch;
};

// The run failed before its commit phase: nothing may be applied.
__device__ __forceinline__ bool flow_failed(const FlowParams& f) {
  const uint32_t e = ld_relaxed_gpu(&f.b.gs->error);
  return e == ERR_DATA || e == ERR_WAIT_FLOW;
}

// ---------------------------------------------------------------------------------------------
// Device-wide exclusive scan of u32 words (sum, or max for position marks), in place, total
// written after the last word: tiles of 4096 words reduced, the tile totals scanned by one CTA,
// then each tile scanned with its carry.
// ---------------------------------------------------------------------------------------------
constexpr uint32_t kScanThreads = 1024, kScanItems = 4, kScanTile = kScanThreads * kScanItems;
constexpr uint32_t kScanMaxTiles = kScanThreads * 16;  // 2^26 words

template <bool MAX>
__device__ __forceinline__ uint32_t scan_op(uint32_t a, uint32_t b) {
  return MAX ? (a > b ? a : b) : a + b;
}

// Exclusive scan of one word per thread over the block (identity 0); *total = the block's total.
// sh: 32 words of shared memory.
template <bool MAX>
__device__ __forceinline__ uint32_t block_exclusive(uint32_t x, uint32_t* total, uint32_t* sh) {
  const uint32_t lane = lane_id(), w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint32_t incl = x;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
    if (lane >= (uint32_t)d) incl = scan_op<MAX>(incl, y);
  }
  uint32_t excl = __shfl_up_sync(0xFFFFFFFFu, incl, 1);
  if (lane == 0) excl = 0u;
  if (lane == 31) sh[w] = incl;
  __syncthreads();
  if (w == 0) {
    uint32_t v = lane < nw ? sh[lane] : 0u;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, v, d);
      if (lane >= (uint32_t)d) v = scan_op<MAX>(v, y);
    }
    __syncwarp();
    sh[lane] = v;  // inclusive over warps
  }
  __syncthreads();
  const uint32_t r = scan_op<MAX>(w ? sh[w - 1] : 0u, excl);
  *total = sh[nw - 1];
  __syncthreads();  // sh is reused by the caller
  return r;
}

template <bool MAX>
__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const uint32_t* in, uint32_t n,
                                                                   uint32_t* agg) {
  __shared__ uint32_t sh[32];
  const uint32_t base = blockIdx.x * kScanTile;
  uint32_t t = 0;
#pragma unroll
  for (uint32_t j = 0; j < kScanItems; j++) {
    const uint32_t idx = base + j * kScanThreads + threadIdx.x;
    if (idx < n) t = scan_op<MAX>(t, in[idx]);
  }
  uint32_t total;
  block_exclusive<MAX>(t, &total, sh);
  if (threadIdx.x == 0) agg[blockIdx.x] = total;
}

template <bool MAX>
__global__ void __launch_bounds__(kScanThreads) scan_tiles_kernel(uint32_t* agg, uint32_t n_tiles,
                                                                  uint32_t* total_out) {
  __shared__ uint32_t sh[32];
  constexpr uint32_t kPer = kScanMaxTiles / kScanThreads;  // 16
  const uint32_t i0 = threadIdx.x * kPer;
  uint32_t x[kPer], run = 0;
#pragma unroll
  for (uint32_t j = 0; j < kPer; j++) {
    x[j] = i0 + j < n_tiles ? agg[i0 + j] : 0u;
    const uint32_t v = x[j];
    x[j] = run;
    run = scan_op<MAX>(run, v);
  }
  uint32_t total;
  const uint32_t pre = block_exclusive<MAX>(run, &total, sh);
#pragma unroll
  for (uint32_t j = 0; j < kPer; j++)
    if (i0 + j < n_tiles) agg[i0 + j] = scan_op<MAX>(pre, x[j]);
  if (threadIdx.x == 0) *total_out = total;
}

template <bool MAX>
__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(uint32_t* data, uint32_t n,
                                                                  const uint32_t* agg) {
  __shared__ uint32_t sh[32];
  const uint32_t i0 = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  uint32_t x[kScanItems], run = 0;
#pragma unroll
  for (uint32_t j = 0; j < kScanItems; j++) {
    const uint32_t v = i0 + j < n ? data[i0 + j] : 0u;
    x[j] = run;
    run = scan_op<MAX>(run, v);
  }
  uint32_t total;
  const uint32_t pre = scan_op<MAX>(agg[blockIdx.x], block_exclusive<MAX>(run, &total, sh));
#pragma unroll
  for (uint32_t j = 0; j < kScanItems; j++)
    if (i0 + j < n) data[i0 + j] = scan_op<MAX>(pre, x[j]);
}

// ---------------------------------------------------------------------------------------------
// Stable LSD radix sort of (key, value) pairs, 8 bits per pass. A tile of 4096 pairs is split
// over 8 warps of 512 consecutive pairs; a warp ranks its pairs 32 at a time in order with
// match.any, so equal digits keep their input order within the tile, and tiles are laid out in
// order by the digit-major scan of the per-tile counts.
// ---------------------------------------------------------------------------------------------
constexpr uint32_t kRadixThreads = 256, kRadixWarps = 8, kRadixTile = 4096;
constexpr uint32_t kRadixPerWarp = kRadixTile / kRadixWarps;

__global__ void __launch_bounds__(kRadixThreads) flow_radix_hist_kernel(const uint32_t* key, uint32_t n,
                                                                        uint32_t shift, uint32_t n_tiles,
                                                                        uint32_t* counts) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0u;
  __syncthreads();
  const uint32_t base = blockIdx.x * kRadixTile;
  for (uint32_t j = threadIdx.x; j < kRadixTile; j += kRadixThreads)
    if (base + j < n) atomicAdd(&h[(key[base + j] >> shift) & 255u], 1u);
  __syncthreads();
  counts[threadIdx.x * n_tiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kRadixThreads) flow_radix_scatter_kernel(
    const uint32_t* kin, const uint32_t* vin, uint32_t n, uint32_t shift, uint32_t n_tiles,
    const uint32_t* offs, uint32_t* kout, uint32_t* vout) {
  __shared__ uint32_t wc[kRadixWarps][256];
  const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
  for (uint32_t j = threadIdx.x; j < kRadixWarps * 256; j += kRadixThreads) (&wc[0][0])[j] = 0u;
  __syncthreads();
  const uint32_t wbase = blockIdx.x * kRadixTile + w * kRadixPerWarp;
  for (uint32_t c = 0; c < kRadixPerWarp; c += 32) {  // the warp's digit counts
    const uint32_t idx = wbase + c + lane;
    const bool valid = idx < n;
    const uint32_t d = valid ? (kin[idx] >> shift) & 255u : 256u;
    const uint32_t m = __match_any_sync(0xFFFFFFFFu, d);
    if (valid && lane == (uint32_t)__ffs(m) - 1u) wc[w][d] += __popc(m);
    __syncwarp();
  }
  __syncthreads();
  {  // thread = digit: start of each warp's run of that digit
    uint32_t run = offs[threadIdx.x * n_tiles + blockIdx.x];
#pragma unroll
    for (uint32_t ww = 0; ww < kRadixWarps; ww++) {
      const uint32_t t = wc[ww][threadIdx.x];
      wc[ww][threadIdx.x] = run;
      run += t;
    }
  }
  __syncthreads();
  for (uint32_t c = 0; c < kRadixPerWarp; c += 32) {
    const uint32_t idx = wbase + c + lane;
    const bool valid = idx < n;
    const uint32_t k = valid ? kin[idx] : 0u;
    const uint32_t d = valid ? (k >> shift) & 255u : 256u;
    const uint32_t m = __match_any_sync(0xFFFFFFFFu, d);
    if (valid) {
      const uint32_t pos = wc[w][d] + __popc(m & lanemask_lt());
      kout[pos] = k;
      vout[pos] = vin[idx];
    }
    __syncwarp();
    if (valid && lane == (uint32_t)__ffs(m) - 1u) wc[w][d] += __popc(m);
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------------------------
// Static analysis
// ---------------------------------------------------------------------------------------------
// Elements per transaction (0 for a malformed one, which raises ERR_DATA). Rounds are 32
// consecutive transactions, read-only or not as a whole (the serial lane's rule). Read-only
// commits are counted here.
__global__ void __launch_bounds__(256) flow_count_kernel(FlowParams f, uint32_t max_reads) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= f.n_txn) return;  // whole warps: n_txn is a multiple of 32
  const uint32_t op = f.b.op[i], off = f.b.off[i];
  const uint32_t nr = CSMV_OP_NREADS(op);
  const bool ro = CSMV_OP_KIND(op) == CSMV_KIND_READONLY;
  const bool all_ro = __all_sync(0xFFFFFFFFu, ro), any_ro = __any_sync(0xFFFFFFFFu, ro);
  bool bad = all_ro != any_ro;
  if (!ro) bad |= nr < 2 || nr > max_reads || CSMV_OP_AMOD(op) == 0;
  for (uint32_t k = 0; k < nr && !bad; k++) bad |= f.b.addr[off + k] >= f.b.n_items;
  uint32_t nw = 0;
  if (!bad && !ro) nw = f.b.addr[off] == f.b.addr[off + 1] ? 1u : 2u;
  f.eoff[i] = bad ? 0u : nr + nw;
  if (bad) raise_error(&f.b.gs->error, ERR_DATA);
  if (!bad && all_ro && lane_id() == 0) atomicAdd(&f.b.stats[ST_COMMIT_RO], 32ull);
  if (!bad && !ro) atomicMax(&f.n_tails[1], nr);
}

__global__ void __launch_bounds__(256) flow_elements_kernel(FlowParams f, uint32_t* key, uint32_t* val) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= f.n_txn) return;
  const uint32_t e = f.eoff[i], n_el = f.eoff[i + 1] - e;
  if (n_el == 0) return;
  const uint32_t op = f.b.op[i], off = f.b.off[i], nr = CSMV_OP_NREADS(op);
  for (uint32_t k = 0; k < nr; k++) {
    key[e + k] = f.b.addr[off + k];
    val[e + k] = i << 7 | k;
  }
  if (n_el > nr) {
    const uint32_t a0 = f.b.addr[off], a1 = f.b.addr[off + 1];
    if (a0 == a1) {  // written once, with the second write's value
      key[e + nr] = a1;
      val[e + nr] = i << 7 | (kFlowWrite + 1u);
    } else {
      key[e + nr] = a0;
      val[e + nr] = i << 7 | kFlowWrite;
      key[e + nr + 1] = a1;
      val[e + nr + 1] = i << 7 | (kFlowWrite + 1u);
    }
  }
}

// wpos[p] = p + 1 for a write element at sorted position p, else 0 (max-scanned next)
__global__ void __launch_bounds__(256) flow_wpos_kernel(const uint32_t* val, uint32_t n, uint32_t* wpos) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) wpos[p] = (val[p] & 127u) >= kFlowWrite ? p + 1u : 0u;
}

__device__ __forceinline__ uint32_t flow_code(uint32_t v) {  // producer name of a write element
  return (v >> 7) * 2u + ((v & 127u) - kFlowWrite);
}

// Producer (or committed value) of every read, and the tail write of every written account.
// wpos: exclusive max-scan of the write marks, 1 + the last write position before p (or 0).
template <int DEPTH>
__global__ void __launch_bounds__(256) flow_src_kernel(FlowParams f, const uint32_t* key,
                                                       const uint32_t* val, const uint32_t* wpos,
                                                       uint32_t n_elem) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_elem) return;
  const uint32_t x = key[p], v = val[p], code = v & 127u;
  const uint32_t q1 = wpos[p];
  const bool prev_in_seg = q1 != 0u && key[q1 - 1u] == x;  // an earlier write of the same account
  if (code < kFlowWrite) {
    unsigned long long s;
    if (prev_in_seg) {
      s = flow_code(val[q1 - 1u]);
    } else {
      unsigned long long sl[DEPTH];
      const unsigned long long* item = f.b.slots + (size_t)x * DEPTH;
#pragma unroll
      for (int d = 0; d < DEPTH; d += 2) ld_relaxed_gpu_v2(item + d, sl[d], sl[d + 1]);
      s = kFlowValue | (uint32_t)latest_of<DEPTH, 8>(sl);
    }
    f.src[f.eoff[v >> 7] + code] = s;
  }
  if (p + 1u == n_elem || key[p + 1u] != x) {  // the account's last access
    const bool has = code >= kFlowWrite || prev_in_seg;
    if (has) {
      const uint32_t last = code >= kFlowWrite ? v : val[q1 - 1u];
      f.tails[atomicAdd(f.n_tails, 1u)] = make_uint2(x, flow_code(last));
    }
  }
}

// ---------------------------------------------------------------------------------------------
// Execution: one CTA of kFlowExecThreads threads (32 warps).
//
// Outputs go to a ring in shared memory (the hand-offs of a dependency chain take a shared-memory
// round trip) and to `out` in global memory (read by consumers far behind their producer and by
// the installs). Ring word of transaction j's slot s, at (2j + s) mod 2R: (j + 1) << 32 | value.
// A warp starts block b only when every block <= b - G has finished (per-warp finished-block
// counters). Then a consumer in block c reads producer block bj from the ring when c - bj < G -
// the ring slot cannot have been reused yet, as its next writer, block bj + R/32, waits for c
// (R/32 >= 2G - 1) - and from `out` otherwise, where the producer has certainly finished.
// ---------------------------------------------------------------------------------------------
constexpr uint32_t kFlowRing = 8192;  // transactions whose outputs the ring holds (R)
constexpr uint32_t kFlowGate = 128;   // blocks a warp may run ahead of the oldest unfinished (G)
static_assert(kFlowRing / 32 >= 2 * kFlowGate - 1, "ring reach");
static_assert((kFlowRing & (kFlowRing - 1)) == 0, "ring size");
// A transfer's producers are held in registers: NR of them, NR = 4 when no transfer of the
// stream reads more than 4 accounts, else 8 (the most a transfer may read).

struct FlowSmem {
  unsigned long long ring[2 * kFlowRing];
  uint32_t prog[32];  // blocks finished by each warp
  uint32_t failed;
};

__device__ __forceinline__ unsigned long long ld_relaxed_cta_shared(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.cta.shared.u64 %0, [%1];"
               : "=l"(v)
               : "r"((uint32_t)__cvta_generic_to_shared(p))
               : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_cta_shared(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.cta.shared.u64 [%0], %1;" ::"r"((uint32_t)__cvta_generic_to_shared(p)),
               "l"(v)
               : "memory");
}

// Value of a read with source word s, for a consumer in block c; false while it has not arrived.
__device__ __forceinline__ bool flow_fetch(const FlowParams& f, FlowSmem& S, unsigned long long s,
                                           uint32_t c, unsigned long long tag, uint32_t& x) {
  if (s & kFlowValue) {
    x = (uint32_t)s;
    return true;
  }
  const uint32_t j = (uint32_t)s >> 1;
  if (c - (j >> 5) < kFlowGate) {
    const unsigned long long wv = ld_relaxed_cta_shared(&S.ring[(uint32_t)s & (2u * kFlowRing - 1u)]);
    x = (uint32_t)wv;
    return (uint32_t)(wv >> 32) == j + 1u;
  }
  const unsigned long long wv = ld_relaxed_cta_global(&f.out[s]);
  x = (uint32_t)wv;
  return (wv & 0xFFFFFFFF00000000ull) == tag;
}

// Entry k (< NR) of a lane's register array, without local memory.
template <uint32_t NR, class T>
__device__ __forceinline__ T pick(const T (&a)[NR], uint32_t k) {
  T s = a[0];
#pragma unroll
  for (uint32_t q = 1; q < NR; q++) s = k == q ? a[q] : s;
  return s;
}

// A transfer's static inputs (producers, committed values, written accounts, divisor) are read
// at the start of its block, and so are the outputs of producers at least G blocks older (they
// have finished); the amount is worked out as soon as its extra reads are in. What is left are
// producers in the ring, with their ring word and tag worked out once: a pass loads all of them
// at once (independent shared-memory loads) and takes them when all have arrived - a ring word
// keeps its producer's value until the consumer's block is done. A finished transfer publishes
// to the ring at once and leaves its global outputs, flags and counts for the end of the block:
// the passes that carry the dependency chain stay short.
template <uint32_t NR>
__global__ void __launch_bounds__(kFlowExecThreads, 1) flow_exec_kernel(FlowParams f) {
  extern __shared__ __align__(16) unsigned char flow_smem_raw[];
  FlowSmem& S = *reinterpret_cast<FlowSmem*>(flow_smem_raw);
  const uint32_t lane = lane_id(), w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const uint32_t nb = f.n_txn / 32u;
  const unsigned long long tag = (unsigned long long)f.epoch << 32;
  uint32_t* err = &f.b.gs->error;
  const uint32_t limit = 1u << f.b.spin_log2;  // spin_log2 <= 30
  for (uint32_t k = threadIdx.x; k < 2u * kFlowRing; k += blockDim.x) S.ring[k] = 0ull;
  if (threadIdx.x < 32) S.prog[threadIdx.x] = 0u;
  if (threadIdx.x == 0) S.failed = ld_relaxed_gpu(err);
  __syncthreads();
  if (S.failed) return;
  // bounded poll bookkeeping: false when the warp must leave (budget spent or an error raised)
  auto keep_polling = [&](uint32_t it) {
    if (it >= limit) {
      if (lane == 0) raise_error(err, ERR_WAIT_FLOW);
      return false;
    }
    if ((it & 1023u) == 1023u) {
      uint32_t e = 0;
      if (lane == 0) e = ld_relaxed_gpu(err);
      if (__shfl_sync(0xFFFFFFFFu, e, 0)) return false;
    }
    return true;
  };  // (called with it = 255, 511, ... by the execution loop: limit >= 1024)
  uint32_t finished = 0;  // this warp's blocks
  uint32_t op_n = 0, e0_n = 0;  // the next block's op and element offset, loaded ahead
  if (w < nb) {
    op_n = f.b.op[w * 32u + lane];
    e0_n = f.eoff[w * 32u + lane];
  }
  for (uint32_t b = w; b < nb; b += nw) {
    const uint32_t i = b * 32u + lane;
    const uint32_t op = op_n, e0 = e0_n;
    if (b + nw < nb) {
      op_n = f.b.op[i + 32u * nw];
      e0_n = f.eoff[i + 32u * nw];
    }
    const uint32_t nr = CSMV_OP_NREADS(op);
    const bool ro = CSMV_OP_KIND(op) == CSMV_KIND_READONLY;
    unsigned long long sv[NR];
    uint32_t a0 = 0, a1 = 0;
    if (!ro) {
      const uint32_t off = f.b.off[i];
#pragma unroll
      for (uint32_t k = 0; k < NR; k++) sv[k] = k < nr ? __ldg(&f.src[e0 + k]) : kFlowValue;
      a0 = f.b.addr[off];
      a1 = f.b.addr[off + 1];
    }
    if (b >= kFlowGate) {  // every block <= b - G finished
      const uint32_t q = b - kFlowGate;
      for (uint32_t it = 0;; ++it) {
        bool ok = true;
        if (lane < nw) ok = ld_acquire_cta(&S.prog[lane]) >= (q >= lane ? (q - lane) / nw + 1u : 0u);
        if (__all_sync(0xFFFFFFFFu, ok)) break;
        if (!keep_polling(it)) return;
      }
      __syncwarp();
    }
    int32_t v0 = 0, v1 = 0;
    uint32_t acc = 0;  // extra reads of a transfer; every read past the first two of a scan
    uint32_t pm = 0;   // a transfer's reads waiting on the ring
    unsigned long long gpend = 0;  // reads waiting on global memory (a scan: all of them)
    auto take = [&](uint32_t k, uint32_t x) {
      v0 = k == 0 ? (int32_t)x : v0;
      v1 = k == 1 ? (int32_t)x : v1;
      acc += k >= 2 ? x : 0u;
    };
    const ModMagic mm(ro ? 1u : CSMV_OP_AMOD(op));
    uint32_t ridx[NR], rtag[NR];
    if (!ro) {
      // committed values, and outputs of producers that finished (all loads issued together)
      unsigned long long gv[NR];
#pragma unroll
      for (uint32_t k = 0; k < NR; k++) {
        const unsigned long long s = sv[k];
        gv[k] = s;
        if (k < nr && !(s & kFlowValue) && b - ((uint32_t)s >> 6) >= kFlowGate)
          gv[k] = ld_relaxed_cta_global(&f.out[s]);
        ridx[k] = (uint32_t)s & (2u * kFlowRing - 1u);
        rtag[k] = ((uint32_t)s >> 1) + 1u;
      }
#pragma unroll
      for (uint32_t k = 0; k < NR; k++) {
        if (k >= nr) continue;
        const unsigned long long s = sv[k];
        if (s & kFlowValue) {
          take(k, (uint32_t)s);
        } else if (b - ((uint32_t)s >> 6) >= kFlowGate) {
          if ((gv[k] & 0xFFFFFFFF00000000ull) == tag)
            take(k, (uint32_t)gv[k]);
          else
            gpend |= 1ull << k;
        } else {
          pm |= 1u << k;
        }
      }
    } else {
      gpend = (1ull << nr) - 1ull;  // a scan: every read through flow_fetch (nr <= 63)
    }
    // the amount, as soon as every extra read is in (usually here, before any wait)
    uint32_t amt = 0;
    bool amt_known = false;
    auto try_amount = [&]() {
      if (!ro && !amt_known && ((pm | (uint32_t)gpend) & ~3u) == 0u) {
        amt = 1u + mm.mod(CSMV_OP_AMT0(op) - 1u + acc);
        amt_known = true;
      }
    };
    try_amount();
    bool done = false, hw = false;
    uint32_t o0 = 0, o1 = 0;
    for (uint32_t it = 0;; ++it) {
      if (!done) {
        if (pm) {  // every ring read polled at once; all are taken when all have arrived
          uint32_t rdy = 0, xv[NR];
#pragma unroll
          for (uint32_t k = 0; k < NR; k++) {
            xv[k] = 0u;
            if ((pm >> k) & 1u) {
              const unsigned long long wv = ld_relaxed_cta_shared(&S.ring[ridx[k]]);
              xv[k] = (uint32_t)wv;
              rdy |= (uint32_t)((uint32_t)(wv >> 32) == rtag[k]) << k;
            }
          }
          if (rdy == pm) {
#pragma unroll
            for (uint32_t k = 0; k < NR; k++)
              if ((pm >> k) & 1u) take(k, xv[k]);
            pm = 0u;
          }
        }
        if (gpend) {
          for (unsigned long long m = gpend; m; m &= m - 1ull) {
            const uint32_t k = (uint32_t)__ffsll((long long)m) - 1u;
            uint32_t x;
            if (flow_fetch(f, S, ro ? __ldg(&f.src[e0 + k]) : pick<NR>(sv, k), b, tag, x)) {
              take(k, x);
              gpend &= ~(1ull << k);
            }
          }
        }
        if (pm == 0u && gpend == 0ull) {
          done = true;
          if (!ro) {
            try_amount();
            hw = CSMV_OP_KIND(op) == CSMV_KIND_TRANSFER_ALWAYS || v0 >= (int32_t)amt;
            o0 = hw ? (uint32_t)v0 - amt : (uint32_t)v0;
            o1 = hw ? (uint32_t)v1 + amt : (uint32_t)v1;
            const unsigned long long rt = (unsigned long long)(i + 1u) << 32;
            const uint32_t r0 = (2u * i) & (2u * kFlowRing - 1u);
            if (a0 != a1) st_relaxed_cta_shared(&S.ring[r0], rt | o0);
            st_relaxed_cta_shared(&S.ring[r0 + 1u], rt | o1);
          }
        } else {
          try_amount();
        }
      }
      if (__all_sync(0xFFFFFFFFu, done)) break;
      // (no warp barrier between passes: a ring word read before its store is only "not yet")
      if ((it & 255u) == 255u && !keep_polling(it)) return;
    }
    // off the chain: global outputs, flags, counts, scan results
    if (ro) {
      if (f.b.log) f.b.result[i] = (int32_t)((uint32_t)v0 + (uint32_t)v1 + acc);
      f.wflag[i] = 0u;
    } else {
      if (a0 != a1) st_relaxed_cta_global(&f.out[2u * i], tag | o0);
      st_relaxed_cta_global(&f.out[2u * i + 1u], tag | o1);
      f.wflag[i] = hw ? 1u : 0u;
      if (hw) {
        atomicAdd(&f.cnt[a0], 1u);
        if (a1 != a0) atomicAdd(&f.cnt[a1], 1u);
      }
    }
    __syncwarp();  // every lane's outputs before the block is announced
    if (lane == 0) st_release_cta(&S.prog[w], ++finished);
  }
}

// ---------------------------------------------------------------------------------------------
// Commit
// ---------------------------------------------------------------------------------------------
// wflag: scanned writer ranks (wflag[i + 1] - wflag[i] = has-write of i).
__global__ void __launch_bounds__(256) flow_finalize_kernel(FlowParams f) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= f.n_txn || flow_failed(f)) return;
  const uint32_t base0 = ld_relaxed_gpu(&f.b.gs->ts_next);
  const uint32_t r = f.wflag[i], hw = f.wflag[i + 1] - r;
  if (f.b.log) {
    if (hw) {
      const uint32_t ts = base0 + r + 1u, li = ts - 1u - f.b.log_base;
      if (li < f.b.log_cap)
        f.b.log_txn[li] = i;
      else
        raise_error(&f.b.gs->error, ERR_CAPACITY);
      f.b.outcome[i] = ts;
    } else {
      f.b.outcome[i] = (base0 + r) | kSnapFlag;  // after every earlier writer
    }
    if (CSMV_OP_KIND(f.b.op[i]) != CSMV_KIND_READONLY) f.b.result[i] = 0;
  }
  if (f.b.txn_aborts) f.b.txn_aborts[i] = 0u;
}

template <int DEPTH>
__global__ void __launch_bounds__(256) flow_install_kernel(FlowParams f) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= *f.n_tails || flow_failed(f)) return;
  const uint32_t base0 = ld_relaxed_gpu(&f.b.gs->ts_next);
  const uint2 tl = f.tails[t];
  const uint32_t x = tl.x, total = f.cnt[x];
  f.cnt[x] = 0u;
  if (total == 0u) return;  // no would-be writer of x wrote
  const uint32_t want = total < (uint32_t)DEPTH ? total : (uint32_t)DEPTH;
  // the last `want` actual writes of x, newest first, along the chain of x's writers
  uint32_t tsv[DEPTH], valv[DEPTH];
#pragma unroll
  for (int d = 0; d < DEPTH; d++) tsv[d] = valv[d] = 0u;
  uint32_t got = 0, c = tl.y;
  for (;;) {
    const uint32_t j = c >> 1, s = c & 1u;
    const uint32_t r = f.wflag[j];
    if (f.wflag[j + 1u] != r) {
      const uint32_t v = (uint32_t)f.out[c];
#pragma unroll
      for (int d = 0; d < DEPTH; d++)
        if ((uint32_t)d == got) {
          tsv[d] = base0 + r + 1u;
          valv[d] = v;
        }
      if (++got == want) break;
    }
    const unsigned long long sp = f.src[f.eoff[j] + s];  // j's read of x (read k = slot s)
    if (sp & kFlowValue) break;                           // j was x's first would-be writer
    c = (uint32_t)sp;
  }
  if (got == 0u) return;  // (the chain holds every would-be writer of x: not reached)
  unsigned long long* item = f.b.slots + (size_t)x * DEPTH;
  unsigned long long sl[DEPTH], nv[DEPTH];
#pragma unroll
  for (int d = 0; d < DEPTH; d += 2) ld_relaxed_gpu_v2(item + d, sl[d], sl[d + 1]);
#pragma unroll
  for (int d = 0; d < DEPTH; d++) nv[d] = sl[d];
#pragma unroll
  for (int e = 0; e < DEPTH; e++) {
    if ((uint32_t)e >= got) break;
    const int slot = victim_rank_slot<DEPTH>(sl, (total - 1u - (uint32_t)e) % (uint32_t)DEPTH);
    const unsigned long long ver = pack_version(tsv[e], (int32_t)valv[e]);
#pragma unroll
    for (int d = 0; d < DEPTH; d++)
      if (d == slot) nv[d] = ver;
  }
#pragma unroll
  for (int d = 0; d < DEPTH; d++)
    if (nv[d] != sl[d]) st_relaxed_gpu(item + d, nv[d]);
  st_relaxed_gpu(&f.b.cw[x], (unsigned long long)tsv[0]);
}

__global__ void __launch_bounds__(256) flow_end_kernel(FlowParams f) {
  if (flow_failed(f)) return;
  const uint32_t base0 = ld_relaxed_gpu(&f.b.gs->ts_next);
  const uint32_t W = f.wflag[f.n_txn], base = base0 + W;
  __syncthreads();  // every thread read the cursor before it moves
  // completion-bitmap words the run's timestamps passed over: cleared as the clock advance of
  // the commit kernel would
  if (base > base0) {
    const uint32_t w_lo = (base0 + 1u) >> 5, w_end = (base + 1u) >> 5;
    const uint32_t cnt = min(w_end > w_lo ? w_end - w_lo : 0u, f.b.done_mask + 1u);
    for (uint32_t i = threadIdx.x; i < cnt; i += blockDim.x)
      st_relaxed_gpu(&f.b.done[(w_lo + i) & f.b.done_mask], 0u);
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    st_relaxed_gpu(&f.b.gs->ts_next, base);
    st_release_gpu(&f.b.gs->clock, base);
    const unsigned long long n_ro = f.b.stats[ST_COMMIT_RO];
    atomicAdd(&f.b.stats[ST_COMMIT_UPDATE], (unsigned long long)W);
    atomicAdd(&f.b.stats[ST_COMMIT_NOWRITE], (unsigned long long)f.n_txn - n_ro - W);
    atomicAdd(&f.b.stats[ST_SECTIONS], (unsigned long long)f.b.n_rounds);
    atomicAdd(&f.b.stats[ST_ROUNDS], (unsigned long long)f.b.n_rounds);
  }
}

}  // namespace csmv
