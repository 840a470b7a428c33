// sched_kernels.cuh - kernels of the learned conflict scheduler (sched_engine.cu).
//
// A chunk of a bank stream is planned as follows (all on the device):
//   count     hashed access counts of every account the chunk's transfers touch (a sketch of
//             2^kSketchLog2 counters: "hashed read/write-set" statistics)
//   features  64 bf16 indicators per transaction: thermometer codes of the sketch counts of the
//             two written accounts and of the hottest other read, and of the recent abort rates
//             of the written accounts' range bins
//   labels    after the chunk's probe slice ran in stream order: 1 if the transfer aborted
//   keys/pos  transfers the network flags as likely to abort are keyed by their hotter written
//             account; the k-th of c transactions with one key gets position (k + u) / c, u a
//             hash in [0, 1), so a key's transactions are spread evenly over the chunk instead
//             of bunching at random; unflagged transfers get position u
//   sort      counting sort of the transfers by position bucket
//   emit      rounds: read-only rounds interleaved evenly with the sorted transfer rounds,
//             optional deferred rounds (the highest predicted risk) at the end
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

#include "../../include/csmv.h"

namespace csmv {

constexpr int kSketchLog2 = 22;
constexpr uint32_t kSketchMask = (1u << kSketchLog2) - 1u;
constexpr int kRateBins = 64;

__host__ __device__ __forceinline__ uint32_t sketch_slot(uint32_t a) {
  return (a * 0x9E3779B1u) >> (32 - kSketchLog2);
}
__device__ __forceinline__ float unit_hash(uint64_t seed, uint32_t i) {
  uint64_t z = seed + 0x9E3779B97F4A7C15ull * (i + 1ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (float)(z >> 40) * (1.0f / 16777216.0f);
}
__device__ __forceinline__ uint32_t rate_bin(uint32_t a, uint32_t n_accounts) {
  const uint32_t b = (uint32_t)(((uint64_t)a * kRateBins) / n_accounts);
  return b < (uint32_t)kRateBins ? b : (uint32_t)kRateBins - 1u;  // out-of-range ids stay in bounds
}

// accesses of transfers only (read-only rounds neither abort nor make transfers abort)
__global__ void sched_count_kernel(const uint32_t* op, const uint32_t* off, const uint32_t* addr,
                                   uint32_t n, uint32_t* sketch) {
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const uint32_t o = op[t];
    if (CSMV_OP_KIND(o) == CSMV_KIND_READONLY) continue;
    const uint32_t nr = CSMV_OP_NREADS(o), base = off[t];
    for (uint32_t k = 0; k < nr; k++) atomicAdd(&sketch[sketch_slot(addr[base + k])], 1u);
  }
}

__device__ __forceinline__ uint32_t count_level(uint32_t c) {
  // thermometer levels: count >= 1 2 3 4 5 6 8 10 12 16 20 24 32 48 64 128
  const uint32_t th[16] = {1, 2, 3, 4, 5, 6, 8, 10, 12, 16, 20, 24, 32, 48, 64, 128};
  uint32_t m = 0;
#pragma unroll
  for (int i = 0; i < 16; i++) m |= (c >= th[i] ? 1u : 0u) << i;
  return m;
}
__device__ __forceinline__ uint32_t rate_level(float r) {
  const float th[8] = {0.005f, 0.01f, 0.02f, 0.05f, 0.1f, 0.2f, 0.3f, 0.5f};
  uint32_t m = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) m |= (r >= th[i] ? 1u : 0u) << i;
  return m;
}

// Features of transactions [t0, t1): 64 bits -> 64 bf16 values 0/1, 128 bytes per row.
__global__ void sched_features_kernel(const uint32_t* op, const uint32_t* off, const uint32_t* addr,
                                      uint32_t t0, uint32_t t1, uint32_t n_accounts,
                                      const uint32_t* sketch, const float* rates,
                                      uint4* __restrict__ x) {
  for (uint32_t t = t0 + blockIdx.x * blockDim.x + threadIdx.x; t < t1; t += gridDim.x * blockDim.x) {
    const uint32_t o = op[t];
    uint64_t bits = 0;
    if (CSMV_OP_KIND(o) != CSMV_KIND_READONLY) {
      const uint32_t nr = CSMV_OP_NREADS(o), base = off[t];
      const uint32_t a0 = addr[base], a1 = addr[base + 1];
      uint32_t cmax = 0;
      for (uint32_t k = 2; k < nr; k++) cmax = max(cmax, sketch[sketch_slot(addr[base + k])]);
      bits = (uint64_t)count_level(sketch[sketch_slot(a0)]) |
             ((uint64_t)count_level(sketch[sketch_slot(a1)]) << 16) |
             ((uint64_t)count_level(cmax) << 32) |
             ((uint64_t)rate_level(rates[rate_bin(a0, n_accounts)]) << 48) |
             ((uint64_t)rate_level(rates[rate_bin(a1, n_accounts)]) << 56);
    }
    // bf16 1.0 = 0x3F80
    uint4* row = x + (size_t)t * 8;
#pragma unroll
    for (int q = 0; q < 8; q++) {
      uint32_t w[4];
#pragma unroll
      for (int h = 0; h < 4; h++) {
        const int i = q * 8 + h * 2;
        w[h] = (((bits >> i) & 1ull) ? 0x3F80u : 0u) | (((bits >> (i + 1)) & 1ull) ? 0x3F800000u : 0u);
      }
      row[q] = make_uint4(w[0], w[1], w[2], w[3]);
    }
  }
}

// Labels of the probe slice (1: the transfer aborted or, under group commit, waited for a lock
// another warp held - a conflict either way) and the per-bin access / conflict counts.
__global__ void sched_labels_kernel(const uint32_t* op, const uint32_t* off, const uint32_t* addr,
                                    uint32_t n, uint32_t n_accounts, const uint32_t* aborts,
                                    const uint32_t* waits, float* y,
                                    unsigned long long* bin_stats) {
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const uint32_t o = op[t];
    const bool upd = CSMV_OP_KIND(o) != CSMV_KIND_READONLY;
    const bool ab = upd && (aborts[t] > 0 || waits[t] != 0u);
    y[t] = ab ? 1.f : 0.f;
    if (!upd) continue;
    const uint32_t base = off[t];
    for (int k = 0; k < 2; k++) {
      const uint32_t b = rate_bin(addr[base + k], n_accounts);
      atomicAdd(&bin_stats[2 * b], 1ull);
      if (ab) atomicAdd(&bin_stats[2 * b + 1], 1ull);
    }
  }
}

__global__ void sched_rates_kernel(unsigned long long* bin_stats, float* rates) {
  const int b = threadIdx.x;
  if (b >= kRateBins) return;
  const unsigned long long acc = bin_stats[2 * b], ab = bin_stats[2 * b + 1];
  if (acc) rates[b] = 0.5f * rates[b] + 0.5f * (float)((double)ab / (double)acc);
  bin_stats[2 * b] = bin_stats[2 * b + 1] = 0;
}

// Transfers [t0, t1) flagged by the network (p > threshold) take a key: the written account
// with the larger sketch count; keyed transactions are counted per key.
__global__ void sched_keys_kernel(const uint32_t* op, const uint32_t* off, const uint32_t* addr,
                                  uint32_t t0, uint32_t t1, const float* p, float threshold,
                                  const uint32_t* sketch, uint32_t* key, uint32_t* key_count,
                                  uint32_t* n_flagged) {
  uint32_t flagged = 0;
  for (uint32_t t = t0 + blockIdx.x * blockDim.x + threadIdx.x; t < t1; t += gridDim.x * blockDim.x) {
    const uint32_t o = op[t];
    uint32_t k = 0xFFFFFFFFu;
    if (CSMV_OP_KIND(o) != CSMV_KIND_READONLY && p[t - t0] > threshold) {
      const uint32_t base = off[t];
      const uint32_t a0 = addr[base], a1 = addr[base + 1];
      const uint32_t s0 = sketch_slot(a0), s1 = sketch_slot(a1);
      k = sketch[s1] > sketch[s0] ? s1 : s0;
      atomicAdd(&key_count[k], 1u);
      flagged++;
    }
    key[t - t0] = k;
  }
  if (flagged) atomicAdd(n_flagged, flagged);
}

// Position bucket of every transfer: keyed (k + u) / c, else u; the deferred bucket (index
// n_buckets) takes transfers with p > defer_threshold.
__global__ void sched_bucket_kernel(const uint32_t* op, uint32_t t0, uint32_t t1, const float* p,
                                    float defer_threshold, const uint32_t* key,
                                    const uint32_t* key_count, uint32_t* key_rank,
                                    uint32_t n_buckets, uint64_t seed, uint32_t* bucket,
                                    uint32_t* bucket_count) {
  for (uint32_t t = t0 + blockIdx.x * blockDim.x + threadIdx.x; t < t1; t += gridDim.x * blockDim.x) {
    const uint32_t i = t - t0;
    if (CSMV_OP_KIND(op[t]) == CSMV_KIND_READONLY) {
      bucket[i] = 0xFFFFFFFFu;
      continue;
    }
    const float u = unit_hash(seed, t);
    float pos = u;
    const uint32_t k = key[i];
    if (k != 0xFFFFFFFFu) {
      const uint32_t r = atomicAdd(&key_rank[k], 1u);
      pos = ((float)r + u) / (float)key_count[k];
    }
    uint32_t b = min((uint32_t)(pos * (float)n_buckets), n_buckets - 1u);
    if (p[i] > defer_threshold) b = n_buckets;
    bucket[i] = b;
    atomicAdd(&bucket_count[b], 1u);
  }
}

// Exclusive scan of n (<= 1024 * 64) counters in one CTA of 1024 threads; out[n] = total.
__global__ void __launch_bounds__(1024) sched_scan_kernel(const uint32_t* in, uint32_t n,
                                                          uint32_t* out) {
  __shared__ uint32_t part[1024];
  const uint32_t per = (n + 1023) / 1024, lo = threadIdx.x * per, hi = min(lo + per, n);
  uint32_t s = 0;
  for (uint32_t i = lo; i < hi; i++) s += in[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (uint32_t d = 1; d < 1024; d <<= 1) {
    const uint32_t v = threadIdx.x >= d ? part[threadIdx.x - d] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t run = part[threadIdx.x] - s;
  for (uint32_t i = lo; i < hi; i++) {
    out[i] = run;
    run += in[i];
  }
  if (threadIdx.x == 1023) out[n] = part[1023];
}

__global__ void sched_scatter_kernel(uint32_t t0, uint32_t t1, const uint32_t* bucket,
                                     const uint32_t* bucket_start, uint32_t* bucket_fill,
                                     uint32_t* order) {
  for (uint32_t t = t0 + blockIdx.x * blockDim.x + threadIdx.x; t < t1; t += gridDim.x * blockDim.x) {
    const uint32_t b = bucket[t - t0];
    if (b == 0xFFFFFFFFu) continue;
    order[bucket_start[b] + atomicAdd(&bucket_fill[b], 1u)] = t;
  }
}

// Flags of read-only rounds among rounds [r0, r1).
__global__ void sched_ro_flags_kernel(const uint32_t* op, uint32_t r0, uint32_t r1, uint32_t* flag) {
  for (uint32_t r = r0 + blockIdx.x * blockDim.x + threadIdx.x; r < r1; r += gridDim.x * blockDim.x)
    flag[r - r0] = CSMV_OP_KIND(op[r * 32u]) == CSMV_KIND_READONLY ? 1u : 0u;
}

__global__ void sched_ro_list_kernel(uint32_t r0, uint32_t n_rounds, const uint32_t* flag,
                                     const uint32_t* flag_scan, uint32_t* ro_list) {
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n_rounds; r += gridDim.x * blockDim.x)
    if (flag[r]) ro_list[flag_scan[r]] = r0 + r;
}

// Planned stream: R_main = R_ro + U_main rounds with the R_ro read-only rounds at positions
// floor(i * R_main / R_ro), transfer rounds in sorted order in between, then the deferred
// transfer rounds. perm[i] = original transaction of planned slot i.
__global__ void sched_emit_kernel(const uint32_t* op, const uint32_t* off, uint32_t n_rounds,
                                  uint32_t r_ro, uint32_t r_main, const uint32_t* ro_list,
                                  const uint32_t* order, uint32_t* perm, uint32_t* op2,
                                  uint32_t* off2) {
  const uint32_t n = n_rounds * 32u;
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    const uint32_t pos = s / 32u, lane = s % 32u;
    uint32_t src;
    if (pos < r_main && r_ro) {
      // read-only slots before pos: ceil(pos * r_ro / r_main)
      const uint32_t i = (uint32_t)(((uint64_t)pos * r_ro + r_main - 1) / r_main);
      const bool is_ro = i < r_ro && (uint32_t)(((uint64_t)i * r_main) / r_ro) == pos;
      src = is_ro ? ro_list[i] * 32u + lane : order[(pos - i) * 32u + lane];
    } else {
      src = order[(pos - r_ro) * 32u + lane];
    }
    perm[s] = src;
    op2[s] = op[src];
    off2[s] = off[src];
  }
}

// ---------------------------------------------------------------------------------------------
// Multi-block exclusive scan of n counters (any n up to 2^28): tiles of 4096 scanned by one CTA
// each, the tile totals by sched_scan_kernel, then the tile offsets added.
// ---------------------------------------------------------------------------------------------
constexpr uint32_t kScanTile = 4096;

__global__ void __launch_bounds__(1024) sched_scan_tiles_kernel(const uint32_t* in, uint32_t n,
                                                                uint32_t* out, uint32_t* tile_sum) {
  __shared__ uint32_t part[1024];
  const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * 4u;
  uint32_t v[4], s = 0;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    v[i] = base + i < n ? in[base + i] : 0u;
    s += v[i];
  }
  part[threadIdx.x] = s;
  __syncthreads();
  for (uint32_t d = 1; d < 1024; d <<= 1) {
    const uint32_t x = threadIdx.x >= d ? part[threadIdx.x - d] : 0u;
    __syncthreads();
    part[threadIdx.x] += x;
    __syncthreads();
  }
  uint32_t run = part[threadIdx.x] - s;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
  if (threadIdx.x == 1023) tile_sum[blockIdx.x] = part[1023];
}

// out[i] += tile_off[i / kScanTile]; out[n] = the total
__global__ void sched_scan_add_kernel(uint32_t* out, uint32_t n, const uint32_t* tile_off,
                                      uint32_t tiles) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += gridDim.x * blockDim.x)
    out[i] = i < n ? out[i] + tile_off[i / kScanTile] : tile_off[tiles];
}

// ---------------------------------------------------------------------------------------------
// Grouped plan: transfers likely to conflict are sorted by the two hottest accounts they touch
// (read or write), so the 32 transfers of a round share their hot accounts and the engine's
// group commit locks each hot account once for all of them; the rounds of one hot account are
// then spread evenly over the plan, so warps queue for many different hot accounts at once.
//   hot account: sketch count >= hot_count; hot index = its rank among hot sketch slots
//   key = hidx(h1) << 6 | hidx(h2) mod 63 (63 when the transfer touches one hot account);
//   transfers not flagged, or touching no hot account (or a hot index >= 65535), take the cold
//   key (2^22 - 1) and keep stream order among themselves
// ---------------------------------------------------------------------------------------------
constexpr uint32_t kGroupKeys = 1u << 22;
constexpr uint32_t kColdKey = kGroupKeys - 1u;
constexpr uint32_t kHotNone = 0xFFFFu;
constexpr uint32_t kMaxLanes = 64;  // hot lanes of a grouped plan at most

__global__ void sched_hot_flags_kernel(const uint32_t* sketch, uint32_t hot_count, uint32_t* flag) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= kSketchMask; i += gridDim.x * blockDim.x)
    flag[i] = sketch[i] >= hot_count ? 1u : 0u;
}

// Heat class of every account of the bank for the engine's lock order: 0 below hot_count, else
// 1 + 4 log2(count / hot_count) (quarter octaves, from the count's two bits below its leading
// one), at most 255. Accounts sharing a sketch slot share its class; any class is a valid order.
__global__ void sched_lock_last_kernel(uint32_t n_accounts, const uint32_t* sketch,
                                       uint32_t hot_count, uint8_t* cls) {
  for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < n_accounts; x += gridDim.x * blockDim.x) {
    const uint32_t c = sketch[sketch_slot(x)];
    uint32_t k = 0;
    if (c >= hot_count) {
      const uint32_t q = c / max(hot_count, 1u);  // >= 1
      const uint32_t l = 31u - __clz(q);
      const uint32_t frac = l >= 2u ? (q >> (l - 2u)) & 3u : (l == 1u ? (q & 1u) << 1 : 0u);
      k = min(255u, 1u + 4u * l + frac);
    }
    cls[x] = (uint8_t)k;
  }
}

// score: 0 = the network's predicted probability p[t - t0]; 1 = the raw sketch-count score
// (count of the transfer's most-accessed account / the chunk's largest count, no network).
// backoff (ns) per transaction: 0 below a score of 1/4, else score x backoff_ns.
__global__ void sched_group_keys_kernel(const uint32_t* op, const uint32_t* off,
                                        const uint32_t* addr, uint32_t t0, uint32_t t1,
                                        const float* p, float threshold, uint32_t score_mode,
                                        const uint32_t* sketch, const uint32_t* max_count,
                                        uint32_t hot_count, const uint32_t* hidx, uint32_t* key,
                                        uint32_t* rank, uint32_t* key_count, uint32_t* n_flagged,
                                        uint32_t* backoff, uint32_t backoff_ns,
                                        uint32_t key_written) {
  uint32_t flagged = 0;
  for (uint32_t t = t0 + blockIdx.x * blockDim.x + threadIdx.x; t < t1; t += gridDim.x * blockDim.x) {
    const uint32_t i = t - t0, o = op[t];
    if (CSMV_OP_KIND(o) == CSMV_KIND_READONLY) {
      key[i] = 0xFFFFFFFFu;
      backoff[i] = 0u;
      continue;
    }
    const uint32_t nr = CSMV_OP_NREADS(o), base = off[t];
    uint32_t c1 = 0, c2 = 0, x1 = kHotNone, x2 = kHotNone, cmax = 0;
    for (uint32_t k = 0; k < nr; k++) {
      const uint32_t sl = sketch_slot(addr[base + k]), c0 = sketch[sl];
      cmax = max(cmax, c0);
      if (c0 < hot_count) continue;
      // key_written: a written account (k < 2) ranks above every read-only one, so a round's
      // transfers share the hot account they WRITE (the lock the group must take)
      const uint32_t c = (key_written && k < 2) ? c0 + 0x40000000u : c0;
      const uint32_t h = min(hidx[sl], kHotNone);
      if (h == x1 || h == x2) continue;  // two accounts hashed to one slot
      if (c > c1 || (c == c1 && h < x1)) {
        c2 = c1;
        x2 = x1;
        c1 = c;
        x1 = h;
      } else if (c > c2 || (c == c2 && h < x2)) {
        c2 = c;
        x2 = h;
      }
    }
    const float sc = score_mode ? (float)cmax / (float)max(1u, *max_count) : p[i];
    const bool hot = sc > threshold && x1 != kHotNone;
    const uint32_t k = hot ? (x1 << 6) | (x2 == kHotNone ? 63u : x2 % 63u) : kColdKey;
    key[i] = k;
    rank[i] = atomicAdd(&key_count[k], 1u);
    backoff[i] = sc >= 0.25f ? (uint32_t)(fminf(sc, 1.f) * (float)backoff_ns) : 0u;
    flagged += hot ? 1u : 0u;
  }
  if (flagged) atomicAdd(n_flagged, flagged);
}

__global__ void sched_max_kernel(const uint32_t* in, uint32_t n, uint32_t* out) {
  uint32_t m = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    m = max(m, in[i]);
  m = __reduce_max_sync(0xFFFFFFFFu, m);
  if ((threadIdx.x & 31u) == 0 && m) atomicMax(out, m);
}

// sorted[key_start[key] + rank] = transaction (transfers of [t0, t1) only); the cold key's
// transfers keep stream order (their rank is replaced by their position among cold transfers,
// computed from a scan of cold flags)
__global__ void sched_group_scatter_kernel(uint32_t t0, uint32_t t1, const uint32_t* key,
                                           const uint32_t* rank, const uint32_t* key_start,
                                           const uint32_t* cold_pos, uint32_t* sorted) {
  for (uint32_t t = t0 + blockIdx.x * blockDim.x + threadIdx.x; t < t1; t += gridDim.x * blockDim.x) {
    const uint32_t i = t - t0, k = key[i];
    if (k == 0xFFFFFFFFu) continue;
    sorted[key_start[k] + (k == kColdKey ? cold_pos[i] : rank[i])] = t;
  }
}

__global__ void sched_cold_flags_kernel(uint32_t n, const uint32_t* key, uint32_t* flag) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    flag[i] = key[i] == kColdKey ? 1u : 0u;
}

// Position bucket of every transfer round of the sorted list: the j-th of the n rounds that start
// within one hot account's keys goes to (j + u) / n of the plan (u a hash of the account in
// [0, 1)), a cold round to a hash of its index.
// Lanes of the hottest accounts (hot_lanes): every hot index whose transfers fill at least
// min_rounds rounds gets a lane of its own, first come first served, while lanes last (lane_of:
// lane, or kHotNone).
__global__ void sched_hot_lanes_kernel(const uint32_t* key_start, uint32_t min_rounds,
                                       uint32_t n_lanes, uint32_t* lane_count, uint32_t* lane_of) {
  for (uint32_t h = blockIdx.x * blockDim.x + threadIdx.x; h < kHotNone; h += gridDim.x * blockDim.x) {
    const uint32_t n = key_start[(h + 1u) << 6] - key_start[h << 6];
    uint32_t q = kHotNone;
    if (n_lanes && n >= 32u * min_rounds) {
      q = atomicAdd(lane_count, 1u);
      if (q >= n_lanes) q = kHotNone;
    }
    lane_of[h] = q;
  }
}

__global__ void sched_round_bucket_kernel(uint32_t t0, uint32_t U, const uint32_t* sorted,
                                          const uint32_t* key, const uint32_t* key_start,
                                          uint64_t seed, const uint32_t* lane_of,
                                          uint32_t* rbucket, uint32_t* bcount) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < U; j += gridDim.x * blockDim.x) {
    const uint32_t k = key[sorted[32u * j] - t0], h1 = k >> 6;
    float pos;
    if (k != kColdKey && h1 < kHotNone && lane_of && lane_of[h1] != kHotNone) {
      // a round of a laned account: bucket U + lane, after every position of the main plan
      rbucket[j] = U + lane_of[h1];
      atomicAdd(&bcount[U + lane_of[h1]], 1u);
      continue;
    }
    if (k == kColdKey || h1 >= kHotNone) {
      pos = unit_hash(seed, j);
    } else {
      const uint32_t S = key_start[h1 << 6], E = key_start[(h1 + 1u) << 6];
      const uint32_t first = (S + 31u) / 32u, last = (E - 1u) / 32u;  // rounds starting in [S, E)
      const uint32_t n = last >= first ? last - first + 1u : 1u;
      const uint32_t idx = j >= first ? j - first : 0u;
      pos = ((float)min(idx, n - 1u) + unit_hash(seed ^ 0xA5A5A5A5ull, h1)) / (float)n;
    }
    const uint32_t b = min((uint32_t)(pos * (float)U), U - 1u);
    rbucket[j] = b;
    atomicAdd(&bcount[b], 1u);
  }
}

__global__ void sched_round_scatter_kernel(uint32_t U, const uint32_t* rbucket,
                                           const uint32_t* bstart, uint32_t* bfill,
                                           uint32_t* round_order) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < U; j += gridDim.x * blockDim.x) {
    const uint32_t b = rbucket[j];
    round_order[bstart[b] + atomicAdd(&bfill[b], 1u)] = j;
  }
}

// lane_start[q] = first planned round of lane q (the laned rounds follow the r_main others)
__global__ void sched_lane_start_kernel(uint32_t U, uint32_t n_lanes, uint32_t r_main,
                                        const uint32_t* bstart, uint32_t* lane_start) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q <= n_lanes) lane_start[q] = r_main + (bstart[U + q] - bstart[U]);
}

// order[32 i + lane] = sorted[32 round_order[i] + lane]
__global__ void sched_expand_rounds_kernel(uint32_t U, const uint32_t* round_order,
                                           const uint32_t* sorted, uint32_t* order) {
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < U * 32u; s += gridDim.x * blockDim.x)
    order[s] = sorted[32u * round_order[s / 32u] + (s & 31u)];
}

// backoff of the planned stream: bo2[s] = backoff of the transaction at planned slot s
__global__ void sched_plan_backoff_kernel(uint32_t n, uint32_t t0, const uint32_t* perm,
                                          const uint32_t* bo, uint32_t* bo2) {
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
    bo2[s] = bo[perm[s] - t0];
}

}  // namespace csmv
