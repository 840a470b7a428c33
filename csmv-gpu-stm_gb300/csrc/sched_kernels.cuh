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

// Labels of the probe slice and the per-bin access / abort counts of its transfers.
__global__ void sched_labels_kernel(const uint32_t* op, const uint32_t* off, const uint32_t* addr,
                                    uint32_t n, uint32_t n_accounts, const uint32_t* aborts,
                                    float* y, unsigned long long* bin_stats) {
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const uint32_t o = op[t];
    const bool upd = CSMV_OP_KIND(o) != CSMV_KIND_READONLY;
    const bool ab = upd && aborts[t] > 0;
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

}  // namespace csmv
