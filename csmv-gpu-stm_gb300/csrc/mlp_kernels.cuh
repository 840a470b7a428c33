// mlp_kernels.cuh - the conflict predictor's network: 64 -> 128 -> 128 -> 1 (ReLU, ReLU,
// sigmoid), bf16 weights, fp32 accumulation, hand-written forward, backward and Adam kernels.
//
// Layout: features X [n][64] bf16 (0/1 indicators here, exact in bf16); weights W1 [64][128],
// W2 [128][128], w3 [128] in bf16 (rounded from fp32 master copies after every step), biases
// fp32. A CTA of 256 threads works on tiles of 64 samples with every operand in shared memory;
// thread (ty, tx) = (tid / 16, tid % 16) owns samples 4ty..4ty+3 x hidden units tx + 16b
// (b < 8) of an activation tile (interleaved so a warp's weight reads hit 16 distinct banks).
// The tile GEMMs run on the FP32 pipes: the whole network is ~25 K multiply-adds per sample,
// well under 1 % of the per-transaction time of the commit kernel whose input it schedules.
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

namespace csmv {

constexpr int kMlpIn = 64, kMlpHid = 128, kMlpTile = 64, kMlpThreads = 256;
// fp32 master parameter block: W1 | b1 | W2 | b2 | w3 | b3 (+3 pad)
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kMlpIn * kMlpHid, kOffW2 = kOffB1 + kMlpHid,
              kOffB2 = kOffW2 + kMlpHid * kMlpHid, kOffW3 = kOffB2 + kMlpHid,
              kOffB3 = kOffW3 + kMlpHid, kMlpParams = kOffB3 + 4;

// padded row strides (floats) keep the 4-sample column reads free of bank conflicts
constexpr int kXs = kMlpIn + 1, kHs = kMlpHid + 1;

struct MlpSmem {
  float w1[kMlpIn * kMlpHid];    // [k][j]
  float w2[kMlpHid * kHs];       // [i][j], row stride kHs
  float b1[kMlpHid], b2[kMlpHid], w3[kMlpHid];
  float x[kMlpTile * kXs];       // [s][k]
  float h1[kMlpTile * kHs];      // [s][i] post-ReLU
  float h2[kMlpTile * kHs];      // [s][j] post-ReLU, then dL/dh2 pre-activation
  float dz[kMlpTile];
  float b3;
};

__device__ __forceinline__ void mlp_load_weights(MlpSmem& sm, const __nv_bfloat16* w1,
                                                 const __nv_bfloat16* w2, const __nv_bfloat16* w3,
                                                 const float* bias) {
  for (int i = threadIdx.x; i < kMlpIn * kMlpHid; i += blockDim.x) sm.w1[i] = __bfloat162float(w1[i]);
  for (int i = threadIdx.x; i < kMlpHid * kMlpHid; i += blockDim.x)
    sm.w2[(i / kMlpHid) * kHs + i % kMlpHid] = __bfloat162float(w2[i]);
  for (int i = threadIdx.x; i < kMlpHid; i += blockDim.x) {
    sm.b1[i] = bias[kOffB1 + i];
    sm.b2[i] = bias[kOffB2 + i];
    sm.w3[i] = __bfloat162float(w3[i]);
  }
  if (threadIdx.x == 0) sm.b3 = bias[kOffB3];
}

// X tile -> smem (rows beyond n are zero)
__device__ __forceinline__ void mlp_load_x(MlpSmem& sm, const __nv_bfloat16* x, uint32_t s0,
                                           uint32_t n) {
  for (int i = threadIdx.x; i < kMlpTile * kMlpIn; i += blockDim.x) {
    const uint32_t s = i / kMlpIn, k = i % kMlpIn;
    sm.x[s * kXs + k] = (s0 + s < n) ? __bfloat162float(x[(size_t)(s0 + s) * kMlpIn + k]) : 0.f;
  }
}

// Forward of one tile; leaves h1, h2 (post-ReLU) and returns z for samples ty*4.. in zq[4]
// (valid in the tx == 0 thread of each row group after the reduction).
__device__ __forceinline__ void mlp_tile_forward(MlpSmem& sm, float zq[4]) {
  const int ty = threadIdx.x / 16, tx = threadIdx.x % 16;
  const int s0 = ty * 4;
  float acc[4][8];
  // layer 1: h1 = relu(x W1 + b1)
#pragma unroll
  for (int q = 0; q < 4; q++)
#pragma unroll
    for (int j = 0; j < 8; j++) acc[q][j] = sm.b1[tx + 16 * j];
#pragma unroll 4
  for (int k = 0; k < kMlpIn; k++) {
    float xv[4], wv[8];
#pragma unroll
    for (int q = 0; q < 4; q++) xv[q] = sm.x[(s0 + q) * kXs + k];
#pragma unroll
    for (int j = 0; j < 8; j++) wv[j] = sm.w1[k * kMlpHid + tx + 16 * j];
#pragma unroll
    for (int q = 0; q < 4; q++)
#pragma unroll
      for (int j = 0; j < 8; j++) acc[q][j] = fmaf(xv[q], wv[j], acc[q][j]);
  }
#pragma unroll
  for (int q = 0; q < 4; q++)
#pragma unroll
    for (int j = 0; j < 8; j++) sm.h1[(s0 + q) * kHs + tx + 16 * j] = fmaxf(acc[q][j], 0.f);
  __syncthreads();
  // layer 2: h2 = relu(h1 W2 + b2)
#pragma unroll
  for (int q = 0; q < 4; q++)
#pragma unroll
    for (int j = 0; j < 8; j++) acc[q][j] = sm.b2[tx + 16 * j];
#pragma unroll 4
  for (int k = 0; k < kMlpHid; k++) {
    float hv[4], wv[8];
#pragma unroll
    for (int q = 0; q < 4; q++) hv[q] = sm.h1[(s0 + q) * kHs + k];
#pragma unroll
    for (int j = 0; j < 8; j++) wv[j] = sm.w2[k * kHs + tx + 16 * j];
#pragma unroll
    for (int q = 0; q < 4; q++)
#pragma unroll
      for (int j = 0; j < 8; j++) acc[q][j] = fmaf(hv[q], wv[j], acc[q][j]);
  }
  // layer 3 partial dot products, then a reduction over the 16 tx lanes of the row group
#pragma unroll
  for (int q = 0; q < 4; q++) {
    float z = 0.f;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const float h = fmaxf(acc[q][j], 0.f);
      sm.h2[(s0 + q) * kHs + tx + 16 * j] = h;
      z = fmaf(h, sm.w3[tx + 16 * j], z);
    }
#pragma unroll
    for (int o = 8; o >= 1; o >>= 1) z += __shfl_xor_sync(0xFFFFFFFFu, z, o);
    zq[q] = z + sm.b3;
  }
}

__device__ __forceinline__ float mlp_sigmoid(float z) { return 1.f / (1.f + expf(-z)); }

// p[s] = sigmoid(z) for every sample. Grid-stride over tiles.
__global__ void __launch_bounds__(kMlpThreads) mlp_forward_kernel(
    const __nv_bfloat16* __restrict__ x, uint32_t n, const __nv_bfloat16* w1,
    const __nv_bfloat16* w2, const __nv_bfloat16* w3, const float* master, float* __restrict__ p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  MlpSmem& sm = *reinterpret_cast<MlpSmem*>(smem_raw);
  mlp_load_weights(sm, w1, w2, w3, master);
  const int ty = threadIdx.x / 16, tx = threadIdx.x % 16;
  for (uint32_t s0 = blockIdx.x * kMlpTile; s0 < n; s0 += gridDim.x * kMlpTile) {
    __syncthreads();  // weights loaded / previous tile's reads done
    mlp_load_x(sm, x, s0, n);
    __syncthreads();
    float zq[4];
    mlp_tile_forward(sm, zq);
    if (tx == 0)
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const uint32_t s = s0 + ty * 4 + q;
        if (s < n) p[s] = mlp_sigmoid(zq[q]);
      }
  }
}

// Gradient of the mean binary cross-entropy over n samples, accumulated (atomicAdd) into
// grad[kMlpParams] (fp32, same packing as the master block); the summed loss into *loss.
// Grid-stride over tiles; each CTA keeps its share of dW1 and dW2 in registers across tiles.
__global__ void __launch_bounds__(kMlpThreads) mlp_grad_kernel(
    const __nv_bfloat16* __restrict__ x, const float* __restrict__ y, uint32_t n,
    const __nv_bfloat16* w1, const __nv_bfloat16* w2, const __nv_bfloat16* w3,
    const float* master, float* grad, float* loss) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  MlpSmem& sm = *reinterpret_cast<MlpSmem*>(smem_raw);
  mlp_load_weights(sm, w1, w2, w3, master);
  const int tid = threadIdx.x, ty = tid / 16, tx = tid % 16;
  const float inv_n = 1.f / (float)n;
  // register accumulators: dW2 rows i = ty*8+a, cols j = tx+16b; dW1 rows k = ty*4+a, cols
  // i = tx+16b
  float gw2[8][8], gw1[4][8];
#pragma unroll
  for (int a = 0; a < 8; a++)
#pragma unroll
    for (int b = 0; b < 8; b++) gw2[a][b] = 0.f;
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 8; b++) gw1[a][b] = 0.f;
  float gb1 = 0.f, gb2 = 0.f, gw3 = 0.f, gb3 = 0.f, lsum = 0.f;  // thread tid < 128 owns unit tid

  for (uint32_t s0 = blockIdx.x * kMlpTile; s0 < n; s0 += gridDim.x * kMlpTile) {
    __syncthreads();
    mlp_load_x(sm, x, s0, n);
    __syncthreads();
    float zq[4];
    mlp_tile_forward(sm, zq);
    if (tx == 0) {
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const uint32_t s = s0 + ty * 4 + q;
        float d = 0.f;
        if (s < n) {
          const float z = zq[q], t = y[s];
          d = (mlp_sigmoid(z) - t) * inv_n;
          // softplus(z) - t z, written to stay finite for large |z|
          lsum += fmaxf(z, 0.f) - t * z + log1pf(expf(-fabsf(z)));
        }
        sm.dz[ty * 4 + q] = d;
      }
    }
    __syncthreads();
    // dw3, db3, db2 partials and dh2 = dz * w3 * relu'(h2), in place over h2
    if (tid < kMlpHid) {
      float a3 = 0.f;
      for (int s = 0; s < kMlpTile; s++) a3 = fmaf(sm.dz[s], sm.h2[s * kHs + tid], a3);
      gw3 += a3;
    }
    if (tid == kMlpHid) {
      float a = 0.f;
      for (int s = 0; s < kMlpTile; s++) a += sm.dz[s];
      gb3 += a;
    }
    __syncthreads();
    for (int e = tid; e < kMlpTile * kMlpHid; e += kMlpThreads) {
      const int s = e / kMlpHid, j = e % kMlpHid;
      const float h = sm.h2[s * kHs + j];
      sm.h2[s * kHs + j] = h > 0.f ? sm.dz[s] * sm.w3[j] : 0.f;
    }
    __syncthreads();
    if (tid < kMlpHid) {
      float a = 0.f;
      for (int s = 0; s < kMlpTile; s++) a += sm.h2[s * kHs + tid];
      gb2 += a;
    }
    // dW2 += h1^T dh2
#pragma unroll 2
    for (int s = 0; s < kMlpTile; s++) {
      float hv[8], dv[8];
#pragma unroll
      for (int a = 0; a < 8; a++) hv[a] = sm.h1[s * kHs + ty * 8 + a];
#pragma unroll
      for (int b = 0; b < 8; b++) dv[b] = sm.h2[s * kHs + tx + 16 * b];
#pragma unroll
      for (int a = 0; a < 8; a++)
#pragma unroll
        for (int b = 0; b < 8; b++) gw2[a][b] = fmaf(hv[a], dv[b], gw2[a][b]);
    }
    // dh1 = (dh2 W2^T) * relu'(h1): thread owns samples ty*4+q and units i = tx + 16*b
    float dh[4][8];
#pragma unroll
    for (int q = 0; q < 4; q++)
#pragma unroll
      for (int b = 0; b < 8; b++) dh[q][b] = 0.f;
#pragma unroll 2
    for (int j = 0; j < kMlpHid; j++) {
      float dv[4], wv[8];
#pragma unroll
      for (int q = 0; q < 4; q++) dv[q] = sm.h2[(ty * 4 + q) * kHs + j];
#pragma unroll
      for (int b = 0; b < 8; b++) wv[b] = sm.w2[(tx + 16 * b) * kHs + j];
#pragma unroll
      for (int q = 0; q < 4; q++)
#pragma unroll
        for (int b = 0; b < 8; b++) dh[q][b] = fmaf(dv[q], wv[b], dh[q][b]);
    }
    __syncthreads();  // every read of h1 (dW2) and dh2 is done: dh1 replaces h1
#pragma unroll
    for (int q = 0; q < 4; q++)
#pragma unroll
      for (int b = 0; b < 8; b++) {
        const int s = ty * 4 + q, i = tx + 16 * b;
        sm.h1[s * kHs + i] = sm.h1[s * kHs + i] > 0.f ? dh[q][b] : 0.f;
      }
    __syncthreads();
    if (tid < kMlpHid) {
      float a = 0.f;
      for (int s = 0; s < kMlpTile; s++) a += sm.h1[s * kHs + tid];
      gb1 += a;
    }
    // dW1 += x^T dh1
#pragma unroll 2
    for (int s = 0; s < kMlpTile; s++) {
      float xv[4], dv[8];
#pragma unroll
      for (int a = 0; a < 4; a++) xv[a] = sm.x[s * kXs + ty * 4 + a];
#pragma unroll
      for (int b = 0; b < 8; b++) dv[b] = sm.h1[s * kHs + tx + 16 * b];
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 8; b++) gw1[a][b] = fmaf(xv[a], dv[b], gw1[a][b]);
    }
  }
#pragma unroll
  for (int a = 0; a < 8; a++)
#pragma unroll
    for (int b = 0; b < 8; b++) atomicAdd(&grad[kOffW2 + (ty * 8 + a) * kMlpHid + tx + 16 * b], gw2[a][b]);
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 8; b++) atomicAdd(&grad[kOffW1 + (ty * 4 + a) * kMlpHid + tx + 16 * b], gw1[a][b]);
  if (tid < kMlpHid) {
    atomicAdd(&grad[kOffB1 + tid], gb1);
    atomicAdd(&grad[kOffB2 + tid], gb2);
    atomicAdd(&grad[kOffW3 + tid], gw3);
  }
  if (tid == kMlpHid) atomicAdd(&grad[kOffB3], gb3);
  if (tx == 0) atomicAdd(loss, lsum);
}

// Adam on the fp32 master block, then the bf16 weight copies; clears the gradient.
__global__ void mlp_adam_kernel(float* master, float* grad, float* m, float* v, float lr,
                                float b1t, float b2t, __nv_bfloat16* w1, __nv_bfloat16* w2,
                                __nv_bfloat16* w3) {
  const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kMlpParams; i += gridDim.x * blockDim.x) {
    const float g = grad[i];
    const float mi = beta1 * m[i] + (1.f - beta1) * g;
    const float vi = beta2 * v[i] + (1.f - beta2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / (1.f - b1t), vh = vi / (1.f - b2t);
    const float w = master[i] - lr * mh / (sqrtf(vh) + eps);
    master[i] = w;
    grad[i] = 0.f;
    if (i < kOffB1)
      w1[i - kOffW1] = __float2bfloat16_rn(w);
    else if (i >= kOffW2 && i < kOffB2)
      w2[i - kOffW2] = __float2bfloat16_rn(w);
    else if (i >= kOffW3 && i < kOffB3)
      w3[i - kOffW3] = __float2bfloat16_rn(w);
  }
}

__global__ void mlp_round_weights_kernel(const float* master, __nv_bfloat16* w1,
                                         __nv_bfloat16* w2, __nv_bfloat16* w3) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kMlpParams; i += gridDim.x * blockDim.x) {
    const float w = master[i];
    if (i < kOffB1)
      w1[i - kOffW1] = __float2bfloat16_rn(w);
    else if (i >= kOffW2 && i < kOffB2)
      w2[i - kOffW2] = __float2bfloat16_rn(w);
    else if (i >= kOffW3 && i < kOffB3)
      w3[i - kOffW3] = __float2bfloat16_rn(w);
  }
}

}  // namespace csmv
