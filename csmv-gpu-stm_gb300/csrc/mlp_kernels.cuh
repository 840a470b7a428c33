// mlp_kernels.cuh - the conflict predictor's network: 64 -> 128 -> 128 -> 1 (ReLU, ReLU,
// sigmoid), bf16 weights, fp32 accumulation, hand-written forward, backward and Adam kernels.
//
// Layout: features X [n][64] bf16 (0/1 indicators here, exact in bf16); weights W1 [64][128],
// W2 [128][128], w3 [128] in bf16 (rounded from fp32 master copies after every step), biases
// fp32. A CTA of 256 threads works on tiles of 64 samples with every operand in shared memory;
// thread (ty, tx) = (tid / 16, tid % 16) owns samples 4ty..4ty+3 x hidden units tx + 16b
// (b < 8) of an activation tile (interleaved so a warp's weight reads hit 16 distinct banks).
// Inference (every planned transaction) runs on the tensor cores (mlp_forward_tc_kernel, bf16
// warp MMAs with fp32 accumulation); training (the probe slice, a few percent of the chunk)
// runs its fused forward + backward tile GEMMs on the FP32 pipes. Both feed layer 2 with bf16
// activations, so they compute the same network.
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
  float h1[kMlpTile * kHs];      // [s][i] post-ReLU, rounded to bf16
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
    for (int j = 0; j < 8; j++)  // layer-2 operands are bf16, as on the tensor-core path
      sm.h1[(s0 + q) * kHs + tx + 16 * j] = __bfloat162float(__float2bfloat16_rn(fmaxf(acc[q][j], 0.f)));
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

// ---------------------------------------------------------------------------------------------
// Inference on the tensor cores: bf16 x bf16 -> fp32 warp MMAs (m16n8k16). A CTA of 8 warps
// takes 128 samples; warp w owns samples 16w..16w+15 and all 128 hidden units (16 n-tiles), so
// layer 2 reads only the layer-1 rows the same warp wrote. Weights sit in shared memory
// transposed (unit-major, k contiguous) so every B fragment register is one 32-bit load; rows
// are padded by 8 bf16 so a warp's fragment loads hit 32 distinct banks.
// ---------------------------------------------------------------------------------------------
constexpr int kTcTile = 128, kTcX = kMlpIn + 8, kTcH = kMlpHid + 8;

struct MlpTcSmem {
  __nv_bfloat16 w1t[kMlpHid * kTcX];   // [j][k]
  __nv_bfloat16 w2t[kMlpHid * kTcH];   // [j][i]
  __nv_bfloat16 x[kTcTile * kTcX];     // [s][k]
  __nv_bfloat16 h1[kTcTile * kTcH];    // [s][i]
  float b1[kMlpHid], b2[kMlpHid], w3[kMlpHid];
  float b3;
};

__device__ __forceinline__ void mma_bf16_16816(float c[4], const uint32_t a[4], uint32_t b0,
                                               uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t ld_pair(const __nv_bfloat16* p) {
  return *reinterpret_cast<const uint32_t*>(p);
}

__global__ void __launch_bounds__(256) mlp_forward_tc_kernel(
    const __nv_bfloat16* __restrict__ x, uint32_t n, const __nv_bfloat16* w1,
    const __nv_bfloat16* w2, const __nv_bfloat16* w3, const float* master, float* __restrict__ p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  MlpTcSmem& sm = *reinterpret_cast<MlpTcSmem*>(smem_raw);
  for (int i = threadIdx.x; i < kMlpIn * kMlpHid; i += blockDim.x)  // W1 [k][j] -> [j][k]
    sm.w1t[(i % kMlpHid) * kTcX + i / kMlpHid] = w1[i];
  for (int i = threadIdx.x; i < kMlpHid * kMlpHid; i += blockDim.x)  // W2 [i][j] -> [j][i]
    sm.w2t[(i % kMlpHid) * kTcH + i / kMlpHid] = w2[i];
  for (int i = threadIdx.x; i < kMlpHid; i += blockDim.x) {
    sm.b1[i] = master[kOffB1 + i];
    sm.b2[i] = master[kOffB2 + i];
    sm.w3[i] = __bfloat162float(w3[i]);
  }
  if (threadIdx.x == 0) sm.b3 = master[kOffB3];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32, g = lane / 4, tig = lane % 4;
  const int r0 = warp * 16;  // this warp's rows
  for (uint32_t s0 = blockIdx.x * kTcTile; s0 < n; s0 += gridDim.x * kTcTile) {
    __syncthreads();
    // x tile: 128 rows x 128 bytes, 16-byte pieces
    for (int i = threadIdx.x; i < kTcTile * 8; i += blockDim.x) {
      const uint32_t s = i / 8, q = i % 8;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (s0 + s < n) v = reinterpret_cast<const uint4*>(x + (size_t)(s0 + s) * kMlpIn)[q];
      *reinterpret_cast<uint4*>(&sm.x[s * kTcX + q * 8]) = v;
    }
    __syncthreads();
    float acc[16][4];
    // layer 1
#pragma unroll
    for (int nt = 0; nt < 16; nt++) {
      const int c = nt * 8 + tig * 2;
      acc[nt][0] = acc[nt][2] = sm.b1[c];
      acc[nt][1] = acc[nt][3] = sm.b1[c + 1];
    }
#pragma unroll
    for (int ks = 0; ks < kMlpIn / 16; ks++) {
      uint32_t a[4];
      const __nv_bfloat16* xa = &sm.x[(r0 + g) * kTcX + ks * 16 + tig * 2];
      a[0] = ld_pair(xa);
      a[1] = ld_pair(xa + 8 * kTcX);
      a[2] = ld_pair(xa + 8);
      a[3] = ld_pair(xa + 8 * kTcX + 8);
#pragma unroll
      for (int nt = 0; nt < 16; nt++) {
        const __nv_bfloat16* wb = &sm.w1t[(nt * 8 + g) * kTcX + ks * 16 + tig * 2];
        mma_bf16_16816(acc[nt], a, ld_pair(wb), ld_pair(wb + 8));
      }
    }
    // ReLU, bf16, into this warp's rows of h1
#pragma unroll
    for (int nt = 0; nt < 16; nt++) {
      const int c = nt * 8 + tig * 2;
      *reinterpret_cast<__nv_bfloat162*>(&sm.h1[(r0 + g) * kTcH + c]) =
          __floats2bfloat162_rn(fmaxf(acc[nt][0], 0.f), fmaxf(acc[nt][1], 0.f));
      *reinterpret_cast<__nv_bfloat162*>(&sm.h1[(r0 + g + 8) * kTcH + c]) =
          __floats2bfloat162_rn(fmaxf(acc[nt][2], 0.f), fmaxf(acc[nt][3], 0.f));
    }
    __syncwarp();
    // layer 2
#pragma unroll
    for (int nt = 0; nt < 16; nt++) {
      const int c = nt * 8 + tig * 2;
      acc[nt][0] = acc[nt][2] = sm.b2[c];
      acc[nt][1] = acc[nt][3] = sm.b2[c + 1];
    }
#pragma unroll
    for (int ks = 0; ks < kMlpHid / 16; ks++) {
      uint32_t a[4];
      const __nv_bfloat16* ha = &sm.h1[(r0 + g) * kTcH + ks * 16 + tig * 2];
      a[0] = ld_pair(ha);
      a[1] = ld_pair(ha + 8 * kTcH);
      a[2] = ld_pair(ha + 8);
      a[3] = ld_pair(ha + 8 * kTcH + 8);
#pragma unroll
      for (int nt = 0; nt < 16; nt++) {
        const __nv_bfloat16* wb = &sm.w2t[(nt * 8 + g) * kTcH + ks * 16 + tig * 2];
        mma_bf16_16816(acc[nt], a, ld_pair(wb), ld_pair(wb + 8));
      }
    }
    // layer 3: rows g and g+8, reduced over the 4 lanes of the group
    float z0 = 0.f, z1 = 0.f;
#pragma unroll
    for (int nt = 0; nt < 16; nt++) {
      const int c = nt * 8 + tig * 2;
      z0 = fmaf(fmaxf(acc[nt][0], 0.f), sm.w3[c], z0);
      z0 = fmaf(fmaxf(acc[nt][1], 0.f), sm.w3[c + 1], z0);
      z1 = fmaf(fmaxf(acc[nt][2], 0.f), sm.w3[c], z1);
      z1 = fmaf(fmaxf(acc[nt][3], 0.f), sm.w3[c + 1], z1);
    }
#pragma unroll
    for (int o = 1; o <= 2; o <<= 1) {
      z0 += __shfl_xor_sync(0xFFFFFFFFu, z0, o);
      z1 += __shfl_xor_sync(0xFFFFFFFFu, z1, o);
    }
    if (tig == 0) {
      const uint32_t sa = s0 + r0 + g, sb = sa + 8;
      if (sa < n) p[sa] = mlp_sigmoid(z0 + sm.b3);
      if (sb < n) p[sb] = mlp_sigmoid(z1 + sm.b3);
    }
  }
}

}  // namespace csmv
