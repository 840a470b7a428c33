// mlp_engine.cu - C-ABI of the conflict predictor's network (include/csmv.h, csmv_mlp_*).
//
// Device state per handle: fp32 master parameters, Adam moments and the gradient accumulator
// (kMlpParams floats each), bf16 copies of W1/W2/w3 for the kernels, one loss word. Every call
// runs on the handle's stream and returns once that stream is idle.
#include <cmath>
#include <cstring>
#include <vector>

#include "common.h"
#include "mlp_kernels.cuh"

using namespace csmv;

static_assert(kMlpParams == CSMV_MLP_PARAMS, "parameter block size");
static_assert(kMlpIn == CSMV_MLP_IN && kMlpHid == CSMV_MLP_HIDDEN, "network shape");

struct csmv_mlp_t {
  int device = 0, n_sms = 0;
  cudaStream_t stream = nullptr;
  float *master = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr, *loss = nullptr;
  __nv_bfloat16 *w1 = nullptr, *w2 = nullptr, *w3 = nullptr;
  uint32_t steps = 0;
};

namespace {
void free_all(csmv_mlp_t* h) {
  cudaFree(h->master);
  cudaFree(h->grad);
  cudaFree(h->m);
  cudaFree(h->v);
  cudaFree(h->loss);
  cudaFree(h->w1);
  cudaFree(h->w2);
  cudaFree(h->w3);
  if (h->stream) cudaStreamDestroy(h->stream);
}

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
}  // namespace

extern "C" csmv_status csmv_mlp_create(int32_t device, uint64_t seed, csmv_mlp_t** out) {
  if (!out) return CSMV_ERR_INVALID_ARG;
  *out = nullptr;
  int n_sms = 0;
  csmv_status st = check_device(device, &n_sms);
  if (st != CSMV_OK) return st;
  CSMV_CUDA(cudaSetDevice(device));
  csmv_mlp_t* h = new csmv_mlp_t;
  h->device = device;
  h->n_sms = n_sms;
  auto fail = [&](csmv_status s) {
    free_all(h);
    delete h;
    return s;
  };
  const size_t pb = kMlpParams * sizeof(float);
  struct {
    void** p;
    size_t bytes;
  } allocs[] = {{(void**)&h->master, pb}, {(void**)&h->grad, pb}, {(void**)&h->m, pb},
                {(void**)&h->v, pb}, {(void**)&h->loss, 16},
                {(void**)&h->w1, kMlpIn * kMlpHid * 2}, {(void**)&h->w2, kMlpHid * kMlpHid * 2},
                {(void**)&h->w3, kMlpHid * 2}};
  for (auto& a : allocs)
    if ((st = cuda_status(cudaMalloc(a.p, a.bytes), "cudaMalloc")) != CSMV_OK) return fail(st);
  if ((st = cuda_status(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "stream")) != CSMV_OK)
    return fail(st);
  if ((st = cuda_status(cudaFuncSetAttribute((const void*)mlp_grad_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)sizeof(MlpSmem)),
                        "cudaFuncSetAttribute")) != CSMV_OK ||
      (st = cuda_status(cudaFuncSetAttribute((const void*)mlp_forward_tc_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)sizeof(MlpTcSmem)),
                        "cudaFuncSetAttribute")) != CSMV_OK)
    return fail(st);
  // uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases
  std::vector<float> p(kMlpParams, 0.f);
  uint64_t s = seed;
  auto uni = [&](float bound) {
    return (float)((double)(splitmix(s) >> 11) * 0x1p-53 * 2.0 - 1.0) * bound;
  };
  for (int i = 0; i < kMlpIn * kMlpHid; i++) p[kOffW1 + i] = uni(1.f / std::sqrt((float)kMlpIn));
  for (int i = 0; i < kMlpHid * kMlpHid; i++) p[kOffW2 + i] = uni(1.f / std::sqrt((float)kMlpHid));
  for (int i = 0; i < kMlpHid; i++) p[kOffW3 + i] = uni(1.f / std::sqrt((float)kMlpHid));
  *out = h;
  if ((st = csmv_mlp_set_params(h, p.data())) != CSMV_OK) {
    *out = nullptr;
    return fail(st);
  }
  return CSMV_OK;
}

extern "C" csmv_status csmv_mlp_set_params(csmv_mlp_t* h, const float* host_params) {
  if (!h || !host_params) return CSMV_ERR_INVALID_ARG;
  CSMV_CUDA(cudaSetDevice(h->device));
  const size_t pb = kMlpParams * sizeof(float);
  CSMV_CUDA(cudaMemcpyAsync(h->master, host_params, pb, cudaMemcpyHostToDevice, h->stream));
  CSMV_CUDA(cudaMemsetAsync(h->grad, 0, pb, h->stream));
  CSMV_CUDA(cudaMemsetAsync(h->m, 0, pb, h->stream));
  CSMV_CUDA(cudaMemsetAsync(h->v, 0, pb, h->stream));
  mlp_round_weights_kernel<<<32, 256, 0, h->stream>>>(h->master, h->w1, h->w2, h->w3);
  CSMV_CUDA(cudaGetLastError());
  CSMV_CUDA(cudaStreamSynchronize(h->stream));
  h->steps = 0;
  return CSMV_OK;
}

extern "C" csmv_status csmv_mlp_get_params(csmv_mlp_t* h, float* host_params) {
  if (!h || !host_params) return CSMV_ERR_INVALID_ARG;
  CSMV_CUDA(cudaSetDevice(h->device));
  CSMV_CUDA(cudaMemcpy(host_params, h->master, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost));
  return CSMV_OK;
}

extern "C" csmv_status csmv_mlp_get_grads(csmv_mlp_t* h, float* host_grads) {
  if (!h || !host_grads) return CSMV_ERR_INVALID_ARG;
  CSMV_CUDA(cudaSetDevice(h->device));
  CSMV_CUDA(cudaMemcpy(host_grads, h->grad, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost));
  return CSMV_OK;
}

// Internal launchers, shared with the scheduler (same stream discipline as the C-ABI calls).
csmv_status csmv_mlp_launch_forward(csmv_mlp_t* h, uint32_t n, const void* dev_x, float* dev_p,
                                    cudaStream_t stream) {
  if (n == 0) return CSMV_OK;
  // two 104 KB CTAs per SM
  const uint32_t tiles = (n + kTcTile - 1) / kTcTile, cap = 2u * (uint32_t)h->n_sms;
  const uint32_t grid = tiles < cap ? tiles : cap;
  mlp_forward_tc_kernel<<<grid, 256, sizeof(MlpTcSmem), stream>>>(
      static_cast<const __nv_bfloat16*>(dev_x), n, h->w1, h->w2, h->w3, h->master, dev_p);
  return cuda_status(cudaGetLastError(), "mlp_forward_tc_kernel");
}

csmv_status csmv_mlp_launch_grad(csmv_mlp_t* h, uint32_t n, const void* dev_x, const float* dev_y,
                                 cudaStream_t stream) {
  if (n == 0) return CSMV_OK;
  const uint32_t tiles = (n + kMlpTile - 1) / kMlpTile;
  const uint32_t grid = tiles < (uint32_t)h->n_sms ? tiles : (uint32_t)h->n_sms;
  CSMV_CUDA(cudaMemsetAsync(h->loss, 0, 4, stream));
  mlp_grad_kernel<<<grid, kMlpThreads, sizeof(MlpSmem), stream>>>(
      static_cast<const __nv_bfloat16*>(dev_x), dev_y, n, h->w1, h->w2, h->w3, h->master, h->grad,
      h->loss);
  return cuda_status(cudaGetLastError(), "mlp_grad_kernel");
}

csmv_status csmv_mlp_launch_adam(csmv_mlp_t* h, float lr, cudaStream_t stream) {
  h->steps++;
  const float b1t = (float)std::pow(0.9, (double)h->steps), b2t = (float)std::pow(0.999, (double)h->steps);
  mlp_adam_kernel<<<32, 256, 0, stream>>>(h->master, h->grad, h->m, h->v, lr, b1t, b2t, h->w1,
                                          h->w2, h->w3);
  return cuda_status(cudaGetLastError(), "mlp_adam_kernel");
}

float* csmv_mlp_loss_ptr(csmv_mlp_t* h) { return h->loss; }

extern "C" csmv_status csmv_mlp_forward(csmv_mlp_t* h, uint32_t n, const uint16_t* dev_x,
                                        float* dev_p) {
  if (!h || (n && (!dev_x || !dev_p))) return CSMV_ERR_INVALID_ARG;
  CSMV_CUDA(cudaSetDevice(h->device));
  csmv_status st = csmv_mlp_launch_forward(h, n, dev_x, dev_p, h->stream);
  if (st != CSMV_OK) return st;
  CSMV_CUDA(cudaStreamSynchronize(h->stream));
  return CSMV_OK;
}

extern "C" csmv_status csmv_mlp_grad(csmv_mlp_t* h, uint32_t n, const uint16_t* dev_x,
                                     const float* dev_y, float* host_loss) {
  if (!h || n == 0 || !dev_x || !dev_y) return CSMV_ERR_INVALID_ARG;
  CSMV_CUDA(cudaSetDevice(h->device));
  csmv_status st = csmv_mlp_launch_grad(h, n, dev_x, dev_y, h->stream);
  if (st != CSMV_OK) return st;
  float l = 0.f;
  CSMV_CUDA(cudaMemcpyAsync(&l, h->loss, 4, cudaMemcpyDeviceToHost, h->stream));
  CSMV_CUDA(cudaStreamSynchronize(h->stream));
  if (host_loss) *host_loss = l / (float)n;
  return CSMV_OK;
}

extern "C" csmv_status csmv_mlp_adam_step(csmv_mlp_t* h, float lr) {
  if (!h || !(lr > 0.f)) return CSMV_ERR_INVALID_ARG;
  CSMV_CUDA(cudaSetDevice(h->device));
  csmv_status st = csmv_mlp_launch_adam(h, lr, h->stream);
  if (st != CSMV_OK) return st;
  CSMV_CUDA(cudaStreamSynchronize(h->stream));
  return CSMV_OK;
}

extern "C" void csmv_mlp_destroy(csmv_mlp_t* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  free_all(h);
  delete h;
}
