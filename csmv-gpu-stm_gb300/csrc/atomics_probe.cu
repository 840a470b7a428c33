// atomics_probe.cu - measures the GPU's L2 atomic rates (csmv_measure_atomics).
//
// The commit path is bound by L2 atomics and by chains of dependent L2 round trips, not by HBM
// streaming: a lock is a CAS on an account's commit word, a timestamp an add on one cursor, and a
// contended account's lock passes from warp to warp through a few dependent round trips. Three
// kernels measure the three rates that bound it:
//   same word  every thread of a full grid runs dependent atomicAdds on ONE 4-byte word (the
//              rate at which one L2 line serialises returning atomics: a hot cursor or lock)
//   spread     every thread runs dependent atomicAdds on pseudo-random words of a 64 MB buffer
//              (L2-resident: the aggregate returning-atomic rate of all L2 slices)
//   CAS chain  one thread runs dependent 64-bit CASes on one word: the latency of one L2 round
//              trip of an atomic, the unit of a contended lock hand-off
// Device time is taken with CUDA events on the probe's own stream.
#include <cstring>

#include "common.h"

namespace {

constexpr uint32_t kSpreadWords = 1u << 24;  // 64 MB
constexpr int kIters = 256;

__global__ void same_word_kernel(uint32_t* word, uint32_t* sink) {
  uint32_t acc = 0;
  for (int i = 0; i < kIters; i++) acc += atomicAdd(word, 1u);
  if (acc == 0xFFFFFFFFu) sink[0] = acc;  // keeps the returned values live
}

__global__ void spread_kernel(uint32_t* words, uint32_t* sink) {
  uint32_t x = (blockIdx.x * blockDim.x + threadIdx.x) * 0x9E3779B1u + 1u, acc = 0;
  for (int i = 0; i < kIters; i++) {
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    acc += atomicAdd(&words[(x + acc) & (kSpreadWords - 1u)], 1u);
  }
  if (acc == 0xFFFFFFFFu) sink[0] = acc;
}

__global__ void cas_chain_kernel(unsigned long long* word, uint32_t n, uint32_t* sink) {
  unsigned long long v = 0;
  for (uint32_t i = 0; i < n; i++) v = atomicCAS(word, v, v + 1ull);  // each CAS needs the last
  sink[1] = (uint32_t)v;
}

}  // namespace

extern "C" csmv_status csmv_measure_atomics(int32_t device, csmv_atomic_rates* out) {
  if (!out) return CSMV_ERR_INVALID_ARG;
  std::memset(out, 0, sizeof(*out));
  int n_sms = 0;
  csmv_status st = csmv::check_device(device, &n_sms);
  if (st != CSMV_OK) return st;
  CSMV_CUDA(cudaSetDevice(device));
  uint32_t* words = nullptr;
  uint32_t* sink = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  auto cleanup = [&]() {
    cudaFree(words);
    cudaFree(sink);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
  };
  auto fail = [&](cudaError_t e, const char* what) {
    csmv_status r = csmv::cuda_status(e, what);
    cleanup();
    return r;
  };
  cudaError_t e;
  if ((e = cudaMalloc(&words, (size_t)kSpreadWords * 4)) != cudaSuccess) return fail(e, "cudaMalloc");
  if ((e = cudaMalloc(&sink, 64)) != cudaSuccess) return fail(e, "cudaMalloc");
  if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess) return fail(e, "stream");
  if ((e = cudaEventCreate(&e0)) != cudaSuccess || (e = cudaEventCreate(&e1)) != cudaSuccess)
    return fail(e, "event");
  if ((e = cudaMemsetAsync(words, 0, (size_t)kSpreadWords * 4, s)) != cudaSuccess) return fail(e, "memset");
  const uint32_t grid = (uint32_t)n_sms * 4u, block = 256u;
  const double ops = (double)grid * block * kIters;
  float ms = 0.f;
  auto timed = [&](auto launch, double* rate_out, double count) -> cudaError_t {
    launch();  // warm-up
    cudaEventRecord(e0, s);
    launch();
    cudaEventRecord(e1, s);
    cudaError_t r = cudaEventSynchronize(e1);
    if (r != cudaSuccess) return r;
    if ((r = cudaGetLastError()) != cudaSuccess) return r;
    cudaEventElapsedTime(&ms, e0, e1);
    out->kernel_ms += ms;
    *rate_out = count / (ms * 1e-3);
    return cudaSuccess;
  };
  if ((e = timed([&] { same_word_kernel<<<grid, block, 0, s>>>(words, sink); },
                 &out->same_word_per_s, ops)) != cudaSuccess)
    return fail(e, "same-word atomics");
  if ((e = timed([&] { spread_kernel<<<grid, block, 0, s>>>(words, sink); }, &out->spread_per_s,
                 ops)) != cudaSuccess)
    return fail(e, "spread atomics");
  const uint32_t chain = 4096;
  double chain_rate = 0;
  if ((e = timed([&] {
         cas_chain_kernel<<<1, 1, 0, s>>>(reinterpret_cast<unsigned long long*>(words + 64), chain,
                                          sink);
       },
                 &chain_rate, chain)) != cudaSuccess)
    return fail(e, "CAS chain");
  out->cas_chain_ns = 1e9 / chain_rate;
  cleanup();
  return CSMV_OK;
}
