// devtest.cu - C-ABI harness around the public device functions of include/csmv_tx.cuh, built as
// lib/libcsmv_devtest.so so the GPU tests can pin each function against the CPU oracle on
// arbitrary inputs: the version read rule, TXPreValidation, TXWriteBack's slot choice, and the
// bounded wait that turns a wait nobody satisfies into an error status instead of a hang.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../../include/csmv_tx.cuh"

using namespace csmv;

namespace {

template <int DEPTH>
__global__ void read_kernel(const unsigned long long* slots, uint32_t n, const uint32_t* snaps,
                            int32_t* out, uint8_t* aborted) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  VersionStore vs{const_cast<unsigned long long*>(slots), n};
  bool ab = false;
  out[i] = TXReadOnly<DEPTH>(vs, i, snaps[i], &ab);
  aborted[i] = ab ? 1 : 0;
}

// one warp per test warp: lanes load their sets and run the warp-collective pre-validation
__global__ void prevalidate_kernel(const uint32_t* rs, const uint32_t* nrs, const uint32_t* ws,
                                   const uint32_t* nws, const uint32_t* active, uint32_t n_warps,
                                   uint32_t* out) {
  const uint32_t w = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  if (w >= n_warps) return;  // warp-uniform
  const uint32_t lane = threadIdx.x & 31u;
  ReadSet<8> r;
  WriteSet<2> x;
  r.n = nrs[w * 32 + lane];
  x.n = nws[w * 32 + lane];
#pragma unroll
  for (int k = 0; k < 8; k++) r.addr[k] = rs[(w * 32 + lane) * 8 + k];
#pragma unroll
  for (int k = 0; k < 2; k++) {
    x.addr[k] = ws[(w * 32 + lane) * 2 + k];
    x.val[k] = 0;
  }
  const uint32_t m = TXPreValidation(r, x, (active[w] >> lane) & 1u);
  if (lane == 0) out[w] = m;
}

// thread i installs item i's writes in order (ts increasing), as the engine's exclusive writer
template <int DEPTH>
__global__ void writeback_kernel(unsigned long long* slots, uint32_t n_items, const uint32_t* start,
                                 const uint32_t* ts, const int32_t* val) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_items) return;
  VersionStore vs{slots, n_items};
  for (uint32_t k = start[i]; k < start[i + 1]; k++) {
    WriteSet<2> x;
    x.n = 1;
    x.addr[0] = i;
    x.val[0] = val[k];
    x.addr[1] = 0;
    x.val[1] = 0;
    TXWriteBack<DEPTH>(ts[k], vs, x);
  }
}

__global__ void bounded_wait_kernel(uint32_t* flag, uint32_t* err, uint32_t limit_log2,
                                    uint32_t* done) {
  const bool ok = bounded_wait([&] { return ld_acquire_gpu(flag) != 0; }, err, ERR_WAIT_TURN,
                               limit_log2);
  if (threadIdx.x == 0) *done = ok ? 1u : 2u;
}

template <class T>
int to_dev(T** d, const T* h, size_t n) {
  if (cudaMalloc(d, n * sizeof(T) + 16) != cudaSuccess) return 3;
  if (h && cudaMemcpy(*d, h, n * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) return 2;
  return 0;
}

}  // namespace

extern "C" {

int csmv_devtest_read(const uint64_t* slots, int depth, uint32_t n, const uint32_t* snaps,
                      int32_t* out, uint8_t* aborted) {
  unsigned long long* ds;
  uint32_t* dn;
  int32_t* dout;
  uint8_t* dab;
  int rc = to_dev(&ds, (const unsigned long long*)slots, (size_t)n * depth) | to_dev(&dn, snaps, n) |
           to_dev(&dout, (const int32_t*)nullptr, n) | to_dev(&dab, (const uint8_t*)nullptr, n);
  if (rc) return rc;
  const uint32_t blocks = (n + 127) / 128;
  switch (depth) {
    case 2: read_kernel<2><<<blocks, 128>>>(ds, n, dn, dout, dab); break;
    case 4: read_kernel<4><<<blocks, 128>>>(ds, n, dn, dout, dab); break;
    case 8: read_kernel<8><<<blocks, 128>>>(ds, n, dn, dout, dab); break;
    case 16: read_kernel<16><<<blocks, 128>>>(ds, n, dn, dout, dab); break;
    default: return 1;
  }
  if (cudaMemcpy(out, dout, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(aborted, dab, n, cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = 2;
  cudaFree(ds);
  cudaFree(dn);
  cudaFree(dout);
  cudaFree(dab);
  return rc;
}

int csmv_devtest_prevalidate(const uint32_t* rs, const uint32_t* nrs, const uint32_t* ws,
                             const uint32_t* nws, const uint32_t* active, uint32_t n_warps,
                             uint32_t* out) {
  uint32_t *drs, *dnrs, *dws, *dnws, *dact, *dout;
  int rc = to_dev(&drs, rs, (size_t)n_warps * 32 * 8) | to_dev(&dnrs, nrs, (size_t)n_warps * 32) |
           to_dev(&dws, ws, (size_t)n_warps * 32 * 2) | to_dev(&dnws, nws, (size_t)n_warps * 32) |
           to_dev(&dact, active, n_warps) | to_dev(&dout, (const uint32_t*)nullptr, n_warps);
  if (rc) return rc;
  prevalidate_kernel<<<(n_warps + 3) / 4, 128>>>(drs, dnrs, dws, dnws, dact, n_warps, dout);
  if (cudaMemcpy(out, dout, n_warps * 4, cudaMemcpyDeviceToHost) != cudaSuccess) rc = 2;
  cudaFree(drs);
  cudaFree(dnrs);
  cudaFree(dws);
  cudaFree(dnws);
  cudaFree(dact);
  cudaFree(dout);
  return rc;
}

int csmv_devtest_writeback(uint64_t* slots, int depth, uint32_t n_items, const uint32_t* start,
                           const uint32_t* ts, const int32_t* val) {
  const uint32_t n_w = start[n_items];
  unsigned long long* ds;
  uint32_t *dst, *dts;
  int32_t* dv;
  int rc = to_dev(&ds, (const unsigned long long*)slots, (size_t)n_items * depth) |
           to_dev(&dst, start, n_items + 1) | to_dev(&dts, ts, n_w + 1) | to_dev(&dv, val, n_w + 1);
  if (rc) return rc;
  const uint32_t blocks = (n_items + 127) / 128;
  switch (depth) {
    case 2: writeback_kernel<2><<<blocks, 128>>>(ds, n_items, dst, dts, dv); break;
    case 4: writeback_kernel<4><<<blocks, 128>>>(ds, n_items, dst, dts, dv); break;
    case 8: writeback_kernel<8><<<blocks, 128>>>(ds, n_items, dst, dts, dv); break;
    case 16: writeback_kernel<16><<<blocks, 128>>>(ds, n_items, dst, dts, dv); break;
    default: return 1;
  }
  if (cudaMemcpy(slots, ds, (size_t)n_items * depth * 8, cudaMemcpyDeviceToHost) != cudaSuccess) rc = 2;
  cudaFree(ds);
  cudaFree(dst);
  cudaFree(dts);
  cudaFree(dv);
  return rc;
}

// A wait whose flag nobody sets must come back with an error word, not hang.
int csmv_devtest_bounded_wait(uint32_t limit_log2, uint32_t* err_out, uint32_t* done_out) {
  uint32_t* d;
  if (cudaMalloc(&d, 12) != cudaSuccess) return 3;
  cudaMemset(d, 0, 12);
  bounded_wait_kernel<<<1, 32>>>(d, d + 1, limit_log2, d + 2);
  uint32_t h[3];
  int rc = cudaMemcpy(h, d, 12, cudaMemcpyDeviceToHost) == cudaSuccess ? 0 : 2;
  *err_out = h[1];
  *done_out = h[2];
  cudaFree(d);
  return rc;
}

}  // extern "C"
