// bank_engine_r4.cu - the commit kernels specialised for transfers of at most four reads
// (csmv_bank_config.max_reads = 4), in a translation unit of their own so they compile in
// parallel with bank_engine.cu. Four-entry read sets halve the per-lane register arrays and the
// unrolled per-read work of every commit step (the bank workloads read 2 or 4 accounts).
#include "bank_internal.h"

namespace csmv {

KernelFn pick_kernel_r4(uint32_t depth) {
  switch (depth) {
    case 2: return bank_kernel<2, 4, 2>;
    case 4: return bank_kernel<4, 4, 2>;
    case 8: return bank_kernel<8, 4, 2>;
    case 16: return bank_kernel<16, 4, 2>;
    default: return nullptr;
  }
}

KernelFn pick_cluster_r4(uint32_t depth) {
  switch (depth) {
    case 2: return bank_cluster_kernel<2, 4, 2>;
    case 4: return bank_cluster_kernel<4, 4, 2>;
    case 8: return bank_cluster_kernel<8, 4, 2>;
    case 16: return bank_cluster_kernel<16, 4, 2>;
    default: return nullptr;
  }
}

size_t cta_shared_bytes_r4(uint32_t n_mail) { return cta_shared_bytes<4, 2>(n_mail); }

}  // namespace csmv
