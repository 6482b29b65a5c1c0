// Relaxed-order quantized-graph search kernel instantiations, one per number of
// subspaces each lane holds (ceil(m / 32) rounded up to a power of two).
#include "kernels.h"
#include "qg_wide.cuh"

namespace ngtg {

QGWideKernelFn qg_wide_kernel_for(uint32_t m, uint32_t blocks) {
  if (blocks == 4) {
    if (m <= 32) return &qg_wide_kernel<1, 4>;
    if (m <= 64) return &qg_wide_kernel<2, 4>;
    if (m <= 128) return &qg_wide_kernel<4, 4>;
    if (m <= 256) return &qg_wide_kernel<8, 4>;
    return nullptr;                                 // 16 subspaces per lane: two blocks at a time only
  }
  if (m <= 32) return &qg_wide_kernel<1, 2>;
  if (m <= 64) return &qg_wide_kernel<2, 2>;
  if (m <= 128) return &qg_wide_kernel<4, 2>;
  if (m <= 256) return &qg_wide_kernel<8, 2>;
  if (m <= 512) return &qg_wide_kernel<16, 2>;
  return nullptr;
}

size_t qg_wide_kernel_smem_bytes(uint32_t row_chunks, uint32_t dim, uint32_t m, const QGWideConfig& c) {
  return qg_wide_smem_bytes(row_chunks, dim, m, c);
}

}  // namespace ngtg
