// Quantized-blob-graph search kernel instantiations, one per number of
// subspaces each lane holds (ceil(m / 32) rounded up to a power of two).
#include "kernels.h"
#include "qbg_search.cuh"

namespace ngtg {

QBGKernelFn qbg_kernel(uint32_t m) {
  if (m <= 32) return &qbg_search_kernel<1>;
  if (m <= 64) return &qbg_search_kernel<2>;
  if (m <= 128) return &qbg_search_kernel<4>;
  if (m <= 256) return &qbg_search_kernel<8>;
  if (m <= 512) return &qbg_search_kernel<16>;
  return nullptr;
}

size_t qbg_kernel_smem_bytes(uint32_t row_chunks, uint32_t dim, uint32_t m, const QBGConfig& c) {
  return qbg_smem_bytes(row_chunks, dim, m, c);
}

QBGScanKernelFn qbg_scan_kernel_for(uint32_t m) {
  if (m <= 32) return &qbg_scan_kernel<1>;
  if (m <= 64) return &qbg_scan_kernel<2>;
  if (m <= 128) return &qbg_scan_kernel<4>;
  if (m <= 256) return &qbg_scan_kernel<8>;
  if (m <= 512) return &qbg_scan_kernel<16>;
  return nullptr;
}

size_t qbg_scan_kernel_smem_bytes(uint32_t row_chunks, uint32_t dim, uint32_t m, uint32_t rcap) {
  return qbg_scan_smem_bytes(row_chunks, dim, m, rcap);
}

QBGRefineKernelFn qbg_refine_kernel_for(bool uint8_rows) {
  return uint8_rows ? &qbg_refine_kernel<ObjType::Uint8> : &qbg_refine_kernel<ObjType::Float>;
}

QBGRefineKernelFn graph_refine_kernel_for(Metric m) {
  switch (m) {
    case Metric::L1: return &qbg_refine_kernel<ObjType::Float, Metric::L1>;
    case Metric::L2: return &qbg_refine_kernel<ObjType::Float, Metric::L2>;
    case Metric::Angle: return &qbg_refine_kernel<ObjType::Float, Metric::Angle>;
    case Metric::Cosine: return &qbg_refine_kernel<ObjType::Float, Metric::Cosine>;
    default: return nullptr;
  }
}

}  // namespace ngtg
