// Instantiations of the CTA-per-query ("wide") batched graph search kernel.
#include "graph_wide.cuh"
#include "kernels.h"

namespace ngtg {

WideKernelFn wide_kernel(ObjType ot, Metric m, bool bf16_rows, uint32_t threads) {
  m = kernel_metric(m);
  if (threads != 128 && threads != 256) return nullptr;
  if (ot == ObjType::Float && bf16_rows && m == Metric::L2)
    return threads == 128 ? &graph_search_wide_kernel<ObjType::Bfloat16, ObjType::Float, Metric::L2, 128>
                          : &graph_search_wide_kernel<ObjType::Bfloat16, ObjType::Float, Metric::L2, 256>;
  if (threads != 256) return nullptr;
  if (ot == ObjType::Float && !bf16_rows && m == Metric::L2)
    return &graph_search_wide_kernel<ObjType::Float, ObjType::Float, Metric::L2, 256>;
  if (ot == ObjType::Uint8 && m == Metric::L2)
    return &graph_search_wide_kernel<ObjType::Uint8, ObjType::Uint8, Metric::L2, 256>;
  return nullptr;
}

size_t wide_kernel_smem_bytes(uint32_t row_chunks, const WideConfig& c) { return wide_smem_bytes(row_chunks, c); }

}  // namespace ngtg
