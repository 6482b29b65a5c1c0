// Instantiations of the CTA-per-query ("wide") batched graph search kernel.
#include <algorithm>
#include "graph_wide.cuh"
#include "kernels.h"

namespace ngtg {

WideKernelFn wide_kernel(ObjType ot, Metric m, SearchRows rows, uint32_t threads) {
  if (ot != ObjType::Qsint8) m = kernel_metric(m);   // qsint8 inner product: its own comparator
  if (threads != 64 && threads != 128 && threads != 256) return nullptr;
  // 64 threads (more queries in flight per SM): the float L2 search rows only
  if (ot == ObjType::Float && rows == SearchRows::Bf16 && m == Metric::L2)
    return threads == 64    ? &graph_search_wide_kernel<ObjType::Bfloat16, ObjType::Float, Metric::L2, 64>
           : threads == 128 ? &graph_search_wide_kernel<ObjType::Bfloat16, ObjType::Float, Metric::L2, 128>
                            : &graph_search_wide_kernel<ObjType::Bfloat16, ObjType::Float, Metric::L2, 256>;
  if (ot == ObjType::Float && rows == SearchRows::Sq8 && m == Metric::L2)
    return threads == 64    ? &graph_search_wide_kernel<ObjType::Uint8, ObjType::Float, Metric::L2, 64>
           : threads == 128 ? &graph_search_wide_kernel<ObjType::Uint8, ObjType::Float, Metric::L2, 128>
                            : &graph_search_wide_kernel<ObjType::Uint8, ObjType::Float, Metric::L2, 256>;
  if (threads == 64) return nullptr;
  if (ot == ObjType::Qsint8 && rows == SearchRows::Native && m == Metric::L2)
    return threads == 128 ? &graph_search_wide_kernel<ObjType::Qsint8, ObjType::Qsint8, Metric::L2, 128>
                          : &graph_search_wide_kernel<ObjType::Qsint8, ObjType::Qsint8, Metric::L2, 256>;
  if (threads != 256 || rows != SearchRows::Native) return nullptr;
  if (ot == ObjType::Float && m == Metric::L2)
    return &graph_search_wide_kernel<ObjType::Float, ObjType::Float, Metric::L2, 256>;
  if (ot == ObjType::Uint8 && m == Metric::L2)
    return &graph_search_wide_kernel<ObjType::Uint8, ObjType::Uint8, Metric::L2, 256>;
  return wide_kernel_native(ot, m);           // the other distances (kern_wide_metrics.cu)
}

size_t wide_kernel_smem_bytes(uint32_t row_chunks, const WideConfig& c) { return wide_smem_bytes(row_chunks, c); }

__global__ void float_rows_to_sq8_kernel(const float* __restrict__ in, uint8_t* __restrict__ out, size_t n,
                                         uint32_t dpad, uint32_t dim, float offset, float scale) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t d = (uint32_t)(i % dpad);
    float c = 0.f;
    if (d < dim) c = fminf(fmaxf(rintf((in[i] - offset) / scale), 0.f), 255.f);
    out[i] = (uint8_t)c;
  }
}

void launch_float_rows_to_sq8(const float* in, uint8_t* out, size_t nrows, uint32_t dpad, uint32_t dim, float offset,
                              float scale, cudaStream_t s) {
  const size_t n = nrows * dpad;
  unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 32);
  float_rows_to_sq8_kernel<<<grid, 256, 0, s>>>(in, out, n, dpad, dim, offset, scale);
}

}  // namespace ngtg
