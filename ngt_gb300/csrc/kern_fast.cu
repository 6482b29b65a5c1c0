// Instantiations of the batched (warp-per-query) graph search kernel, and the
// conversion of float object rows to the bf16 search rows it reads.
#include <cuda_bf16.h>
#include <algorithm>
#include "graph_fast.cuh"
#include "kernels.h"

namespace ngtg {

#define NGT_FAST_CASE(ST, OT, M) \
  case Metric::M: return &graph_search_fast_kernel<ObjType::ST, ObjType::OT, Metric::M>;

FastKernelFn fast_kernel(ObjType ot, Metric m, bool bf16_rows, uint32_t rows_in_flight, uint32_t ctas_per_sm) {
  if (ot != ObjType::Qsint8) m = kernel_metric(m);   // qsint8 inner product: its own comparator
  if (rows_in_flight == 0) rows_in_flight = 4;
  if (ctas_per_sm == 0) ctas_per_sm = rows_in_flight > 4 ? 4 : 5;
  if (ot == ObjType::Float && bf16_rows && m == Metric::L2 && !(rows_in_flight == 4 && ctas_per_sm == 5)) {
    // other row pipelines / register budgets for the L2 bf16 search
#define NGT_FAST_L2(U, B) \
  if (rows_in_flight == U && ctas_per_sm == B) \
    return &graph_search_fast_kernel<ObjType::Bfloat16, ObjType::Float, Metric::L2, U, B>;
    NGT_FAST_L2(6, 4) NGT_FAST_L2(8, 4) NGT_FAST_L2(6, 5) NGT_FAST_L2(4, 6) NGT_FAST_L2(2, 8)
#undef NGT_FAST_L2
    return nullptr;
  }
  if (!(rows_in_flight == 4 && ctas_per_sm == 5)) return nullptr;
  if (ot == ObjType::Float && bf16_rows) {
    switch (m) {
      NGT_FAST_CASE(Bfloat16, Float, L2) NGT_FAST_CASE(Bfloat16, Float, L1) NGT_FAST_CASE(Bfloat16, Float, Cosine)
      NGT_FAST_CASE(Bfloat16, Float, Angle) NGT_FAST_CASE(Bfloat16, Float, NormalizedCosine)
      NGT_FAST_CASE(Bfloat16, Float, NormalizedAngle) NGT_FAST_CASE(Bfloat16, Float, NormalizedL2)
      default: return nullptr;
    }
  }
  if (ot == ObjType::Float) {
    switch (m) {
      NGT_FAST_CASE(Float, Float, L2) NGT_FAST_CASE(Float, Float, NormalizedCosine)
      NGT_FAST_CASE(Float, Float, Poincare) NGT_FAST_CASE(Float, Float, Lorentz)   // searched on the fp32 rows
      default: return nullptr;
    }
  }
  if (ot == ObjType::Uint8) {
    switch (m) {
      NGT_FAST_CASE(Uint8, Uint8, L2) NGT_FAST_CASE(Uint8, Uint8, L1) NGT_FAST_CASE(Uint8, Uint8, Hamming)
      NGT_FAST_CASE(Uint8, Uint8, Jaccard)
      default: return nullptr;
    }
  }
  if (ot == ObjType::Float16) {
    switch (m) { NGT_FAST_CASE(Float16, Float16, L2) NGT_FAST_CASE(Float16, Float16, L1) default: return nullptr; }
  }
  if (ot == ObjType::Qsint8) {
    switch (m) { NGT_FAST_CASE(Qsint8, Qsint8, L2) default: return nullptr; }
  }
  return nullptr;
}

// rows x dpad floats -> rows x dpad bf16 (round to nearest even), 16-byte chunks.
__global__ void float_rows_to_bf16_kernel(const float4* __restrict__ in, uint2* __restrict__ out, size_t n4) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
    float4 v = in[i];
    uint32_t a = __bfloat16_as_ushort(__float2bfloat16_rn(v.x)) | ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v.y)) << 16);
    uint32_t b = __bfloat16_as_ushort(__float2bfloat16_rn(v.z)) | ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v.w)) << 16);
    out[i] = make_uint2(a, b);
  }
}

void launch_float_rows_to_bf16(const void* in, void* out, size_t nfloats, cudaStream_t s) {
  size_t n4 = nfloats / 4;
  unsigned grid = (unsigned)std::min<size_t>((n4 + 255) / 256, 152 * 32);
  float_rows_to_bf16_kernel<<<grid, 256, 0, s>>>(static_cast<const float4*>(in), static_cast<uint2*>(out), n4);
}

}  // namespace ngtg
