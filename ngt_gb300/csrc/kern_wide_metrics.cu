// Instantiations of the CTA-per-query ("wide") batched graph search for the
// distances other than L2: the objects themselves are the search rows, 256
// threads per query.  A translation unit of its own so that they compile in
// parallel with the L2 instantiations.
#include "graph_wide.cuh"
#include "kernels.h"

namespace ngtg {

WideKernelFn wide_kernel_native(ObjType ot, Metric m) {
#define NGT_WIDE(OT, M) \
  case Metric::M: return &graph_search_wide_kernel<ObjType::OT, ObjType::OT, Metric::M, 256>;
  switch (ot) {
    case ObjType::Float:
      switch (m) {
        NGT_WIDE(Float, L1) NGT_WIDE(Float, Cosine) NGT_WIDE(Float, Angle) NGT_WIDE(Float, NormalizedCosine)
        NGT_WIDE(Float, NormalizedAngle) NGT_WIDE(Float, NormalizedL2) NGT_WIDE(Float, Poincare)
        NGT_WIDE(Float, Lorentz)
        default: return nullptr;
      }
    case ObjType::Uint8:
      switch (m) {
        NGT_WIDE(Uint8, L1) NGT_WIDE(Uint8, Hamming) NGT_WIDE(Uint8, Jaccard)
        default: return nullptr;
      }
    case ObjType::Float16:
      switch (m) {
        NGT_WIDE(Float16, L2) NGT_WIDE(Float16, L1)
        default: return nullptr;
      }
    default: return nullptr;
  }
#undef NGT_WIDE
}

}  // namespace ngtg
