// FP32-object instantiations of the search kernels.
#include "graph_exact.cuh"
#include "linear_search.cuh"
#include "kernels.h"

namespace ngtg {
#define NGT_OT ObjType::Float
#define NGT_METRICS(X) X(L1) X(L2) X(Angle) X(Cosine) X(NormalizedAngle) X(NormalizedCosine) X(NormalizedL2) X(Poincare) X(Lorentz)
#define NGT_SUFFIX float
#include "kern_table.inc"
}  // namespace ngtg
