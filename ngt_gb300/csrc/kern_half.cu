// FP16-object instantiations of the search kernels.
#include "graph_exact.cuh"
#include "linear_search.cuh"
#include "kernels.h"

namespace ngtg {
#define NGT_OT ObjType::Float16
#define NGT_METRICS(X) X(L1) X(L2) X(Angle) X(Cosine) X(NormalizedAngle) X(NormalizedCosine) X(NormalizedL2) X(Poincare) X(Lorentz)
#define NGT_SUFFIX half
#include "kern_table.inc"
}  // namespace ngtg
