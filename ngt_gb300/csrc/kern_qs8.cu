// Instantiations of the search kernels for scalar-quantized (int8) objects.
#include "graph_exact.cuh"
#include "linear_search.cuh"
#include "kernels.h"

namespace ngtg {
#define NGT_OT ObjType::Qsint8
#define NGT_METRICS(X) X(L2) X(InnerProduct) X(NormalizedCosine)
#define NGT_SUFFIX qs8
#include "kern_table.inc"
}  // namespace ngtg
