// uint8-object instantiations of the search kernels.
#include "graph_exact.cuh"
#include "linear_search.cuh"
#include "kernels.h"

namespace ngtg {
#define NGT_OT ObjType::Uint8
#define NGT_METRICS(X) X(L1) X(L2) X(Hamming) X(Jaccard) X(Angle) X(Cosine)
#define NGT_SUFFIX u8
#include "kern_table.inc"
}  // namespace ngtg
