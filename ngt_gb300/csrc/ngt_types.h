// Shared enums and small POD types of the GB300 NGT search library.
//
// Enum values follow NGT's ObjectSpace::DistanceType / ObjectType
// (lib/NGT/ObjectSpace.h:223-259) so an index's property file maps 1:1.
#pragma once
#include <cstdint>
#include <cstddef>

namespace ngtg {

enum class Metric : int32_t {
  L1 = 0,
  L2 = 1,
  Hamming = 2,
  Angle = 3,
  Cosine = 4,
  NormalizedAngle = 5,
  NormalizedCosine = 6,
  Jaccard = 7,
  SparseJaccard = 8,
  NormalizedL2 = 9,
  InnerProduct = 10,  // stored as L2 over the (D+1) augmented space
  Poincare = 100,
  Lorentz = 101,
  // internal only: the squared L2 over unsigned bytes, the tree comparator of
  // scalar-quantized inner-product and normalized-cosine indexes
  // (ComparatorL2Quint8Quint8, lib/NGT/ObjectSpaceRepository.h:514-533)
  Quint8L2 = 200,
};

// Qsint8: NGT's scalar-quantized objects (ObjectType "QSUInteger-8B",
// lib/NGT/ObjectSpace.h:250): int8 codes rint(x / QuantizationScale x 127.5).
enum class ObjType : int32_t { Float = 0, Uint8 = 1, Float16 = 2, Bfloat16 = 3, Qsint8 = 4 };

inline size_t objtype_size(ObjType t) {
  switch (t) {
    case ObjType::Float: return 4;
    case ObjType::Uint8:
    case ObjType::Qsint8: return 1;
    default: return 2;
  }
}

// Search semantics of the two NGT graph-search variants.
//  ReadOnly : NeighborhoodGraph::searchReadOnlyGraph (lib/NGT/Graph.cpp:716-835),
//             used by ngt_open_index_as_read_only.
//  Updatable: NeighborhoodGraph::search (lib/NGT/Graph.cpp:840-1024), used by
//             ngt_open_index; differs only in how the result heap is updated.
enum class GraphMode : int32_t { ReadOnly = 0, Updatable = 1 };

// Packed (id, distance) with NGT's ordering: distance, then id
// (ObjectDistance::operator<, lib/NGT/Common.h:2337-2360).
struct ObjDist {
  uint32_t id;
  float distance;
};

}  // namespace ngtg
