// Device-resident index layout and per-query parameter blocks shared by the
// host engine and the kernels.
//
// HBM layout (all arrays 16-byte aligned, row 0 is NGT's dummy object so that
// object ids index rows directly):
//   objects  : [nrows][row_chunks] uint4  -- the object's native type, zero padded
//              to ((dim-1)/16+1)*16 elements like the reference's padded rows
//              (lib/NGT/ObjectSpace.h:354)
//   offsets  : [nrows+1] uint32           -- CSR of the graph (edge order kept)
//   edges    : [E] uint32                 -- neighbour ids
//   internals: DVP-tree internal nodes, pivots: [npivots][row_chunks] uint4
//   leaf_seed_off/ids : per-leaf seed lists, already thinned on the host exactly
//              as GraphAndTreeIndex::getSeedsFromTree does (lib/NGT/Index.h:2173-2220)
#pragma once
#include <cstdint>
#include "ngt_types.h"

namespace ngtg {

struct DevInternal {
  uint32_t pivot;
  uint32_t nchildren;
  uint32_t children[5];
  float borders[4];
  uint32_t pad;
};

struct DevGraph {
  const uint4* objects = nullptr;
  uint32_t row_chunks = 0;      // 16-byte chunks per row
  uint32_t nrows = 0;
  const uint32_t* offsets = nullptr;
  const uint32_t* edges = nullptr;
  const DevInternal* internals = nullptr;
  uint32_t ninternals = 0;
  const uint4* pivots = nullptr;
  uint32_t root = 0;            // raw node id (bit 31 = leaf)
  uint32_t nleaves = 0;
  const uint32_t* leaf_seed_off = nullptr;
  const uint32_t* leaf_seed_ids = nullptr;
};

// Per-query search parameters (one SearchContainer of the reference,
// lib/NGT/Common.h:2456-2534, after the C API and getEdgeSize have resolved
// the defaults).
struct QueryParams {
  uint32_t size;         // sc.size as used during the search (after RESULT_DEFINED_RANGE expansion)
  uint32_t size_out;     // number of results kept at the end (sizeBackup or size)
  float radius;          // initial sc.radius
  float coef;            // coefficient applied to the radius to get explorationRadius
  uint32_t edge_size;    // neighbours read per expanded node
  uint32_t seed_off;     // explicit seeds: offset into the seed list (tree seeds: unused)
  uint32_t seed_cnt;     // explicit seeds: count; 0xffffffff = take seeds from the tree
  uint32_t out_off;      // offset of this query's results in the output arrays
};

// Quantized graph in HBM (NGTQG, lib/NGT/NGTQ/QuantizedGraph.h):
//   rotation   : [dim][dim] float, element [p*dim + c] (null: no rotation)
//   gcentroid  : [dim] float (the single global centroid)
//   lcentroids : [m][16][ld] float
//   offsets/ids: CSR of the quantized graph (each node's first <= E edges)
//   codes      : per node, blocks of 16 neighbours x ma subspaces x 4 bits
//                (8*ma bytes per block; neighbour o of a block has subspace s's
//                code in byte 8*s + o/2, low nibble for even o), starting at
//                byte 16*code_off16[node]
struct DevQG {
  const float* rotation = nullptr;
  const float* gcentroid = nullptr;
  const float* lcentroids = nullptr;
  const uint32_t* offsets = nullptr;
  const uint32_t* ids = nullptr;
  const uint32_t* code_off16 = nullptr;
  const uint8_t* codes = nullptr;
  uint32_t dim = 0, m = 0, ld = 0, ma = 0, nnodes = 0;
};

// Per-query parameters of a quantized-graph search (NGTQG::SearchContainer
// after ngtqg_search_index_, lib/NGT/NGTQ/Capi.cpp:81-127).
struct QGParams {
  uint32_t size;         // result-set size during the search: size x result expansion when that is > 1
  uint32_t k;            // requested size
  float radius;          // initial radius (FLT_MAX for none)
  float coef;            // exploration coefficient (1 + epsilon)
  uint32_t rerank;       // 1 when result expansion >= 1: exact re-rank, radius cut, truncation to k
  uint32_t seed_off;     // as QueryParams
  uint32_t seed_cnt;
  uint32_t out_off;
};

// Per-query parameters of a quantized-blob-graph search (QBG::SearchContainer
// after qbg_search_index_, lib/NGT/NGTQ/Capi.cpp:549-574).
struct QBGParams {
  uint32_t size;         // result size: number_of_results x result_expansion when that is >= 1
  float coef;            // 1 + epsilon
  float bcoef;           // 1 + blob_epsilon
  uint32_t explored;     // number_of_explored_blobs
  uint32_t edge_size;    // global-graph neighbours read per expanded node
  uint32_t seed_off;     // tree-seed table of the global index (seed_cnt 0xffffffff)
  uint32_t seed_cnt;
  uint32_t fb_off;       // the fixed random seeds used when the tree gives none
  uint32_t fb_cnt;
  uint32_t out_off;
};

// Per-query counters written by the kernels.
struct QueryStats {
  uint32_t distance_computations;
  uint32_t expansions;
  uint32_t visited;
  uint32_t edges_read;   // adjacency entries read (sum over expanded nodes of min(degree, edge size))
  uint32_t status;       // bit flags below
};

// Search rows of the CTA-per-query kernel: the objects themselves, bf16 copies of
// float objects, or 8-bit codes of float objects (WideConfig::sq8).
enum class SearchRows : uint32_t { Native = 0, Bf16 = 1, Sq8 = 2 };

enum StatusBits : uint32_t {
  kStatusCandidateOverflow = 1u,   // candidate list hit its capacity (result may differ)
  kStatusVisitedSpill = 2u,        // visited set moved to the global bitmap
  kStatusEmptySeeds = 4u,          // no seed was available
  kStatusTreeError = 8u,           // tree descent exceeded its depth bound
  kStatusIterationLimit = 16u,     // search loop hit its iteration bound
};

}  // namespace ngtg
