// Readers for the on-disk NGT index directory (prf / obj / grp / tre).
//
// The formats are fixed by the reference and must be read byte-for-byte:
//   prf : text "key<TAB>value" lines               (lib/NGT/Common.h:915-1000 PropertySet,
//                                                    keys written by lib/NGT/Index.h:121-200
//                                                    and lib/NGT/Graph.h:627-739)
//   obj : Repository<Object>: size_t n, then per slot '-' or '+' and
//         Dimension*sizeof(type) raw bytes          (lib/NGT/Common.h:2181-2238,
//                                                    lib/NGT/ObjectSpace.h:620-640)
//   grp : Repository<GraphNode>: size_t n, per slot '-' or '+' then
//         uint32 count + count*{uint32 id,float d}  (lib/NGT/Graph.h:153-160,
//                                                    lib/NGT/ObjectSpace.h:72-80)
//   tre : leaf repository then internal repository (lib/NGT/Tree.h:347-355,
//                                                    lib/NGT/Node.h:88-110,218-280,441-510)
#pragma once
#include <map>
#include <string>
#include <vector>
#include <cstdint>
#include "ngt_types.h"

namespace ngtg {

struct Property {
  std::map<std::string, std::string> kv;
  int dimension = 0;               // user dimension (prf "Dimension")
  Metric metric = Metric::L2;
  ObjType otype = ObjType::Float;
  bool has_tree = true;            // IndexType GraphAndTree
  int edge_size_for_search = 40;
  int dynamic_edge_size_base = 30;
  int dynamic_edge_size_rate = 20;
  int seed_size = 10;
  int seed_type = 0;               // SeedType (lib/NGT/Graph.h:297-304)
  int epsilon_type = 0;            // EpsilonType (lib/NGT/Graph.h:306)
  float quantization_scale = 0.f;  // QuantizationScale (Qsint8 objects)
  std::string graph_type;
  std::string get(const std::string& k, const std::string& dflt = "") const;
};

// DVP tree with the pivots flattened into one arena.
struct HostTree {
  // Node ids keep the reference's raw encoding: bit 31 = leaf, low bits = index.
  struct Internal {
    uint32_t pivot = 0;            // row in pivots (in units of padded rows)
    uint32_t children[5] = {0, 0, 0, 0, 0};
    float borders[4] = {0, 0, 0, 0};
    uint32_t nchildren = 0;
  };
  struct Leaf {
    uint32_t first = 0;            // offset into leaf_ids
    uint32_t count = 0;
  };
  std::vector<Internal> internals;  // index = node index (slot 0 unused)
  std::vector<uint8_t> internal_present;
  std::vector<Leaf> leaves;
  std::vector<uint8_t> leaf_present;
  std::vector<uint32_t> leaf_ids;   // object ids stored in leaves, in stored order
  std::vector<uint8_t> pivots;      // [npivots][dpad] elements of the object type
  uint32_t npivots = 0;
  uint32_t root = 0;                // raw id of the root node
};

struct HostIndex {
  std::string path;
  Property prop;
  uint32_t nrows = 0;               // repository size including the dummy row 0
  uint32_t dim = 0;                 // stored dimension (D, or D+1 for inner product)
  uint32_t dpad = 0;                // ((dim-1)/16+1)*16
  std::vector<uint8_t> objects;     // [nrows][dpad] elements, zero padded
  std::vector<uint8_t> present;     // 1 if the object slot is occupied
  std::vector<uint32_t> offsets;    // CSR of the graph, nrows+1 entries
  std::vector<uint32_t> edges;
  HostTree tree;
  // refinement objects (robj, RefinementObjectType Float-4): float rows of rdim_pad
  // elements (the user dimension rounded up to 4), slot 0 unused; empty when absent
  std::vector<float> robj;
  uint32_t robj_rows = 0, rdim_pad = 0;
  size_t elem_size() const { return objtype_size(prop.otype); }
  size_t row_bytes() const { return (size_t)dpad * elem_size(); }
};

// Quantized graph of an index (<index>/qg, written by `qbg create-qg` and
// `qbg build-qg`), as NGTQG::Index reads it:
//   qg/prf     NGTQ::Property text file           (lib/NGT/NGTQ/Quantizer.h:560-700)
//   qg/qr      uint32 n, n floats: the rotation   (lib/NGT/NGTQ/Quantizer.h:164-186)
//   qg/rqcb    uint32 size, dimension, padded dimension, size floats: the
//              (rotated) global codebook, one centroid for QG
//                                                 (lib/NGT/NGTQ/Quantizer.h:355-378,3790-3805)
//   qg/local-i NGT index whose objects 1..16 are subspace i's centroids
//   qg/grp     uint64 subspaces, uint64 n, then per node: uint32 subspace id,
//              uint32 count, count neighbour ids, and the neighbours' 4-bit codes
//              (QuantizedGraphRepository::serialize, lib/NGT/NGTQ/QuantizedGraph.h:170-226;
//              code layout of QuantizedObjectProcessingStream,
//              lib/NGT/NGTQ/Quantizer.h:1040-1180)
struct HostQG {
  uint32_t dim = 0;                 // quantizer dimension
  uint32_t m = 0;                   // subspaces (LocalDivisionNo)
  uint32_t ld = 0;                  // dimensions per subspace
  uint32_t ma = 0;                  // m rounded up to even
  std::vector<float> rotation;      // dim*dim, [p*dim + c]; empty = none
  std::vector<float> gcentroid;     // [ncentroids][dim]: QG has one, QBG one per blob subspace id
  uint32_t ncentroids = 1;
  std::vector<float> lcentroids;    // [m][16][ld]
  std::vector<uint32_t> sid;        // per node: its subspace id (the codebook centroid of its table)
  uint32_t nnodes = 0;
  std::vector<uint32_t> offsets;    // nnodes+1
  std::vector<uint32_t> ids;
  std::vector<uint32_t> code_off16; // start of each node's code stream, in 16-byte units
  std::vector<uint8_t> codes;       // every stream padded to 16 bytes
  size_t block_bytes() const { return (size_t)8 * ma; }   // 16 neighbours
};

// Every node of a graph file with its edges' distances (Repository<GraphNode>,
// lib/NGT/Graph.h:153-160): slot count, presence, CSR offsets, ids and distances, and
// the raw bytes of the trailing prevsize vector (GraphRepository::serialize).
struct GraphEdges {
  uint64_t n = 0;
  std::vector<uint8_t> present;
  std::vector<uint64_t> off;        // n+1
  std::vector<uint32_t> ids;
  std::vector<float> dists;
  std::vector<char> trailer;
};
GraphEdges read_graph_edges(const std::string& path);
void write_graph_edges(const std::string& path, const GraphEdges& g);

// Throws std::runtime_error with a message on any format or I/O error.
Property load_property(const std::string& dir);
// The key/value pairs of <dir>/prf without interpreting them (NGTQ property files).
Property load_property_raw(const std::string& dir);
void load_index(const std::string& dir, HostIndex& out);
// Reads <index_dir>/qg; nrows bounds the neighbour ids.
void load_qg(const std::string& index_dir, uint32_t nrows, HostQG& out);
// Reads the blobs of a QBG index directory (same files at its top level:
// prf, qr, rqcb, local-*/obj, grp); blobs = nodes of its global index, at most
// nblobs of them; the object ids in a blob are not bounded here.
void load_qbg(const std::string& qbg_dir, uint32_t nblobs, HostQG& out);

}  // namespace ngtg
