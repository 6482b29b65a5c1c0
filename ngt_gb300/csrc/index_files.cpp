// Readers for the NGT index directory.  See index_files.h for the format
// citations.  Every read is bounds-checked; a truncated or corrupted file is
// rejected with a message instead of producing a partial index.
#include "index_files.h"

#include <algorithm>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace ngtg {

namespace {

[[noreturn]] void fail(const std::string& msg) { throw std::runtime_error(msg); }

struct Reader {
  std::vector<char> buf;
  size_t pos = 0;
  std::string name;
  explicit Reader(const std::string& path) : name(path) {
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    if (!f.is_open()) fail("cannot open " + path);
    std::streamsize n = f.tellg();
    f.seekg(0);
    buf.resize((size_t)n);
    if (n > 0 && !f.read(buf.data(), n)) fail("cannot read " + path);
  }
  template <typename T>
  T get() {
    if (pos + sizeof(T) > buf.size()) fail("truncated file " + name);
    T v;
    std::memcpy(&v, buf.data() + pos, sizeof(T));
    pos += sizeof(T);
    return v;
  }
  const char* take(size_t n) {
    if (pos + n > buf.size()) fail("truncated file " + name);
    const char* p = buf.data() + pos;
    pos += n;
    return p;
  }
  bool at_end() const { return pos == buf.size(); }
};

Metric parse_metric(const std::string& s) {
  if (s == "L1") return Metric::L1;
  if (s == "L2") return Metric::L2;
  if (s == "Hamming") return Metric::Hamming;
  if (s == "Jaccard") return Metric::Jaccard;
  if (s == "SparseJaccard") return Metric::SparseJaccard;
  if (s == "Angle") return Metric::Angle;
  if (s == "Cosine") return Metric::Cosine;
  if (s == "NormalizedAngle") return Metric::NormalizedAngle;
  if (s == "NormalizedCosine") return Metric::NormalizedCosine;
  if (s == "NormalizedL2") return Metric::NormalizedL2;
  if (s == "InnerProduct") return Metric::InnerProduct;
  if (s == "Poincare") return Metric::Poincare;
  if (s == "Lorentz") return Metric::Lorentz;
  fail("unsupported DistanceType '" + s + "'");
}

ObjType parse_objtype(const std::string& s) {
  if (s == "Float-4") return ObjType::Float;
  if (s == "Integer-1") return ObjType::Uint8;
  if (s == "Float-2") return ObjType::Float16;
  if (s == "QSUInteger-8B") return ObjType::Qsint8;
  fail("unsupported ObjectType '" + s + "'");
}

int to_int(const std::string& s, const char* key) {
  try {
    size_t used = 0;
    long v = std::stol(s, &used);
    return (int)v;
  } catch (...) {
    fail(std::string("invalid integer for ") + key + ": '" + s + "'");
  }
}

}  // namespace

std::string Property::get(const std::string& k, const std::string& dflt) const {
  auto it = kv.find(k);
  return it == kv.end() ? dflt : it->second;
}

Property load_property_raw(const std::string& dir) {
  Property p;
  std::ifstream f(dir + "/prf");
  if (!f.is_open()) fail("cannot open " + dir + "/prf");
  std::string line;
  while (std::getline(f, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    auto tab = line.find('\t');
    if (tab != std::string::npos) p.kv[line.substr(0, tab)] = line.substr(tab + 1);
  }
  return p;
}

Property load_property(const std::string& dir) {
  Property p;
  std::ifstream f(dir + "/prf");
  if (!f.is_open()) fail("cannot open " + dir + "/prf");
  std::string line;
  while (std::getline(f, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    auto tab = line.find('\t');
    if (tab == std::string::npos) continue;
    p.kv[line.substr(0, tab)] = line.substr(tab + 1);
  }
  p.dimension = to_int(p.get("Dimension", "0"), "Dimension");
  if (p.dimension <= 0) fail("invalid Dimension in " + dir + "/prf");
  p.metric = parse_metric(p.get("DistanceType", "L2"));
  p.otype = parse_objtype(p.get("ObjectType", "Float-4"));
  p.has_tree = p.get("IndexType", "GraphAndTree") == "GraphAndTree";
  p.edge_size_for_search = to_int(p.get("EdgeSizeForSearch", "40"), "EdgeSizeForSearch");
  p.dynamic_edge_size_base = to_int(p.get("DynamicEdgeSizeBase", "30"), "DynamicEdgeSizeBase");
  p.dynamic_edge_size_rate = to_int(p.get("DynamicEdgeSizeRate", "20"), "DynamicEdgeSizeRate");
  p.seed_size = to_int(p.get("SeedSize", "10"), "SeedSize");
  std::string st = p.get("SeedType", "None");
  p.seed_type = st == "RandomNodes" ? 1 : st == "FixedNodes" ? 2 : st == "FirstNode" ? 3 : st == "AllLeafNodes" ? 4 : 0;
  std::string et = p.get("EpsilonType", "None");
  p.epsilon_type = et == "ByQuery" ? 1 : et == "ResultSize" ? 2 : 0;
  p.graph_type = p.get("GraphType", "ANNG");
  if (p.metric == Metric::SparseJaccard) fail("SparseJaccard indexes are not supported");
  if (p.otype == ObjType::Qsint8) {
    // the read-only search specializes L2, the inner product and the normalized cosine
    // for these objects (lib/NGT/Graph.h:357-363); the others are not supported here
    if (p.metric != Metric::L2 && p.metric != Metric::InnerProduct && p.metric != Metric::NormalizedCosine)
      fail("QSUInteger-8B objects are supported with the L2, inner-product and normalized-cosine distances");
    try {
      p.quantization_scale = std::stof(p.get("QuantizationScale", "0"));
    } catch (...) {
      fail("invalid QuantizationScale in " + dir + "/prf");
    }
    if (!(p.quantization_scale > 0.f)) fail("QSUInteger-8B index without a positive QuantizationScale");
  }
  return p;
}

static void read_objects(const std::string& path, HostIndex& ix) {
  Reader r(path);
  uint64_t n = r.get<uint64_t>();
  if (n == 0 || n > 0xFFFFFFF0ull) fail("invalid object count in " + path);
  const size_t es = ix.elem_size();
  const size_t file_row = (size_t)ix.dim * es;
  ix.nrows = (uint32_t)n;
  ix.objects.assign((size_t)n * ix.row_bytes(), 0);
  ix.present.assign(n, 0);
  for (uint64_t i = 0; i < n; i++) {
    char t = r.get<char>();
    if (t == '-') continue;
    if (t != '+') fail("corrupted object file " + path);
    const char* src = r.take(file_row);
    std::memcpy(ix.objects.data() + i * ix.row_bytes(), src, file_row);
    ix.present[i] = 1;
  }
  if (!r.at_end()) fail("trailing bytes in object file " + path);
}

static void read_graph(const std::string& path, HostIndex& ix) {
  Reader r(path);
  uint64_t n = r.get<uint64_t>();
  if (n > 0xFFFFFFF0ull) fail("invalid node count in " + path);
  ix.offsets.assign(ix.nrows + 1, 0);
  ix.edges.clear();
  std::vector<uint32_t> start(ix.nrows, 0), deg(ix.nrows, 0);
  for (uint64_t i = 0; i < n; i++) {
    char t = r.get<char>();
    if (t == '-') continue;
    if (t != '+') fail("corrupted graph file " + path);
    uint32_t cnt = r.get<uint32_t>();
    const char* p = r.take((size_t)cnt * 8);
    if (i >= ix.nrows) fail("graph node beyond the object repository in " + path);
    start[i] = (uint32_t)ix.edges.size();
    deg[i] = cnt;
    for (uint32_t e = 0; e < cnt; e++) {
      uint32_t id;
      std::memcpy(&id, p + (size_t)e * 8, 4);
      if (id == 0 || id >= ix.nrows) fail("edge to an invalid object id in " + path);
      ix.edges.push_back(id);
    }
  }
  // A trailing uint32-counted vector of uint16 (GraphRepository::prevsize) may follow.
  if (!r.at_end()) {
    uint32_t m = r.get<uint32_t>();
    r.take((size_t)m * 2);
    if (!r.at_end()) fail("trailing bytes in graph file " + path);
  }
  // Rows are laid out in id order already; offsets is the CSR prefix.
  uint32_t acc = 0;
  for (uint32_t i = 0; i < ix.nrows; i++) {
    if (deg[i] && start[i] != acc) fail("internal error: non-monotone graph layout");
    ix.offsets[i] = acc;
    acc += deg[i];
  }
  ix.offsets[ix.nrows] = acc;
}

GraphEdges read_graph_edges(const std::string& path) {
  Reader r(path);
  GraphEdges g;
  g.n = r.get<uint64_t>();
  if (g.n > 0xFFFFFFF0ull) fail("invalid node count in " + path);
  g.present.assign(g.n, 0);
  g.off.assign(g.n + 1, 0);
  for (uint64_t i = 0; i < g.n; i++) {
    char t = r.get<char>();
    if (t == '+') {
      uint32_t cnt = r.get<uint32_t>();
      const char* p = r.take((size_t)cnt * 8);
      g.present[i] = 1;
      for (uint32_t e = 0; e < cnt; e++) {
        uint32_t id;
        float d;
        std::memcpy(&id, p + (size_t)e * 8, 4);
        std::memcpy(&d, p + (size_t)e * 8 + 4, 4);
        if (id == 0 || id >= g.n) fail("edge to an invalid node id in " + path);
        g.ids.push_back(id);
        g.dists.push_back(d);
      }
    } else if (t != '-') {
      fail("corrupted graph file " + path);
    }
    g.off[i + 1] = g.ids.size();
  }
  g.trailer.assign(r.buf.begin() + (std::ptrdiff_t)r.pos, r.buf.end());
  return g;
}

void write_graph_edges(const std::string& path, const GraphEdges& g) {
  std::ofstream f(path, std::ios::binary | std::ios::trunc);
  if (!f.is_open()) fail("cannot write " + path);
  f.write(reinterpret_cast<const char*>(&g.n), 8);
  std::vector<char> rec;
  for (uint64_t i = 0; i < g.n; i++) {
    if (!g.present[i]) {
      f.put('-');
      continue;
    }
    const uint32_t cnt = (uint32_t)(g.off[i + 1] - g.off[i]);
    rec.resize(1 + 4 + (size_t)cnt * 8);
    rec[0] = '+';
    std::memcpy(rec.data() + 1, &cnt, 4);
    for (uint32_t e = 0; e < cnt; e++) {
      std::memcpy(rec.data() + 5 + (size_t)e * 8, &g.ids[g.off[i] + e], 4);
      std::memcpy(rec.data() + 9 + (size_t)e * 8, &g.dists[g.off[i] + e], 4);
    }
    f.write(rec.data(), (std::streamsize)rec.size());
  }
  f.write(g.trailer.data(), (std::streamsize)g.trailer.size());
  if (!f.good()) fail("cannot write " + path);
}

static void read_tree(const std::string& path, HostIndex& ix) {
  Reader r(path);
  HostTree& t = ix.tree;
  const size_t es = ix.elem_size();
  const size_t file_row = (size_t)ix.dim * es;
  const size_t row = ix.row_bytes();
  auto add_pivot = [&](const char* src) {
    t.pivots.resize((size_t)(t.npivots + 1) * row, 0);
    std::memcpy(t.pivots.data() + (size_t)t.npivots * row, src, file_row);
    return t.npivots++;
  };
  // leaves
  uint64_t nl = r.get<uint64_t>();
  if (nl > 0xFFFFFFFull) fail("invalid leaf count in " + path);
  t.leaves.assign(nl, {});
  t.leaf_present.assign(nl, 0);
  for (uint64_t i = 0; i < nl; i++) {
    char c = r.get<char>();
    if (c == '-') continue;
    if (c != '+') fail("corrupted tree file " + path);
    r.get<uint32_t>();                 // node id
    uint32_t parent = r.get<uint32_t>();
    uint16_t cnt = r.get<uint16_t>();
    t.leaves[i].first = (uint32_t)t.leaf_ids.size();
    t.leaves[i].count = cnt;
    for (uint16_t k = 0; k < cnt; k++) {
      uint32_t id = r.get<uint32_t>();
      r.get<float>();
      t.leaf_ids.push_back(id);
    }
    if (!((parent & 0x7fffffffu) == 0 && cnt == 0)) r.take(file_row);  // leaf pivot (unused for seeds)
    t.leaf_present[i] = 1;
  }
  // internal nodes
  uint64_t ni = r.get<uint64_t>();
  if (ni > 0xFFFFFFFull) fail("invalid internal-node count in " + path);
  t.internals.assign(ni, {});
  t.internal_present.assign(ni, 0);
  for (uint64_t i = 0; i < ni; i++) {
    char c = r.get<char>();
    if (c == '-') continue;
    if (c != '+') fail("corrupted tree file " + path);
    r.get<uint32_t>();
    r.get<uint32_t>();
    HostTree::Internal in;
    in.pivot = add_pivot(r.take(file_row));
    uint64_t cs = r.get<uint64_t>();
    if (cs < 2 || cs > 5) fail("unsupported internal fan-out in " + path);
    in.nchildren = (uint32_t)cs;
    for (uint64_t k = 0; k < cs; k++) in.children[k] = r.get<uint32_t>();
    for (uint64_t k = 0; k + 1 < cs; k++) in.borders[k] = r.get<float>();
    t.internals[i] = in;
    t.internal_present[i] = 1;
  }
  if (!r.at_end()) fail("trailing bytes in tree file " + path);
  // Root is node 1: internal if present, otherwise the leaf (lib/NGT/Tree.h:217-233).
  if (ni > 1 && t.internal_present[1]) t.root = 1u;
  else if (nl > 1 && t.leaf_present[1]) t.root = 0x80000000u | 1u;
  else fail("tree has no root node in " + path);
  // Validate child references so the device never follows a bad id.
  for (uint64_t i = 0; i < ni; i++) {
    if (!t.internal_present[i]) continue;
    for (uint32_t k = 0; k < t.internals[i].nchildren; k++) {
      uint32_t raw = t.internals[i].children[k];
      uint32_t idx = raw & 0x7fffffffu;
      bool leaf = (raw & 0x80000000u) != 0;
      if (leaf ? (idx >= nl || !t.leaf_present[idx]) : (idx >= ni || !t.internal_present[idx]))
        fail("tree child reference out of range in " + path);
    }
  }
  for (uint32_t id : t.leaf_ids)
    if (id == 0 || id >= ix.nrows) fail("tree leaf holds an invalid object id in " + path);
}

// The refinement object file robj (lib/NGT/Index.cpp:1207, ObjectSpace::deserialize): the
// object-file layout of float rows of the user dimension.  Absent, or holding only the
// count, when the index has no refinement objects.
static void read_refinement(const std::string& path, HostIndex& ix) {
  std::ifstream f(path, std::ios::binary | std::ios::ate);
  if (!f.is_open() || (size_t)f.tellg() <= 8) return;
  if (ix.prop.get("RefinementObjectType", "Float-4") != "Float-4") return;
  f.close();
  Reader r(path);
  uint64_t n = r.get<uint64_t>();
  if (n == 0 || n > 0xFFFFFFF0ull) fail("invalid object count in " + path);
  // an inner-product index's refinement objects are augmented like its objects
  // (GraphIndex::constructObjectSpace, lib/NGT/Index.cpp:1127-1189)
  const uint32_t d = (uint32_t)ix.prop.dimension + (ix.prop.metric == Metric::InnerProduct ? 1u : 0u);
  ix.rdim_pad = (d + 3) / 4 * 4;
  ix.robj.assign((size_t)n * ix.rdim_pad, 0.f);
  for (uint64_t i = 0; i < n; i++) {
    char t = r.get<char>();
    if (t == '-') continue;
    if (t != '+') fail("corrupted refinement object file " + path);
    std::memcpy(ix.robj.data() + i * ix.rdim_pad, r.take((size_t)d * 4), (size_t)d * 4);
  }
  if (!r.at_end()) fail("trailing bytes in refinement object file " + path);
  ix.robj_rows = (uint32_t)n;
}

void load_index(const std::string& dir, HostIndex& ix) {
  ix.path = dir;
  ix.prop = load_property(dir);
  ix.dim = (uint32_t)ix.prop.dimension + (ix.prop.metric == Metric::InnerProduct ? 1u : 0u);
  ix.dpad = ((ix.dim - 1) / 16 + 1) * 16;
  read_objects(dir + "/obj", ix);
  read_graph(dir + "/grp", ix);
  read_refinement(dir + "/robj", ix);
  if (ix.prop.has_tree) {
    read_tree(dir + "/tre", ix);
  }
}

namespace {

std::vector<float> read_float_rows(const std::string& path, uint32_t dim, uint32_t& n_out) {
  Reader r(path);
  uint64_t n = r.get<uint64_t>();
  if (n == 0 || n > 0xFFFFFFFull) fail("invalid object count in " + path);
  std::vector<float> rows((size_t)n * dim, 0.f);
  for (uint64_t i = 0; i < n; i++) {
    char t = r.get<char>();
    if (t == '-') continue;
    if (t != '+') fail("corrupted object file " + path);
    std::memcpy(rows.data() + i * dim, r.take((size_t)dim * 4), (size_t)dim * 4);
  }
  if (!r.at_end()) fail("trailing bytes in object file " + path);
  n_out = (uint32_t)n;
  return rows;
}

}  // namespace

static void load_quantized(const std::string& dir, uint32_t id_bound, uint32_t node_bound, bool blobs, HostQG& q);

void load_qg(const std::string& index_dir, uint32_t nrows, HostQG& q) {
  load_quantized(index_dir + "/qg", nrows, nrows, false, q);
}

void load_qbg(const std::string& qbg_dir, uint32_t nblobs, HostQG& q) {
  load_quantized(qbg_dir, 0xFFFFFFFFu, nblobs, true, q);
}

static void load_quantized(const std::string& dir, uint32_t nrows, uint32_t node_bound, bool blobs, HostQG& q) {
  {
    std::ifstream f(dir + "/prf");
    if (!f.is_open()) fail("no quantized graph: cannot open " + dir + "/prf");
  }
  Property p = load_property_raw(dir);
  int dim = to_int(p.get("Dimension", "0"), "Dimension");
  int m = to_int(p.get("LocalDivisionNo", "0"), "LocalDivisionNo");
  if (dim <= 0 || m <= 0 || dim % m != 0) fail("invalid Dimension / LocalDivisionNo in " + dir + "/prf");
  if (to_int(p.get("LocalCentroidLimit", "16"), "LocalCentroidLimit") != 16)
    fail("a quantized graph needs 16 local centroids per subspace");
  if (to_int(p.get("SingleLocalCodebook", "0"), "SingleLocalCodebook") != 0)
    fail("a single shared local codebook is not supported for the quantized graph");
  if (m > 512) fail("more than 512 subspaces are not supported");
  q.dim = (uint32_t)dim;
  q.m = (uint32_t)m;
  q.ld = q.dim / q.m;
  q.ma = (q.m + 1) / 2 * 2;
  {
    Reader r(dir + "/qr");
    q.rotation.clear();
    if (!r.at_end()) {
      uint32_t n = r.get<uint32_t>();
      if (n != 0) {
        if ((uint64_t)n != (uint64_t)q.dim * q.dim) fail("rotation size does not match the dimension in " + dir);
        q.rotation.resize(n);
        std::memcpy(q.rotation.data(), r.take((size_t)n * 4), (size_t)n * 4);
      }
    }
  }
  {
    Reader r(dir + "/rqcb");
    uint32_t size = r.get<uint32_t>();
    (void)r.get<uint32_t>();
    uint32_t pdim = r.get<uint32_t>();
    if (pdim == 0 || size < pdim || size % pdim != 0) fail("invalid global codebook in " + dir + "/rqcb");
    const char* src = r.take((size_t)size * 4);
    q.ncentroids = blobs ? size / pdim : 1u;
    q.gcentroid.assign((size_t)q.ncentroids * q.dim, 0.f);
    for (uint32_t c = 0; c < q.ncentroids; c++)
      std::memcpy(q.gcentroid.data() + (size_t)c * q.dim, src + (size_t)c * pdim * 4, (size_t)std::min(pdim, q.dim) * 4);
  }
  q.lcentroids.assign((size_t)q.m * 16 * q.ld, 0.f);
  for (uint32_t i = 0; i < q.m; i++) {
    uint32_t n = 0;
    std::vector<float> rows = read_float_rows(dir + "/local-" + std::to_string(i) + "/obj", q.ld, n);
    if (n != 17) fail("local codebook " + std::to_string(i) + " does not hold 16 centroids");
    std::memcpy(q.lcentroids.data() + (size_t)i * 16 * q.ld, rows.data() + q.ld, (size_t)16 * q.ld * 4);
  }
  {
    Reader r(dir + "/grp");
    (void)r.get<uint64_t>();
    uint64_t n = r.get<uint64_t>();
    if (n > node_bound) fail("quantized graph has more nodes than the object repository in " + dir);
    q.nnodes = (uint32_t)n;
    q.offsets.assign(n + 1, 0);
    q.code_off16.assign(n, 0);
    q.sid.assign(n, 0);
    q.ids.clear();
    q.codes.clear();
    for (uint64_t i = 0; i < n; i++) {
      uint32_t sid = r.get<uint32_t>();
      if (blobs && sid >= q.ncentroids) fail("blob subspace id beyond the codebook in " + dir + "/grp");
      q.sid[i] = blobs ? sid : 0u;
      uint32_t cnt = r.get<uint32_t>();
      const char* src = r.take((size_t)cnt * 4);
      size_t base = q.ids.size();
      q.ids.resize(base + cnt);
      std::memcpy(q.ids.data() + base, src, (size_t)cnt * 4);
      for (size_t j = base; j < base + cnt; j++)
        if (q.ids[j] == 0 || q.ids[j] >= nrows) fail("quantized graph edge to an invalid object id in " + dir);
      q.offsets[i + 1] = (uint32_t)q.ids.size();
      size_t bytes = cnt ? (size_t)((cnt + 15) / 16) * q.block_bytes() : 0;
      if (q.codes.size() / 16 > 0xFFFFFFFFull) fail("quantized graph codes exceed 64 GB");
      q.code_off16[i] = (uint32_t)(q.codes.size() / 16);
      const char* cs = r.take(bytes);
      q.codes.insert(q.codes.end(), cs, cs + bytes);
      q.codes.resize((q.codes.size() + 15) / 16 * 16, 0);
    }
    if (!r.at_end()) fail("trailing bytes in " + dir + "/grp");
  }
}

}  // namespace ngtg
