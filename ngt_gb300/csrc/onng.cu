// ONNG construction from an ANNG on the GPU: the graph `ngt reconstruct-graph -m S`
// writes (GraphOptimizer::execute, lib/NGT/GraphOptimizer.h:268-367), edge for edge.
//
//   1. reconstructGraph (lib/NGT/GraphReconstructor.h:645-813): every node keeps its
//      `outgoing` nearest edges (all of them when it has fewer) and receives, from each
//      node, a reverse edge for that node's `incoming` nearest edges; lists are sorted
//      by (distance, id) and repeated ids dropped.  Host, linear in the edges.
//   2. adjustPathsEffectively (lib/NGT/GraphReconstructor.h:200-409): an edge src->d is
//      a removal candidate through p when p and d are both neighbours of src with
//      dist(src,p) < dist(src,d) and dist(p,d) < dist(src,d) and p->d is an edge.
//      Finding them reads every neighbour list of every neighbour (deg^2 per node):
//      the GPU kernel below, one CTA per node with its neighbours in a shared-memory
//      hash (a binary search over an id-sorted copy for nodes of more than 4096
//      neighbours), then each node's candidates sorted by (rank of d, p) in shared
//      memory.  The edges are then added rank by rank over all nodes, skipping an edge
//      when one of its candidates already has both edges src->p and p->d in the graph
//      being built -- a pass whose order decides the result, so it runs on the host
//      exactly in the reference's order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "index_files.h"

extern "C" {
#include "../../include/ngtgpu.h"
}

namespace ngtg {
namespace {

#define ONNG_CUDA(x)                                                                                \
  do {                                                                                              \
    cudaError_t e_ = (x);                                                                           \
    if (e_ != cudaSuccess)                                                                          \
      throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e_) + " in " #x);     \
  } while (0)

struct Edge {
  uint32_t id;
  float d;
};
inline bool edge_less(const Edge& a, const Edge& b) { return a.d != b.d ? a.d < b.d : a.id < b.id; }
// GraphReconstructor::edgeComp: nodes being built are kept sorted by id
inline bool id_less(const Edge& a, const Edge& b) { return (a.id & 0x7FFFFFFFu) < (b.id & 0x7FFFFFFFu); }

constexpr uint32_t kHashMax = 4096;     // neighbours held in the shared-memory hash
constexpr uint32_t kHashCap = 8192;
constexpr uint32_t kSortMax = 4096;     // candidate lists sorted in shared memory
constexpr uint32_t kNone = 0xffffffffu;

__device__ __forceinline__ uint32_t hash_slot(uint32_t id, uint32_t mask) { return (id * 2654435761u) & mask; }

// Count (FILL = false) or write (FILL = true) the removal candidates of every node:
// key (rank of d in src's list) << 32 | p.
template <bool FILL>
__global__ void __launch_bounds__(256)
onng_candidates_kernel(const uint64_t* __restrict__ off, const uint32_t* __restrict__ ids,
                       const float* __restrict__ ds, uint32_t n, const uint32_t* __restrict__ hub_slot,
                       const uint64_t* __restrict__ hub_off, const uint32_t* __restrict__ hub_ids,
                       const uint32_t* __restrict__ hub_rank, unsigned long long* __restrict__ counts,
                       const unsigned long long* __restrict__ cand_off, unsigned long long* __restrict__ cand) {
  extern __shared__ uint32_t onng_smem[];              // kHashCap keys, then kHashCap ranks
  uint32_t* keys = onng_smem;
  uint32_t* vals = onng_smem + kHashCap;
  __shared__ unsigned int s_count;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5, nwarps = blockDim.x >> 5;
  for (uint32_t src = blockIdx.x + 1; src < n; src += gridDim.x) {
    const uint64_t b = off[src];
    const uint32_t deg = (uint32_t)(off[src + 1] - b);
    const uint32_t hs = hub_slot[src];
    uint32_t mask = 0;
    if (hs == kNone) {
      uint32_t H = 64;
      while (H < 2 * deg) H <<= 1;                 // deg <= kHashMax: H <= kHashCap
      mask = H - 1;
      for (uint32_t i = tid; i < H; i += blockDim.x) {
        keys[i] = 0u;
        vals[i] = 0u;
      }
      __syncthreads();
      for (uint32_t r = tid; r < deg; r += blockDim.x) {
        const uint32_t id = ids[b + r];
        uint32_t h = hash_slot(id, mask);
        for (uint32_t it = 0; it < H; it++) {      // H >= 2 deg: a free slot exists
          const uint32_t old = atomicCAS(&keys[h], 0u, id);
          if (old == 0u || old == id) {
            atomicMax(&vals[h], r);                // a repeated id keeps its last rank (std::map)
            break;
          }
          h = (h + 1) & mask;
        }
      }
    }
    if (tid == 0) s_count = 0u;
    __syncthreads();
    const unsigned long long base = FILL ? cand_off[src] : 0ull;
    for (uint32_t j = warp; j < deg; j += nwarps) {
      const uint32_t p = ids[b + j];
      const float dp = ds[b + j];
      const uint64_t pb = off[p];
      const uint32_t pdeg = (uint32_t)(off[p + 1] - pb);
      for (uint32_t t = lane; t < pdeg; t += 32) {
        const uint32_t q = ids[pb + t];
        uint32_t r = kNone;
        if (hs == kNone) {
          uint32_t h = hash_slot(q, mask);
          for (uint32_t it = 0; it <= mask; it++) {
            const uint32_t k = keys[h];
            if (k == q) {
              r = vals[h];
              break;
            }
            if (k == 0u) break;
            h = (h + 1) & mask;
          }
        } else {
          uint64_t lo = hub_off[hs], hi = hub_off[hs + 1];
          const uint64_t end = hi;
          while (lo < hi) {
            const uint64_t mid = (lo + hi) >> 1;
            if (hub_ids[mid] < q) lo = mid + 1;
            else hi = mid;
          }
          if (lo < end && hub_ids[lo] == q) r = hub_rank[lo];
        }
        if (r != kNone) {
          const float dd = ds[b + r];
          if (dp < dd && ds[pb + t] < dd) {
            const unsigned int slot = atomicAdd(&s_count, 1u);
            if (FILL) cand[base + slot] = ((unsigned long long)r << 32) | p;
          }
        }
      }
    }
    __syncthreads();
    if (!FILL && tid == 0) counts[src] = s_count;
    __syncthreads();                                // the hash is rebuilt for the next node
  }
}

// Each node's candidate keys ascending (lists of at most kSortMax; longer ones are
// sorted on the host).
__global__ void __launch_bounds__(256)
onng_sort_kernel(const unsigned long long* __restrict__ cand_off, unsigned long long* __restrict__ cand, uint32_t n) {
  __shared__ unsigned long long buf[kSortMax];
  for (uint32_t src = blockIdx.x + 1; src < n; src += gridDim.x) {
    const unsigned long long b = cand_off[src];
    const uint32_t len = (uint32_t)(cand_off[src + 1] - b);
    if (len <= 1 || len > kSortMax) continue;
    uint32_t P = 2;
    while (P < len) P <<= 1;
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) buf[i] = i < len ? cand[b + i] : ~0ull;
    __syncthreads();
    for (uint32_t k = 2; k <= P; k <<= 1)
      for (uint32_t j = k >> 1; j > 0; j >>= 1) {
        for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
          const uint32_t l = i ^ j;
          if (l > i) {
            const unsigned long long x = buf[i], y = buf[l];
            if ((x > y) == ((i & k) == 0)) {
              buf[i] = y;
              buf[l] = x;
            }
          }
        }
        __syncthreads();
      }
    for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) cand[b + i] = buf[i];
    __syncthreads();
  }
}

template <typename T>
T* to_device(const std::vector<T>& v, std::vector<void*>& owned) {
  T* d = nullptr;
  ONNG_CUDA(cudaMalloc(&d, std::max<size_t>(v.size(), 1) * sizeof(T)));
  if (!v.empty()) ONNG_CUDA(cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  owned.push_back(d);
  return d;
}

// GraphReconstructor::reconstructGraph over the ANNG's edge lists.
std::vector<std::vector<Edge>> reconstruct(const GraphEdges& in, int64_t outgoing, int64_t incoming,
                                           int64_t max_edges) {
  const uint64_t n = in.n;
  std::vector<std::vector<Edge>> g(n);
  for (uint64_t id = 1; id < n; id++) {
    if (!in.present[id]) continue;
    const uint64_t cnt = in.off[id + 1] - in.off[id];
    // a node with fewer edges than `outgoing` keeps all of them (the reference warns)
    const uint64_t keep = outgoing == 0 ? 0 : std::min<uint64_t>(cnt, (uint64_t)outgoing);
    for (uint64_t e = 0; e < keep; e++) g[id].push_back(Edge{in.ids[in.off[id] + e], in.dists[in.off[id] + e]});
  }
  if (max_edges == 0) max_edges = std::max(outgoing, incoming);
  for (uint64_t id = 1; id < n; id++) {
    const uint64_t cnt = in.present[id] ? in.off[id + 1] - in.off[id] : 0;
    const uint64_t rsize = std::min<uint64_t>((uint64_t)std::max<int64_t>(incoming, 0), cnt);
    for (uint64_t i = 0; i < rsize; i++) {
      const uint32_t to = in.ids[in.off[id] + i];
      const float d = in.dists[in.off[id] + i];
      if (to >= n || !in.present[to]) continue;
      std::vector<Edge>& l = g[to];
      const Edge x{(uint32_t)id, d};
      if ((int64_t)l.size() >= max_edges) {
        if (l.back().d > d || (l.back().d == d && l.back().id > to)) {
          l.insert(std::lower_bound(l.begin(), l.end(), x, edge_less), x);
          l.resize((size_t)max_edges);
        }
      } else {
        l.push_back(x);
        if ((int64_t)l.size() >= max_edges) std::sort(l.begin(), l.end(), edge_less);
      }
    }
  }
  for (uint64_t id = 1; id < n; id++) {
    std::vector<Edge>& l = g[id];
    std::sort(l.begin(), l.end(), edge_less);
    size_t w = 0;
    uint32_t prev = 0;
    for (size_t r = 0; r < l.size(); r++) {
      if (l[r].id == prev) continue;
      prev = l[r].id;
      l[w++] = l[r];
    }
    l.resize(w);
  }
  return g;
}

// The removal candidates of every node on the GPU: CSR offsets (n+1) and keys.
void candidates(const std::vector<std::vector<Edge>>& g, std::vector<unsigned long long>& coff,
                std::vector<unsigned long long>& cand) {
  const uint32_t n = (uint32_t)g.size();
  std::vector<uint64_t> off(n + 1, 0);
  for (uint32_t i = 0; i < n; i++) off[i + 1] = off[i] + g[i].size();
  std::vector<uint32_t> ids(off[n]);
  std::vector<float> ds(off[n]);
  std::vector<uint32_t> hub_slot(n, kNone);
  std::vector<uint64_t> hub_off(1, 0);
  std::vector<uint32_t> hub_ids, hub_rank;
  for (uint32_t i = 0; i < n; i++) {
    for (size_t e = 0; e < g[i].size(); e++) {
      ids[off[i] + e] = g[i][e].id;
      ds[off[i] + e] = g[i][e].d;
    }
    if (g[i].size() > kHashMax) {
      // an id-sorted copy of the neighbours (a repeated id keeps its last rank)
      std::vector<std::pair<uint32_t, uint32_t>> s;
      for (uint32_t r = 0; r < (uint32_t)g[i].size(); r++) s.emplace_back(g[i][r].id, r);
      std::sort(s.begin(), s.end());
      hub_slot[i] = (uint32_t)(hub_off.size() - 1);
      for (size_t k = 0; k < s.size(); k++) {
        if (k + 1 < s.size() && s[k + 1].first == s[k].first) continue;
        hub_ids.push_back(s[k].first);
        hub_rank.push_back(s[k].second);
      }
      hub_off.push_back(hub_ids.size());
    }
  }
  std::vector<void*> owned;
  try {
    const uint64_t* d_off = to_device(off, owned);
    const uint32_t* d_ids = to_device(ids, owned);
    const float* d_ds = to_device(ds, owned);
    const uint32_t* d_hub_slot = to_device(hub_slot, owned);
    const uint64_t* d_hub_off = to_device(hub_off, owned);
    const uint32_t* d_hub_ids = to_device(hub_ids, owned);
    const uint32_t* d_hub_rank = to_device(hub_rank, owned);
    std::vector<unsigned long long> counts(n, 0);
    unsigned long long* d_counts = to_device(counts, owned);
    int dev = 0, sms = 0;
    ONNG_CUDA(cudaGetDevice(&dev));
    ONNG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const unsigned grid = (unsigned)std::max<uint32_t>(1, std::min<uint32_t>(n, (uint32_t)sms * 3));
    const int smem = (int)(2 * kHashCap * sizeof(uint32_t));
    ONNG_CUDA(cudaFuncSetAttribute((const void*)onng_candidates_kernel<false>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    ONNG_CUDA(cudaFuncSetAttribute((const void*)onng_candidates_kernel<true>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    onng_candidates_kernel<false><<<grid, 256, smem>>>(d_off, d_ids, d_ds, n, d_hub_slot, d_hub_off, d_hub_ids,
                                                  d_hub_rank, d_counts, nullptr, nullptr);
    ONNG_CUDA(cudaGetLastError());
    ONNG_CUDA(cudaMemcpy(counts.data(), d_counts, n * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    coff.assign(n + 1, 0);
    for (uint32_t i = 0; i < n; i++) coff[i + 1] = coff[i] + counts[i];
    cand.assign(coff[n], 0);
    const unsigned long long* d_coff = to_device(coff, owned);
    unsigned long long* d_cand = to_device(cand, owned);
    onng_candidates_kernel<true><<<grid, 256, smem>>>(d_off, d_ids, d_ds, n, d_hub_slot, d_hub_off, d_hub_ids,
                                                 d_hub_rank, nullptr, d_coff, d_cand);
    ONNG_CUDA(cudaGetLastError());
    onng_sort_kernel<<<grid, 256>>>(d_coff, d_cand, n);
    ONNG_CUDA(cudaGetLastError());
    if (!cand.empty())
      ONNG_CUDA(cudaMemcpy(cand.data(), d_cand, cand.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  } catch (...) {
    for (void* p : owned) cudaFree(p);
    throw;
  }
  for (void* p : owned) cudaFree(p);
  for (uint32_t i = 1; i < n; i++)
    if (coff[i + 1] - coff[i] > kSortMax) std::sort(cand.begin() + (std::ptrdiff_t)coff[i], cand.begin() + (std::ptrdiff_t)coff[i + 1]);
}

bool has_edge(const std::vector<Edge>& node, uint32_t id) {
  auto it = std::lower_bound(node.begin(), node.end(), Edge{id, 0.f}, id_less);
  return it != node.end() && it->id == id;
}

// GraphReconstructor::adjustPathsEffectively: the edges of `tmp` added rank by rank.
std::vector<std::vector<Edge>> adjust(const std::vector<std::vector<Edge>>& tmp, const std::vector<uint8_t>& present,
                                      int64_t min_edges) {
  const uint32_t n = (uint32_t)tmp.size();
  std::vector<unsigned long long> coff, cand;
  candidates(tmp, coff, cand);
  std::vector<unsigned long long> next(coff.begin(), coff.end() - 1);   // first unused candidate per node
  std::vector<std::vector<Edge>> out(n);
  std::vector<uint32_t> active;
  for (uint32_t id = 1; id < n; id++) active.push_back(id);
  for (size_t rank = 0; !active.empty(); rank++) {
    size_t w = 0;
    for (size_t a = 0; a < active.size(); a++) {
      const uint32_t id = active[a];
      const std::vector<Edge>& src = tmp[id];
      if (rank >= src.size()) continue;               // finished: leaves the list
      active[w++] = id;
      if (!present[id]) continue;
      if (next[id] < coff[id + 1] && (int64_t)(out[id].size() + src.size() - rank) > min_edges) {
        bool exist = false;
        // this rank's candidates, ascending p (candidates of an earlier rank left over
        // when the edge count condition failed stay in front and stop the scan, as the
        // reference's list does)
        while (next[id] < coff[id + 1] && (cand[next[id]] >> 32) == rank) {
          const uint32_t p = (uint32_t)cand[next[id]];
          next[id]++;
          if (has_edge(out[id], p) && has_edge(out[p], src[rank].id)) {
            exist = true;
            while (next[id] < coff[id + 1] && (cand[next[id]] >> 32) == rank) next[id]++;
            break;
          }
        }
        if (exist) continue;
      }
      std::vector<Edge>& l = out[id];
      l.insert(std::lower_bound(l.begin(), l.end(), src[rank], id_less), src[rank]);
    }
    active.resize(w);
  }
  for (auto& l : out) std::sort(l.begin(), l.end(), edge_less);
  return out;
}

void set_graph_type_onng(const std::string& dir) {
  const std::string path = dir + "/prf";
  std::ifstream f(path);
  if (!f.is_open()) throw std::runtime_error("cannot open " + path);
  std::stringstream out;
  std::string line;
  bool found = false;
  while (std::getline(f, line)) {
    if (line.rfind("GraphType\t", 0) == 0) {
      line = "GraphType\tONNG";
      found = true;
    }
    out << line << "\n";
  }
  if (!found) out << "GraphType\tONNG\n";
  f.close();
  std::ofstream o(path, std::ios::trunc);
  o << out.str();
  if (!o.good()) throw std::runtime_error("cannot write " + path);
}

}  // namespace

void build_onng(const std::string& anng, const std::string& onng, int64_t outgoing, int64_t incoming,
                int64_t min_edges) {
  namespace fs = std::filesystem;
  if (fs::exists(onng)) throw std::runtime_error("the specified index exists: " + onng);
  Property prop = load_property(anng);
  if (outgoing < 0) outgoing = std::stoll(prop.get("OutgoingEdge", "-1"));
  if (incoming < 0) incoming = std::stoll(prop.get("IncomingEdge", "-1"));
  GraphEdges in = read_graph_edges(anng + "/grp");
  if (in.n >= 0xFFFFFFFFull || in.ids.size() >= (1ull << 40)) throw std::runtime_error("graph too large");
  fs::copy(anng, onng, fs::copy_options::recursive);
  std::vector<std::vector<Edge>> g;
  const bool rebuilt = outgoing > 0 || incoming > 0;
  if (rebuilt) {
    g = reconstruct(in, outgoing, incoming, INT64_MAX);
  } else {
    g.assign(in.n, {});
    for (uint64_t id = 0; id < in.n; id++)
      for (uint64_t e = in.off[id]; e < in.off[id + 1]; e++) g[id].push_back(Edge{in.ids[e], in.dists[e]});
  }
  std::vector<std::vector<Edge>> out = adjust(g, in.present, min_edges);
  GraphEdges res;
  res.n = in.n;
  res.present = in.present;
  res.trailer = in.trailer;
  res.off.assign(in.n + 1, 0);
  for (uint64_t id = 0; id < in.n; id++) {
    for (const Edge& e : out[id]) {
      res.ids.push_back(e.id);
      res.dists.push_back(e.d);
    }
    res.off[id + 1] = res.ids.size();
  }
  write_graph_edges(onng + "/grp", res);
  if (rebuilt) set_graph_type_onng(onng);
}

}  // namespace ngtg

extern "C" {

bool ngtgpu_build_onng(const char* anng_index, const char* onng_index, int32_t outgoing, int32_t incoming,
                       int64_t min_edges, NGTError error) {
  try {
    if (anng_index == nullptr || onng_index == nullptr) throw std::runtime_error("index path is NULL");
    ngtg::build_onng(anng_index, onng_index, outgoing, incoming, min_edges);
    return true;
  } catch (std::exception& ex) {
    const std::string msg = std::string("Capi : ngtgpu_build_onng() : Error: ") + ex.what();
    if (error != nullptr) *static_cast<std::string*>(error) = msg;
    else std::fprintf(stderr, "%s\n", msg.c_str());
    return false;
  }
}

}  // extern "C"
