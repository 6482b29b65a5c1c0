// Host engine implementation: uploads an opened index to HBM, converts
// queries, resolves per-query parameters like the reference's C API and
// search containers do, and launches the search kernels.
#include "engine.h"

#include <cuda_fp16.h>
#include <algorithm>
#include <cfloat>
#include <cstdlib>
#include <fstream>
#include <climits>
#include <cmath>
#include <cstring>
#include <exception>
#include <stdexcept>
#include <sstream>
#include <string>
#include <thread>

#include "graph_exact.cuh"
#include "graph_fast.cuh"
#include "graph_wide.cuh"
#include "qg_search.cuh"
#include "qg_wide.cuh"
#include "qbg_search.cuh"
#include "kernels.h"
#include "linear_select.cuh"
#include "seed_rng.h"

namespace ngtg {

#define NGT_CUDA(x)                                                                                 \
  do {                                                                                              \
    cudaError_t e_ = (x);                                                                           \
    if (e_ != cudaSuccess)                                                                          \
      throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e_) + " in " #x);     \
  } while (0)

namespace {

template <typename T>
T* dmalloc_copy(const void* src, size_t bytes) {
  void* p = nullptr;
  size_t n = bytes ? bytes : 16;
  NGT_CUDA(cudaMalloc(&p, n));
  if (bytes) NGT_CUDA(cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice));
  return static_cast<T*>(p);
}

uint32_t next_pow2(uint32_t v) {
  uint32_t p = 1;
  while (p < v) p <<= 1;
  return p;
}

ExactKernelFn exact_kernel(ObjType t, Metric m) {
  if (t != ObjType::Qsint8) m = kernel_metric(m);   // qsint8 inner product: its own comparator
  switch (t) {
    case ObjType::Float: return exact_kernel_float(m);
    case ObjType::Float16: return exact_kernel_half(m);
    case ObjType::Uint8: return exact_kernel_u8(m);
    case ObjType::Qsint8: return exact_kernel_qs8(m);
    default: return nullptr;
  }
}

LinearKernelFn linear_kernel(ObjType t, Metric m) {
  if (t != ObjType::Qsint8) m = kernel_metric(m);   // qsint8 inner product: its own comparator
  switch (t) {
    case ObjType::Float: return linear_kernel_float(m);
    case ObjType::Float16: return linear_kernel_half(m);
    case ObjType::Uint8: return linear_kernel_u8(m);
    case ObjType::Qsint8: return linear_kernel_qs8(m);
    default: return nullptr;
  }
}

double query_elem(const void* q, QueryType qt, size_t i) {
  switch (qt) {
    case QueryType::Float32: return static_cast<const float*>(q)[i];
    case QueryType::Float64: return static_cast<const double*>(q)[i];
    case QueryType::Uint8: return static_cast<const uint8_t*>(q)[i];
    case QueryType::Float16: return __half2float(static_cast<const __half*>(q)[i]);
  }
  return 0.0;
}

bool is_normalized(Metric m) {
  return m == Metric::NormalizedAngle || m == Metric::NormalizedCosine || m == Metric::NormalizedL2;
}

}  // namespace

GraphEngine::GraphEngine(const std::string& path, GraphMode mode, bool quantized) : mode_(mode) {
  load_index(path, host_);
  if (!exact_kernel(host_.prop.otype, host_.prop.metric))
    throw std::runtime_error("unsupported combination of object type and distance type in " + path);
  if (is_normalized(host_.prop.metric) && host_.prop.otype == ObjType::Uint8)
    throw std::runtime_error("normalized distances over uint8 objects are not supported");
  if (quantized) read_qg();
  NGT_CUDA(cudaGetDevice(&device_));
  NGT_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  upload();
  if (quantized) upload_qg();
  // The no-allocation search's fixed scratch and the exact kernel live in modules
  // that CUDA loads lazily; loading them here, while the index opens, keeps that
  // search's first call free of the module loads (and the reservation they make).
  noalloc_prepare_device(device_, (const void*)exact_kernel(host_.prop.otype, host_.prop.metric));
}

GraphEngine::GraphEngine(const std::string& qbg_dir, bool blobs) : mode_(GraphMode::Updatable) {
  if (!blobs) throw std::runtime_error("invalid QBG open");
  load_index(qbg_dir + "/global", host_);
  if (host_.prop.otype != ObjType::Float || host_.prop.metric != Metric::L2)
    throw std::runtime_error("the QBG global index must hold float L2 centroids");
  load_qbg(qbg_dir, host_.nrows, qb_);
  qbg_dir_ = qbg_dir;
  {
    Property qp = load_property_raw(qbg_dir);
    try {
      qbg_genuine_dim_ = (uint32_t)std::stoul(qp.get("GenuineDimension", std::to_string(qb_.dim)));
    } catch (...) {
      qbg_genuine_dim_ = 0;
    }
    if (qbg_genuine_dim_ == 0 || qbg_genuine_dim_ > host_.dim)
      throw std::runtime_error("invalid GenuineDimension in " + qbg_dir + "/prf");
  }
  if (!qg_kernel(qb_.m)) throw std::runtime_error("too many subspaces in the QBG index");
  uint32_t mx = 1;
  for (uint32_t b = 0; b < qb_.nnodes; b++) mx = std::max(mx, qb_.offsets[b + 1] - qb_.offsets[b]);
  blob_cap_ = (mx + 15) / 16 * 16;
  // getRandomSeeds(repository, seeds, 20) (lib/NGT/Index.h:1270-1302) for a query whose
  // tree leaf is empty, drawn from a generator seeded with 1
  {
    size_t n = host_.nrows ? host_.nrows - 1 : 0;
    size_t ss = std::min<size_t>(n, 20);
    GlibcRand rng(1);
    size_t empty = 0;
    while (qbg_fallback_seeds_.size() < ss) {
      size_t idx = (size_t)std::floor((double)n * rng.unit()) + 1;
      if (!host_.present[idx]) {
        if (++empty > n) break;
        continue;
      }
      if (std::find(qbg_fallback_seeds_.begin(), qbg_fallback_seeds_.end(), (uint32_t)idx) !=
          qbg_fallback_seeds_.end())
        continue;
      qbg_fallback_seeds_.push_back((uint32_t)idx);
    }
  }
  NGT_CUDA(cudaGetDevice(&device_));
  NGT_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  upload();
  auto up = [&](const void* src, size_t bytes) {
    void* p = dmalloc_copy<void>(src, bytes);
    qg_buffers_.push_back(p);
    return p;
  };
  dqb_.rotation = qb_.rotation.empty() ? nullptr
                                       : static_cast<const float*>(up(qb_.rotation.data(), qb_.rotation.size() * 4));
  dqb_.gcentroid = static_cast<const float*>(up(qb_.gcentroid.data(), qb_.gcentroid.size() * 4));
  dqb_.lcentroids = static_cast<const float*>(up(qb_.lcentroids.data(), qb_.lcentroids.size() * 4));
  dqb_.offsets = static_cast<const uint32_t*>(up(qb_.offsets.data(), qb_.offsets.size() * 4));
  dqb_.ids = static_cast<const uint32_t*>(up(qb_.ids.data(), qb_.ids.size() * 4));
  dqb_.code_off16 = static_cast<const uint32_t*>(up(qb_.code_off16.data(), qb_.code_off16.size() * 4));
  dqb_.codes = static_cast<const uint8_t*>(up(qb_.codes.data(), qb_.codes.size()));
  dqb_.dim = qb_.dim;
  dqb_.m = qb_.m;
  dqb_.ld = qb_.ld;
  dqb_.ma = qb_.ma;
  dqb_.nnodes = qb_.nnodes;
  d_blob_sid_ = static_cast<uint32_t*>(up(qb_.sid.data(), qb_.sid.size() * 4));
  qbg_loaded_ = true;
}

GraphEngine::~GraphEngine() {
  cudaSetDevice(device_);
  if (staging_) cudaFreeHost(staging_);
  for (auto& l : co_lanes_) {
    if (l.stream) cudaStreamSynchronize(l.stream);
    cudaFree(l.bitmaps);
    cudaFree(l.overflow);
    cudaFree(l.dev);
    if (l.staging) cudaFreeHost(l.staging);
    if (l.stream) cudaStreamDestroy(l.stream);
  }
  cudaFree(d_objects_);
  cudaFree(d_offsets_);
  cudaFree(d_edges_);
  cudaFree(d_internals_);
  cudaFree(d_pivots_);
  cudaFree(d_present_);
  cudaFree(d_seed_off_);
  cudaFree(d_seed_ids_);
  cudaFree(d_bitmaps_);
  cudaFree(d_overflow_);
  for (auto& sc : fast_scratch_) {
    cudaFree(sc.bitmaps);
    cudaFree(sc.spill);
    cudaFree(sc.work);
  }
  cudaFree(d_bf16_);
  cudaFree(d_sq8_);
  for (void* p : qg_buffers_) cudaFree(p);
  cudaFree(d_qbg_ovf_);
  cudaFree(d_blob_dist_);
  cudaFree(d_olist_);
  cudaFree(d_robj_);
  for (QbgScratch& q : qbg_scratch_) {
    cudaFree(q.bitmaps);
    cudaFree(q.exact_ovf);
    cudaFree(q.qbg_ovf);
    cudaFree(q.blob_dist);
  }
  tc_release(tc_);
  if (stream_) cudaStreamDestroy(stream_);
}

void GraphEngine::upload() {
  const HostIndex& h = host_;
  d_objects_ = dmalloc_copy<void>(h.objects.data(), h.objects.size());
  d_present_ = dmalloc_copy<uint8_t>(h.present.data(), h.present.size());
  d_offsets_ = dmalloc_copy<uint32_t>(h.offsets.data(), h.offsets.size() * 4);
  d_edges_ = dmalloc_copy<uint32_t>(h.edges.data(), h.edges.size() * 4);
  std::vector<DevInternal> ins(h.tree.internals.size());
  for (size_t i = 0; i < ins.size(); i++) {
    const auto& s = h.tree.internals[i];
    DevInternal d{};
    d.pivot = s.pivot;
    d.nchildren = s.nchildren;
    for (int k = 0; k < 5; k++) d.children[k] = s.children[k];
    for (int k = 0; k < 4; k++) d.borders[k] = s.borders[k];
    ins[i] = d;
  }
  d_internals_ = dmalloc_copy<DevInternal>(ins.data(), ins.size() * sizeof(DevInternal));
  d_pivots_ = dmalloc_copy<void>(h.tree.pivots.data(), h.tree.pivots.size());
  nleaves_ = (uint32_t)h.tree.leaves.size();
  dev_.objects = static_cast<const uint4*>(d_objects_);
  dev_.row_chunks = (uint32_t)(h.row_bytes() / 16);
  dev_.nrows = h.nrows;
  dev_.offsets = d_offsets_;
  dev_.edges = d_edges_;
  dev_.internals = d_internals_;
  dev_.ninternals = (uint32_t)ins.size();
  dev_.pivots = static_cast<const uint4*>(d_pivots_);
  dev_.root = h.tree.root;
  dev_.nleaves = nleaves_;
}

// Thinned seed lists of every leaf for one effective seed size, concatenated
// after the tables built so far.  Table t's offsets start at t*(nleaves+1).
uint32_t GraphEngine::seed_table(size_t seed_size) {
  auto it = seed_tables_.find(seed_size);
  if (it != seed_tables_.end()) return it->second;
  const HostTree& t = host_.tree;
  uint32_t table = (uint32_t)seed_tables_.size();
  std::vector<uint32_t> ids;
  for (uint32_t leaf = 0; leaf < nleaves_; leaf++) {
    h_seed_off_.push_back((uint32_t)h_seed_ids_.size());
    if (!t.leaf_present[leaf]) continue;
    const auto& L = t.leaves[leaf];
    ids.assign(t.leaf_ids.begin() + L.first, t.leaf_ids.begin() + L.first + L.count);
    thin_leaf_seeds(ids, leaf, seed_size);
    h_seed_ids_.insert(h_seed_ids_.end(), ids.begin(), ids.end());
  }
  h_seed_off_.push_back((uint32_t)h_seed_ids_.size());
  // launches on any stream (serving and coalescing lanes) may still read the
  // previous tables: they finish before the tables are replaced
  if (d_seed_off_ || d_seed_ids_) NGT_CUDA(cudaDeviceSynchronize());
  cudaFree(d_seed_off_);
  cudaFree(d_seed_ids_);
  d_seed_off_ = dmalloc_copy<uint32_t>(h_seed_off_.data(), h_seed_off_.size() * 4);
  d_seed_ids_ = dmalloc_copy<uint32_t>(h_seed_ids_.data(), h_seed_ids_.size() * 4);
  dev_.leaf_seed_off = d_seed_off_;
  dev_.leaf_seed_ids = d_seed_ids_;
  seed_tables_[seed_size] = table;
  return table;
}

// NeighborhoodGraph::getEdgeSize (lib/NGT/Graph.h:991-1010).
size_t GraphEngine::edge_size_for(const SearchArgs& a) const {
  int64_t esize = a.edge_size == -1 ? host_.prop.edge_size_for_search : a.edge_size;
  if (esize == 0) return INT_MAX;
  if (esize > 0) return (size_t)esize;
  if (esize == -2) {
    float coef = a.epsilon + 1.0f;
    double add = std::pow(10.0, ((double)coef - 1.0) * (double)(float)host_.prop.dynamic_edge_size_rate);
    return add >= (double)INT_MAX ? (size_t)INT_MAX : (size_t)(host_.prop.dynamic_edge_size_base + add);
  }
  throw std::runtime_error("invalid edge size parameter " + std::to_string(a.edge_size));
}

float GraphEngine::epsilon_for_accuracy(double accuracy) const {
  // the table "eps:accuracy,eps:accuracy,..." (AccuracyTable::set, lib/NGT/Index.h:424-440)
  std::vector<std::pair<float, double>> table;
  const std::string str = host_.prop.get("AccuracyTable", "");
  std::stringstream ss(str);
  std::string tok;
  while (std::getline(ss, tok, ',')) {
    if (tok.empty()) continue;
    const size_t c = tok.find(':');
    if (c == std::string::npos || tok.find(':', c + 1) != std::string::npos)
      throw std::runtime_error("AccuracyTable: invalid accuracy table string " + tok + ":" + str);
    table.emplace_back((float)std::strtod(tok.substr(0, c).c_str(), nullptr),
                       std::strtod(tok.substr(c + 1).c_str(), nullptr));
  }
  if (table.size() <= 2)
    throw std::runtime_error("AccuracyTable: the accuracy table is not set yet. The table size=" +
                             std::to_string(table.size()));
  if (accuracy > 1.0) accuracy = 1.0;
  size_t i = 0;
  while (i < table.size() && table[i].second < accuracy) i++;
  if (i == table.size()) i -= 2;
  else if (i != 0) i--;
  const std::pair<float, double> lower = table[i], upper = table[i + 1];
  float e = (float)(lower.first + (upper.first - lower.first) * (accuracy - lower.second) /
                                      (upper.second - lower.second));
  if (e < -0.9f) e = -0.9f;
  return e;
}

void GraphEngine::build_params(const SearchArgs* args, size_t nargs, size_t nq, size_t kmax,
                               std::vector<QueryParams>& params, std::vector<uint32_t>& seed_list,
                               uint32_t& max_size) {
  params.resize(nq);
  seed_list.clear();
  max_size = 0;
  uint32_t shared_seeds = UINT32_MAX;
  for (size_t i = 0; i < nq; i++) {
    if (nargs == 1 && i > 0) {
      // one parameter set for the whole batch: every query's parameters (seeds
      // included) equal the first one's but for its output slot
      params[i] = params[0];
      params[i].out_off = (uint32_t)(i * kmax);
      continue;
    }
    SearchArgs a = args[nargs == 1 ? 0 : i];
    if (a.accuracy > 0.0f) {
      // GraphIndex::search sets epsilon from the expected accuracy before the edge size
      // and the exploration coefficient are derived from it (lib/NGT/Index.h:1700-1702)
      a.epsilon = epsilon_for_accuracy(a.accuracy);
      a.accuracy = -1.0f;
    }
    QueryParams qp{};
    float coef = a.epsilon + 1.0f;                     // SearchContainer::setEpsilon
    if (coef == 0.0f) coef = 1.1f;                     // NGT_EXPLORATION_COEFFICIENT
    size_t size = a.size;
    size_t size_out = size;
    bool size_backup = result_size_rule();
    if (size_backup) {
      size = (size_t)std::round(coef * (float)size);
      coef = 1.0f;
      // Only the read-only search cuts the results back to the requested size
      // (lib/NGT/Graph.cpp:821-828); the updatable search returns them all.
      if (mode_ == GraphMode::Updatable) size_out = size;
    }
    if (size_out > kmax) throw std::runtime_error("result size larger than the output capacity");
    qp.size = (uint32_t)size;
    qp.size_out = (uint32_t)size_out;
    qp.radius = a.radius < 0.0f ? FLT_MAX : a.radius;
    qp.coef = coef;
    qp.edge_size = (uint32_t)std::min<size_t>(edge_size_for(a), 0xffffffffu);
    qp.out_off = (uint32_t)(i * kmax);
    seed_params(a.size, qp.seed_off, qp.seed_cnt, seed_list, &shared_seeds);
    params[i] = qp;
    max_size = std::max<uint32_t>(max_size, qp.size);
  }
  if (seed_list.empty()) seed_list.push_back(0);
}

void GraphEngine::seed_params(size_t k, uint32_t& seed_off, uint32_t& seed_cnt, std::vector<uint32_t>& seed_list,
                              uint32_t* shared_off) {
  const Property& p = host_.prop;
  if (p.has_tree) {
    // GraphAndTreeIndex::getSeedsFromTree: seedSize = SeedSize or size, capped by size;
    // AllLeafNodes keeps the whole leaf.
    size_t seed_size = p.seed_size == 0 ? k : (size_t)p.seed_size;
    if (seed_size > k) seed_size = k;
    if (p.seed_type == 4) seed_size = SIZE_MAX;
    uint32_t t = seed_table(seed_size == 0 ? 1 : seed_size);
    seed_off = t * (nleaves_ + 1);
    seed_cnt = 0xffffffffu;
    return;
  }
  // Graph-only index: GraphIndex::getSeedsFromGraph (lib/NGT/Index.h:1658-1679).
  size_t n = host_.nrows ? host_.nrows - 1 : 0;
  size_t ss = std::min<size_t>(n, (size_t)p.seed_size);
  seed_off = (uint32_t)seed_list.size();
  if (p.seed_type == 2) {
    for (size_t s = 1; s <= ss; s++) seed_list.push_back((uint32_t)s);
  } else if (p.seed_type == 3) {
    seed_list.push_back(1u);
  } else {
    // getRandomSeeds draws from the process-global rand() without reseeding;
    // here every query draws from a generator seeded with 1 so that results
    // are reproducible -- the same seeds for every query, drawn once.
    std::call_once(random_seeds_once_, [&] {
      GlibcRand rng(1);
      size_t empty = 0;
      while (random_seeds_.size() < ss) {
        double r = rng.unit();
        size_t idx = (size_t)std::floor((double)n * r) + 1;
        if (!host_.present[idx]) {
          if (++empty > n) break;
          continue;
        }
        if (std::find(random_seeds_.begin(), random_seeds_.end(), (uint32_t)idx) != random_seeds_.end()) continue;
        random_seeds_.push_back((uint32_t)idx);
      }
    });
    if (shared_off && *shared_off != UINT32_MAX) {
      seed_off = *shared_off;
      seed_cnt = (uint32_t)random_seeds_.size();
      return;
    }
    seed_list.insert(seed_list.end(), random_seeds_.begin(), random_seeds_.end());
    if (shared_off) *shared_off = seed_off;
  }
  seed_cnt = (uint32_t)(seed_list.size() - seed_off);
}

// EpsilonType ResultSize: search for round((1+epsilon) x k) results with the
// exploration coefficient 1; the updatable search applies it to quantized
// objects under EpsilonType None too (lib/NGT/Graph.cpp:845-852).
bool GraphEngine::result_size_rule() const {
  const Property& p = host_.prop;
  return p.epsilon_type == 2 ||
         (mode_ == GraphMode::Updatable && p.epsilon_type == 0 && p.otype == ObjType::Qsint8);
}

size_t GraphEngine::output_size(const SearchArgs& a) const {
  if (result_size_rule() && mode_ == GraphMode::Updatable) {
    float coef = (a.accuracy > 0.0f ? epsilon_for_accuracy(a.accuracy) : a.epsilon) + 1.0f;
    if (coef == 0.0f) coef = 1.1f;
    return (size_t)std::round(coef * (float)a.size);
  }
  return a.size;
}

void GraphEngine::convert_queries(const void* queries, QueryType qt, size_t nq, size_t qdim,
                                  std::vector<uint8_t>& rows) const {
  rows.resize(nq * host_.row_bytes());
  convert_queries(queries, qt, nq, qdim, rows.data());
}

void GraphEngine::convert_queries(const void* queries, QueryType qt, size_t nq, size_t qdim, uint8_t* rows) const {
  const size_t user_dim = (size_t)host_.prop.dimension;
  if (qdim != host_.dim && !(host_.prop.metric == Metric::InnerProduct && qdim == user_dim))
    throw std::runtime_error("the query dimension " + std::to_string(qdim) + " differs from the index dimension " +
                             std::to_string(user_dim));
  const size_t rb = host_.row_bytes();
  const bool norm = is_normalized(host_.prop.metric);
  const bool plain_copy = host_.prop.otype == ObjType::Float && qt == QueryType::Float32 && !norm;
  // bytes of a row the query's elements fill; the rest of the row is zero padding
  const size_t esize = host_.prop.otype == ObjType::Float ? 4 : host_.prop.otype == ObjType::Float16 ? 2 : 1;
  const size_t filled = std::min(rb, qdim * esize);
  // queries [q_begin, q_end): each query's arithmetic is independent of the others
  auto convert_range = [&](size_t q_begin, size_t q_end) {
    for (size_t q = q_begin; q < q_end; q++) std::memset(rows + q * rb + filled, 0, rb - filled);
    if (plain_copy) {
      // float rows are the queries themselves, zero padded
      const float* src = static_cast<const float*>(queries);
      for (size_t q = q_begin; q < q_end; q++) std::memcpy(rows + q * rb, src + q * qdim, qdim * sizeof(float));
      return;
    }
    std::vector<float> tmp(qdim);
    for (size_t q = q_begin; q < q_end; q++) {
      uint8_t* dst = rows + q * rb;
      for (size_t i = 0; i < qdim; i++) tmp[i] = (float)query_elem(queries, qt, q * qdim + i);
      switch (host_.prop.otype) {
        case ObjType::Float: {
          float* o = reinterpret_cast<float*>(dst);
          for (size_t i = 0; i < qdim; i++) o[i] = qt == QueryType::Float64
                                                     ? (float)static_cast<const double*>(queries)[q * qdim + i]
                                                     : tmp[i];
          if (norm) {
            // ObjectSpace::normalize (lib/NGT/ObjectSpace.h:356-384): float sum, sqrt, divide.
            float sum = 0.0f;
            for (size_t i = 0; i < qdim; i++) sum += o[i] * o[i];
            if (sum == 0.0f) throw std::runtime_error("the query is a zero vector; it cannot be normalized");
            sum = (float)std::sqrt(sum);
            for (size_t i = 0; i < qdim; i++) o[i] = o[i] / sum;
          }
          break;
        }
        case ObjType::Float16: {
          __half* o = reinterpret_cast<__half*>(dst);
          for (size_t i = 0; i < qdim; i++) o[i] = __float2half_rn(tmp[i]);
          if (norm) {
            float sum = 0.0f;
            for (size_t i = 0; i < qdim; i++) {
              float v = __half2float(o[i]);
              sum += v * v;
            }
            if (sum == 0.0f) throw std::runtime_error("the query is a zero vector; it cannot be normalized");
            sum = (float)std::sqrt(sum);
            for (size_t i = 0; i < qdim; i++) o[i] = __float2half_rn(__half2float(o[i]) / sum);
          }
          break;
        }
        case ObjType::Uint8: {
          for (size_t i = 0; i < qdim; i++) {
            double v = query_elem(queries, qt, q * qdim + i);
            dst[i] = (uint8_t)(int)v;       // static_cast<uint8_t> truncates toward zero
          }
          break;
        }
        case ObjType::Qsint8: {
          // ObjectSpace::quantizeSymmetrically (lib/NGT/ObjectSpace.h:432-441): the
          // division in float, the product with 127.5 and the rounding in double; under a
          // normalized distance the float query is normalized first
          // (ObjectSpaceRepository::allocateNormalizedObject, ObjectSpaceRepository.h:1120-1160)
          const float scale = host_.prop.quantization_scale;
          if (norm) {
            float sum = 0.0f;
            for (size_t i = 0; i < qdim; i++) sum += tmp[i] * tmp[i];
            if (sum == 0.0f) throw std::runtime_error("the query is a zero vector; it cannot be normalized");
            sum = (float)std::sqrt(sum);
            for (size_t i = 0; i < qdim; i++) tmp[i] = tmp[i] / sum;
          }
          for (size_t i = 0; i < qdim; i++) {
            float fv = tmp[i];
            fv = (float)std::round((double)(fv / scale) * 127.5);
            fv = fv < -127.0f ? -127.0f : fv;
            fv = fv > 127.0f ? 127.0f : fv;
            dst[i] = (uint8_t)(int8_t)fv;
          }
          break;
        }
        default: throw std::runtime_error("unsupported object type");
      }
    }
  };
  // large batches that are more than a copy are converted by several host threads
  const size_t hw = std::max<size_t>(1, std::thread::hardware_concurrency());
  const size_t nt = plain_copy || nq * qdim < ((size_t)1 << 20) ? 1 : std::min<size_t>({hw, (size_t)16, nq});
  if (nt <= 1) {
    convert_range(0, nq);
    return;
  }
  std::vector<std::thread> threads;
  std::vector<std::exception_ptr> errors(nt);
  for (size_t t = 0; t < nt; t++)
    threads.emplace_back([&, t] {
      try {
        convert_range(nq * t / nt, nq * (t + 1) / nt);
      } catch (...) {
        errors[t] = std::current_exception();
      }
    });
  for (auto& th : threads) th.join();
  for (auto& e : errors)
    if (e) std::rethrow_exception(e);
}

void GraphEngine::ensure_scratch(size_t grid) {
  if (grid <= bitmap_grid_) return;
  NGT_CUDA(cudaStreamSynchronize(stream_));   // earlier launches may still use the old buffers
  cudaFree(d_bitmaps_);
  cudaFree(d_overflow_);
  d_bitmaps_ = nullptr;
  d_overflow_ = nullptr;
  size_t words = (host_.nrows + 31) / 32;
  NGT_CUDA(cudaMalloc(&d_bitmaps_, grid * words * 4));
  NGT_CUDA(cudaMemsetAsync(d_bitmaps_, 0, grid * words * 4, stream_));
  NGT_CUDA(cudaMalloc(&d_overflow_, grid * 2 * (size_t)kOverflowCapacity * 8));
  NGT_CUDA(cudaStreamSynchronize(stream_));
  bitmap_grid_ = grid;
}

bool GraphEngine::fast_supported(Kernel k) const {
  if (k == Kernel::Exact) return true;
  if (k == Kernel::Wide)
    return wide_kernel(host_.prop.otype, host_.prop.metric,
                       host_.prop.otype == ObjType::Float && kernel_metric(host_.prop.metric) == Metric::L2
                           ? SearchRows::Bf16 : SearchRows::Native, 256) != nullptr;
  const bool hyperbolic = host_.prop.metric == Metric::Poincare || host_.prop.metric == Metric::Lorentz;
  return fast_kernel(host_.prop.otype, host_.prop.metric, k == Kernel::Fast && !hyperbolic) != nullptr;
}

void GraphEngine::ensure_fast_scratch(FastScratch& sc, size_t slots, cudaStream_t stream) {
  if (slots <= sc.slots) return;
  NGT_CUDA(cudaStreamSynchronize(stream));   // earlier launches on this set may still use it
  cudaFree(sc.bitmaps);
  cudaFree(sc.spill);
  sc.bitmaps = nullptr;
  sc.spill = nullptr;
  size_t words = ((host_.nrows + 31) / 32 + 3) / 4 * 4;
  NGT_CUDA(cudaMalloc(&sc.bitmaps, slots * words * 4));
  NGT_CUDA(cudaMalloc(&sc.spill, slots * 2 * (size_t)kSpillCapacity * 8));
  NGT_CUDA(cudaMemsetAsync(sc.bitmaps, 0, slots * words * 4, stream));
  if (!sc.work) NGT_CUDA(cudaMalloc(&sc.work, 16));
  NGT_CUDA(cudaStreamSynchronize(stream));
  sc.slots = slots;
}

void GraphEngine::reserve_scratch_sets(size_t n) {
  std::lock_guard<std::mutex> lock(mu_);
  if (fast_scratch_.size() < n) fast_scratch_.resize(n);
}

void GraphEngine::reserve_scratch_slots(size_t set, size_t slots) {
  std::lock_guard<std::mutex> lock(mu_);
  if (set >= fast_scratch_.size()) fast_scratch_.resize(set + 1);
  NGT_CUDA(cudaSetDevice(device_));
  ensure_fast_scratch(fast_scratch_[set], slots, stream_);
}

size_t GraphEngine::batched_scratch_bytes(size_t nq) const {
  size_t words = ((host_.nrows + 31) / 32 + 3) / 4 * 4;
  return nq * (words * 4 + 2 * (size_t)kSpillCapacity * 8) + nq * (sizeof(QueryParams) + 64);
}

void GraphEngine::ensure_bf16_rows() {
  if (d_bf16_ || host_.prop.otype != ObjType::Float) return;
  size_t nfloats = (size_t)host_.nrows * host_.dpad;
  NGT_CUDA(cudaMalloc(&d_bf16_, nfloats * 2));
  launch_float_rows_to_bf16(d_objects_, d_bf16_, nfloats, stream_);
  NGT_CUDA(cudaGetLastError());
  NGT_CUDA(cudaStreamSynchronize(stream_));
}

void GraphEngine::ensure_sq8_stats() {
  std::call_once(sq8_once_, [this] { compute_sq8_stats(); });
}

void GraphEngine::compute_sq8_stats() {
  const float* x = reinterpret_cast<const float*>(host_.objects.data());
  const uint32_t dim = host_.prop.dimension, dpad = host_.dpad;
  float lo = FLT_MAX, hi = -FLT_MAX;
  bool integral = true;
  for (size_t r = 1; r < host_.nrows; r++) {          // row 0 is the unused slot
    if (!host_.present[r]) continue;                   // removed objects
    const float* row = x + r * dpad;
    for (uint32_t d = 0; d < dim; d++) {
      const float v = row[d];
      lo = std::min(lo, v);
      hi = std::max(hi, v);
      integral = integral && std::nearbyint(v) == v;
    }
  }
  if (!(lo <= hi)) { lo = 0.f; hi = 0.f; }
  sq8_lossless_ = integral && hi - lo <= 255.f;
  sq8_offset_ = lo;
  sq8_scale_ = sq8_lossless_ || hi == lo ? 1.f : (hi - lo) / 255.f;
}

void GraphEngine::ensure_sq8_rows() {
  if (d_sq8_ || host_.prop.otype != ObjType::Float) return;
  ensure_sq8_stats();
  NGT_CUDA(cudaMalloc(&d_sq8_, (size_t)host_.nrows * host_.dpad));
  launch_float_rows_to_sq8(static_cast<const float*>(d_objects_), static_cast<uint8_t*>(d_sq8_), host_.nrows,
                           host_.dpad, host_.prop.dimension, sq8_offset_, sq8_scale_, stream_);
  NGT_CUDA(cudaGetLastError());
  NGT_CUDA(cudaStreamSynchronize(stream_));
}

SearchRows GraphEngine::wide_search_rows() {
  if (host_.prop.otype != ObjType::Float || kernel_metric(host_.prop.metric) != Metric::L2) return SearchRows::Native;
  if (tuning_.search_rows == 1) return SearchRows::Bf16;
  if (tuning_.search_rows == 2) return SearchRows::Sq8;
  ensure_sq8_stats();
  return sq8_lossless_ ? SearchRows::Sq8 : SearchRows::Bf16;
}

void GraphEngine::search_device(const uint4* d_rows, size_t nq, const SearchArgs* args, size_t nargs, ObjDist* d_out,
                                uint32_t* d_counts, QueryStats* d_stats, size_t kmax, cudaStream_t stream,
                                Kernel kernel) {
  std::lock_guard<std::mutex> lock(mu_);
  NGT_CUDA(cudaSetDevice(device_));
  if (nq == 0) return;
  if (!fast_supported(kernel)) throw std::runtime_error("the batched kernel does not support this index type");
  std::vector<QueryParams> params;
  std::vector<uint32_t> seeds;
  uint32_t max_size = 0;
  build_params(args, nargs, nq, kmax, params, seeds, max_size);
  QueryParams* d_params = nullptr;
  uint32_t* d_seeds = nullptr;
  NGT_CUDA(cudaMallocAsync(&d_params, nq * sizeof(QueryParams), stream));
  NGT_CUDA(cudaMallocAsync(&d_seeds, seeds.size() * 4, stream));
  NGT_CUDA(cudaMemcpyAsync(d_params, params.data(), nq * sizeof(QueryParams), cudaMemcpyHostToDevice, stream));
  NGT_CUDA(cudaMemcpyAsync(d_seeds, seeds.data(), seeds.size() * 4, cudaMemcpyHostToDevice, stream));
  if (kernel == Kernel::Exact)
    launch_exact(d_rows, nq, d_params, d_seeds, max_size, d_out, d_counts, d_stats, stream);
  else if (kernel == Kernel::Wide)
    launch_wide(d_rows, nq, d_params, d_seeds, max_size, d_out, d_counts, d_stats, stream, fast_scratch_[0]);
  else
    launch_fast(d_rows, nq, d_params, d_seeds, max_size, d_out, d_counts, d_stats, stream, kernel,
                fast_scratch_[0]);
  NGT_CUDA(cudaFreeAsync(d_params, stream));
  NGT_CUDA(cudaFreeAsync(d_seeds, stream));
}

void GraphEngine::search_device_slot(const uint4* d_rows, size_t nq, const SearchArgs* args, size_t nargs,
                                     ObjDist* d_out, uint32_t* d_counts, QueryStats* d_stats, size_t kmax,
                                     cudaStream_t stream, size_t slot, Kernel kernel) {
  std::lock_guard<std::mutex> lock(mu_);
  NGT_CUDA(cudaSetDevice(device_));
  if (nq == 0) return;
  if (slot == 0 || slot >= fast_scratch_.size()) throw std::runtime_error("invalid scratch set");
  if (kernel == Kernel::Exact || !fast_supported(kernel))
    throw std::runtime_error("the batched kernel does not support this index type");
  std::vector<QueryParams> params;
  std::vector<uint32_t> seeds;
  uint32_t max_size = 0;
  build_params(args, nargs, nq, kmax, params, seeds, max_size);
  QueryParams* d_params = nullptr;
  uint32_t* d_seeds = nullptr;
  NGT_CUDA(cudaMallocAsync(&d_params, nq * sizeof(QueryParams), stream));
  NGT_CUDA(cudaMallocAsync(&d_seeds, seeds.size() * 4, stream));
  NGT_CUDA(cudaMemcpyAsync(d_params, params.data(), nq * sizeof(QueryParams), cudaMemcpyHostToDevice, stream));
  NGT_CUDA(cudaMemcpyAsync(d_seeds, seeds.data(), seeds.size() * 4, cudaMemcpyHostToDevice, stream));
  if (kernel == Kernel::Wide)
    launch_wide(d_rows, nq, d_params, d_seeds, max_size, d_out, d_counts, d_stats, stream, fast_scratch_[slot]);
  else
    launch_fast(d_rows, nq, d_params, d_seeds, max_size, d_out, d_counts, d_stats, stream, kernel,
                fast_scratch_[slot]);
  NGT_CUDA(cudaFreeAsync(d_params, stream));
  NGT_CUDA(cudaFreeAsync(d_seeds, stream));
  // the pageable host parameter copies above are complete once they return
}

// Shared-memory visited hash of the exact-order kernels (QG included): a query moves
// its visited set to the global bitmap once the hash is half full, which every
// query of a large index does after a few thousand visits, so large indexes get a
// small hash (more CTAs per SM) and small ones a large hash (no bitmap at all).
uint32_t GraphEngine::visited_hash_capacity() const { return host_.nrows >= (1u << 18) ? 2048u : 8192u; }
// Shared-memory tier of the exact-order kernels' candidate queue: 512 keys on large
// indexes (the overflow tier behind it keeps the queue exact; a smaller tier means
// more CTAs per SM: 1M x 128: plain kernel +17 %, QG +18 %, results unchanged).
uint32_t GraphEngine::candidate_list_capacity() const { return host_.nrows >= (1u << 18) ? 512u : 1024u; }

size_t GraphEngine::exact_launch_config(uint32_t max_size, ExactConfig& cfg) const {
  cfg = ExactConfig{};
  cfg.kcap = max_size + 1;
  cfg.ccap = std::max<uint32_t>(candidate_list_capacity(), std::min<uint32_t>(1024, next_pow2(cfg.kcap)));
  cfg.hcap = visited_hash_capacity();
  cfg.mode = (uint32_t)mode_;
  cfg.group = std::min<uint32_t>(32, next_pow2((uint32_t)dev_.row_chunks));
  cfg.bitmap_words = (host_.nrows + 31) / 32;
  cfg.ocap = kOverflowCapacity;
  int max_smem = 0;
  NGT_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, device_));
  size_t smem = exact_smem_bytes(dev_.row_chunks, cfg);
  while (smem > (size_t)max_smem && cfg.hcap > 2048) {
    cfg.hcap >>= 1;
    smem = exact_smem_bytes(dev_.row_chunks, cfg);
  }
  while (smem > (size_t)max_smem && cfg.ccap > 256) {
    cfg.ccap >>= 1;
    smem = exact_smem_bytes(dev_.row_chunks, cfg);
  }
  if (smem > (size_t)max_smem) throw std::runtime_error("result size too large for the on-chip search state");
  return smem;
}

void GraphEngine::launch_exact(const uint4* d_rows, size_t nq, const QueryParams* d_params, const uint32_t* d_seeds,
                               uint32_t max_size, ObjDist* d_out, uint32_t* d_counts, QueryStats* d_stats,
                               cudaStream_t stream, uint32_t* bitmaps, unsigned long long* overflow,
                               size_t grid_cap) {
  ExactConfig cfg;
  const size_t smem = exact_launch_config(max_size, cfg);
  ExactKernelFn fn = exact_kernel(host_.prop.otype, host_.prop.metric);
  NGT_CUDA(cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0, sms = 0;
  NGT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)fn, kExactThreads, smem));
  NGT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
  size_t grid = std::min<size_t>(nq, (size_t)std::max(1, per_sm) * sms);
  if (bitmaps) {
    grid = std::min(grid, grid_cap);
  } else {
    ensure_scratch(grid);
    bitmaps = d_bitmaps_;
    overflow = d_overflow_;
  }
  fn<<<(unsigned)grid, kExactThreads, smem, stream>>>(dev_, d_rows, (uint32_t)nq, d_params, d_seeds, d_out, d_counts,
                                                       d_stats, bitmaps, overflow, cfg);
  NGT_CUDA(cudaGetLastError());
  launches_++;
}

void GraphEngine::launch_wide(const uint4* d_rows, size_t nq, const QueryParams* d_params, const uint32_t* d_seeds,
                              uint32_t max_size, ObjDist* d_out, uint32_t* d_counts, QueryStats* d_stats,
                              cudaStream_t stream, FastScratch& scratch) {
  const SearchRows rows = wide_search_rows();
  const bool bf16 = rows == SearchRows::Bf16, sq8 = rows == SearchRows::Sq8;
  const uint32_t threads = tuning_.cta_threads ? tuning_.cta_threads : 256u;
  WideKernelFn fn = wide_kernel(host_.prop.otype, host_.prop.metric, rows, threads);
  if (!fn) throw std::runtime_error("the wide kernel does not support this index type or CTA size");
  if (bf16) ensure_bf16_rows();
  if (sq8) ensure_sq8_rows();
  WideConfig cfg{};
  // automatic list: 4 x the result size, at least 256, at most 1024 (and never below size + 1)
  uint32_t L = tuning_.list_cap ? next_pow2(tuning_.list_cap)
                                : std::min<uint32_t>(1024, next_pow2(std::max<uint32_t>(256, 4 * max_size)));
  L = std::max<uint32_t>(L, next_pow2(max_size + 1));
  if (L > 1024) throw std::runtime_error("result size too large for the wide kernel (at most 1023)");
  cfg.list_cap = L;
  cfg.parents = tuning_.parents ? std::min<uint32_t>(tuning_.parents, 32) : 8;
  float rf = tuning_.rerank_factor > 0.f ? tuning_.rerank_factor : 2.0f;
  uint32_t rerank_max = std::min<uint32_t>(L, (uint32_t)std::ceil(rf * (float)max_size) + 1);
  cfg.nbr_cap = tuning_.nbr_cap ? std::max<uint32_t>({next_pow2(tuning_.nbr_cap), next_pow2(rerank_max), L})
                                : std::max<uint32_t>({512u, next_pow2(rerank_max), L,
                                                      std::min<uint32_t>(4096, next_pow2(cfg.parents * 100))});
  cfg.search_chunks = bf16 ? dev_.row_chunks / 2 : sq8 ? dev_.row_chunks / 4 : dev_.row_chunks;
  if (sq8) {
    cfg.sq8 = 1;
    cfg.dim = host_.prop.dimension;
    cfg.sq_offset = sq8_offset_;
    cfg.sq_in = 256.f / sq8_scale_;
    cfg.sq_out = sq8_scale_ / 256.f;
  }
  // 64 KB of staged rows by default (two 256-thread CTAs share an SM)
  const uint32_t stage_bytes = (tuning_.stage_kb ? tuning_.stage_kb : 64u) * 1024u;
  cfg.stage_rows = std::max<uint32_t>(16, std::min<uint32_t>(512, stage_bytes / (cfg.search_chunks * 16)));
  // two chunks per lane; one for 8-bit rows (whose unpacked query chunk is 16 floats)
  cfg.sgroup = std::min<uint32_t>(32, next_pow2(sq8 ? cfg.search_chunks : (cfg.search_chunks + 1) / 2));
  cfg.ngroup = std::min<uint32_t>(32, next_pow2(dev_.row_chunks));
  cfg.rerank_x16 = (uint32_t)std::ceil(rf * 16.0f);
  cfg.bitmap_words = ((host_.nrows + 31) / 32 + 3) / 4 * 4;
  cfg.max_iters = 1u << 22;
  cfg.spill_cap = kSpillCapacity;
  // default: visited bitmaps kept in L2, staged rows streamed through it
  cfg.l2_policy = tuning_.l2_policy ? tuning_.l2_policy - 1 : 2u;
  // rows_in_flight: rows per lane group scored at once (1, 2 or 4; default 4)
  cfg.score_rows = tuning_.rows_in_flight ? std::min<uint32_t>(tuning_.rows_in_flight, 4) : 4u;
  size_t smem = wide_kernel_smem_bytes(dev_.row_chunks, cfg);
  int max_smem = 0, per_sm = 0, sms = 0;
  NGT_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, device_));
  while (smem > (size_t)max_smem && cfg.stage_rows > 16) {
    cfg.stage_rows /= 2;
    smem = wide_kernel_smem_bytes(dev_.row_chunks, cfg);
  }
  if (smem > (size_t)max_smem) throw std::runtime_error("wide search state does not fit in shared memory");
  NGT_CUDA(cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  NGT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)fn, (int)threads, smem));
  NGT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
  size_t grid = std::min<size_t>(nq, (size_t)std::max(1, per_sm) * sms);
  ensure_fast_scratch(scratch, grid, stream);
  NGT_CUDA(cudaMemsetAsync(scratch.work, 0, 4, stream));
  const uint4* srows = bf16 ? static_cast<const uint4*>(d_bf16_) : sq8 ? static_cast<const uint4*>(d_sq8_)
                                                                       : dev_.objects;
  fn<<<(unsigned)grid, threads, smem, stream>>>(dev_, srows, d_rows, (uint32_t)nq, d_params, d_seeds, d_out,
                                                d_counts, d_stats, scratch.bitmaps, scratch.work, scratch.spill, cfg);
  NGT_CUDA(cudaGetLastError());
  launches_++;
}

void GraphEngine::launch_fast(const uint4* d_rows, size_t nq, const QueryParams* d_params, const uint32_t* d_seeds,
                              uint32_t max_size, ObjDist* d_out, uint32_t* d_counts, QueryStats* d_stats,
                              cudaStream_t stream, Kernel kernel, FastScratch& scratch) {
  // hyperbolic metrics search on the fp32 rows: acosh near 1 magnifies bf16 rounding
  // of the coordinates far beyond what the exact re-rank of a few candidates can repair
  const bool hyperbolic = host_.prop.metric == Metric::Poincare || host_.prop.metric == Metric::Lorentz;
  const bool bf16 = kernel == Kernel::Fast && host_.prop.otype == ObjType::Float && !hyperbolic;
  FastKernelFn fn = fast_kernel(host_.prop.otype, host_.prop.metric, bf16, tuning_.rows_in_flight,
                                tuning_.ctas_per_sm);
  if (!fn) throw std::runtime_error("the batched kernel does not support this index type or tuning");
  if (bf16) ensure_bf16_rows();
  FastConfig cfg{};
  // automatic list: 4 x the result size, at least 512, at most 1024 (and never below size + 1)
  uint32_t L = tuning_.list_cap ? next_pow2(tuning_.list_cap)
                                : std::min<uint32_t>(1024, next_pow2(std::max<uint32_t>(512, 4 * max_size)));
  L = std::max<uint32_t>(L, next_pow2(max_size + 1));
  if (L > 1024) throw std::runtime_error("result size too large for the batched kernel (at most 1023)");
  cfg.list_cap = L;
  // neighbour buffer: P parents' edges per iteration, and the re-rank set (sorted in place)
  cfg.parents = tuning_.parents ? std::min<uint32_t>(tuning_.parents, 16) : 4;
  float rf0 = tuning_.rerank_factor > 0.f ? tuning_.rerank_factor : 2.0f;
  uint32_t rerank_max = std::min<uint32_t>(L, (uint32_t)std::ceil(rf0 * (float)max_size) + 1);
  cfg.nbr_cap = tuning_.nbr_cap ? std::max<uint32_t>({next_pow2(tuning_.nbr_cap), next_pow2(rerank_max), L})
                                : std::max<uint32_t>({512u, next_pow2(rerank_max), L, next_pow2(cfg.parents * 128)});
  // nd doubles as the 256-bin refill histogram
  cfg.nbr_cap = std::max<uint32_t>(cfg.nbr_cap, 256u);
  cfg.search_chunks = bf16 ? dev_.row_chunks / 2 : dev_.row_chunks;
  cfg.sgroup = std::min<uint32_t>(32, next_pow2((cfg.search_chunks + 1) / 2));   // two chunks per lane
  cfg.ngroup = std::min<uint32_t>(32, next_pow2(dev_.row_chunks));
  float rf = tuning_.rerank_factor > 0.f ? tuning_.rerank_factor : 2.0f;
  cfg.rerank_x16 = (uint32_t)std::ceil(rf * 16.0f);
  cfg.bitmap_words = ((host_.nrows + 31) / 32 + 3) / 4 * 4;
  cfg.max_iters = 1u << 22;
  cfg.spill_cap = kSpillCapacity;
  size_t smem = kFastWarps * fast_smem_per_warp(dev_.row_chunks, cfg);
  int max_smem = 0, per_sm = 0, sms = 0;
  NGT_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, device_));
  if (smem > (size_t)max_smem) throw std::runtime_error("batched search state does not fit in shared memory");
  NGT_CUDA(cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  NGT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)fn, kFastThreads, smem));
  NGT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
  size_t grid = std::min<size_t>((nq + kFastWarps - 1) / kFastWarps, (size_t)std::max(1, per_sm) * sms);
  ensure_fast_scratch(scratch, grid * kFastWarps, stream);
  NGT_CUDA(cudaMemsetAsync(scratch.work, 0, 4, stream));
  const uint4* srows = bf16 ? static_cast<const uint4*>(d_bf16_) : dev_.objects;
  fn<<<(unsigned)grid, kFastThreads, smem, stream>>>(dev_, srows, d_rows, (uint32_t)nq, d_params, d_seeds, d_out,
                                                      d_counts, d_stats, scratch.bitmaps, scratch.work,
                                                      scratch.spill, cfg);
  NGT_CUDA(cudaGetLastError());
  launches_++;
}

void GraphEngine::search(const void* queries, QueryType qt, size_t nq, size_t qdim, const SearchArgs* args,
                         size_t nargs, SearchOutput& out, Kernel kernel) {
  NGT_CUDA(cudaSetDevice(device_));
  bool refine = false;
  for (size_t i = 0; i < nargs; i++) refine = refine || args[i].refinement_expansion >= 1.0f;
  if (refine) {
    search_refined(queries, qt, nq, qdim, args, nargs, out, kernel);
    return;
  }
  std::lock_guard<std::mutex> staging(staging_mu_);
  // the query rows are converted straight into a pinned staging buffer (kept between calls)
  const size_t row_total = nq * host_.row_bytes();
  if (staging_bytes_ < row_total) {
    if (staging_) NGT_CUDA(cudaFreeHost(staging_));
    staging_ = nullptr;
    staging_bytes_ = 0;
    NGT_CUDA(cudaMallocHost(&staging_, std::max<size_t>(row_total, 1)));
    staging_bytes_ = std::max<size_t>(row_total, 1);
  }
  convert_queries(queries, qt, nq, qdim, static_cast<uint8_t*>(staging_));
  size_t kmax = 1;
  for (size_t i = 0; i < nargs; i++) kmax = std::max(kmax, output_size(args[i]));
  out.kmax = kmax;
  out.results.assign(nq * kmax, ObjDist{0, 0.f});
  out.counts.assign(nq, 0);
  out.stats.assign(nq, QueryStats{});
  if (nq == 0) return;
  uint4* d_rows = nullptr;
  ObjDist* d_out = nullptr;
  uint32_t* d_counts = nullptr;
  QueryStats* d_stats = nullptr;
  cudaStream_t s = stream_;
  NGT_CUDA(cudaMallocAsync(&d_rows, row_total, s));
  NGT_CUDA(cudaMallocAsync(&d_out, nq * kmax * sizeof(ObjDist), s));
  NGT_CUDA(cudaMallocAsync(&d_counts, nq * 4, s));
  NGT_CUDA(cudaMallocAsync(&d_stats, nq * sizeof(QueryStats), s));
  NGT_CUDA(cudaMemcpyAsync(d_rows, staging_, row_total, cudaMemcpyHostToDevice, s));
  search_device(d_rows, nq, args, nargs, d_out, d_counts, d_stats, kmax, s, kernel);
  NGT_CUDA(cudaMemcpyAsync(out.results.data(), d_out, nq * kmax * sizeof(ObjDist), cudaMemcpyDeviceToHost, s));
  NGT_CUDA(cudaMemcpyAsync(out.counts.data(), d_counts, nq * 4, cudaMemcpyDeviceToHost, s));
  NGT_CUDA(cudaMemcpyAsync(out.stats.data(), d_stats, nq * sizeof(QueryStats), cudaMemcpyDeviceToHost, s));
  NGT_CUDA(cudaFreeAsync(d_rows, s));
  NGT_CUDA(cudaFreeAsync(d_out, s));
  NGT_CUDA(cudaFreeAsync(d_counts, s));
  NGT_CUDA(cudaFreeAsync(d_stats, s));
  NGT_CUDA(cudaStreamSynchronize(s));
}

void GraphEngine::linear_search_tc_host(const float* queries, size_t nq, size_t qdim, size_t size,
                                        size_t candidates, ObjDist* results, size_t kmax, uint32_t* counts,
                                        uint32_t* status, bool fp8, bool fp64_ties, bool pair) {
  NGT_CUDA(cudaSetDevice(device_));
  if (nq == 0) return;
  std::lock_guard<std::mutex> staging(staging_mu_);
  const size_t row_total = nq * host_.row_bytes();
  if (staging_bytes_ < row_total) {
    if (staging_) NGT_CUDA(cudaFreeHost(staging_));
    staging_ = nullptr;
    staging_bytes_ = 0;
    NGT_CUDA(cudaMallocHost(&staging_, row_total));
    staging_bytes_ = row_total;
  }
  convert_queries(queries, QueryType::Float32, nq, qdim, static_cast<uint8_t*>(staging_));
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t o_out = al(row_total), o_cnt = o_out + al(nq * kmax * sizeof(ObjDist));
  const size_t o_st = o_cnt + al(nq * 4), total = o_st + al(nq * 4);
  cudaStream_t s = stream_;
  uint8_t* d = nullptr;
  NGT_CUDA(cudaMallocAsync(&d, total, s));
  try {
    NGT_CUDA(cudaMemcpyAsync(d, staging_, row_total, cudaMemcpyHostToDevice, s));
    linear_search_tc_device(reinterpret_cast<const uint4*>(d), nq, size, candidates,
                            reinterpret_cast<ObjDist*>(d + o_out), kmax, reinterpret_cast<uint32_t*>(d + o_cnt),
                            reinterpret_cast<uint32_t*>(d + o_st), s, fp8, fp64_ties, pair);
    NGT_CUDA(cudaMemcpyAsync(results, d + o_out, nq * kmax * sizeof(ObjDist), cudaMemcpyDeviceToHost, s));
    NGT_CUDA(cudaMemcpyAsync(counts, d + o_cnt, nq * 4, cudaMemcpyDeviceToHost, s));
    NGT_CUDA(cudaMemcpyAsync(status, d + o_st, nq * 4, cudaMemcpyDeviceToHost, s));
  } catch (...) {
    cudaFreeAsync(d, s);
    cudaStreamSynchronize(s);
    throw;
  }
  NGT_CUDA(cudaFreeAsync(d, s));
  NGT_CUDA(cudaStreamSynchronize(s));
}

void GraphEngine::search_refined(const void* queries, QueryType qt, size_t nq, size_t qdim, const SearchArgs* args,
                                 size_t nargs, SearchOutput& out, Kernel kernel) {
  // GraphIndex::search(SearchQuery&) with a refinement expansion (lib/NGT/Index.h:1146-1236):
  // the search keeps size x expansion results, whose exact distances over the float
  // refinement objects (the comparator of the index's distance) order them, and the size
  // best by (distance, id) are returned
  if (host_.robj_rows == 0) throw std::runtime_error("the index has no refinement objects (robj)");
  if (qt != QueryType::Float32 || qdim != (size_t)host_.prop.dimension)
    throw std::runtime_error("a refined search takes float queries of the index dimension");
  QBGRefineKernelFn rf = graph_refine_kernel_for(host_.prop.metric);
  if (!rf) throw std::runtime_error("the refinement supports the L1, L2, angle and cosine distances");
  std::vector<SearchArgs> exp(nargs);
  std::vector<uint32_t> exact(nq);
  uint32_t max_search = 1;
  for (size_t i = 0; i < nargs; i++) {
    if (args[i].refinement_expansion < 1.0f)
      throw std::runtime_error("refined and unrefined queries in one call");
    exp[i] = args[i];
    exp[i].size = (size_t)((float)args[i].size * args[i].refinement_expansion);
    exp[i].refinement_expansion = 0.0f;
    max_search = std::max<uint32_t>(max_search, (uint32_t)output_size(exp[i]));
  }
  if (max_search > 4096) throw std::runtime_error("size x refinement expansion above 4096");
  size_t kmax = 1;
  for (size_t q = 0; q < nq; q++) {
    exact[q] = (uint32_t)args[nargs == 1 ? 0 : q].size;
    kmax = std::max<size_t>(kmax, exact[q]);
  }
  SearchOutput cand;
  search(queries, qt, nq, qdim, exp.data(), nargs, cand, kernel);
  {
    std::lock_guard<std::mutex> lock(mu_);
    if (!d_robj_) d_robj_ = dmalloc_copy<void>(host_.robj.data(), host_.robj.size() * 4);
  }
  cudaStream_t s = stream_;
  ObjDist *d_cand = nullptr, *d_out = nullptr;
  uint32_t *d_cc = nullptr, *d_exact = nullptr, *d_counts = nullptr;
  float* d_q = nullptr;
  NGT_CUDA(cudaMallocAsync(&d_cand, cand.results.size() * sizeof(ObjDist), s));
  NGT_CUDA(cudaMallocAsync(&d_cc, nq * 4, s));
  NGT_CUDA(cudaMallocAsync(&d_exact, nq * 4, s));
  NGT_CUDA(cudaMallocAsync(&d_q, nq * qdim * 4, s));
  NGT_CUDA(cudaMallocAsync(&d_out, nq * kmax * sizeof(ObjDist), s));
  NGT_CUDA(cudaMallocAsync(&d_counts, nq * 4, s));
  NGT_CUDA(cudaMemcpyAsync(d_cand, cand.results.data(), cand.results.size() * sizeof(ObjDist),
                           cudaMemcpyHostToDevice, s));
  NGT_CUDA(cudaMemcpyAsync(d_cc, cand.counts.data(), nq * 4, cudaMemcpyHostToDevice, s));
  NGT_CUDA(cudaMemcpyAsync(d_exact, exact.data(), nq * 4, cudaMemcpyHostToDevice, s));
  NGT_CUDA(cudaMemcpyAsync(d_q, queries, nq * qdim * 4, cudaMemcpyHostToDevice, s));
  int sms = 0;
  NGT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
  const uint32_t P = next_pow2(std::max<uint32_t>((uint32_t)cand.kmax, 2));
  const uint32_t rchunks = host_.rdim_pad / 4;
  const size_t smem = (size_t)rchunks * 16 + (size_t)P * 8;
  NGT_CUDA(cudaFuncSetAttribute((const void*)rf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  rf<<<(unsigned)std::min<size_t>(nq, (size_t)sms * 8), 256, smem, s>>>(
      d_cand, d_cc, (uint32_t)cand.kmax, d_q, (uint32_t)qdim, static_cast<const uint4*>(d_robj_), rchunks,
      (uint32_t)host_.prop.dimension, host_.robj_rows, d_exact, (uint32_t)nq, P, d_out, (uint32_t)kmax, d_counts);
  NGT_CUDA(cudaGetLastError());
  launches_++;
  out.kmax = kmax;
  out.results.assign(nq * kmax, ObjDist{0, 0.f});
  out.counts.assign(nq, 0);
  out.stats = cand.stats;
  NGT_CUDA(cudaMemcpyAsync(out.results.data(), d_out, nq * kmax * sizeof(ObjDist), cudaMemcpyDeviceToHost, s));
  NGT_CUDA(cudaMemcpyAsync(out.counts.data(), d_counts, nq * 4, cudaMemcpyDeviceToHost, s));
  for (void* p : {(void*)d_cand, (void*)d_cc, (void*)d_exact, (void*)d_q, (void*)d_out, (void*)d_counts})
    NGT_CUDA(cudaFreeAsync(p, s));
  NGT_CUDA(cudaStreamSynchronize(s));
}

void GraphEngine::search_one(const void* query, QueryType qt, size_t qdim, const SearchArgs& args,
                             SearchOutput& out) {
  auto call = std::make_shared<CoalescedCall>();
  convert_queries(query, qt, 1, qdim, call->row);
  call->args = args;
  (void)output_size(args);
  std::unique_lock<std::mutex> lock(co_mu_);
  co_pending_.push_back(call);
  while (!call->done) {
    CoLane* lane = nullptr;
    if (!co_pending_.empty())
      for (size_t i = 0; i < co_nlanes_; i++)
        if (!co_lanes_[i].busy) {
          lane = &co_lanes_[i];
          break;
        }
    if (lane) {
      // a free lane: this caller launches everything waiting (its own query, unless a
      // caller before it took that one already)
      lane->busy = true;
      std::vector<std::shared_ptr<CoalescedCall>> batch;
      batch.swap(co_pending_);
      lock.unlock();
      std::string err;
      try {
        run_coalesced(batch, *lane);
      } catch (std::exception& ex) {
        err = ex.what();
      }
      lock.lock();
      for (auto& c : batch) {
        c->error = err;
        c->done = true;
      }
      lane->busy = false;
      co_cv_.notify_all();
    } else {
      co_cv_.wait(lock);
    }
  }
  lock.unlock();
  if (!call->error.empty()) throw std::runtime_error(call->error);
  out = std::move(call->out);
}

void GraphEngine::run_coalesced(std::vector<std::shared_ptr<CoalescedCall>>& batch, CoLane& lane) {
  // Every copy goes between the lane's pinned block and its device block (one upload
  // of rows + parameters + seeds, one download of results + counts + statistics), so
  // the lanes' launches and copies overlap; pageable copies would serialize them.
  NGT_CUDA(cudaSetDevice(device_));
  const size_t nq = batch.size(), rb = host_.row_bytes();
  const size_t words = (host_.nrows + 31) / 32;
  if (!lane.stream) {
    NGT_CUDA(cudaStreamCreateWithFlags(&lane.stream, cudaStreamNonBlocking));
    NGT_CUDA(cudaMalloc(&lane.bitmaps, kLaneCtas * words * 4));
    NGT_CUDA(cudaMemsetAsync(lane.bitmaps, 0, kLaneCtas * words * 4, lane.stream));
    NGT_CUDA(cudaMalloc(&lane.overflow, kLaneCtas * 2 * (size_t)kOverflowCapacity * 8));
  }
  std::vector<SearchArgs> args(nq);
  size_t kmax = 1;
  for (size_t i = 0; i < nq; i++) {
    args[i] = batch[i]->args;
    kmax = std::max(kmax, output_size(args[i]));
  }
  std::vector<QueryParams> params;
  std::vector<uint32_t> seeds;
  uint32_t max_size = 0;
  {
    // the parameters may create a seed table (engine state shared with every lane)
    std::lock_guard<std::mutex> lock(mu_);
    build_params(args.data(), nq, nq, kmax, params, seeds, max_size);
  }
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t o_par = al(nq * rb), o_seed = o_par + al(nq * sizeof(QueryParams));
  const size_t o_out = o_seed + al(seeds.size() * 4), o_cnt = o_out + al(nq * kmax * sizeof(ObjDist));
  const size_t o_st = o_cnt + al(nq * 4), total = o_st + al(nq * sizeof(QueryStats));
  if (lane.staging_bytes < total) {
    if (lane.staging) NGT_CUDA(cudaFreeHost(lane.staging));
    if (lane.dev) NGT_CUDA(cudaFree(lane.dev));
    lane.staging = nullptr;
    lane.dev = nullptr;
    lane.staging_bytes = 0;
    const size_t bytes = std::max<size_t>(total, 64 << 10);
    NGT_CUDA(cudaMallocHost(&lane.staging, bytes));
    NGT_CUDA(cudaMalloc(&lane.dev, bytes));
    lane.staging_bytes = bytes;
  }
  uint8_t* h = static_cast<uint8_t*>(lane.staging);
  uint8_t* d = static_cast<uint8_t*>(lane.dev);
  for (size_t i = 0; i < nq; i++) std::memcpy(h + i * rb, batch[i]->row.data(), rb);
  std::memcpy(h + o_par, params.data(), nq * sizeof(QueryParams));
  std::memcpy(h + o_seed, seeds.data(), seeds.size() * 4);
  cudaStream_t s = lane.stream;
  NGT_CUDA(cudaMemcpyAsync(d, h, o_out, cudaMemcpyHostToDevice, s));
  {
    std::lock_guard<std::mutex> lock(mu_);
    launch_exact(reinterpret_cast<const uint4*>(d), nq, reinterpret_cast<const QueryParams*>(d + o_par),
                 reinterpret_cast<const uint32_t*>(d + o_seed), max_size, reinterpret_cast<ObjDist*>(d + o_out),
                 reinterpret_cast<uint32_t*>(d + o_cnt), reinterpret_cast<QueryStats*>(d + o_st), s, lane.bitmaps,
                 lane.overflow, kLaneCtas);
  }
  NGT_CUDA(cudaMemcpyAsync(h + o_out, d + o_out, total - o_out, cudaMemcpyDeviceToHost, s));
  NGT_CUDA(cudaStreamSynchronize(s));
  co_queries_ += nq;
  co_launches_++;
  const ObjDist* res = reinterpret_cast<const ObjDist*>(h + o_out);
  const uint32_t* counts = reinterpret_cast<const uint32_t*>(h + o_cnt);
  const QueryStats* stats = reinterpret_cast<const QueryStats*>(h + o_st);
  for (size_t i = 0; i < nq; i++) {
    SearchOutput& o = batch[i]->out;
    o.kmax = kmax;
    o.results.assign(res + i * kmax, res + (i + 1) * kmax);
    o.counts.assign(1, counts[i]);
    o.stats.assign(1, stats[i]);
  }
}

void GraphEngine::linear_search(const void* queries, QueryType qt, size_t nq, size_t qdim, size_t size,
                                SearchOutput& out) {
  std::lock_guard<std::mutex> lock(mu_);
  NGT_CUDA(cudaSetDevice(device_));
  std::vector<uint8_t> rows;
  convert_queries(queries, qt, nq, qdim, rows);
  size = std::min<size_t>(size, host_.nrows ? host_.nrows - 1 : 0);   // never more results than objects
  size_t kmax = std::max<size_t>(size, 1);
  out.kmax = kmax;
  out.results.assign(nq * kmax, ObjDist{0, 0.f});
  out.counts.assign(nq, 0);
  out.stats.assign(nq, QueryStats{});
  if (nq == 0 || size == 0) return;
  if (size > 12288) throw std::runtime_error("linear search supports at most 12288 results per query");
  LinearKernelFn fn = linear_kernel(host_.prop.otype, host_.prop.metric);
  if (!fn) throw std::runtime_error("unsupported distance for linear search");
  cudaStream_t s = stream_;
  const uint32_t rc = dev_.row_chunks;
  const size_t nrows = host_.nrows;
  size_t qb = std::max<size_t>(1, std::min<size_t>({nq, (size_t)(1u << 28) / nrows, (size_t)65535}));
  uint4* d_rows = nullptr;
  float* d_dist = nullptr;
  ObjDist* d_out = nullptr;
  uint32_t* d_counts = nullptr;
  NGT_CUDA(cudaMallocAsync(&d_rows, rows.size(), s));
  NGT_CUDA(cudaMallocAsync(&d_dist, qb * nrows * 4, s));
  NGT_CUDA(cudaMallocAsync(&d_out, nq * kmax * sizeof(ObjDist), s));
  NGT_CUDA(cudaMallocAsync(&d_counts, nq * 4, s));
  NGT_CUDA(cudaMemcpyAsync(d_rows, rows.data(), rows.size(), cudaMemcpyHostToDevice, s));
  const uint32_t group = std::min<uint32_t>(32, next_pow2(rc));
  const size_t sel_smem = (256 + 16) * 4 + 2 * kmax * 8;
  NGT_CUDA(cudaFuncSetAttribute((const void*)linear_select_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)sel_smem));
  for (size_t q0 = 0; q0 < nq; q0 += qb) {
    size_t nb = std::min(qb, nq - q0);
    dim3 grid((unsigned)((nrows + kLinRowsPerBlock - 1) / kLinRowsPerBlock), (unsigned)nb);
    fn<<<grid, kLinThreads, rc * 16, s>>>(dev_, d_rows, (uint32_t)q0, (uint32_t)nb, d_present_, d_dist, group);
    NGT_CUDA(cudaGetLastError());
    linear_select_kernel<<<(unsigned)nb, 512, sel_smem, s>>>(d_dist, (uint32_t)nrows, (uint32_t)q0, (uint32_t)nb,
                                                               (uint32_t)size, FLT_MAX, d_out, d_counts);
    NGT_CUDA(cudaGetLastError());
    launches_ += 2;
  }
  NGT_CUDA(cudaMemcpyAsync(out.results.data(), d_out, nq * kmax * sizeof(ObjDist), cudaMemcpyDeviceToHost, s));
  NGT_CUDA(cudaMemcpyAsync(out.counts.data(), d_counts, nq * 4, cudaMemcpyDeviceToHost, s));
  NGT_CUDA(cudaFreeAsync(d_rows, s));
  NGT_CUDA(cudaFreeAsync(d_dist, s));
  NGT_CUDA(cudaFreeAsync(d_out, s));
  NGT_CUDA(cudaFreeAsync(d_counts, s));
  NGT_CUDA(cudaStreamSynchronize(s));
}

}  // namespace ngtg

namespace ngtg {

void GraphEngine::search_device_noalloc(void* scratch, size_t scratch_bytes, const uint4* d_rows, size_t nq,
                                        const SearchArgs* args, size_t nargs, ObjDist* d_out, uint32_t* d_counts,
                                        QueryStats* d_stats, size_t kmax, cudaStream_t stream) {
  std::lock_guard<std::mutex> lock(mu_);
  NGT_CUDA(cudaSetDevice(device_));
  if (nq == 0) return;
  const Property& p = host_.prop;
  // every seed table the queries need must exist already (building one allocates)
  if (p.has_tree) {
    for (size_t i = 0; i < nargs; i++) {
      const SearchArgs& a = args[i];
      float coef = a.epsilon + 1.0f;
      if (coef == 0.0f) coef = 1.1f;
      size_t ss = p.seed_size == 0 ? a.size : (size_t)p.seed_size;
      if (ss > a.size) ss = a.size;
      if (p.seed_type == 4) ss = SIZE_MAX;
      if (ss == 0) ss = 1;
      if (!seed_tables_.count(ss))
        throw std::runtime_error("no seed table for result size " + std::to_string(a.size) +
                                 " yet: run one regular search with this result size on the index first");
    }
  }
  std::vector<QueryParams> params;
  std::vector<uint32_t> seeds;
  uint32_t max_size = 0;
  build_params(args, nargs, nq, kmax, params, seeds, max_size);
  ExactConfig cfg;
  const size_t smem = exact_launch_config(max_size, cfg);
  // scratch layout: params | seeds | bitmaps[grid] | overflow[grid], each 256-byte aligned
  auto up = [](size_t v) { return (v + 255) & ~(size_t)255; };
  const size_t params_bytes = up(nq * sizeof(QueryParams));
  const size_t seeds_bytes = up(seeds.size() * 4);
  const size_t bitmap_bytes = up((size_t)cfg.bitmap_words * 4);
  const size_t overflow_bytes = (size_t)2 * cfg.ocap * 8;
  const size_t per_cta = bitmap_bytes + overflow_bytes;
  const size_t fixed = params_bytes + seeds_bytes;
  if (fixed + per_cta > scratch_bytes) {
    std::ostringstream m;
    m << "the no-allocation search needs " << fixed + per_cta << " bytes of scratch for " << nq
      << " queries on this index, more than its fixed " << scratch_bytes << "-byte scratch; use fewer queries per call";
    throw std::runtime_error(m.str());
  }
  ExactKernelFn fn = exact_kernel(host_.prop.otype, host_.prop.metric);
  NGT_CUDA(cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0, sms = 0;
  NGT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)fn, kExactThreads, smem));
  NGT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
  size_t grid = std::min<size_t>({nq, (size_t)std::max(1, per_sm) * sms, (scratch_bytes - fixed) / per_cta});
  unsigned char* base = static_cast<unsigned char*>(scratch);
  QueryParams* d_params = reinterpret_cast<QueryParams*>(base);
  uint32_t* d_seeds = reinterpret_cast<uint32_t*>(base + params_bytes);
  uint32_t* d_bitmaps = reinterpret_cast<uint32_t*>(base + fixed);
  unsigned long long* d_overflow = reinterpret_cast<unsigned long long*>(base + fixed + grid * bitmap_bytes);
  NGT_CUDA(cudaMemcpyAsync(d_params, params.data(), nq * sizeof(QueryParams), cudaMemcpyHostToDevice, stream));
  NGT_CUDA(cudaMemcpyAsync(d_seeds, seeds.data(), seeds.size() * 4, cudaMemcpyHostToDevice, stream));
  NGT_CUDA(cudaMemsetAsync(d_bitmaps, 0, grid * bitmap_bytes, stream));   // the kernel expects clear bitmaps
  cfg.bitmap_words = (uint32_t)(bitmap_bytes / 4);
  fn<<<(unsigned)grid, kExactThreads, smem, stream>>>(dev_, d_rows, (uint32_t)nq, d_params, d_seeds, d_out, d_counts,
                                                       d_stats, d_bitmaps, d_overflow, cfg);
  NGT_CUDA(cudaGetLastError());
  // the host parameter vectors must outlive the copies above
  NGT_CUDA(cudaStreamSynchronize(stream));
  launches_++;
}

// ---- quantized graph --------------------------------------------------------

void GraphEngine::read_qg() {
  if (host_.prop.otype != ObjType::Float || host_.prop.metric != Metric::L2)
    throw std::runtime_error("the quantized graph search supports float objects with the L2 distance only");
  load_qg(host_.path, host_.nrows, qg_);
  if (!qg_kernel(qg_.m)) throw std::runtime_error("too many subspaces in the quantized graph");
}

void GraphEngine::upload_qg() {
  NGT_CUDA(cudaSetDevice(device_));
  auto up = [&](const void* src, size_t bytes) {
    void* p = dmalloc_copy<void>(src, bytes);
    qg_buffers_.push_back(p);
    return p;
  };
  dqg_.rotation = qg_.rotation.empty() ? nullptr
                                       : static_cast<const float*>(up(qg_.rotation.data(), qg_.rotation.size() * 4));
  dqg_.gcentroid = static_cast<const float*>(up(qg_.gcentroid.data(), qg_.gcentroid.size() * 4));
  dqg_.lcentroids = static_cast<const float*>(up(qg_.lcentroids.data(), qg_.lcentroids.size() * 4));
  dqg_.offsets = static_cast<const uint32_t*>(up(qg_.offsets.data(), qg_.offsets.size() * 4));
  dqg_.ids = static_cast<const uint32_t*>(up(qg_.ids.data(), qg_.ids.size() * 4));
  dqg_.code_off16 = static_cast<const uint32_t*>(up(qg_.code_off16.data(), qg_.code_off16.size() * 4));
  dqg_.codes = static_cast<const uint8_t*>(up(qg_.codes.data(), qg_.codes.size()));
  dqg_.dim = qg_.dim;
  dqg_.m = qg_.m;
  dqg_.ld = qg_.ld;
  dqg_.ma = qg_.ma;
  dqg_.nnodes = qg_.nnodes;
  qg_loaded_ = true;
}

void GraphEngine::open_qg() {
  std::lock_guard<std::mutex> lock(mu_);
  if (qg_loaded_) return;
  read_qg();
  upload_qg();
}

void GraphEngine::qg_search_device(const uint4* d_rows, size_t nq, const QGArgs* args, size_t nargs,
                                   ObjDist* d_out, uint32_t* d_counts, QueryStats* d_stats, size_t kmax,
                                   cudaStream_t stream, uint32_t* bitmaps, unsigned long long* overflow,
                                   size_t grid_cap) {
  if (!qg_loaded_) open_qg();
  std::lock_guard<std::mutex> lock(mu_);
  NGT_CUDA(cudaSetDevice(device_));
  if (nq == 0) return;
  // ngtqg_search_index_ / NGTQG::Index::search (lib/NGT/NGTQ/Capi.cpp:81-127,
  // lib/NGT/NGTQ/QuantizedGraph.h:283-296,449-497)
  std::vector<QGParams> params(nq);
  std::vector<uint32_t> seeds;
  uint32_t max_size = 1;
  for (size_t i = 0; i < nq; i++) {
    const QGArgs& a = args[nargs == 1 ? 0 : i];
    if (a.size > kmax) throw std::runtime_error("result size larger than the output capacity");
    QGParams qp{};
    float coef = a.epsilon + 1.0f;
    if (coef == 0.0f) coef = 1.1f;
    size_t size = a.size;
    if (a.result_expansion > 1.0f) size = (size_t)((float)a.size * a.result_expansion);
    qp.size = (uint32_t)std::min<size_t>(size, 0xffffffffu);
    qp.k = (uint32_t)a.size;
    qp.radius = a.radius < 0.0f ? FLT_MAX : a.radius;
    qp.coef = coef;
    qp.rerank = a.result_expansion >= 1.0f ? 1u : 0u;
    qp.out_off = (uint32_t)(i * kmax);
    if (a.size > 0) seed_params(a.size, qp.seed_off, qp.seed_cnt, seeds);
    params[i] = qp;
    max_size = std::max<uint32_t>(max_size, qp.size);
  }
  if (seeds.empty()) seeds.push_back(0);
  ExactConfig cfg{};
  cfg.kcap = max_size + 1;
  cfg.ccap = std::max<uint32_t>(candidate_list_capacity(), std::min<uint32_t>(1024, next_pow2(cfg.kcap)));
  cfg.hcap = visited_hash_capacity();
  cfg.mode = (uint32_t)GraphMode::Updatable;
  cfg.group = std::min<uint32_t>(32, next_pow2((uint32_t)dev_.row_chunks));
  cfg.bitmap_words = (host_.nrows + 31) / 32;
  cfg.ocap = kOverflowCapacity;
  if (cfg.kcap > cfg.ccap) throw std::runtime_error("size x result expansion too large for the quantized graph search");
  int max_smem = 0;
  NGT_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, device_));
  size_t smem = qg_kernel_smem_bytes(dev_.row_chunks, qg_.dim, qg_.m, cfg);
  while (smem > (size_t)max_smem && cfg.hcap > 2048) {
    cfg.hcap >>= 1;
    smem = qg_kernel_smem_bytes(dev_.row_chunks, qg_.dim, qg_.m, cfg);
  }
  if (smem > (size_t)max_smem) throw std::runtime_error("quantized graph search state does not fit in shared memory");
  QGKernelFn fn = qg_kernel(qg_.m);
  NGT_CUDA(cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0, sms = 0;
  NGT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)fn, kExactThreads, smem));
  NGT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
  size_t grid = std::min<size_t>(nq, (size_t)std::max(1, per_sm) * sms);
  if (bitmaps) {
    grid = std::min(grid, grid_cap);
  } else {
    ensure_scratch(grid);
    bitmaps = d_bitmaps_;
    overflow = d_overflow_;
  }
  QGParams* d_params = nullptr;
  uint32_t* d_seeds = nullptr;
  NGT_CUDA(cudaMallocAsync(&d_params, nq * sizeof(QGParams), stream));
  NGT_CUDA(cudaMallocAsync(&d_seeds, seeds.size() * 4, stream));
  NGT_CUDA(cudaMemcpyAsync(d_params, params.data(), nq * sizeof(QGParams), cudaMemcpyHostToDevice, stream));
  NGT_CUDA(cudaMemcpyAsync(d_seeds, seeds.data(), seeds.size() * 4, cudaMemcpyHostToDevice, stream));
  fn<<<(unsigned)grid, kExactThreads, smem, stream>>>(dev_, dqg_, d_rows, (uint32_t)nq, d_params, d_seeds, d_out,
                                                       d_counts, d_stats, bitmaps, overflow, cfg);
  NGT_CUDA(cudaGetLastError());
  launches_++;
  NGT_CUDA(cudaFreeAsync(d_params, stream));
  NGT_CUDA(cudaFreeAsync(d_seeds, stream));
  // the pageable host parameter copies above are complete once they return
}

void GraphEngine::qg_search_device_relaxed(const uint4* d_rows, size_t nq, const QGArgs* args, size_t nargs,
                                           ObjDist* d_out, uint32_t* d_counts, QueryStats* d_stats, size_t kmax,
                                           cudaStream_t stream, size_t slot) {
  if (!qg_loaded_) open_qg();
  std::lock_guard<std::mutex> lock(mu_);
  NGT_CUDA(cudaSetDevice(device_));
  if (nq == 0) return;
  if (slot >= fast_scratch_.size()) throw std::runtime_error("invalid scratch set");
  std::vector<QGParams> params(nq);
  std::vector<uint32_t> seeds;
  uint32_t max_size = 1;
  for (size_t i = 0; i < nq; i++) {
    const QGArgs& a = args[nargs == 1 ? 0 : i];
    if (a.size > kmax) throw std::runtime_error("result size larger than the output capacity");
    QGParams qp{};
    float coef = a.epsilon + 1.0f;
    if (coef == 0.0f) coef = 1.1f;
    size_t size = a.size;
    if (a.result_expansion > 1.0f) size = (size_t)((float)a.size * a.result_expansion);
    qp.size = (uint32_t)std::min<size_t>(size, 0xffffffffu);
    qp.k = (uint32_t)a.size;
    qp.radius = a.radius < 0.0f ? FLT_MAX : a.radius;
    qp.coef = coef;
    qp.rerank = a.result_expansion >= 1.0f ? 1u : 0u;
    qp.out_off = (uint32_t)(i * kmax);
    if (a.size > 0) seed_params(a.size, qp.seed_off, qp.seed_cnt, seeds);
    params[i] = qp;
    max_size = std::max<uint32_t>(max_size, qp.size);
  }
  if (seeds.empty()) seeds.push_back(0);
  QGWideConfig cfg{};
  uint32_t L = tuning_.list_cap ? next_pow2(tuning_.list_cap)
                                : std::min<uint32_t>(1024, next_pow2(std::max<uint32_t>(256, 4 * max_size)));
  L = std::max<uint32_t>(L, next_pow2(max_size + 1));
  if (L > 1024) throw std::runtime_error("result set too large for the relaxed quantized graph search (at most 1023)");
  cfg.list_cap = L;
  cfg.parents = tuning_.parents ? std::min<uint32_t>(tuning_.parents, 32) : 8;
  // neighbour slots: the code blocks of the largest node, and about P typical nodes
  uint32_t maxdeg = 0;
  for (uint32_t i = 0; i < qg_.nnodes; i++) maxdeg = std::max(maxdeg, qg_.offsets[i + 1] - qg_.offsets[i]);
  const uint32_t meandeg = qg_.nnodes ? (uint32_t)(qg_.offsets[qg_.nnodes] / qg_.nnodes) : 0u;
  uint32_t NB = next_pow2(std::max<uint32_t>({512u, (maxdeg + 15) / 16 * 16,
                                              cfg.parents * ((meandeg + 15) / 16 * 16), L}));
  cfg.nbr_cap = std::min<uint32_t>(NB, std::max<uint32_t>(4096u, L));
  cfg.group = std::min<uint32_t>(32, next_pow2((uint32_t)dev_.row_chunks));
  cfg.bitmap_words = ((host_.nrows + 31) / 32 + 3) / 4 * 4;
  cfg.max_iters = 1u << 22;
  // rows_in_flight of the batched tuning: code blocks each warp loads at a time (2 or 4)
  QGWideKernelFn fn = qg_wide_kernel_for(qg_.m, tuning_.rows_in_flight == 4 ? 4u : 2u);
  if (!fn) fn = qg_wide_kernel_for(qg_.m, 2u);
  if (!fn) throw std::runtime_error("too many subspaces in the quantized graph");
  const size_t smem = qg_wide_kernel_smem_bytes(dev_.row_chunks, qg_.dim, qg_.m, cfg);
  int max_smem = 0, per_sm = 0, sms = 0;
  NGT_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, device_));
  if (smem > (size_t)max_smem) throw std::runtime_error("relaxed quantized graph search state does not fit in shared memory");
  NGT_CUDA(cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  NGT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)fn, (int)kQGWideThreads, smem));
  NGT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
  const size_t grid = std::min<size_t>(nq, (size_t)std::max(1, per_sm) * sms);
  FastScratch& scratch = fast_scratch_[slot];
  ensure_fast_scratch(scratch, grid, stream);
  NGT_CUDA(cudaMemsetAsync(scratch.work, 0, 4, stream));
  QGParams* d_params = nullptr;
  uint32_t* d_seeds = nullptr;
  NGT_CUDA(cudaMallocAsync(&d_params, nq * sizeof(QGParams), stream));
  NGT_CUDA(cudaMallocAsync(&d_seeds, seeds.size() * 4, stream));
  NGT_CUDA(cudaMemcpyAsync(d_params, params.data(), nq * sizeof(QGParams), cudaMemcpyHostToDevice, stream));
  NGT_CUDA(cudaMemcpyAsync(d_seeds, seeds.data(), seeds.size() * 4, cudaMemcpyHostToDevice, stream));
  fn<<<(unsigned)grid, kQGWideThreads, smem, stream>>>(dev_, dqg_, d_rows, (uint32_t)nq, d_params, d_seeds,
                                                             d_out, d_counts, d_stats, scratch.bitmaps, scratch.work,
                                                             cfg);
  NGT_CUDA(cudaGetLastError());
  launches_++;
  NGT_CUDA(cudaFreeAsync(d_params, stream));
  NGT_CUDA(cudaFreeAsync(d_seeds, stream));
  // the pageable host parameter copies above are complete once they return
}

void GraphEngine::qg_search(const void* queries, QueryType qt, size_t nq, size_t qdim, const QGArgs* args,
                            size_t nargs, SearchOutput& out, bool relaxed) {
  if (!qg_loaded_) open_qg();
  NGT_CUDA(cudaSetDevice(device_));
  std::vector<uint8_t> rows;
  convert_queries(queries, qt, nq, qdim, rows);
  size_t kmax = 1;                                  // a quantized-graph query returns at most its size
  for (size_t i = 0; i < nargs; i++) kmax = std::max(kmax, args[i].size);
  out.kmax = kmax;
  out.results.assign(nq * kmax, ObjDist{0, 0.f});
  out.counts.assign(nq, 0);
  out.stats.assign(nq, QueryStats{});
  if (nq == 0) return;
  uint4* d_rows = nullptr;
  ObjDist* d_out = nullptr;
  uint32_t* d_counts = nullptr;
  QueryStats* d_stats = nullptr;
  cudaStream_t s = stream_;
  NGT_CUDA(cudaMallocAsync(&d_rows, rows.size(), s));
  NGT_CUDA(cudaMallocAsync(&d_out, nq * kmax * sizeof(ObjDist), s));
  NGT_CUDA(cudaMallocAsync(&d_counts, nq * 4, s));
  NGT_CUDA(cudaMallocAsync(&d_stats, nq * sizeof(QueryStats), s));
  NGT_CUDA(cudaMemcpyAsync(d_rows, rows.data(), rows.size(), cudaMemcpyHostToDevice, s));
  if (relaxed) qg_search_device_relaxed(d_rows, nq, args, nargs, d_out, d_counts, d_stats, kmax, s);
  else qg_search_device(d_rows, nq, args, nargs, d_out, d_counts, d_stats, kmax, s);
  NGT_CUDA(cudaMemcpyAsync(out.results.data(), d_out, nq * kmax * sizeof(ObjDist), cudaMemcpyDeviceToHost, s));
  NGT_CUDA(cudaMemcpyAsync(out.counts.data(), d_counts, nq * 4, cudaMemcpyDeviceToHost, s));
  NGT_CUDA(cudaMemcpyAsync(out.stats.data(), d_stats, nq * sizeof(QueryStats), cudaMemcpyDeviceToHost, s));
  NGT_CUDA(cudaFreeAsync(d_rows, s));
  NGT_CUDA(cudaFreeAsync(d_out, s));
  NGT_CUDA(cudaFreeAsync(d_counts, s));
  NGT_CUDA(cudaFreeAsync(d_stats, s));
  NGT_CUDA(cudaStreamSynchronize(s));
}

// ---- quantized blob graph ---------------------------------------------------

void GraphEngine::ensure_object_list() {
  if (d_olist_) return;
  // the array file of the object list (lib/NGT/ArrayFile.h): a 16-byte head (record
  // size, reserved), then per object a 16-byte flag block and the object; record 0
  // is the unused slot.  GenuineDataType: 0 uint8, 1 float (ObjectFile::DataType).
  Property qp = load_property_raw(qbg_dir_);
  const int gdt = std::atoi(qp.get("GenuineDataType", "0").c_str());
  if (gdt != 0 && gdt != 1) throw std::runtime_error("the object list's data type is neither uint8 nor float");
  const std::string path = qbg_dir_ + "/obj";
  std::ifstream f(path, std::ios::binary | std::ios::ate);
  if (!f.is_open()) throw std::runtime_error("the refinement needs the object list " + path);
  const size_t bytes = (size_t)f.tellg();
  f.seekg(0);
  uint64_t head[2] = {0, 0};
  if (bytes < 16 || !f.read(reinterpret_cast<char*>(head), 16)) throw std::runtime_error("truncated " + path);
  const size_t rs = head[0], es = gdt == 0 ? 1 : 4;
  if (rs == 0 || rs % es != 0 || (bytes - 16) % (16 + rs) != 0) throw std::runtime_error("corrupted " + path);
  const size_t n = (bytes - 16) / (16 + rs);
  if (n > 0xffffffffull) throw std::runtime_error("object list too large");
  const size_t chunks = (rs + 15) / 16;
  std::vector<uint8_t> rows(n * chunks * 16, 0), rec(16 + rs);
  for (size_t i = 0; i < n; i++) {
    if (!f.read(reinterpret_cast<char*>(rec.data()), (std::streamsize)rec.size())) throw std::runtime_error("truncated " + path);
    std::memcpy(rows.data() + i * chunks * 16, rec.data() + 16, rs);
  }
  d_olist_ = dmalloc_copy<void>(rows.data(), rows.size());
  olist_chunks_ = (uint32_t)chunks;
  olist_dim_ = (uint32_t)(rs / es);
  olist_rows_ = (uint32_t)n;
  olist_uint8_ = gdt == 0;
}

GraphEngine::QbgScratch& GraphEngine::qbg_slot(size_t slot, size_t grid, cudaStream_t stream) {
  if (slot >= qbg_scratch_.size()) qbg_scratch_.resize(slot + 1);
  QbgScratch& q = qbg_scratch_[slot];
  if (grid <= q.grid) return q;
  NGT_CUDA(cudaStreamSynchronize(stream));     // earlier launches of this slot may still use the old buffers
  cudaFree(q.bitmaps);
  cudaFree(q.exact_ovf);
  cudaFree(q.qbg_ovf);
  cudaFree(q.blob_dist);
  q = QbgScratch{};
  const size_t words = (host_.nrows + 31) / 32;
  const size_t qocap = std::min<size_t>(65536, 2 * (size_t)host_.nrows + 256);
  NGT_CUDA(cudaMalloc(&q.bitmaps, grid * words * 4));
  NGT_CUDA(cudaMemsetAsync(q.bitmaps, 0, grid * words * 4, stream));     // the kernels leave them clear
  NGT_CUDA(cudaMalloc(&q.exact_ovf, grid * 2 * (size_t)kOverflowCapacity * 8));
  NGT_CUDA(cudaMalloc(&q.qbg_ovf, grid * 4 * qocap * 8));
  NGT_CUDA(cudaMalloc(&q.blob_dist, grid * (size_t)blob_cap_ * 4));
  NGT_CUDA(cudaStreamSynchronize(stream));
  q.grid = grid;
  return q;
}

void GraphEngine::reserve_qbg_slot(size_t slot, size_t max_queries, cudaStream_t stream) {
  std::lock_guard<std::mutex> lock(mu_);
  NGT_CUDA(cudaSetDevice(device_));
  int sms = 0;
  NGT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
  // the largest grid any of the QBG kernels launches: one CTA per query, at most 16 per SM
  qbg_slot(slot, std::min<size_t>(max_queries, (size_t)sms * 16), stream);
}

void GraphEngine::qbg_probe_blobs(const uint4* d_rows, size_t nq, const QBGArgs* args, size_t nargs,
                                  ObjDist* d_blobs, uint32_t* d_bcounts, size_t bstride, cudaStream_t stream,
                                  size_t slot) {
  // searchInTwoSteps' global search (QuantizedBlobGraph.h:1224-1237): NGT::Index::search
  // of the read-only global index with size = the probes, epsilon = (1 + blob_epsilon) - 1
  // and the index's own edge size
  std::vector<SearchArgs> sa(nargs);
  for (size_t i = 0; i < nargs; i++) {
    sa[i].size = args[i].explored_blobs;
    sa[i].epsilon = (args[i].blob_epsilon + 1.0f) - 1.0f;
    sa[i].radius = FLT_MAX;
    sa[i].edge_size = -1;
  }
  const GraphMode saved = mode_;
  mode_ = GraphMode::ReadOnly;
  try {
    std::vector<QueryParams> params;
    std::vector<uint32_t> seeds;
    uint32_t max_size = 0;
    build_params(sa.data(), nargs, nq, bstride, params, seeds, max_size);
    QueryParams* d_params = nullptr;
    uint32_t* d_seeds = nullptr;
    QueryStats* d_st = nullptr;
    NGT_CUDA(cudaMallocAsync(&d_params, nq * sizeof(QueryParams), stream));
    NGT_CUDA(cudaMallocAsync(&d_seeds, seeds.size() * 4, stream));
    NGT_CUDA(cudaMallocAsync(&d_st, nq * sizeof(QueryStats), stream));
    NGT_CUDA(cudaMemcpyAsync(d_params, params.data(), nq * sizeof(QueryParams), cudaMemcpyHostToDevice, stream));
    NGT_CUDA(cudaMemcpyAsync(d_seeds, seeds.data(), seeds.size() * 4, cudaMemcpyHostToDevice, stream));
    if (slot == 0) {
      launch_exact(d_rows, nq, d_params, d_seeds, max_size, d_blobs, d_bcounts, d_st, stream);
    } else {
      QbgScratch& q = qbg_scratch_.at(slot);
      launch_exact(d_rows, nq, d_params, d_seeds, max_size, d_blobs, d_bcounts, d_st, stream, q.bitmaps,
                   q.exact_ovf, q.grid);
    }
    // (the copies above read pageable host memory: staged before they return)
    NGT_CUDA(cudaFreeAsync(d_params, stream));
    NGT_CUDA(cudaFreeAsync(d_seeds, stream));
    NGT_CUDA(cudaFreeAsync(d_st, stream));
  } catch (...) {
    mode_ = saved;
    throw;
  }
  mode_ = saved;
}

void GraphEngine::qbg_search_device(const uint4* d_rows, size_t nq, const QBGArgs* args, size_t nargs,
                                    ObjDist* d_out, uint32_t* d_counts, QueryStats* d_stats, size_t kmax,
                                    cudaStream_t stream, size_t slot) {
  if (!qbg_loaded_) throw std::runtime_error("not a QBG index");
  std::lock_guard<std::mutex> lock(mu_);
  NGT_CUDA(cudaSetDevice(device_));
  if (nq == 0) return;
  if (nargs != 1 && nargs != nq) throw std::runtime_error("one parameter block, or one per query");
  const bool two_step = args[0].two_step;
  bool refine = false;
  for (size_t i = 0; i < nargs; i++) {
    if (args[i].two_step != two_step) throw std::runtime_error("one-step and two-step queries in one call");
    refine = refine || (args[i].refine && args[i].result_expansion >= 1.0f);
  }
  if (refine) ensure_object_list();
  // qbg_search_index_ (lib/NGT/NGTQ/Capi.cpp:549-574), searchInOneStep
  // (lib/NGT/NGTQ/QuantizedBlobGraph.h:1332-1381) and searchInTwoSteps (:1190-1330)
  std::vector<QBGParams> params(nq);
  std::vector<uint32_t> seeds(qbg_fallback_seeds_);
  std::vector<uint32_t> exact(nq, 0);
  uint32_t max_size = 1;
  size_t max_probes = 1;
  for (size_t i = 0; i < nq; i++) {
    const QBGArgs& a = args[nargs == 1 ? 0 : i];
    const size_t size = qbg_search_size(a);
    const bool ref = a.refine && a.result_expansion >= 1.0f;
    if (qbg_result_size(a) > kmax) throw std::runtime_error("result size larger than the output capacity");
    if (size > 4096) throw std::runtime_error("number_of_results x result_expansion above 4096 is not supported");
    exact[i] = ref ? (uint32_t)a.size : 0u;
    QBGParams qp{};
    qp.size = (uint32_t)size;
    float coef = a.epsilon + 1.0f;
    if (coef == 0.0f) coef = 1.1f;
    qp.coef = coef;
    qp.bcoef = a.blob_epsilon + 1.0f;
    qp.explored = (uint32_t)std::min<size_t>(a.explored_blobs, 0xffffffffu);
    SearchArgs sa;
    sa.size = size;
    sa.epsilon = a.epsilon;
    sa.edge_size = (int64_t)(int)a.edges;
    qp.edge_size = (uint32_t)std::min<size_t>(edge_size_for(sa), 0xffffffffu);
    qp.fb_off = 0;
    qp.fb_cnt = (uint32_t)qbg_fallback_seeds_.size();
    qp.out_off = 0;                                    // set below, once the stride is known
    if (size > 0 && !two_step) {
      // the tree seeds are thinned with the container's size: the result size before a
      // refinement expansion (QuantizedBlobGraph.h:1336-1345)
      if (host_.prop.has_tree) seed_params(ref ? a.size : size, qp.seed_off, qp.seed_cnt, seeds);
      else { qp.seed_off = 0; qp.seed_cnt = 0; }
    }
    params[i] = qp;
    max_size = std::max<uint32_t>(max_size, qp.size);
    max_probes = std::max<size_t>(max_probes, a.explored_blobs);
  }
  // refined results pass through a buffer as wide as the largest search size
  const size_t stride = refine ? (size_t)max_size : kmax;
  for (size_t i = 0; i < nq; i++) params[i].out_off = (uint32_t)(i * stride);
  if (seeds.empty()) seeds.push_back(0);
  int max_smem = 0, sms = 0;
  NGT_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, device_));
  NGT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
  // the search's own output: the caller's buffers, or a temporary one before the refinement
  ObjDist* d_sout = d_out;
  uint32_t* d_scount = d_counts;
  if (refine) {
    NGT_CUDA(cudaMallocAsync(&d_sout, nq * stride * sizeof(ObjDist), stream));
    NGT_CUDA(cudaMallocAsync(&d_scount, nq * 4, stream));
  }
  QBGParams* d_params = nullptr;
  uint32_t* d_seeds = nullptr;
  NGT_CUDA(cudaMallocAsync(&d_params, nq * sizeof(QBGParams), stream));
  NGT_CUDA(cudaMallocAsync(&d_seeds, seeds.size() * 4, stream));
  NGT_CUDA(cudaMemcpyAsync(d_params, params.data(), nq * sizeof(QBGParams), cudaMemcpyHostToDevice, stream));
  NGT_CUDA(cudaMemcpyAsync(d_seeds, seeds.data(), seeds.size() * 4, cudaMemcpyHostToDevice, stream));
  auto ensure_blob_dist = [&](size_t grid, uint32_t ocap) {
    if (grid > qbg_grid_ || ocap != qbg_ocap_) {
      NGT_CUDA(cudaStreamSynchronize(stream));
      cudaFree(d_qbg_ovf_);
      cudaFree(d_blob_dist_);
      d_qbg_ovf_ = nullptr;
      d_blob_dist_ = nullptr;
      size_t g2 = std::max(grid, qbg_grid_);
      NGT_CUDA(cudaMalloc(&d_qbg_ovf_, g2 * 4 * (size_t)std::max<uint32_t>(ocap, 1) * 8));
      NGT_CUDA(cudaMalloc(&d_blob_dist_, g2 * (size_t)blob_cap_ * 4));
      qbg_grid_ = g2;
      qbg_ocap_ = ocap;
    }
  };
  if (two_step) {
    ObjDist* d_blobs = nullptr;
    uint32_t* d_bcounts = nullptr;
    NGT_CUDA(cudaMallocAsync(&d_blobs, nq * max_probes * sizeof(ObjDist), stream));
    NGT_CUDA(cudaMallocAsync(&d_bcounts, nq * 4, stream));
    qbg_probe_blobs(d_rows, nq, args, nargs, d_blobs, d_bcounts, max_probes, stream, slot);
    QBGScanKernelFn fn = qbg_scan_kernel_for(qb_.m);
    if (!fn) throw std::runtime_error("too many subspaces in the QBG index");
    const size_t smem = qbg_scan_kernel_smem_bytes(dev_.row_chunks, qb_.dim, qb_.m, max_size);
    if (smem > (size_t)max_smem) throw std::runtime_error("QBG search state does not fit in shared memory");
    NGT_CUDA(cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    NGT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)fn, kExactThreads, smem));
    size_t grid = std::min<size_t>(nq, (size_t)std::max(1, per_sm) * sms);
    float* bdist = nullptr;
    if (slot == 0) {
      ensure_blob_dist(grid, qbg_ocap_);
      bdist = d_blob_dist_;
    } else {
      QbgScratch& q = qbg_scratch_.at(slot);
      grid = std::min(grid, q.grid);
      bdist = q.blob_dist;
    }
    fn<<<(unsigned)grid, kExactThreads, smem, stream>>>(dqb_, d_blob_sid_, d_rows, dev_.row_chunks, (uint32_t)nq,
                                                         d_params, d_blobs, d_bcounts, (uint32_t)max_probes, d_sout,
                                                         d_scount, d_stats, bdist, blob_cap_, max_size);
    NGT_CUDA(cudaGetLastError());
    launches_++;
    NGT_CUDA(cudaFreeAsync(d_blobs, stream));
    NGT_CUDA(cudaFreeAsync(d_bcounts, stream));
  } else {
    QBGConfig cfg{};
    cfg.rcap = max_size;
    cfg.qcap = 1024;
    cfg.ocap = (uint32_t)std::min<size_t>(65536, 2 * (size_t)host_.nrows + 256);
    cfg.bitmap_words = (host_.nrows + 31) / 32;
    cfg.blob_cap = blob_cap_;
    cfg.group = std::min<uint32_t>(32, next_pow2((uint32_t)dev_.row_chunks));
    size_t smem = qbg_kernel_smem_bytes(dev_.row_chunks, qb_.dim, qb_.m, cfg);
    while (smem > (size_t)max_smem && cfg.qcap > 256) {
      cfg.qcap >>= 1;
      smem = qbg_kernel_smem_bytes(dev_.row_chunks, qb_.dim, qb_.m, cfg);
    }
    if (smem > (size_t)max_smem) throw std::runtime_error("QBG search state does not fit in shared memory");
    QBGKernelFn fn = qbg_kernel(qb_.m);
    NGT_CUDA(cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    NGT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)fn, kExactThreads, smem));
    size_t grid = std::min<size_t>(nq, (size_t)std::max(1, per_sm) * sms);
    uint32_t* bitmaps = nullptr;
    unsigned long long* qovf = nullptr;
    float* bdist = nullptr;
    if (slot == 0) {
      ensure_scratch(grid);
      ensure_blob_dist(grid, cfg.ocap);
      bitmaps = d_bitmaps_;
      qovf = d_qbg_ovf_;
      bdist = d_blob_dist_;
    } else {
      QbgScratch& q = qbg_scratch_.at(slot);
      grid = std::min(grid, q.grid);
      bitmaps = q.bitmaps;
      qovf = q.qbg_ovf;
      bdist = q.blob_dist;
    }
    fn<<<(unsigned)grid, kExactThreads, smem, stream>>>(dev_, dqb_, d_blob_sid_, d_rows, (uint32_t)nq, d_params,
                                                         d_seeds, d_sout, d_scount, d_stats, bitmaps, qovf, bdist,
                                                         cfg);
    NGT_CUDA(cudaGetLastError());
    launches_++;
  }
  if (refine) {
    uint32_t* d_exact = nullptr;
    NGT_CUDA(cudaMallocAsync(&d_exact, nq * 4, stream));
    NGT_CUDA(cudaMemcpyAsync(d_exact, exact.data(), nq * 4, cudaMemcpyHostToDevice, stream));
    const uint32_t P = next_pow2(std::max<uint32_t>(max_size, 2));
    const size_t smem = (size_t)olist_chunks_ * 16 + (size_t)P * 8;
    QBGRefineKernelFn rf = qbg_refine_kernel_for(olist_uint8_);
    NGT_CUDA(cudaFuncSetAttribute((const void*)rf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const unsigned grid = (unsigned)std::min<size_t>(nq, (size_t)sms * 8);
    rf<<<grid, 256, smem, stream>>>(d_sout, d_scount, (uint32_t)stride, reinterpret_cast<const float*>(d_rows),
                                    (uint32_t)(dev_.row_chunks * 4), static_cast<const uint4*>(d_olist_),
                                    olist_chunks_, olist_dim_, olist_rows_, d_exact, (uint32_t)nq, P, d_out,
                                    (uint32_t)kmax, d_counts);
    NGT_CUDA(cudaGetLastError());
    launches_++;
    NGT_CUDA(cudaFreeAsync(d_exact, stream));
    NGT_CUDA(cudaFreeAsync(d_sout, stream));
    NGT_CUDA(cudaFreeAsync(d_scount, stream));
  }
  // (the host vectors were read by copies from pageable memory, staged before they returned)
  NGT_CUDA(cudaFreeAsync(d_params, stream));
  NGT_CUDA(cudaFreeAsync(d_seeds, stream));
}

void GraphEngine::qbg_search(const void* queries, QueryType qt, size_t nq, size_t qdim, const QBGArgs* args,
                             size_t nargs, SearchOutput& out) {
  if (!qbg_loaded_) throw std::runtime_error("not a QBG index");
  NGT_CUDA(cudaSetDevice(device_));
  if (qdim != qbg_genuine_dim_)
    throw std::runtime_error("the query dimension " + std::to_string(qdim) + " differs from the index dimension " +
                             std::to_string(qbg_genuine_dim_));
  // the query as floats, zero-padded to the global index dimension
  // (searchInOneStep resizes the object vector, QuantizedBlobGraph.h:1336-1339)
  std::vector<float> padded(nq * host_.dim, 0.f);
  for (size_t q = 0; q < nq; q++)
    for (size_t i = 0; i < qdim; i++) padded[q * host_.dim + i] = (float)query_elem(queries, qt, q * qdim + i);
  std::vector<uint8_t> rows;
  convert_queries(padded.data(), QueryType::Float32, nq, host_.dim, rows);
  size_t kmax = 1;
  for (size_t i = 0; i < nargs; i++) kmax = std::max(kmax, qbg_result_size(args[i]));
  out.kmax = kmax;
  out.results.assign(nq * kmax, ObjDist{0, 0.f});
  out.counts.assign(nq, 0);
  out.stats.assign(nq, QueryStats{});
  if (nq == 0) return;
  uint4* d_rows = nullptr;
  ObjDist* d_out = nullptr;
  uint32_t* d_counts = nullptr;
  QueryStats* d_stats = nullptr;
  cudaStream_t s = stream_;
  NGT_CUDA(cudaMallocAsync(&d_rows, rows.size(), s));
  NGT_CUDA(cudaMallocAsync(&d_out, nq * kmax * sizeof(ObjDist), s));
  NGT_CUDA(cudaMallocAsync(&d_counts, nq * 4, s));
  NGT_CUDA(cudaMallocAsync(&d_stats, nq * sizeof(QueryStats), s));
  NGT_CUDA(cudaMemcpyAsync(d_rows, rows.data(), rows.size(), cudaMemcpyHostToDevice, s));
  qbg_search_device(d_rows, nq, args, nargs, d_out, d_counts, d_stats, kmax, s);
  NGT_CUDA(cudaMemcpyAsync(out.results.data(), d_out, nq * kmax * sizeof(ObjDist), cudaMemcpyDeviceToHost, s));
  NGT_CUDA(cudaMemcpyAsync(out.counts.data(), d_counts, nq * 4, cudaMemcpyDeviceToHost, s));
  NGT_CUDA(cudaMemcpyAsync(out.stats.data(), d_stats, nq * sizeof(QueryStats), cudaMemcpyDeviceToHost, s));
  NGT_CUDA(cudaFreeAsync(d_rows, s));
  NGT_CUDA(cudaFreeAsync(d_out, s));
  NGT_CUDA(cudaFreeAsync(d_counts, s));
  NGT_CUDA(cudaFreeAsync(d_stats, s));
  NGT_CUDA(cudaStreamSynchronize(s));
}

}  // namespace ngtg
