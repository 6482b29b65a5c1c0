// Autotuner of the batched graph-search kernels (ngtgpu_autotune).
//
// For one index, result size and epsilon it times a fixed list of candidate
// configurations -- the warp-per-query kernel with its row pipelines and register
// budgets, the CTA-per-query kernel with its CTA sizes, staged rows and parents per
// step -- on a sample of the caller's queries (device resident, CUDA events, median
// of three launches), and keeps the fastest whose tie-aware recall@k against the
// exact answer (the index's exhaustive search) is at least a floor: the caller's, or
// (floor < 0) the exact-order kernel's own recall at the same epsilon, i.e. the
// reference's.  With epsilon < 0 each configuration runs at the smallest epsilon of
// a sweep that reaches the floor, and the epsilon becomes part of the choice.  The
// winner becomes the index's tuning, and is remembered in a JSON cache keyed by (rows,
// dimension, object type, distance, k, epsilon) -- the file named by
// NGTGPU_TUNE_CACHE, if set -- so that a later process skips the timing.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "engine.h"
#include "kernels.h"

extern "C" {
#include "../../include/ngtgpu.h"
}

namespace ngtg {
namespace {

#define AT_CUDA(x)                                                                                 \
  do {                                                                                             \
    cudaError_t e_ = (x);                                                                          \
    if (e_ != cudaSuccess)                                                                         \
      throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e_) + " in " #x);    \
  } while (0)

struct Candidate {
  uint32_t kernel;                 // NGTGPU_KERNEL_BATCHED or NGTGPU_KERNEL_WIDE
  FastTuning t;
};

std::vector<Candidate> candidates(bool float_l2) {
  std::vector<Candidate> c;
  auto warp = [&](uint32_t P, uint32_t R, uint32_t C, uint32_t NB) {
    Candidate x{NGTGPU_KERNEL_BATCHED, FastTuning{}};
    x.t.parents = P;
    x.t.rows_in_flight = R;
    x.t.ctas_per_sm = C;
    x.t.nbr_cap = NB;
    c.push_back(x);
  };
  auto wide = [&](uint32_t P, uint32_t T, uint32_t stage) {
    Candidate x{NGTGPU_KERNEL_WIDE, FastTuning{}};
    x.t.parents = P;
    x.t.cta_threads = T;
    x.t.stage_kb = stage;
    c.push_back(x);
  };
  warp(3, 4, 5, 256);
  if (float_l2) warp(4, 6, 4, 0);
  for (uint32_t P : {8u, 10u, 12u, 16u}) wide(P, 128, 16);
  wide(8, 128, 32);
  if (float_l2) {
    wide(16, 256, 32);
    wide(32, 256, 64);
  }
  return c;
}

std::string cache_key(const HostIndex& h, size_t k, float eps) {
  std::ostringstream s;
  s << h.nrows << "x" << h.dim << ":" << (int)h.prop.otype << ":" << (int)h.prop.metric << ":k" << k << ":e"
    << std::lround(eps * 1000.0);
  return s.str();
}

std::mutex g_cache_mu;

// The cache is a flat JSON object of key -> [kernel, parents, rows, ctas, nbr, threads, stage, qps, epsilon].
std::map<std::string, std::vector<double>> read_cache(const std::string& path) {
  std::map<std::string, std::vector<double>> m;
  std::ifstream f(path);
  if (!f.is_open()) return m;
  std::string text((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  size_t pos = 0;
  while ((pos = text.find('"', pos)) != std::string::npos) {
    size_t end = text.find('"', pos + 1);
    if (end == std::string::npos) break;
    std::string key = text.substr(pos + 1, end - pos - 1);
    size_t lb = text.find('[', end), rb = text.find(']', end);
    if (lb == std::string::npos || rb == std::string::npos || rb < lb) break;
    std::vector<double> v;
    std::stringstream vs(text.substr(lb + 1, rb - lb - 1));
    std::string item;
    while (std::getline(vs, item, ',')) v.push_back(std::atof(item.c_str()));
    if (v.size() == 9) m[key] = v;
    pos = rb + 1;
  }
  return m;
}

void write_cache(const std::string& path, const std::map<std::string, std::vector<double>>& m) {
  std::ofstream f(path + ".tmp");
  if (!f.is_open()) return;
  f << "{\n";
  size_t i = 0;
  for (const auto& kv : m) {
    f << "  \"" << kv.first << "\": [";
    for (size_t j = 0; j < kv.second.size(); j++) f << (j ? ", " : "") << kv.second[j];
    f << "]" << (++i < m.size() ? "," : "") << "\n";
  }
  f << "}\n";
  f.close();
  std::rename((path + ".tmp").c_str(), path.c_str());
}

}  // namespace

// Tie-aware recall of device results against the k-th exact distance per query.
static double recall_of(const std::vector<ObjDist>& res, const std::vector<uint32_t>& cnt, size_t kmax,
                        const std::vector<float>& kth, size_t k) {
  size_t hit = 0;
  for (size_t q = 0; q < cnt.size(); q++)
    for (size_t i = 0; i < std::min<size_t>(cnt[q], k); i++)
      if (res[q * kmax + i].distance <= kth[q]) hit++;
  return (double)hit / (double)(k * cnt.size());
}

}  // namespace ngtg

extern "C" bool ngtgpu_autotune(NGTIndex index, const float* queries, size_t nq, int32_t dim, size_t k,
                                float epsilon, float recall_floor, NGTGPUBatchedTuning* best, uint32_t* best_kernel,
                                float* best_qps, float* best_epsilon, NGTError error) {
  using namespace ngtg;
  auto fail = [&](const std::string& msg) {
    std::string s = std::string("Capi : ") + __FUNCTION__ + "() : Error: " + msg;
    if (error) *static_cast<std::string*>(error) = s;
    else fprintf(stderr, "%s\n", s.c_str());
    return false;
  };
  if (index == nullptr || queries == nullptr || nq == 0 || dim <= 0 || k == 0 || best == nullptr ||
      best_kernel == nullptr || (epsilon < 0.0f && recall_floor < 0.0f))
    return fail("parametor error: index, queries, k, outputs, or an epsilon sweep without a recall floor");
  try {
    GraphEngine* e = static_cast<GraphEngine*>(index);
    const HostIndex& h = e->host();
    const char* cpath = std::getenv("NGTGPU_TUNE_CACHE");
    const std::string key = cache_key(h, k, epsilon);
    auto apply = [&](uint32_t kernel, const FastTuning& t, float qps, float eps) {
      if (best_epsilon) *best_epsilon = eps;
      e->set_tuning(t);
      std::memset(best, 0, sizeof(*best));
      best->parents = t.parents;
      best->rows_in_flight = t.rows_in_flight;
      best->ctas_per_sm = t.ctas_per_sm;
      best->neighbour_capacity = t.nbr_cap;
      best->cta_threads = t.cta_threads;
      best->stage_kilobytes = t.stage_kb;
      *best_kernel = kernel;
      if (best_qps) *best_qps = qps;
    };
    if (cpath && *cpath) {
      std::lock_guard<std::mutex> lock(g_cache_mu);
      auto m = read_cache(cpath);
      auto it = m.find(key);
      if (it != m.end()) {
        const auto& v = it->second;
        FastTuning t{};
        t.parents = (uint32_t)v[1];
        t.rows_in_flight = (uint32_t)v[2];
        t.ctas_per_sm = (uint32_t)v[3];
        t.nbr_cap = (uint32_t)v[4];
        t.cta_threads = (uint32_t)v[5];
        t.stage_kb = (uint32_t)v[6];
        apply((uint32_t)v[0], t, (float)v[7], (float)v[8]);
        return true;
      }
    }
    std::vector<uint8_t> rows;
    e->convert_queries(queries, QueryType::Float32, nq, (size_t)dim, rows);
    AT_CUDA(cudaSetDevice(e->device()));
    cudaStream_t s = e->stream();
    // the exact answer of the sample: the exhaustive search (tensor-core pre-selection of
    // 8k candidates for float objects, the plain linear search otherwise)
    std::vector<float> kth(nq, 3.402823466e+38f);
    if (e->tc_supported()) {
      void *d_q = nullptr, *d_o = nullptr, *d_c = nullptr, *d_s = nullptr;
      AT_CUDA(cudaMalloc(&d_q, rows.size()));
      AT_CUDA(cudaMalloc(&d_o, nq * k * sizeof(ObjDist)));
      AT_CUDA(cudaMalloc(&d_c, nq * 4));
      AT_CUDA(cudaMalloc(&d_s, nq * 4));
      struct FreeGt {
        void* p[4];
        ~FreeGt() {
          for (void* x : p) cudaFree(x);
        }
      } fg{{d_q, d_o, d_c, d_s}};
      AT_CUDA(cudaMemcpy(d_q, rows.data(), rows.size(), cudaMemcpyHostToDevice));
      e->linear_search_tc_device(static_cast<const uint4*>(d_q), nq, k, std::min<size_t>(4096, std::max<size_t>(8 * k, 400)),
                                 static_cast<ObjDist*>(d_o), k, static_cast<uint32_t*>(d_c),
                                 static_cast<uint32_t*>(d_s), s, false, true);
      std::vector<ObjDist> o(nq * k);
      std::vector<uint32_t> c(nq);
      AT_CUDA(cudaMemcpy(o.data(), d_o, o.size() * sizeof(ObjDist), cudaMemcpyDeviceToHost));
      AT_CUDA(cudaMemcpy(c.data(), d_c, nq * 4, cudaMemcpyDeviceToHost));
      for (size_t q = 0; q < nq; q++)
        if (c[q] >= k) kth[q] = o[q * k + k - 1].distance;
    } else {
      SearchOutput gt;
      e->linear_search(queries, QueryType::Float32, nq, (size_t)dim, k, gt);
      for (size_t q = 0; q < nq; q++)
        if (gt.counts[q] >= k) kth[q] = gt.results[q * gt.kmax + k - 1].distance;
    }
    // the epsilon sweep (epsilon < 0): every configuration at the smallest of these
    // that reaches the floor
    static const float kSweep[] = {0.0f, 0.02f, 0.04f, 0.06f, 0.07f, 0.075f, 0.08f, 0.085f, 0.09f,
                                   0.1f, 0.12f, 0.15f, 0.2f, 0.3f};
    SearchArgs a;
    a.size = k;
    a.epsilon = epsilon < 0.0f ? kSweep[sizeof(kSweep) / sizeof(kSweep[0]) - 1] : epsilon;
    const size_t kmax = e->output_size(a);
    uint4* d_rows = nullptr;
    ObjDist* d_out = nullptr;
    uint32_t* d_cnt = nullptr;
    QueryStats* d_st = nullptr;
    AT_CUDA(cudaMalloc(&d_rows, rows.size()));
    AT_CUDA(cudaMalloc(&d_out, nq * kmax * sizeof(ObjDist)));
    AT_CUDA(cudaMalloc(&d_cnt, nq * 4));
    AT_CUDA(cudaMalloc(&d_st, nq * sizeof(QueryStats)));
    struct Free {
      void* p[4];
      ~Free() {
        for (void* x : p) cudaFree(x);
      }
    } fr{{d_rows, d_out, d_cnt, d_st}};
    AT_CUDA(cudaMemcpy(d_rows, rows.data(), rows.size(), cudaMemcpyHostToDevice));
    cudaEvent_t e0, e1;
    AT_CUDA(cudaEventCreate(&e0));
    AT_CUDA(cudaEventCreate(&e1));
    std::vector<ObjDist> res(nq * kmax);
    std::vector<uint32_t> cnt(nq);
    // times one configuration: median of three launches after one warm-up; its recall
    auto run = [&](Kernel kernel, double& ms_out) {
      std::vector<float> ms;
      for (int i = 0; i < 4; i++) {
        AT_CUDA(cudaEventRecord(e0, s));
        e->search_device(d_rows, nq, &a, 1, d_out, d_cnt, d_st, kmax, s, kernel);
        AT_CUDA(cudaEventRecord(e1, s));
        AT_CUDA(cudaEventSynchronize(e1));
        float t = 0.f;
        AT_CUDA(cudaEventElapsedTime(&t, e0, e1));
        if (i > 0) ms.push_back(t);
      }
      std::sort(ms.begin(), ms.end());
      ms_out = ms[1];
      AT_CUDA(cudaMemcpy(res.data(), d_out, res.size() * sizeof(ObjDist), cudaMemcpyDeviceToHost));
      AT_CUDA(cudaMemcpy(cnt.data(), d_cnt, nq * 4, cudaMemcpyDeviceToHost));
      return recall_of(res, cnt, kmax, kth, k);
    };
    const FastTuning saved = e->tuning();
    double floor = recall_floor;
    if (floor < 0.0) {
      double ms = 0.0;
      floor = run(Kernel::Exact, ms);
    }
    const bool float_l2 = h.prop.otype == ObjType::Float && kernel_metric(h.prop.metric) == Metric::L2;
    double best_ms = 1e30;
    float win_eps = epsilon;
    Candidate winner{};
    bool found = false;
    for (const Candidate& c : candidates(float_l2)) {
      const Kernel kern = c.kernel == NGTGPU_KERNEL_WIDE ? Kernel::Wide : Kernel::Fast;
      e->set_tuning(c.t);
      if (!e->fast_supported(kern)) continue;
      std::vector<float> eps_list;
      if (epsilon < 0.0f) eps_list.assign(std::begin(kSweep), std::end(kSweep));
      else eps_list.push_back(epsilon);
      for (float ev : eps_list) {
        a.epsilon = ev;
        double ms = 0.0, r = 0.0;
        try {
          r = run(kern, ms);
        } catch (std::exception&) {
          break;                  // a configuration this index does not build (reported by search_device)
        }
        if (r + 1e-12 >= floor) {
          if (ms < best_ms) {
            best_ms = ms;
            winner = c;
            win_eps = ev;
            found = true;
          }
          break;
        }
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!found) {
      e->set_tuning(saved);
      return fail("no batched configuration reaches the recall floor at this epsilon");
    }
    const float qps = (float)(nq / (best_ms * 1e-3));
    apply(winner.kernel, winner.t, qps, win_eps);
    if (cpath && *cpath) {
      std::lock_guard<std::mutex> lock(g_cache_mu);
      auto m = read_cache(cpath);
      m[key] = {(double)winner.kernel, (double)winner.t.parents, (double)winner.t.rows_in_flight,
                (double)winner.t.ctas_per_sm, (double)winner.t.nbr_cap, (double)winner.t.cta_threads,
                (double)winner.t.stage_kb, (double)qps, (double)win_eps};
      write_cache(cpath, m);
    }
    return true;
  } catch (std::exception& ex) {
    return fail(ex.what());
  }
}
