// Serving loop: continuous batching of search requests over one opened index.
//
// The index (objects, graph, seeds) stays resident in HBM.  Callers submit
// requests of any size (up to the batch capacity) with their own k / epsilon /
// radius / edge size, from any thread.  A dispatcher thread keeps up to
// `inflight` batched-kernel launches on the device at once, each on its own
// stream with its own scratch set; whenever a launch slot is free and requests
// are waiting, it admits the waiting requests in arrival order (as many as fit
// the slot's query capacity), uploads them, launches, and queues the result
// download -- so requests arriving while others run join the next launch and
// overlap with them on the GPU.  Completed launches are harvested by polling
// their events; each request's latency is measured from submit to completion.
// A request's results depend only on its queries and parameters (the batched
// kernel handles every query independently), so they are the same alone and
// in any mix.
//
// Admission follows each request's footprint.  Scratch memory (visited bitmaps,
// spill tiers, queue overflows, blob distances) is reserved per lane for
// max_batch queries when the server starts, so a launch admits queries up to that
// count and nothing is allocated while serving.  Shared memory per CTA grows with
// a request's result size (the candidate list of the graph kernels, the result
// set and sort width of the QBG kernels), and a launch runs with the largest one
// it holds; so requests are grouped by that class: a launch takes the oldest
// waiting request and, in arrival order, the waiting requests of the same class
// that fit -- a small-k request never runs at a large-k request's occupancy, and
// the oldest request always goes first (no starvation).
//
// The same loop serves quantized-blob-graph indexes (qbg_* handles): one-step or
// two-step searches, optionally refined, with per-lane scratch sets so that the
// launches overlap; and quantized-graph indexes (ngtqg_* handles), each lane with its
// own visited bitmaps and overflow lists for the exact-order quantized-graph kernel.
//
// A request that waits longer than the server's admission deadline (if one is set)
// completes unlaunched with a "deadline exceeded" error, and a waiting request can be
// cancelled; a request already on the device always runs to completion.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "engine.h"

extern "C" {
#include "../../include/ngtgpu.h"
#include "../../include/ngtq_capi.h"
}

namespace ngtg {

namespace {

#define SRV_CUDA(x)                                                                                \
  do {                                                                                             \
    cudaError_t e_ = (x);                                                                          \
    if (e_ != cudaSuccess)                                                                         \
      throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e_) + " in " #x);    \
  } while (0)

using Clock = std::chrono::steady_clock;

struct Request {
  int64_t ticket = 0;
  std::vector<uint8_t> rows;          // converted query rows
  size_t nq = 0;
  std::vector<SearchArgs> args;       // 1 or nq entries (graph search)
  std::vector<QBGArgs> qargs;         // 1 or nq entries (quantized blob graph)
  std::vector<QGArgs> gargs;          // 1 or nq entries (quantized graph)
  uint32_t cls = 0;                   // shared-memory class (admission groups a launch by it)
  size_t kmax = 0;
  Clock::time_point arrival;
  Clock::time_point deadline = Clock::time_point::max();   // latest admission
  std::vector<ObjDist> results;       // nq * kmax
  std::vector<uint32_t> counts;
  bool done = false;
  std::string error;
  double latency_ms = 0.0;
};

struct Lane {
  cudaStream_t stream = nullptr;
  cudaEvent_t done_event = nullptr;
  size_t slot = 0;                    // scratch set of the engine
  uint4* d_rows = nullptr;
  ObjDist* d_out = nullptr;
  uint32_t* d_counts = nullptr;
  QueryStats* d_stats = nullptr;
  uint8_t* h_rows = nullptr;          // pinned staging
  ObjDist* h_out = nullptr;
  uint32_t* h_counts = nullptr;
  uint32_t* bitmaps = nullptr;        // quantized graph: visited bitmaps of kQgLaneCtas CTAs
  unsigned long long* overflow = nullptr;
  bool busy = false;
  size_t kmax = 0;
  std::vector<std::shared_ptr<Request>> batch;
};

}  // namespace

// Shared-memory class of a result size: powers of two from 16 (sizes up to 16 share one).
uint32_t size_class(size_t size) {
  uint32_t c = 0;
  while (c < 31 && ((size_t)16 << c) < size) c++;
  return c;
}

enum class ServedIndex { Graph, Qbg, Qg };

class Server {
 public:
  // CTAs of one quantized-graph launch (its lane holds their bitmaps and overflow lists)
  static constexpr size_t kQgLaneCtas = 256;

  Server(GraphEngine* e, size_t max_batch, size_t inflight, size_t max_k, Kernel kernel = Kernel::Fast,
         ServedIndex kind = ServedIndex::Graph, uint32_t qbg_flags = 0)
      : e_(e), max_batch_(max_batch), max_k_(max_k), row_bytes_(e->host().row_bytes()), kernel_(kernel),
        qbg_(kind == ServedIndex::Qbg), qg_(kind == ServedIndex::Qg), qbg_flags_(qbg_flags) {
    if (max_batch == 0 || inflight == 0 || max_k == 0) throw std::runtime_error("invalid server sizes");
    if (qbg_ && !e->is_qbg()) throw std::runtime_error("not a QBG index");
    SRV_CUDA(cudaSetDevice(e->device()));
    if (qg_) e->open_qg();
    if (qbg_ && (qbg_flags & 2u)) e->prepare_refinement();
    e->reserve_scratch_sets(inflight + 1);
    lanes_.resize(inflight);
    for (size_t i = 0; i < inflight; i++) {
      Lane& l = lanes_[i];
      l.slot = i + 1;
      SRV_CUDA(cudaStreamCreateWithFlags(&l.stream, cudaStreamNonBlocking));
      SRV_CUDA(cudaEventCreateWithFlags(&l.done_event, cudaEventDisableTiming));
      SRV_CUDA(cudaMalloc(&l.d_rows, max_batch * row_bytes_));
      SRV_CUDA(cudaMalloc(&l.d_out, max_batch * max_k * sizeof(ObjDist)));
      SRV_CUDA(cudaMalloc(&l.d_counts, max_batch * 4));
      SRV_CUDA(cudaMalloc(&l.d_stats, max_batch * sizeof(QueryStats)));
      SRV_CUDA(cudaMallocHost(&l.h_rows, max_batch * row_bytes_));
      SRV_CUDA(cudaMallocHost(&l.h_out, max_batch * max_k * sizeof(ObjDist)));
      SRV_CUDA(cudaMallocHost(&l.h_counts, max_batch * 4));
      // a launch uses at most one scratch slot per query (plus the rounding of its
      // last CTA's warps): no reallocation while serving
      if (qbg_) {
        e->reserve_qbg_slot(l.slot, max_batch, l.stream);
      } else if (qg_ && kernel == Kernel::Wide) {
        e->reserve_scratch_slots(l.slot, max_batch + 8);   // the relaxed-order QG kernel's bitmaps
      } else if (qg_) {
        const size_t ctas = std::min(max_batch, kQgLaneCtas);
        SRV_CUDA(cudaMalloc(&l.bitmaps, ctas * e->cta_bitmap_bytes()));
        SRV_CUDA(cudaMemsetAsync(l.bitmaps, 0, ctas * e->cta_bitmap_bytes(), l.stream));
        SRV_CUDA(cudaMalloc(&l.overflow, ctas * GraphEngine::cta_overflow_bytes()));
      } else {
        e->reserve_scratch_slots(l.slot, max_batch + 8);
      }
    }
    worker_ = std::thread([this] { run(); });
  }

  ~Server() {
    {
      std::lock_guard<std::mutex> lock(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    if (worker_.joinable()) worker_.join();
    cudaSetDevice(e_->device());
    for (Lane& l : lanes_) {
      if (l.stream) cudaStreamSynchronize(l.stream);
      cudaFree(l.d_rows);
      cudaFree(l.d_out);
      cudaFree(l.d_counts);
      cudaFree(l.d_stats);
      cudaFreeHost(l.h_rows);
      cudaFreeHost(l.h_out);
      cudaFreeHost(l.h_counts);
      cudaFree(l.bitmaps);
      cudaFree(l.overflow);
      if (l.done_event) cudaEventDestroy(l.done_event);
      if (l.stream) cudaStreamDestroy(l.stream);
    }
  }

  int64_t submit(const float* queries, size_t nq, size_t dim, const SearchArgs* args, size_t nargs,
                 double deadline_ms = -1.0) {
    if (qbg_ || qg_) throw std::runtime_error("this server serves a quantized index: submit its parameters");
    if (nq == 0 || nq > max_batch_)
      throw std::runtime_error("request size must be 1.." + std::to_string(max_batch_) + " queries");
    if (!(nargs == 1 || nargs == nq)) throw std::runtime_error("parameters must be 1 or one per query");
    auto r = std::make_shared<Request>();
    e_->convert_queries(queries, QueryType::Float32, nq, dim, r->rows);
    r->nq = nq;
    r->args.assign(args, args + nargs);
    size_t kmax = 1, smax = 1;
    for (const auto& a : r->args) {
      kmax = std::max(kmax, e_->output_size(a));
      smax = std::max(smax, a.size);
    }
    if (kmax > max_k_) throw std::runtime_error("result size above the server's maximum " + std::to_string(max_k_));
    r->kmax = kmax;
    r->cls = size_class(smax);
    return enqueue(r, deadline_ms);
  }

  int64_t submit_qg(const float* queries, size_t nq, size_t dim, const QGArgs* args, size_t nargs) {
    if (!qg_) throw std::runtime_error("this server does not serve a quantized graph");
    if (nq == 0 || nq > max_batch_)
      throw std::runtime_error("request size must be 1.." + std::to_string(max_batch_) + " queries");
    if (!(nargs == 1 || nargs == nq)) throw std::runtime_error("parameters must be 1 or one per query");
    auto r = std::make_shared<Request>();
    e_->convert_queries(queries, QueryType::Float32, nq, dim, r->rows);
    r->nq = nq;
    r->gargs.assign(args, args + nargs);
    size_t kmax = 1, smax = 1;
    for (const auto& a : r->gargs) {
      kmax = std::max(kmax, a.size);
      smax = std::max(smax, a.result_expansion > 1.0f ? (size_t)((float)a.size * a.result_expansion) : a.size);
    }
    if (kmax > max_k_) throw std::runtime_error("result size above the server's maximum " + std::to_string(max_k_));
    r->kmax = kmax;
    r->cls = size_class(smax);
    return enqueue(r);
  }

  // Withdraws a request that has not been launched: true, and its wait reports
  // "cancelled"; false when it is on the device or complete (its wait delivers it).
  bool cancel(int64_t ticket) {
    std::lock_guard<std::mutex> lock(mu_);
    if (!tickets_.count(ticket)) throw std::runtime_error("unknown ticket " + std::to_string(ticket));
    for (auto it = pending_.begin(); it != pending_.end(); ++it)
      if ((*it)->ticket == ticket) {
        (*it)->error = "cancelled";
        (*it)->done = true;
        pending_.erase(it);
        done_cv_.notify_all();
        return true;
      }
    return false;
  }

  // Admission deadline of later submits (ms from submission; <= 0: none).
  void set_deadline(double ms) {
    std::lock_guard<std::mutex> lock(mu_);
    deadline_ms_ = ms;
  }

  int64_t submit_qbg(const float* queries, size_t nq, size_t dim, const QBGArgs* args, size_t nargs) {
    if (!qbg_) throw std::runtime_error("this server serves a graph index: submit graph parameters");
    if (nq == 0 || nq > max_batch_)
      throw std::runtime_error("request size must be 1.." + std::to_string(max_batch_) + " queries");
    if (!(nargs == 1 || nargs == nq)) throw std::runtime_error("parameters must be 1 or one per query");
    if (dim != e_->qbg_genuine_dimension())
      throw std::runtime_error("the query dimension differs from the index dimension");
    auto r = std::make_shared<Request>();
    // the query zero-padded to the global index dimension, as the QBG searches resize it
    const size_t gd = e_->host().dim;
    std::vector<float> padded(nq * gd, 0.f);
    for (size_t q = 0; q < nq; q++) std::memcpy(padded.data() + q * gd, queries + q * dim, dim * sizeof(float));
    e_->convert_queries(padded.data(), QueryType::Float32, nq, gd, r->rows);
    r->nq = nq;
    r->qargs.assign(args, args + nargs);
    size_t kmax = 1, smax = 1;
    for (auto& a : r->qargs) {
      a.two_step = (qbg_flags_ & 1u) != 0;
      a.refine = (qbg_flags_ & 2u) != 0;
      kmax = std::max(kmax, GraphEngine::qbg_result_size(a));
      smax = std::max(smax, GraphEngine::qbg_search_size(a));
    }
    if (kmax > max_k_) throw std::runtime_error("result size above the server's maximum " + std::to_string(max_k_));
    if (smax > 4096) throw std::runtime_error("number_of_results x result_expansion above 4096");
    r->kmax = kmax;
    r->cls = size_class(smax);
    return enqueue(r);
  }

  int64_t enqueue(const std::shared_ptr<Request>& r, double deadline_ms = -1.0) {
    r->arrival = Clock::now();
    std::lock_guard<std::mutex> lock(mu_);
    const double ms = deadline_ms > 0.0 ? deadline_ms : deadline_ms_;
    if (ms > 0.0)
      r->deadline = r->arrival + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double, std::milli>(ms));
    r->ticket = next_ticket_++;
    pending_.push_back(r);
    tickets_[r->ticket] = r;
    cv_.notify_all();
    return r->ticket;
  }

  void wait(int64_t ticket, ObjDist* out, size_t kmax, uint32_t* counts, double* latency_ms) {
    std::shared_ptr<Request> r;
    std::unique_lock<std::mutex> lock(mu_);
    auto it = tickets_.find(ticket);
    if (it == tickets_.end()) throw std::runtime_error("unknown ticket " + std::to_string(ticket));
    r = it->second;
    done_cv_.wait(lock, [&] { return r->done; });
    tickets_.erase(ticket);
    lock.unlock();
    if (!r->error.empty()) throw std::runtime_error(r->error);
    for (size_t q = 0; q < r->nq; q++) {
      uint32_t n = r->counts[q];
      if (n > kmax) throw std::runtime_error("kmax smaller than the results of the request");
      counts[q] = n;
      std::memcpy(out + q * kmax, r->results.data() + q * r->kmax, n * sizeof(ObjDist));
    }
    if (latency_ms) *latency_ms = r->latency_ms;
  }

 private:
  // Dispatcher: harvest finished lanes, then admit waiting requests into free lanes.
  void run() {
    cudaSetDevice(e_->device());
    while (true) {
      bool any_busy = false;
      for (Lane& l : lanes_) {
        if (!l.busy) continue;
        cudaError_t q = cudaEventQuery(l.done_event);
        if (q == cudaErrorNotReady) {
          any_busy = true;
          continue;
        }
        finish(l, q == cudaSuccess ? std::string() : std::string(cudaGetErrorString(q)));
      }
      std::vector<std::shared_ptr<Request>> batch;
      Lane* free_lane = nullptr;
      {
        std::unique_lock<std::mutex> lock(mu_);
        if (stop_ && pending_.empty() && !any_busy) break;
        expire(Clock::now());
        for (Lane& l : lanes_)
          if (!l.busy) { free_lane = &l; break; }
        if (free_lane && !pending_.empty()) {
          // the oldest request, and then in arrival order the waiting requests of its
          // shared-memory class that fit the lane's query capacity
          const uint32_t cls = pending_.front()->cls;
          size_t total = 0;
          for (auto it = pending_.begin(); it != pending_.end();) {
            if ((*it)->cls == cls && total + (*it)->nq <= max_batch_) {
              total += (*it)->nq;
              batch.push_back(*it);
              it = pending_.erase(it);
            } else {
              ++it;
            }
          }
        } else if (!any_busy) {
          cv_.wait_for(lock, std::chrono::milliseconds(2), [&] { return stop_ || !pending_.empty(); });
          continue;
        }
      }
      if (!batch.empty()) {
        launch(*free_lane, batch);
      } else if (any_busy) {
        std::this_thread::sleep_for(std::chrono::microseconds(20));
      }
    }
  }

  // Completes, unlaunched, the waiting requests whose admission deadline has passed
  // (called with mu_ held).
  void expire(Clock::time_point now) {
    bool any = false;
    for (auto it = pending_.begin(); it != pending_.end();) {
      if ((*it)->deadline < now) {
        (*it)->error = "deadline exceeded before launch";
        (*it)->latency_ms = std::chrono::duration<double, std::milli>(now - (*it)->arrival).count();
        (*it)->done = true;
        it = pending_.erase(it);
        any = true;
      } else {
        ++it;
      }
    }
    if (any) done_cv_.notify_all();
  }

  void launch(Lane& l, std::vector<std::shared_ptr<Request>>& batch) {
    l.batch = batch;
    l.kmax = 1;
    size_t nq = 0;
    std::vector<SearchArgs> args;
    std::vector<QBGArgs> qargs;
    std::vector<QGArgs> gargs;
    for (auto& r : batch) {
      std::memcpy(l.h_rows + nq * row_bytes_, r->rows.data(), r->nq * row_bytes_);
      for (size_t q = 0; q < r->nq; q++) {
        if (qbg_) qargs.push_back(r->qargs[r->qargs.size() == 1 ? 0 : q]);
        else if (qg_) gargs.push_back(r->gargs[r->gargs.size() == 1 ? 0 : q]);
        else args.push_back(r->args[r->args.size() == 1 ? 0 : q]);
      }
      nq += r->nq;
      l.kmax = std::max(l.kmax, r->kmax);
    }
    try {
      SRV_CUDA(cudaMemcpyAsync(l.d_rows, l.h_rows, nq * row_bytes_, cudaMemcpyHostToDevice, l.stream));
      if (qbg_)
        e_->qbg_search_device(l.d_rows, nq, qargs.data(), qargs.size(), l.d_out, l.d_counts, l.d_stats, l.kmax,
                              l.stream, l.slot);
      else if (qg_ && kernel_ == Kernel::Wide)
        e_->qg_search_device_relaxed(l.d_rows, nq, gargs.data(), gargs.size(), l.d_out, l.d_counts, l.d_stats,
                                     l.kmax, l.stream, l.slot);
      else if (qg_)
        e_->qg_search_device(l.d_rows, nq, gargs.data(), gargs.size(), l.d_out, l.d_counts, l.d_stats, l.kmax,
                             l.stream, l.bitmaps, l.overflow, std::min(max_batch_, kQgLaneCtas));
      else
        e_->search_device_slot(l.d_rows, nq, args.data(), args.size(), l.d_out, l.d_counts, l.d_stats, l.kmax,
                               l.stream, l.slot, kernel_);
      SRV_CUDA(cudaMemcpyAsync(l.h_out, l.d_out, nq * l.kmax * sizeof(ObjDist), cudaMemcpyDeviceToHost, l.stream));
      SRV_CUDA(cudaMemcpyAsync(l.h_counts, l.d_counts, nq * 4, cudaMemcpyDeviceToHost, l.stream));
      SRV_CUDA(cudaEventRecord(l.done_event, l.stream));
      l.busy = true;
    } catch (std::exception& ex) {
      l.busy = true;
      finish(l, ex.what());
    }
  }

  void finish(Lane& l, const std::string& err) {
    auto now = Clock::now();
    size_t off = 0;
    for (auto& r : l.batch) {
      if (err.empty()) {
        r->results.resize(r->nq * r->kmax);
        r->counts.resize(r->nq);
        for (size_t q = 0; q < r->nq; q++) {
          uint32_t n = std::min<uint32_t>(l.h_counts[off + q], (uint32_t)r->kmax);
          r->counts[q] = n;
          std::memcpy(r->results.data() + q * r->kmax, l.h_out + (off + q) * l.kmax, n * sizeof(ObjDist));
        }
      } else {
        r->error = err;
      }
      off += r->nq;
      r->latency_ms = std::chrono::duration<double, std::milli>(now - r->arrival).count();
    }
    {
      std::lock_guard<std::mutex> lock(mu_);
      for (auto& r : l.batch) r->done = true;
    }
    done_cv_.notify_all();
    l.batch.clear();
    l.busy = false;
  }

  GraphEngine* e_;
  size_t max_batch_, max_k_, row_bytes_;
  Kernel kernel_;
  bool qbg_ = false, qg_ = false;
  uint32_t qbg_flags_ = 0;
  double deadline_ms_ = -1.0;
  std::vector<Lane> lanes_;
  std::deque<std::shared_ptr<Request>> pending_;
  std::map<int64_t, std::shared_ptr<Request>> tickets_;
  int64_t next_ticket_ = 0;
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  bool stop_ = false;
  std::thread worker_;
};

}  // namespace ngtg

namespace {
void server_error(const char* fn, const std::string& msg, NGTError error) {
  std::string s = std::string("Capi : ") + fn + "() : Error: " + msg;
  if (error) *static_cast<std::string*>(error) = s;
  else fprintf(stderr, "%s\n", s.c_str());
}

std::vector<ngtg::SearchArgs> server_args(const NGTQueryParameters* params, size_t nparams) {
  std::vector<ngtg::SearchArgs> a(nparams);
  for (size_t i = 0; i < nparams; i++) {
    int es = (int)params[i].edge_size;
    a[i].size = params[i].size;
    a[i].epsilon = params[i].epsilon;
    a[i].radius = params[i].radius < 0.0f ? 3.402823466e+38f : params[i].radius;
    a[i].edge_size = es == INT32_MIN ? -1 : es;
  }
  return a;
}
}  // namespace

extern "C" {

NGTGPUServer ngtgpu_server_create(NGTIndex index, uint32_t max_batch_queries, uint32_t inflight, uint32_t max_k,
                                  NGTError error) {
  return ngtgpu_server_create_ex(index, max_batch_queries, inflight, max_k, NGTGPU_KERNEL_BATCHED, error);
}

NGTGPUServer ngtgpu_server_create_ex(NGTIndex index, uint32_t max_batch_queries, uint32_t inflight, uint32_t max_k,
                                     uint32_t kernel, NGTError error) {
  if (index == nullptr || !(kernel == NGTGPU_KERNEL_BATCHED || kernel == NGTGPU_KERNEL_BATCHED_FP32 ||
                            kernel == NGTGPU_KERNEL_WIDE)) {
    server_error(__FUNCTION__, "parametor error: index is NULL or the kernel is not a batched one", error);
    return nullptr;
  }
  try {
    ngtg::Kernel k = kernel == NGTGPU_KERNEL_WIDE ? ngtg::Kernel::Wide
                     : kernel == NGTGPU_KERNEL_BATCHED_FP32 ? ngtg::Kernel::FastFp32 : ngtg::Kernel::Fast;
    return new ngtg::Server(static_cast<ngtg::GraphEngine*>(index), max_batch_queries, inflight, max_k, k);
  } catch (std::exception& ex) {
    server_error(__FUNCTION__, ex.what(), error);
    return nullptr;
  }
}

int64_t ngtgpu_server_submit(NGTGPUServer server, const float* queries, size_t nq, int32_t dim,
                             const NGTQueryParameters* params, size_t nparams, NGTError error) {
  if (server == nullptr || queries == nullptr || params == nullptr || dim <= 0) {
    server_error(__FUNCTION__, "parametor error: server, queries or params", error);
    return -1;
  }
  try {
    auto a = server_args(params, nparams);
    return static_cast<ngtg::Server*>(server)->submit(queries, nq, (size_t)dim, a.data(), a.size());
  } catch (std::exception& ex) {
    server_error(__FUNCTION__, ex.what(), error);
    return -1;
  }
}

bool ngtgpu_server_wait(NGTGPUServer server, int64_t ticket, NGTObjectDistance* results, size_t kmax,
                        uint32_t* counts, double* latency_ms, NGTError error) {
  if (server == nullptr || results == nullptr || counts == nullptr) {
    server_error(__FUNCTION__, "parametor error: server or output buffers", error);
    return false;
  }
  try {
    static_cast<ngtg::Server*>(server)->wait(ticket, reinterpret_cast<ngtg::ObjDist*>(results), kmax, counts,
                                             latency_ms);
    return true;
  } catch (std::exception& ex) {
    server_error(__FUNCTION__, ex.what(), error);
    return false;
  }
}

void ngtgpu_server_destroy(NGTGPUServer server) { delete static_cast<ngtg::Server*>(server); }

int64_t ngtgpu_server_submit_deadline(NGTGPUServer server, const float* queries, size_t nq, int32_t dim,
                                      const NGTQueryParameters* params, size_t nparams, double deadline_ms,
                                      NGTError error) {
  if (server == nullptr || queries == nullptr || params == nullptr || dim <= 0) {
    server_error(__FUNCTION__, "parametor error: server, queries or params", error);
    return -1;
  }
  try {
    auto a = server_args(params, nparams);
    return static_cast<ngtg::Server*>(server)->submit(queries, nq, (size_t)dim, a.data(), a.size(), deadline_ms);
  } catch (std::exception& ex) {
    server_error(__FUNCTION__, ex.what(), error);
    return -1;
  }
}

bool ngtgpu_server_cancel(NGTGPUServer server, int64_t ticket, NGTError error) {
  if (server == nullptr) {
    server_error(__FUNCTION__, "parametor error: server is NULL", error);
    return false;
  }
  try {
    return static_cast<ngtg::Server*>(server)->cancel(ticket);
  } catch (std::exception& ex) {
    server_error(__FUNCTION__, ex.what(), error);
    return false;
  }
}

bool ngtgpu_server_set_deadline(NGTGPUServer server, double deadline_ms, NGTError error) {
  if (server == nullptr) {
    server_error(__FUNCTION__, "parametor error: server is NULL", error);
    return false;
  }
  static_cast<ngtg::Server*>(server)->set_deadline(deadline_ms);
  return true;
}

void* ngtgpu_qg_server_create(NGTQGIndex index, uint32_t max_batch_queries, uint32_t inflight, uint32_t max_k,
                              NGTQGError error) {
  return ngtgpu_qg_server_create_ex(index, max_batch_queries, inflight, max_k, NGTGPU_KERNEL_EXACT, error);
}

void* ngtgpu_qg_server_create_ex(NGTQGIndex index, uint32_t max_batch_queries, uint32_t inflight, uint32_t max_k,
                                 uint32_t kernel, NGTQGError error) {
  if (index == nullptr || (kernel != NGTGPU_KERNEL_EXACT && kernel != NGTGPU_KERNEL_WIDE)) {
    server_error(__FUNCTION__, "parametor error: index is NULL or unknown kernel", error);
    return nullptr;
  }
  try {
    return new ngtg::Server(static_cast<ngtg::GraphEngine*>(index), max_batch_queries, inflight, max_k,
                            kernel == NGTGPU_KERNEL_WIDE ? ngtg::Kernel::Wide : ngtg::Kernel::Exact,
                            ngtg::ServedIndex::Qg);
  } catch (std::exception& ex) {
    server_error(__FUNCTION__, ex.what(), error);
    return nullptr;
  }
}

int64_t ngtgpu_qg_server_submit(void* server, const float* queries, size_t nq, int32_t dim,
                                const NGTQGQueryParameters* params, size_t nparams, NGTQGError error) {
  if (server == nullptr || queries == nullptr || params == nullptr || dim <= 0) {
    server_error(__FUNCTION__, "parametor error: server, queries or params", error);
    return -1;
  }
  try {
    std::vector<ngtg::QGArgs> a(nparams);
    for (size_t i = 0; i < nparams; i++) {
      a[i].size = params[i].size;
      a[i].epsilon = params[i].epsilon;
      a[i].result_expansion = params[i].result_expansion;
      a[i].radius = params[i].radius < 0.0f ? FLT_MAX : params[i].radius;   // ngtqg_search_index_
    }
    return static_cast<ngtg::Server*>(server)->submit_qg(queries, nq, (size_t)dim, a.data(), a.size());
  } catch (std::exception& ex) {
    server_error(__FUNCTION__, ex.what(), error);
    return -1;
  }
}

void* ngtgpu_qbg_server_create(QBGIndex index, uint32_t max_batch_queries, uint32_t inflight, uint32_t max_k,
                                      uint32_t flags, NGTError error) {
  if (index == nullptr || (flags & ~(NGTGPU_QBG_TWO_STEP | NGTGPU_QBG_REFINE)) != 0) {
    server_error(__FUNCTION__, "parametor error: index is NULL or unknown flags", error);
    return nullptr;
  }
  try {
    return new ngtg::Server(static_cast<ngtg::GraphEngine*>(index), max_batch_queries, inflight, max_k,
                            ngtg::Kernel::Exact, ngtg::ServedIndex::Qbg, flags);
  } catch (std::exception& ex) {
    server_error(__FUNCTION__, ex.what(), error);
    return nullptr;
  }
}

int64_t ngtgpu_qbg_server_submit(void* server, const float* queries, size_t nq, int32_t dim,
                                 const QBGQueryParameters* params, size_t nparams, NGTError error) {
  if (server == nullptr || queries == nullptr || params == nullptr || dim <= 0) {
    server_error(__FUNCTION__, "parametor error: server, queries or params", error);
    return -1;
  }
  try {
    std::vector<ngtg::QBGArgs> a(nparams);
    for (size_t i = 0; i < nparams; i++) {
      a[i].size = params[i].number_of_results;
      a[i].epsilon = params[i].epsilon;
      a[i].blob_epsilon = params[i].blob_epsilon;
      a[i].result_expansion = params[i].result_expansion;
      a[i].explored_blobs = params[i].number_of_explored_blobs;
      a[i].edges = params[i].number_of_edges;
    }
    return static_cast<ngtg::Server*>(server)->submit_qbg(queries, nq, (size_t)dim, a.data(), a.size());
  } catch (std::exception& ex) {
    server_error(__FUNCTION__, ex.what(), error);
    return -1;
  }
}

}  // extern "C"
