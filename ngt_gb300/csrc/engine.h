// Host engine: one opened index resident in HBM plus the launch logic of the
// search kernels.  The C ABI (capi.cpp) and the batched extension entry points
// are thin wrappers around this class.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <atomic>
#include <condition_variable>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>
#include "device_index.h"
#include "index_files.h"

namespace ngtg {
struct ExactConfig;
// Resolves the no-allocation search's fixed scratch on `device` (current) and loads
// the module of `exact_fn` (defined in noalloc.cu; called when an index opens).
void noalloc_prepare_device(int device, const void* exact_fn);
}  // namespace ngtg

namespace ngtg {

// Search parameters of one query, as the reference's C API receives them
// (ngt_search_index_ in lib/NGT/Capi.cpp:514-532).
struct SearchArgs {
  size_t size = 10;
  float epsilon = 0.1f;
  float radius = -1.0f;            // < 0 means FLT_MAX
  int64_t edge_size = -1;          // -1: index default (EdgeSizeForSearch)
  // > 0: the expected accuracy of the C++ API's search container, which replaces
  // epsilon by the index's AccuracyTable (lib/NGT/Index.h:1700-1702); the reference's
  // C API never passes it, so only the batched extensions set it
  float accuracy = -1.0f;
  // >= 1: the C++ API's refinement expansion (GraphIndex::search(SearchQuery&),
  // lib/NGT/Index.h:1146-1236): size x expansion results re-ranked by exact distances
  // over the index's refinement objects (robj) to the size best
  float refinement_expansion = 0.0f;
};

// Query element type accepted at the boundary.
enum class QueryType { Float32 = 0, Float64 = 1, Uint8 = 2, Float16 = 3 };

// Exact: reference-order search, one query per CTA (results equal the reference's).
// Fast: batched warp-per-query search on bf16 rows (float objects) or the native
//       rows (other types), with an exact re-rank.  FastFp32: the same on fp32 rows.
// Wide: the batched search with one query per CTA (rows of an iteration staged in
//       shared memory at once), for low per-query latency.
enum class Kernel { Exact = 0, Fast = 1, FastFp32 = 2, Wide = 3 };

// Knobs of the batched kernel (0 = automatic).
struct FastTuning {
  uint32_t list_cap = 0;       // candidate list length (power of two)
  uint32_t parents = 0;        // nodes expanded per iteration
  float rerank_factor = 0.f;   // re-ranked entries = ceil(size * factor)
  uint32_t rows_in_flight = 0; // rows per lane group in flight in the distance loop (2, 4, 6 or 8)
  uint32_t ctas_per_sm = 0;    // register budget of the instantiation (4..8)
  uint32_t nbr_cap = 0;        // neighbour slots per iteration (power of two >= 256)
  uint32_t cta_threads = 0;    // wide kernel: threads per CTA (128 or 256)
  uint32_t stage_kb = 0;       // wide kernel: shared memory for staged rows (KB)
  uint32_t l2_policy = 0;      // wide kernel: 0 automatic, else WideConfig::l2_policy + 1
  uint32_t search_rows = 0;    // wide kernel, float objects: 0 automatic (8-bit when lossless, else bf16),
                               // 1 bf16, 2 8-bit codes
};

// Parameters of one quantized-graph query (NGTQGQueryParameters,
// lib/NGT/NGTQ/Capi.h; defaults of ngtqg_initialize_query_parameters).
struct QGArgs {
  size_t size = 20;
  float epsilon = 0.03f;
  float result_expansion = 3.0f;
  float radius = -1.0f;            // < 0 means FLT_MAX
};

// Parameters of one quantized-blob-graph query (QBGQueryParameters,
// lib/NGT/NGTQ/Capi.h; defaults of qbg_initialize_query_parameters).
struct QBGArgs {
  size_t size = 20;                 // number_of_results
  float epsilon = 0.1f;
  float blob_epsilon = 0.0f;
  float result_expansion = 3.0f;
  size_t explored_blobs = 256;
  size_t edges = 0;                 // global-graph edge size (0: all)
  // searchInTwoSteps (lib/NGT/NGTQ/QuantizedBlobGraph.h:1190-1330): explored_blobs
  // blobs probed, found by the global index's graph search; else searchInOneStep
  bool two_step = false;
  // result_expansion read as the refinement expansion of the reference's search
  // container: size x expansion quantized results re-ranked by exact distances over
  // the object list (refineDistances, QuantizedBlobGraph.h:1136-1185) to `size`
  bool refine = false;
};

struct SearchOutput {
  std::vector<ObjDist> results;    // nq * kmax
  std::vector<uint32_t> counts;    // nq
  std::vector<QueryStats> stats;   // nq
  size_t kmax = 0;
};

class CudaError;
struct TcState;                     // tensor-core linear search state (tc_linear.cu)
void tc_release(TcState* s);

class GraphEngine {
 public:
  // quantized = true also reads the quantized graph (<path>/qg) before any
  // device work, so that a damaged one is reported like a damaged index.
  GraphEngine(const std::string& path, GraphMode mode, bool quantized = false);
  // A QBG index: `qbg_dir` holds the blobs, qbg_dir/global the global index
  // (blob centroids, their graph and tree) that this engine searches.
  GraphEngine(const std::string& qbg_dir, bool blobs);
  ~GraphEngine();
  GraphEngine(const GraphEngine&) = delete;
  GraphEngine& operator=(const GraphEngine&) = delete;

  const HostIndex& host() const { return host_; }
  GraphMode mode() const { return mode_; }
  uint32_t dimension() const { return (uint32_t)host_.prop.dimension; }

  // Graph search over host queries (row-major nq x qdim).
  // One query through the exact-order kernel, coalesced with the other single-query
  // calls that arrive from other host threads while a launch is on the GPU (the
  // OpenMP loop of ngtpy's batch_search over ngt_search_index_as_float): the first
  // caller launches at once; callers arriving meanwhile wait and the next of them
  // launches all waiting queries together.  Results equal a lone call's (the kernel
  // handles every query independently).
  void search_one(const void* query, QueryType qt, size_t qdim, const SearchArgs& args, SearchOutput& out);
  // queries coalesced so far and launches they took (statistics)
  uint64_t coalesced_queries() const { return co_queries_; }
  uint64_t coalesced_launches() const { return co_launches_; }
  void set_coalescing_lanes(size_t n) {
    if (n < 1 || n > kCoLanes) throw std::runtime_error("coalescing lanes must be 1..16");
    std::lock_guard<std::mutex> lock(co_mu_);
    co_nlanes_ = n;
  }
  // search() of arguments with a refinement expansion (all of them): the expanded
  // search, then the exact re-rank over the refinement objects
  void search_refined(const void* queries, QueryType qt, size_t nq, size_t qdim, const SearchArgs* args,
                      size_t nargs, SearchOutput& out, Kernel kernel);
  void search(const void* queries, QueryType qt, size_t nq, size_t qdim, const SearchArgs* args, size_t nargs,
              SearchOutput& out, Kernel kernel = Kernel::Exact);
  // Quantized graph (<index>/qg): loads it on first use; throws when the index
  // has none or it cannot be searched here (float objects, L2 only).
  void open_qg();
  bool has_qg() const { return qg_loaded_; }
 private:
  void read_qg();
  void upload_qg();
 public:
  const HostQG& qg_host() const { return qg_; }
  // ngtqg_search_index over host queries (row-major nq x qdim).
  void qg_search(const void* queries, QueryType qt, size_t nq, size_t qdim, const QGArgs* args, size_t nargs,
                 SearchOutput& out, bool relaxed = false);
  // The same over converted query rows resident on the device.
  // bitmaps / overflow: a caller's own visited bitmaps and overflow lists for at most
  // grid_cap CTAs (launches on several streams at once); null: the engine's own.
  void qg_search_device(const uint4* d_rows, size_t nq, const QGArgs* args, size_t nargs, ObjDist* d_out,
                        uint32_t* d_counts, QueryStats* d_stats, size_t kmax, cudaStream_t stream,
                        uint32_t* bitmaps = nullptr, unsigned long long* overflow = nullptr, size_t grid_cap = 0);
  // The relaxed-order quantized-graph search (qg_wide.cuh): several parents per step,
  // the batched tuning's parents (default 8) and list capacity (default 4 x the
  // result-set size, at least 256).
  // slot: scratch set (0: the engine's own; >= 1: one reserved by reserve_scratch_slots).
  void qg_search_device_relaxed(const uint4* d_rows, size_t nq, const QGArgs* args, size_t nargs, ObjDist* d_out,
                                uint32_t* d_counts, QueryStats* d_stats, size_t kmax, cudaStream_t stream,
                                size_t slot = 0);
  // bytes of the visited bitmap and of the overflow lists of one CTA of the exact-order
  // kernels (the quantized graph's included)
  size_t cta_bitmap_bytes() const { return (host_.nrows + 31) / 32 * 4; }
  static size_t cta_overflow_bytes() { return 2 * (size_t)kOverflowCapacity * 8; }
  // qbg_search_index over host queries (nq x qdim, qdim = the QBG genuine
  // dimension); results ascending (distance, id) with quantized distances,
  // size x result_expansion of them when the expansion is >= 1.
  void qbg_search(const void* queries, QueryType qt, size_t nq, size_t qdim, const QBGArgs* args, size_t nargs,
                  SearchOutput& out);
  // slot 0: the engine's own scratch; slot >= 1: scratch set `slot`, reserved by
  // reserve_qbg_slot (the serving loop's lanes, whose launches overlap)
  void reserve_qbg_slot(size_t slot, size_t max_queries, cudaStream_t stream);
  // loads the QBG object list the refinement reads (done on the first refined search)
  void prepare_refinement() {
    std::lock_guard<std::mutex> lock(mu_);
    ensure_object_list();
  }
  void qbg_search_device(const uint4* d_rows, size_t nq, const QBGArgs* args, size_t nargs, ObjDist* d_out,
                         uint32_t* d_counts, QueryStats* d_stats, size_t kmax, cudaStream_t stream,
                         size_t slot = 0);
  bool is_qbg() const { return qbg_loaded_; }
  uint32_t qbg_genuine_dimension() const { return qbg_genuine_dim_; }
  // results the blob search keeps, and results returned
  static size_t qbg_search_size(const QBGArgs& a) {
    return a.result_expansion >= 1.0f ? (size_t)((float)a.size * a.result_expansion) : a.size;
  }
  static size_t qbg_result_size(const QBGArgs& a) {
    return a.refine && a.result_expansion >= 1.0f ? a.size : qbg_search_size(a);
  }
  // Exhaustive search with a tensor-core pre-selection (tc_linear.cu): bf16
  // scores of every (query, row) with fp32 accumulation, the `candidates` best
  // per query re-ranked with the exact comparator, the first `size` returned
  // ascending by (distance, id).  d_rows: nq converted query rows; d_status[q]
  // bit 1 = candidate list overflow.  Float objects; L2, inner product, cosine,
  // angle and their normalized forms.
  // fp8: scores from per-row / per-query scaled E4M3 copies (kind::f8f6f4) instead
  // of bf16; fp64_ties: the candidates tied with the size-th one within the fp32
  // evaluation error are ordered by FP64 distance at the cut (status bit 4: tie
  // window too wide, fp32 order kept).
  void linear_search_tc_device(const uint4* d_rows, size_t nq, size_t size, size_t candidates, ObjDist* d_out,
                               size_t kmax, uint32_t* d_counts, uint32_t* d_status, cudaStream_t stream,
                               bool fp8 = false, bool fp64_ties = false, bool pair = false);
  // The same from host float queries into host buffers: the query rows are converted
  // into the pinned staging buffer and copied from there.
  void linear_search_tc_host(const float* queries, size_t nq, size_t qdim, size_t size, size_t candidates,
                             ObjDist* results, size_t kmax, uint32_t* counts, uint32_t* status, bool fp8,
                             bool fp64_ties, bool pair);
  // The approximate scores alone: d_scores[q * ld + row] (-inf for the unused
  // row 0 and removed objects).
  void tc_scores_device(const uint4* d_rows, size_t nq, float* d_scores, size_t ld, cudaStream_t stream);
  bool tc_supported() const;
  // CUDA-event times (ms) of the last query batch of linear_search_tc_device:
  // dense part with its selection, filtered part, final re-rank
  void tc_phase_ms(float* out) const;
  // rows scored densely before the threshold filter (0: automatic, 8192)
  void set_tc_first_rows(size_t rows) { tc_first_rows_ = rows; }
  // Tensor-core searches replay captured CUDA graphs of their launch sequence (one
  // per shape, buffers and options; off: launched directly).
  void set_tc_graphs(bool on);
  // the tensor-core search covers rows [begin, end) only (a shard of a row-range
  // split; begin a multiple of 128; end 0 = the last row)
  void set_tc_row_range(size_t begin, size_t end) {
    if (begin % 128 != 0) throw std::runtime_error("a shard must begin at a multiple of 128 rows");
    if (end != 0 && end <= begin) throw std::runtime_error("empty shard");
    tc_row_begin_ = (uint32_t)begin;
    tc_row_end_ = (uint32_t)end;
  }
  // Exhaustive search (exact ids, ties broken by id).
  void linear_search(const void* queries, QueryType qt, size_t nq, size_t qdim, size_t size, SearchOutput& out);

  // Converts user queries to padded object rows exactly as the reference's
  // allocateObject does (cast to the object type, normalisation for the
  // normalised metrics, zero augmentation for inner product).
  void convert_queries(const void* queries, QueryType qt, size_t nq, size_t qdim, std::vector<uint8_t>& rows) const;
  void convert_queries(const void* queries, QueryType qt, size_t nq, size_t qdim, uint8_t* rows) const;

  // Device-side entry used by the batched extension: queries already converted
  // and resident on the device.
  void search_device(const uint4* d_rows, size_t nq, const SearchArgs* args, size_t nargs, ObjDist* d_out,
                     uint32_t* d_counts, QueryStats* d_stats, size_t kmax, cudaStream_t stream,
                     Kernel kernel = Kernel::Exact);
  // The batched kernel with scratch set `slot` (1 .. scratch_sets-1 are free for
  // concurrent launches on different streams; slot 0 belongs to search_device).
  void search_device_slot(const uint4* d_rows, size_t nq, const SearchArgs* args, size_t nargs, ObjDist* d_out,
                          uint32_t* d_counts, QueryStats* d_stats, size_t kmax, cudaStream_t stream, size_t slot,
                          Kernel kernel = Kernel::Fast);
  void reserve_scratch_sets(size_t n);
  // sizes scratch set `set` for launches of up to `slots` CTAs now, so that no
  // later launch reallocates it (a reallocation waits for the whole device)
  void reserve_scratch_slots(size_t set, size_t slots);
  // Bytes of device scratch one batched launch of nq queries uses (admission).
  size_t batched_scratch_bytes(size_t nq) const;
  // The exact search with every scratch buffer carved from the caller-provided
  // device memory `scratch` (scratch_bytes long) instead of allocated: query
  // parameters, seed lists, per-CTA visited bitmaps and overflow tiers.  Throws
  // when the scratch cannot hold one CTA's share, or when a seed table the
  // queries need has not been built by an earlier regular search.
  void search_device_noalloc(void* scratch, size_t scratch_bytes, const uint4* d_rows, size_t nq,
                             const SearchArgs* args, size_t nargs, ObjDist* d_out, uint32_t* d_counts,
                             QueryStats* d_stats, size_t kmax, cudaStream_t stream);
  // The exact kernel's configuration for result sizes up to max_size: fills cfg and
  // returns its dynamic shared memory (shared by every exact launch path).
  size_t exact_launch_config(uint32_t max_size, ExactConfig& cfg) const;
  void set_tuning(const FastTuning& t) { tuning_ = t; }
  const FastTuning& tuning() const { return tuning_; }
  bool fast_supported(Kernel k) const;

  // AccuracyTable::getEpsilon (lib/NGT/Index.h:442-472) over the index's
  // AccuracyTable property: the epsilon expected to give `accuracy`
  float epsilon_for_accuracy(double accuracy) const;
  // Number of results a query can return (larger than args.size only for the
  // updatable search on an index with EpsilonType ResultSize).
  size_t output_size(const SearchArgs& a) const;

  cudaStream_t stream() const { return stream_; }
  int device() const { return device_; }
  size_t row_chunks() const { return host_.row_bytes() / 16; }
  // Number of launches of our kernels since the engine was created.
  uint64_t launches() const { return launches_; }

 private:
  // Scratch of the batched kernel: one visited bitmap and one spill tier
  // (2 x kSpillCapacity keys) per warp slot, and the work counter.  Set 0 serves
  // search_device; the serving loop owns one set per in-flight launch.
  struct FastScratch {
    uint32_t* bitmaps = nullptr;
    unsigned long long* spill = nullptr;
    uint32_t* work = nullptr;
    size_t slots = 0;
  };
  void upload();
  // seed_table, build_params and seed_params may add a seed table (shared state):
  // callers hold mu_
  uint32_t seed_table(size_t seed_size);        // index of the thinned-seed table
  void build_params(const SearchArgs* args, size_t nargs, size_t nq, size_t kmax, std::vector<QueryParams>& params,
                    std::vector<uint32_t>& seed_list, uint32_t& max_size);
  // Seeds of one query of requested size k: tree seeds thinned to k, or graph seeds.
  // shared_off: when given, queries of one launch share one copy of the graph-only
  // random seeds (UINT32_MAX before the first)
  void seed_params(size_t k, uint32_t& seed_off, uint32_t& seed_cnt, std::vector<uint32_t>& seed_list,
                   uint32_t* shared_off = nullptr);
  std::once_flag random_seeds_once_;
  std::vector<uint32_t> random_seeds_;                    // graph-only index: the seeds of rand() seeded with 1
  size_t edge_size_for(const SearchArgs& a) const;
  void ensure_scratch(size_t grid);
  void ensure_fast_scratch(FastScratch& sc, size_t slots, cudaStream_t stream);
  void ensure_bf16_rows();
  bool result_size_rule() const;
  uint32_t visited_hash_capacity() const;
  uint32_t candidate_list_capacity() const;
  // 8-bit codes of float objects; the affine map is lossless when every
  // coordinate is an integer and they span at most 256 values
  void ensure_sq8_stats();
  void compute_sq8_stats();
  void ensure_sq8_rows();
 public:
  // search rows the wide kernel uses for this index and tuning
  SearchRows wide_search_rows();
 private:
  // bitmaps / overflow: a caller's scratch for `grid_cap` CTAs (nullptr: the engine's own)
  void launch_exact(const uint4* d_rows, size_t nq, const QueryParams* d_params, const uint32_t* d_seeds,
                    uint32_t max_size, ObjDist* d_out, uint32_t* d_counts, QueryStats* d_stats, cudaStream_t stream,
                    uint32_t* bitmaps = nullptr, unsigned long long* overflow = nullptr, size_t grid_cap = 0);
  void launch_fast(const uint4* d_rows, size_t nq, const QueryParams* d_params, const uint32_t* d_seeds,
                   uint32_t max_size, ObjDist* d_out, uint32_t* d_counts, QueryStats* d_stats, cudaStream_t stream,
                   Kernel kernel, FastScratch& scratch);
  void launch_wide(const uint4* d_rows, size_t nq, const QueryParams* d_params, const uint32_t* d_seeds,
                   uint32_t max_size, ObjDist* d_out, uint32_t* d_counts, QueryStats* d_stats, cudaStream_t stream,
                   FastScratch& scratch);

  HostIndex host_;
  GraphMode mode_;
  // quantized blob graph
  HostQG qb_;
  bool qbg_loaded_ = false;
  uint32_t qbg_genuine_dim_ = 0;
  DevQG dqb_;
  uint32_t* d_blob_sid_ = nullptr;
  uint32_t blob_cap_ = 16;
  std::vector<uint32_t> qbg_fallback_seeds_;
  unsigned long long* d_qbg_ovf_ = nullptr;
  float* d_blob_dist_ = nullptr;
  // the QBG object list (qbg_dir/obj), loaded on the first refined search: rows of
  // olist_chunks_ 16-byte chunks (uint8 or float), row 0 unused
  std::string qbg_dir_;
  void* d_olist_ = nullptr;
  uint32_t olist_chunks_ = 0, olist_dim_ = 0, olist_rows_ = 0;
  bool olist_uint8_ = true;
  void ensure_object_list();
  // the global index's read-only graph search for the two-step search (mu_ held)
  void qbg_probe_blobs(const uint4* d_rows, size_t nq, const QBGArgs* args, size_t nargs, ObjDist* d_blobs,
                       uint32_t* d_bcounts, size_t bstride, cudaStream_t stream, size_t slot);
  // per-slot scratch of the QBG searches: the exact kernel's (probe search) visited
  // bitmaps and overflow tiers, the one-step kernel's queue overflow, the blob distances
  struct QbgScratch {
    uint32_t* bitmaps = nullptr;
    unsigned long long* exact_ovf = nullptr;
    unsigned long long* qbg_ovf = nullptr;
    float* blob_dist = nullptr;
    size_t grid = 0;
  };
  std::vector<QbgScratch> qbg_scratch_;
  void* d_robj_ = nullptr;                 // refinement objects on the device (uploaded on first use)
  // coalescing of single-query calls
  struct CoalescedCall {
    std::vector<uint8_t> row;
    SearchArgs args;
    SearchOutput out;
    bool done = false;
    std::string error;
  };
  // A lane is one exact-kernel launch in flight: its own stream, visited bitmaps and
  // overflow lists (kLaneCtas CTAs), and pinned query staging.  Several lanes run at
  // once, so one slow query does not hold back the calls that arrive after it.
  struct CoLane {
    cudaStream_t stream = nullptr;
    uint32_t* bitmaps = nullptr;
    unsigned long long* overflow = nullptr;
    void* staging = nullptr;               // pinned: rows, parameters, seeds | results, counts, stats
    void* dev = nullptr;                   // the same layout on the device
    size_t staging_bytes = 0;
    bool busy = false;
  };
  static constexpr size_t kCoLanes = 16, kLaneCtas = 8;
  std::mutex co_mu_;
  std::condition_variable co_cv_;
  std::vector<std::shared_ptr<CoalescedCall>> co_pending_;
  CoLane co_lanes_[kCoLanes];
  size_t co_nlanes_ = kCoLanes;            // lanes in use (1..kCoLanes)
  std::atomic<uint64_t> co_queries_{0}, co_launches_{0};
  void run_coalesced(std::vector<std::shared_ptr<CoalescedCall>>& batch, CoLane& lane);
  QbgScratch& qbg_slot(size_t slot, size_t grid, cudaStream_t stream);
  size_t qbg_grid_ = 0;
  uint32_t qbg_ocap_ = 0;
  // quantized graph
  HostQG qg_;
  bool qg_loaded_ = false;
  DevQG dqg_;
  std::vector<void*> qg_buffers_;
  int device_ = 0;
  cudaStream_t stream_ = nullptr;
  std::mutex mu_;
  std::mutex staging_mu_;                                 // the pinned query staging of search()
  void* staging_ = nullptr;
  size_t staging_bytes_ = 0;
  uint64_t launches_ = 0;
  // device data
  void* d_objects_ = nullptr;
  uint32_t* d_offsets_ = nullptr;
  uint32_t* d_edges_ = nullptr;
  DevInternal* d_internals_ = nullptr;
  void* d_pivots_ = nullptr;
  uint8_t* d_present_ = nullptr;
  uint32_t* d_seed_off_ = nullptr;
  uint32_t* d_seed_ids_ = nullptr;
  std::map<size_t, uint32_t> seed_tables_;
  std::vector<uint32_t> h_seed_off_, h_seed_ids_;
  uint32_t nleaves_ = 0;
  // scratch (grown on demand, reused across calls)
  uint32_t* d_bitmaps_ = nullptr;
  unsigned long long* d_overflow_ = nullptr;
  size_t bitmap_grid_ = 0;
  static constexpr uint32_t kOverflowCapacity = 65536;   // candidate keys per CTA beyond shared memory
  static constexpr uint32_t kSpillCapacity = 32768;
  std::vector<FastScratch> fast_scratch_ = std::vector<FastScratch>(1);
  void* d_bf16_ = nullptr;                                // bf16 copy of float object rows
  void* d_sq8_ = nullptr;                                 // 8-bit codes of float object rows
  std::once_flag sq8_once_;                               // the statistics are computed once
  bool sq8_lossless_ = false;
  float sq8_offset_ = 0.f, sq8_scale_ = 1.f;
  FastTuning tuning_;
  DevGraph dev_;
  void ensure_tc_rows();
  void ensure_tc_rows8();
  TcState* tc_ = nullptr;
  size_t tc_first_rows_ = 0;
  bool tc_graphs_ = false;
  uint32_t tc_row_begin_ = 0, tc_row_end_ = 0;
};

}  // namespace ngtg
