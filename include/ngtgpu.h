/*
 * Extensions of the GB300 NGT search library that have no counterpart in the
 * reference C API: batched search of many queries in one call (the
 * reference's only batch path is the OpenMP loop of ngtpy.Index.batch_search,
 * python/src/ngtpy.cpp:422-458) and device-resident variants for callers that
 * keep queries and results in GPU memory.
 *
 * Handles, result structs and error objects are the ones of ngt_capi.h.
 */
#pragma once
#include "ngt_capi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Kernel selection for the batched calls. */
#define NGTGPU_KERNEL_EXACT 0u     /* reference-order search, one query per CTA (results equal the reference's) */
#define NGTGPU_KERNEL_BATCHED 1u   /* warp per query, persistent, bf16 search rows for float objects,
                                      exact re-rank of the best candidates (checked by recall) */
#define NGTGPU_KERNEL_BATCHED_FP32 2u  /* the batched kernel on the full-precision rows */
#define NGTGPU_KERNEL_WIDE 3u      /* the same search with one query per 256-thread CTA: rows of an
                                      iteration copied to shared memory all at once (low latency per
                                      query; float L2 and uint8 L2 indexes) */

/* Per-query statistics: distance computations, expanded nodes, visited ids,
 * adjacency entries read, and status bits (1: candidate overflow tier full,
 * the result may differ from the reference's; 2: visited set moved to global
 * memory; 4: no seed; 8: tree error; 16: iteration bound). */
typedef struct {
  uint32_t distance_computations;
  uint32_t expansions;
  uint32_t visited;
  uint32_t edges_read;
  uint32_t status;
} NGTGPUQueryStats;

/* Dimension of the objects of an open index (the user dimension). */
int32_t ngtgpu_get_dimension(NGTIndex, NGTError);

/* Graph search of nq float queries (row-major nq x dim) in one call.
 * params holds nparams entries: 1 (shared by every query) or nq.  Results of
 * query i are written to results[i*kmax .. i*kmax+counts[i]) ascending by
 * (distance, id); kmax must be >= every params[].size.  stats may be NULL. */
bool ngtgpu_search_batch_float(NGTIndex, const float *queries, size_t nq, int32_t dim,
                               const NGTQueryParameters *params, size_t nparams, NGTObjectDistance *results,
                               size_t kmax, uint32_t *counts, NGTGPUQueryStats *stats, uint32_t kernel, NGTError);

/* ngtgpu_search_batch_float with the search container's expected accuracy, as the
 * reference's C++ API takes it (NGT::SearchContainer::setExpectedAccuracy; the C API
 * has no way to pass it, and ignores NGTQuery.accuracy): accuracy > 0 replaces
 * epsilon by the epsilon the index's AccuracyTable property gives for it
 * (AccuracyTable::getEpsilon, lib/NGT/Index.h:442-472; GraphIndex::search,
 * lib/NGT/Index.h:1700-1702), before the edge size and the exploration coefficient
 * are derived from it.  An index without a table fails the call. */
typedef struct {
  size_t size;
  float epsilon;
  float accuracy;   /* expected accuracy; <= 0: use epsilon */
  float radius;     /* < 0: no radius (FLT_MAX); a range search returns at most size objects within it */
  size_t edge_size;
  float refinement_expansion;  /* >= 1 (every query of the call): the search container's refinement
                                  expansion of the C++ API (GraphIndex::search(SearchQuery&),
                                  lib/NGT/Index.h:1146-1236): size x expansion results re-ranked by exact
                                  distances over the index's float refinement objects (robj; L1, L2,
                                  angle and cosine distances) to the size best; 0: none */
} NGTGPUSearchParameters;
bool ngtgpu_search_batch_ex_float(NGTIndex, const float *queries, size_t nq, int32_t dim,
                                  const NGTGPUSearchParameters *params, size_t nparams, NGTObjectDistance *results,
                                  size_t kmax, uint32_t *counts, NGTGPUQueryStats *stats, uint32_t kernel, NGTError);

/* Size in bytes of one converted query row (padded object layout). */
size_t ngtgpu_query_row_bytes(NGTIndex, NGTError);

/* Converts nq float queries to the padded object rows the device calls take
 * (object type, normalisation and augmentation as the index requires). */
bool ngtgpu_convert_queries_float(NGTIndex, const float *queries, size_t nq, int32_t dim, void *rows_out,
                                  NGTError);

/* Same search as ngtgpu_search_batch_float on device memory: d_rows holds nq
 * converted rows, d_results / d_counts / d_stats are device buffers, and the
 * work is queued on `stream` (a cudaStream_t; NULL = the index's own stream)
 * without synchronising. */
bool ngtgpu_search_batch_device(NGTIndex, const void *d_rows, size_t nq, const NGTQueryParameters *params,
                                size_t nparams, NGTObjectDistance *d_results, size_t kmax, uint32_t *d_counts,
                                NGTGPUQueryStats *d_stats, void *stream, uint32_t kernel, NGTError);

/* Tuning of the batched kernel for this index (0 = automatic): candidate
 * list length (rounded up to a power of two, >= size+1, <= 1024; automatic:
 * 4 x size, at least 256 for NGTGPU_KERNEL_WIDE and 512 for the warp kernel,
 * at most 1024, so the batched kernels take result sizes up to 1023), nodes
 * expanded per iteration (<= 16), and re-ranked candidates per query as a
 * multiple of size. */
bool ngtgpu_set_batched_tuning(NGTIndex, uint32_t list_capacity, uint32_t parents, float rerank_factor, NGTError);
/* Rows each lane group of the batched kernel keeps in flight while computing
 * distances: 4 (default), 6 or 8 (float L2 indexes; deeper pipelines trade
 * registers, so fewer CTAs per SM).  0 restores the default. */
bool ngtgpu_set_batched_rows_in_flight(NGTIndex, uint32_t rows, NGTError);

/* All knobs of the batched kernel at once (0 = automatic for each).  The
 * (rows_in_flight, ctas_per_sm) pairs built are (4, 5) for every index type and
 * (6, 4), (8, 4), (6, 5), (4, 6), (2, 8) for float L2 indexes; a search with a
 * pair that is not built fails with an error.  neighbour_capacity bounds the
 * neighbour slots of one iteration (each parent reads at most
 * neighbour_capacity / parents edges) and sets the shared memory per query.
 * parents: at most 32 (the warp-per-query kernel uses at most 16 of them).
 * NGTGPU_KERNEL_WIDE reads rows_in_flight as the rows each lane group scores at
 * once from shared memory (1, 2 or 4; default 4). */
typedef struct {
  uint32_t list_capacity;
  uint32_t parents;
  float rerank_factor;
  uint32_t rows_in_flight;
  uint32_t ctas_per_sm;
  uint32_t neighbour_capacity;
  uint32_t cta_threads;        /* NGTGPU_KERNEL_WIDE: 64, 128 or 256 threads per query (64: float L2 only) */
  uint32_t stage_kilobytes;    /* NGTGPU_KERNEL_WIDE: shared memory for staged rows (default 64) */
  uint32_t l2_policy;          /* NGTGPU_KERNEL_WIDE: 1 plain caching, 2 visited bitmaps kept in L2,
                                  3 (default) as 2 and staged rows streamed through L2 (evict-first) */
  uint32_t search_rows;        /* NGTGPU_KERNEL_WIDE, float L2 objects: 0 automatic (8-bit codes when they
                                  are lossless, else bf16), 1 bf16, 2 8-bit codes */
} NGTGPUBatchedTuning;
bool ngtgpu_set_batched_tuning_ex(NGTIndex, const NGTGPUBatchedTuning *tuning, NGTError);

/* Autotuner of the batched kernels for this index, a result size k and an epsilon
 * (or, epsilon < 0, the smallest epsilon of a sweep from 0 to 0.3 reaching the floor,
 * chosen per configuration and returned in *best_epsilon, which may be NULL):
 * a fixed list of configurations (the warp-per-query kernel's row pipelines and
 * register budgets, the CTA-per-query kernel's threads, staged rows and parents per
 * step) is timed on the nq sample queries (CUDA events, median of three launches),
 * and the fastest whose tie-aware recall@k against the exhaustive search of the
 * sample is >= recall_floor -- or, with recall_floor < 0, >= the exact-order kernel's
 * recall at the same epsilon -- becomes the index's tuning.  *best and *best_kernel
 * (NGTGPU_KERNEL_BATCHED or NGTGPU_KERNEL_WIDE) receive it, *best_qps (may be NULL)
 * its queries/s on the sample.  With the environment variable NGTGPU_TUNE_CACHE
 * naming a file, results are kept there as JSON keyed by (objects, dimension, object
 * type, distance, k, epsilon) and reused without timing.  Fails when no configuration
 * reaches the floor. */
bool ngtgpu_autotune(NGTIndex, const float *queries, size_t nq, int32_t dim, size_t k, float epsilon,
                     float recall_floor, NGTGPUBatchedTuning *best, uint32_t *best_kernel, float *best_qps,
                     float *best_epsilon, NGTError);

/* Exact graph search (results equal ngtgpu_search_batch_device with
 * NGTGPU_KERNEL_EXACT) that allocates no device memory, for callers that cannot
 * call cudaMalloc while they search: hosts that own and budget all device
 * memory themselves, and serving paths that must never enter the allocator.
 * No counterpart in the reference.  Its scratch (query parameters, seed lists,
 * per-CTA visited bitmaps and candidate overflow tiers) lives in one fixed
 * 32 MiB device array.  The library reserves that array on a GPU when it opens
 * the first index there (the array's address lookup loads its module) and holds
 * it until the process exits; the search itself reserves nothing.  Calls share
 * the array: calls that overlap on the GPU race.  A call is rejected with an
 * error when its parameters plus one CTA's scratch exceed 32 MiB, and when a
 * query's result size has no seed table yet (run one regular search with that
 * size on the index first).  Buffers are device memory, as in
 * ngtgpu_search_batch_device.  The call is synchronous: it copies its
 * parameters from host memory and returns after the search completed. */
bool ngtgpu_search_exact_noalloc(NGTIndex, const void *d_rows, size_t nq, const NGTQueryParameters *params,
                                 size_t nparams, NGTObjectDistance *d_results, size_t kmax, uint32_t *d_counts,
                                 NGTGPUQueryStats *d_stats, void *stream, NGTError);

/* Exhaustive k-NN with a tensor-core pre-selection (the precision path of
 * ngt_linear_search_index, lib/NGT/Capi.cpp; exact search semantics of
 * ObjectSpaceRepository::linearSearch, lib/NGT/ObjectSpaceRepository.h:860-922).
 * Float objects with L2, inner product, cosine, angle or their normalized forms.
 * Every (query, object) pair is scored on the tensor cores from bf16 copies with
 * fp32 accumulation; the `candidates` best scores per query (0: max(4 x size,
 * 64); at most 4096, at least size) are re-ranked with the index's exact
 * comparator on the fp32 objects, and the `size` nearest are returned ascending
 * by (distance, id), with the distances of the plain linear search.  The ids
 * equal the plain linear search's whenever the true nearest objects are among
 * the candidates.  d_status[q] bit 1: the query's candidate list overflowed (the
 * result may miss objects).  Device buffers; d_rows holds nq rows converted by
 * ngtgpu_convert_queries_float; queued on `stream` (NULL = the index's stream),
 * returns after completion. */
bool ngtgpu_linear_search_tc_device(NGTIndex, const void *d_rows, size_t nq, size_t size, size_t candidates,
                                    NGTObjectDistance *d_results, size_t kmax, uint32_t *d_counts,
                                    uint32_t *d_status, void *stream, NGTError);
/* The same over host buffers: nq float queries (row-major nq x dim), results of
 * query i in results[i*kmax ..], counts[i], status[i]. */
bool ngtgpu_linear_search_tc_float(NGTIndex, const float *queries, size_t nq, int32_t dim, size_t size,
                                   size_t candidates, NGTObjectDistance *results, size_t kmax, uint32_t *counts,
                                   uint32_t *status, NGTError);
/* Precision of the tensor-core scores, and options, of the _ex calls below. */
#define NGTGPU_TC_BF16 0u        /* bf16 copies, fp32 accumulation (kind::f16) */
#define NGTGPU_TC_FP8 1u         /* per-row and per-query scaled E4M3 copies, fp32 accumulation
                                    (kind::f8f6f4): half the bytes and twice the tensor rate of bf16,
                                    coarser scores, so more candidates are needed for the same ids */
#define NGTGPU_TC_FP64_TIES 1u   /* flag: the candidates whose fp32 distance ties the size-th one within
                                    the fp32 evaluation error (1e-4 x max(d, 1)) are ordered by their FP64
                                    distance at the cut, so the returned ids are the FP64 top `size` among
                                    the candidates (status bit 4: more than 64 such ties, fp32 order kept) */
#define NGTGPU_TC_PAIR 2u         /* flag: the score kernel runs on the two-SM MMA (cta_group::2): pairs
                                    of CTAs compute 256-row x 256-query tiles, each staging its own rows
                                    and half of the query tile; the scores and results are the same */
/* ngtgpu_linear_search_tc_device / _float with a score precision and flags. */
bool ngtgpu_linear_search_tc_ex(NGTIndex, const void *d_rows, size_t nq, size_t size, size_t candidates,
                                uint32_t precision, uint32_t flags, NGTObjectDistance *d_results, size_t kmax,
                                uint32_t *d_counts, uint32_t *d_status, void *stream, NGTError);
bool ngtgpu_linear_search_tc_float_ex(NGTIndex, const float *queries, size_t nq, int32_t dim, size_t size,
                                      size_t candidates, uint32_t precision, uint32_t flags,
                                      NGTObjectDistance *results, size_t kmax, uint32_t *counts, uint32_t *status,
                                      NGTError);
/* The approximate scores of the tensor-core pre-selection alone:
 * d_scores[q * ld + id] (ld >= the number of object slots, id 0 unused), larger
 * = closer: a * (q . x) + b over bf16 copies with a = 1, b = -|x|^2 / 2 for L2
 * and inner product, a = 1 / |x| for cosine and angle, a = 1 for the normalized
 * forms; -inf for id 0 and removed objects. */
bool ngtgpu_tc_scores_device(NGTIndex, const void *d_rows, size_t nq, float *d_scores, size_t ld, void *stream,
                             NGTError);
/* CUDA-event times in milliseconds of the last query batch (up to 16384
 * queries) of ngtgpu_linear_search_tc_*: [0] query conversion, dense part and
 * its selection, [1] the score kernel over the remaining objects (the
 * threshold filter), [2] the final exact re-rank. */
bool ngtgpu_tc_phase_times(NGTIndex, float *ms3, NGTError);
/* Objects scored densely before the per-query threshold filter of the
 * tensor-core search (rounded up to a multiple of 128, at least `candidates`,
 * at most 16384; 0 = automatic, 8192).  Results do not depend on it. */
bool ngtgpu_set_tc_first_rows(NGTIndex, size_t rows, NGTError);
/* enable != 0: ngtgpu_linear_search_tc_* on this handle capture their launch
 * sequence (about 2 launches per part of the objects, 17 for 1M objects) into a
 * CUDA graph on the first call of a given shape, buffers and options (up to 8
 * kept) and replay it on later calls that match; ngtgpu_tc_phase_times then
 * reports a replay's whole time as [1].  A call on a stream that the caller is
 * capturing is recorded into the caller's capture.  enable = 0 (default):
 * launched directly; the kept graphs are released.  Results are the same. */
bool ngtgpu_set_tc_graphs(NGTIndex, int enable, NGTError);
/* Row-range shard of the tensor-core exhaustive search: later ngtgpu_linear_search_tc_*
 * calls on this handle search objects [begin, end) only (begin a multiple of 128,
 * end 0 = through the last object; 0, 0 restores the whole index).  Each GPU of a
 * row-range split searches its shard for the size best and a host merge by
 * (distance, id) gives the whole index's result (ngt_gb300/shard.py). */
bool ngtgpu_set_tc_row_range(NGTIndex, size_t begin, size_t end, NGTError);
/* Serving loop (continuous batching).  A server keeps up to `inflight`
 * batched-kernel launches on the GPU at once, each on its own stream and
 * scratch set; requests submitted from any thread while others run join the
 * next launch that has room (`max_batch_queries` queries per launch), so their
 * work overlaps on the device.  A request holds 1..max_batch_queries queries
 * with one parameter block or one per query, result sizes up to max_k.
 * ngtgpu_server_submit copies the queries and returns a ticket (>= 0, or -1 on
 * error); ngtgpu_server_wait blocks until that request completed, writes its
 * results (results[q*kmax ..], counts[q]) and its latency from submission to
 * completion in milliseconds.  A request's results do not depend on what else
 * is in flight. */
typedef void *NGTGPUServer;
NGTGPUServer ngtgpu_server_create(NGTIndex, uint32_t max_batch_queries, uint32_t inflight, uint32_t max_k,
                                  NGTError);
/* The same with the kernel the launches use: NGTGPU_KERNEL_BATCHED (throughput),
 * NGTGPU_KERNEL_BATCHED_FP32, or NGTGPU_KERNEL_WIDE (lowest latency per query). */
NGTGPUServer ngtgpu_server_create_ex(NGTIndex, uint32_t max_batch_queries, uint32_t inflight, uint32_t max_k,
                                     uint32_t kernel, NGTError);
int64_t ngtgpu_server_submit(NGTGPUServer, const float *queries, size_t nq, int32_t dim,
                             const NGTQueryParameters *params, size_t nparams, NGTError);
bool ngtgpu_server_wait(NGTGPUServer, int64_t ticket, NGTObjectDistance *results, size_t kmax, uint32_t *counts,
                        double *latency_ms, NGTError);
void ngtgpu_server_destroy(NGTGPUServer);
/* Admission deadlines and cancellation (any server).  A request not launched within
 * deadline_ms of its submission completes unlaunched: its wait returns false with
 * "deadline exceeded before launch".  ngtgpu_server_submit_deadline sets it per
 * request; ngtgpu_server_set_deadline sets the default of later submits (<= 0: none).
 * ngtgpu_server_cancel withdraws a request not yet launched (true; its wait returns
 * false with "cancelled"); a request on the device runs to completion (false). */
int64_t ngtgpu_server_submit_deadline(NGTGPUServer, const float *queries, size_t nq, int32_t dim,
                                      const NGTQueryParameters *params, size_t nparams, double deadline_ms,
                                      NGTError);
bool ngtgpu_server_set_deadline(NGTGPUServer, double deadline_ms, NGTError);
bool ngtgpu_server_cancel(NGTGPUServer, int64_t ticket, NGTError);

/* The single-query graph searches (ngt_search_index, _as_float, _as_uint8,
 * _as_float16, _with_query*) of concurrent host threads are coalesced: up to 16
 * exact-order launches run at once, each on its own stream and scratch; a caller
 * that finds one of them free launches every waiting query at once, and callers
 * arriving while all 16 run wait and are launched together by the next free one,
 * so a loop of these calls over many threads (ngtpy's batch_search pattern) fills
 * the GPU.  Every result equals
 * a lone call's.  The queries coalesced so far, and the launches they took. */
bool ngtgpu_coalescing_stats(NGTIndex, uint64_t *queries, uint64_t *launches, NGTError);
/* How many coalesced launches may run at once (1..16, default 16). */
bool ngtgpu_set_coalescing_lanes(NGTIndex, uint32_t lanes, NGTError);

/* ONNG construction (replaces `ngt reconstruct-graph -m S -o outgoing -i incoming -E
 * min_edges anng onng`, GraphOptimizer::execute, lib/NGT/GraphOptimizer.h:268-367):
 * copies the index directory anng_index to onng_index (which must not exist), rebuilds
 * its graph with GraphReconstructor::reconstructGraph and adjustPathsEffectively
 * (lib/NGT/GraphReconstructor.h:200-409,645-813) -- the same graph, edge for edge --
 * with the path-adjustment candidates found on the GPU, and sets GraphType ONNG.
 * outgoing / incoming < 0 take the index's OutgoingEdge / IncomingEdge; both 0 only
 * adjust the paths of the ANNG.  The reference command's later search-parameter
 * optimization (ngt optimize-search-parameters) is not part of it. */
bool ngtgpu_build_onng(const char *anng_index, const char *onng_index, int32_t outgoing, int32_t incoming,
                       int64_t min_edges, NGTError);

/* Number of kernel launches issued by this index since it was opened. */
uint64_t ngtgpu_kernel_launches(NGTIndex, NGTError);

/* Search rows NGTGPU_KERNEL_WIDE uses for this index under its tuning: 0 the
 * objects themselves, 1 bf16 copies, 2 8-bit codes rint((x - min) / s) with s = 1
 * when every coordinate is an integer and they span at most 256 values (the
 * codes are then lossless), else (max - min) / 255.  UINT32_MAX on error. */
uint32_t ngtgpu_get_wide_search_rows(NGTIndex, NGTError);

#ifdef __cplusplus
}
#endif
