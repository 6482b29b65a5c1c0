/*
 * C ABI of the GB300 quantized-graph (NGTQG) search in libngtgpu.so.
 *
 * Drop-in subset of NGT's quantized C API, lib/NGT/NGTQ/Capi.h: the QG types
 * and search functions keep the reference's names, signatures, struct layouts
 * and error conventions.  An index is quantized with the reference tools
 * (`qbg create-qg` + `qbg build-qg`, or ngtqg_quantize) and opened here
 * unchanged; the search runs on the GPU and returns the reference's results
 * (same ids and distances, in the same order).  The QBG search subset
 * (qbg_open_index .. qbg_get_dimension) follows the same rule for indexes built
 * by `qbg create` / `qbg append` / `qbg build`.  Index construction
 * (ngtqg_quantize, qbg_create, qbg_append_object, qbg_build_index, ...) stays
 * with the reference.
 */
#pragma once

#ifdef __cplusplus
extern "C" {
#endif

#include <stdint.h>
#include <stdbool.h>
#include "ngt_capi.h"

/* lib/NGT/NGTQ/Capi.h:27-30 */
typedef void *NGTQGIndex;
typedef NGTError NGTQGError;

/* lib/NGT/NGTQ/Capi.h:33-39 */
typedef struct {
  float *query;
  size_t size;              /* number of results */
  float epsilon;
  float result_expansion;   /* size x this many candidates are kept, then re-ranked exactly (>= 1) */
  float radius;
} NGTQGQuery;

/* lib/NGT/NGTQ/Capi.h:41-46 */
typedef struct {
  size_t size;
  float epsilon;
  float result_expansion;
  float radius;
} NGTQGQueryParameters;

/* lib/NGT/NGTQ/Capi.h:48-61 */
typedef struct {
  float *query;
  NGTQGQueryParameters params;
} NGTQGQueryFloat;

typedef struct {
  uint8_t *query;
  NGTQGQueryParameters params;
} NGTQGQueryUint8;

typedef struct {
  NGTFloat16 *query;
  NGTQGQueryParameters params;
} NGTQGQueryFloat16;

/* Opens <index_path> and its quantized graph <index_path>/qg (float objects,
 * L2); replaces lib/NGT/NGTQ/Capi.h:68 / Capi.cpp:61-73. */
NGTQGIndex ngtqg_open_index(const char *index_path, NGTQGError error);
/* lib/NGT/NGTQ/Capi.h:70 */
void ngtqg_close_index(NGTQGIndex index);
/* Defaults size 20, epsilon 0.03, result_expansion 3.0, radius FLT_MAX
 * (lib/NGT/NGTQ/Capi.cpp:46-59). */
void ngtqg_initialize_query_parameters(NGTQGQueryParameters *parameters);
void ngtqg_initialize_query(NGTQGQuery *query);
/* lib/NGT/NGTQ/Capi.h:80-86: one query; results ascending by (distance, id). */
bool ngtqg_search_index(NGTQGIndex index, NGTQGQuery query, NGTObjectDistances results, NGTQGError error);
bool ngtqg_search_index_float(NGTQGIndex index, NGTQGQueryFloat query, NGTObjectDistances results,
                              NGTQGError error);
bool ngtqg_search_index_uint8(NGTQGIndex index, NGTQGQueryUint8 query, NGTObjectDistances results,
                              NGTQGError error);
bool ngtqg_search_index_float16(NGTQGIndex index, NGTQGQueryFloat16 query, NGTObjectDistances results,
                                NGTQGError error);

/* ---- extensions (no reference counterpart) ---------------------------------
 * Many queries in one launch (replaces a loop over ngtqg_search_index_float):
 * queries nq x dim row-major; params one per query or one for all; results
 * nq x kmax (kmax >= every size); counts nq; stats NULL or nq entries of
 * NGTGPUQueryStats (declared in ngtgpu.h, five uint32 counters). */
bool ngtqg_gpu_search_batch_float(NGTQGIndex index, const float *queries, size_t nq, int32_t dim,
                                  const NGTQGQueryParameters *params, size_t nparams, NGTObjectDistance *results,
                                  size_t kmax, uint32_t *counts, void *stats, NGTQGError error);
/* The same over device-resident query rows (converted with
 * ngtgpu_convert_queries_float), device outputs and a cudaStream_t (NULL: the
 * index's stream); returns after the launch is queued. */
bool ngtqg_gpu_search_batch_device(NGTQGIndex index, const void *d_rows, size_t nq,
                                   const NGTQGQueryParameters *params, size_t nparams, NGTObjectDistance *d_results,
                                   size_t kmax, uint32_t *d_counts, void *d_stats, void *stream, NGTQGError error);
/* The same two with a kernel: NGTGPU_KERNEL_EXACT (the reference's expansion order,
 * results equal ngtqg_search_index_float's) or NGTGPU_KERNEL_WIDE (relaxed order:
 * several parents per step, the quantized distances and the exact re-rank
 * unchanged; recall at a given epsilon at least the exact kernel's in the tests).
 * The relaxed kernel takes its parents per step and list capacity from the
 * index's batched tuning (ngtgpu_set_batched_tuning_ex; defaults 8 and 4 x the
 * result-set size, at least 256). */
bool ngtqg_gpu_search_batch_ex_float(NGTQGIndex index, const float *queries, size_t nq, int32_t dim,
                                     const NGTQGQueryParameters *params, size_t nparams, NGTObjectDistance *results,
                                     size_t kmax, uint32_t *counts, void *stats, uint32_t kernel, NGTQGError error);
bool ngtqg_gpu_search_batch_ex_device(NGTQGIndex index, const void *d_rows, size_t nq,
                                      const NGTQGQueryParameters *params, size_t nparams,
                                      NGTObjectDistance *d_results, size_t kmax, uint32_t *d_counts, void *d_stats,
                                      void *stream, uint32_t kernel, NGTQGError error);

/* ---- quantized blob graph (QBG) search, lib/NGT/NGTQ/Capi.h ---------------- */

/* lib/NGT/NGTQ/Capi.h:101-103 */
typedef void *QBGIndex;
typedef NGTError QBGError;
typedef NGTObjectDistances QBGObjectDistances;

/* lib/NGT/NGTQ/Capi.h:129-137 */
typedef struct {
  size_t number_of_results;
  float epsilon;
  float blob_epsilon;
  float result_expansion;          /* >= 1: number_of_results x this many results (quantized distances) */
  size_t number_of_explored_blobs;
  size_t number_of_edges;
  float radius;                    /* accepted and ignored, as by the reference */
} QBGQueryParameters;

/* lib/NGT/NGTQ/Capi.h:139-148 */
typedef struct {
  float *query;
  size_t number_of_results;
  float epsilon;
  float blob_epsilon;
  float result_expansion;
  size_t number_of_explored_blobs;
  size_t number_of_edges;
  float radius;
} QBGQuery;

/* lib/NGT/NGTQ/Capi.h:150-163 */
typedef struct {
  float *query;
  QBGQueryParameters params;
} QBGQueryFloat;

typedef struct {
  uint8_t *query;
  QBGQueryParameters params;
} QBGQueryUint8;

typedef struct {
  NGTFloat16 *query;
  QBGQueryParameters params;
} QBGQueryFloat16;

/* Opens a built QBG index (its blobs and the global index in <path>/global);
 * replaces lib/NGT/NGTQ/Capi.h:183 / Capi.cpp:239-250.  An index that has not
 * been built is rejected here whatever `prebuilt` says. */
QBGIndex qbg_open_index(const char *index_path, bool prebuilt, QBGError error);
/* lib/NGT/NGTQ/Capi.h:185 */
void qbg_close_index(QBGIndex index);
/* Defaults: 20 results, epsilon 0.1, blob_epsilon 0, result_expansion 3,
 * 256 explored blobs, 0 edges (all), radius 0 (lib/NGT/NGTQ/Capi.cpp:528-547). */
void qbg_initialize_query_parameters(QBGQueryParameters *parameters);
void qbg_initialize_query(QBGQuery *query);
/* lib/NGT/NGTQ/Capi.h:205-211: one query of the genuine dimension; results
 * ascending by (distance, id), quantized distances. */
bool qbg_search_index(QBGIndex index, QBGQuery query, QBGObjectDistances results, QBGError error);
bool qbg_search_index_float(QBGIndex index, QBGQueryFloat query, QBGObjectDistances results, QBGError error);
bool qbg_search_index_uint8(QBGIndex index, QBGQueryUint8 query, QBGObjectDistances results, QBGError error);
bool qbg_search_index_float16(QBGIndex index, QBGQueryFloat16 query, QBGObjectDistances results, QBGError error);
/* lib/NGT/NGTQ/Capi.h:115-119 */
uint32_t qbg_get_result_size(QBGObjectDistances results, NGTError error);
NGTObjectDistance qbg_get_result(const QBGObjectDistances results, const uint32_t idx, NGTError error);
void qbg_destroy_results(QBGObjectDistances results);
/* lib/NGT/NGTQ/Capi.h:226: the genuine (query) dimension. */
size_t qbg_get_dimension(QBGIndex index, QBGError error);

/* Extension: many queries in one launch (replaces a loop over
 * qbg_search_index_float): results nq x kmax with kmax >= every query's
 * number_of_results x result_expansion; counts nq; stats NULL or nq
 * NGTGPUQueryStats (the visited counter holds the blobs judged). */
bool qbg_gpu_search_batch_float(QBGIndex index, const float *queries, size_t nq, int32_t dim,
                                const QBGQueryParameters *params, size_t nparams, NGTObjectDistance *results,
                                size_t kmax, uint32_t *counts, void *stats, QBGError error);

/* Extension flags: the searches of the reference's C++ API (QBG::Index, as its `qbg
 * search` command and ngtpy drive it) rather than its C API's. */
#define NGTGPU_QBG_TWO_STEP 1u   /* searchInTwoSteps (lib/NGT/NGTQ/QuantizedBlobGraph.h:1190-1330): the
                                    number_of_explored_blobs blobs nearest the query, found by the global
                                    index's graph search (epsilon = blob_epsilon), are all judged in order;
                                    epsilon is not used.  Without it: searchInOneStep (:1332-1594). */
#define NGTGPU_QBG_REFINE 2u     /* result_expansion is the refinement expansion: the search keeps
                                    number_of_results x result_expansion (>= 1) quantized results, re-ranked by
                                    exact distances over the index's object list (qbg_dir/obj, loaded on the
                                    first refined call; refineDistances, QuantizedBlobGraph.h:1136-1185) to the
                                    number_of_results best.  The one-step search then thins its tree seeds with
                                    number_of_results, as the reference's container does. */
/* qbg_gpu_search_batch_float with the flags above (0: identical to it). */
bool qbg_gpu_search_batch_ex(QBGIndex index, const float *queries, size_t nq, int32_t dim,
                             const QBGQueryParameters *params, size_t nparams, uint32_t flags,
                             NGTObjectDistance *results, size_t kmax, uint32_t *counts, void *stats, QBGError error);
/* The same on device memory: d_rows holds nq float rows of the global index's
 * dimension (converted by ngtgpu_convert_queries_float on this handle), d_stats nq
 * NGTGPUQueryStats; queued on `stream` (NULL: the index's stream); returns after
 * completion. */
bool qbg_gpu_search_batch_device(QBGIndex index, const void *d_rows, size_t nq, const QBGQueryParameters *params,
                                 size_t nparams, uint32_t flags, NGTObjectDistance *d_results, size_t kmax,
                                 uint32_t *d_counts, void *d_stats, void *stream, QBGError error);

/* Extension: the serving loop of ngtgpu_server_create_ex over a QBG index.  Every
 * request runs the search the flags above select (0: the C API's one-step search);
 * up to `inflight` launches of up to max_batch_queries queries overlap on the
 * device, each lane with scratch reserved at creation (and the object list loaded,
 * with NGTGPU_QBG_REFINE).  Requests of 1..max_batch_queries queries with one
 * parameter block or one per query; results up to max_k per query (with the
 * refinement: number_of_results).  Returns an NGTGPUServer (ngtgpu.h): results are
 * taken with ngtgpu_server_wait and the loop ends with ngtgpu_server_destroy. */
void *ngtgpu_qbg_server_create(QBGIndex index, uint32_t max_batch_queries, uint32_t inflight, uint32_t max_k,
                               uint32_t flags, QBGError error);
int64_t ngtgpu_qbg_server_submit(void *server, const float *queries, size_t nq, int32_t dim,
                                 const QBGQueryParameters *params, size_t nparams, QBGError error);

/* The serving loop over a quantized graph (no reference counterpart; it serves the
 * requests of ngtqg_search_index_float, lib/NGT/NGTQ/Capi.h:68-83): each launch runs
 * the exact-order quantized-graph kernel over the waiting requests of one
 * shared-memory class, with per-lane visited bitmaps; results equal
 * ngtqg_search_index_float's.  Returns an NGTGPUServer (ngtgpu.h). */
void *ngtgpu_qg_server_create(NGTQGIndex index, uint32_t max_batch_queries, uint32_t inflight, uint32_t max_k,
                              NGTQGError error);
/* The same with the kernel each launch runs: NGTGPU_KERNEL_EXACT (above) or
 * NGTGPU_KERNEL_WIDE (the relaxed-order QG kernel of ngtqg_gpu_search_batch_ex_float;
 * a request's results equal that call's on the same queries). */
void *ngtgpu_qg_server_create_ex(NGTQGIndex index, uint32_t max_batch_queries, uint32_t inflight, uint32_t max_k,
                                 uint32_t kernel, NGTQGError error);
int64_t ngtgpu_qg_server_submit(void *server, const float *queries, size_t nq, int32_t dim,
                                const NGTQGQueryParameters *params, size_t nparams, NGTQGError error);

#ifdef __cplusplus
}
#endif
