/*
 * C ABI of the GB300 quantized-graph (NGTQG) search in libngtgpu.so.
 *
 * Drop-in subset of NGT's quantized C API, lib/NGT/NGTQ/Capi.h: the QG types
 * and search functions keep the reference's names, signatures, struct layouts
 * and error conventions.  An index is quantized with the reference tools
 * (`qbg create-qg` + `qbg build-qg`, or ngtqg_quantize) and opened here
 * unchanged; the search runs on the GPU and returns the reference's results
 * (same ids and distances, in the same order).  ngtqg_quantize and the QBG
 * functions of that header are not provided.
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

#ifdef __cplusplus
}
#endif
