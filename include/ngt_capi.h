/*
 * C ABI of the GB300 NGT graph-search library (libngtgpu.so).
 *
 * Drop-in subset of NGT's C API: the types and the search-side functions below
 * keep the exact names, signatures, struct layouts, ownership and error
 * conventions of the reference header lib/NGT/Capi.h, so a program (or a
 * ctypes / cgo binding) built against NGT links against this library
 * unchanged for opening an index and searching it.  Index construction and
 * property editing stay with the reference tools.
 *
 * Conventions kept from the reference (lib/NGT/Capi.cpp):
 *   - functions return false / NULL / 0 on error and write a message into the
 *     NGTError object (or to stderr when the error object is NULL);
 *   - object ids are 1-based; results come back ascending by (distance, id);
 *   - a negative radius means "no radius" (FLT_MAX);
 *   - search clears and fills the caller's NGTObjectDistances.
 */
#pragma once

#ifdef __cplusplus
extern "C" {
#endif

#include <stdio.h>
#include <stdint.h>
#include <stdbool.h>

/* lib/NGT/Capi.h:27-34 */
typedef unsigned int ObjectID;
typedef void *NGTIndex;
typedef void *NGTProperty;
typedef void *NGTObjectSpace;
typedef void *NGTObjectDistances;
typedef void *NGTError;
typedef void NGTFloat16;

/* lib/NGT/Capi.h:36-39 */
typedef struct {
  ObjectID id;
  float distance;
} NGTObjectDistance;

/* lib/NGT/Capi.h:41-48 */
typedef struct {
  float *query;
  size_t size;      /* # of returned objects */
  float epsilon;
  float accuracy;   /* expected accuracy (accuracy tables are not supported; ignored) */
  float radius;
  size_t edge_size; /* # of edges to explore for each node */
} NGTQuery;

/* lib/NGT/Capi.h:50-55 */
typedef struct {
  size_t size;
  float epsilon;
  float radius;
  size_t edge_size;
} NGTQueryParameters;

/* lib/NGT/Capi.h:57-70 */
typedef struct {
  float *query;
  NGTQueryParameters params;
} NGTQueryFloat;

typedef struct {
  uint8_t *query;
  NGTQueryParameters params;
} NGTQueryUint8;

typedef struct {
  NGTFloat16 *query;
  NGTQueryParameters params;
} NGTQueryFloat16;

/* Open / close.  Replaces lib/NGT/Capi.h:160-162 (impl lib/NGT/Capi.cpp:41-69)
 * and ngt_close_index (lib/NGT/Capi.h:322).  ngt_open_index searches with the
 * updatable-graph semantics (NeighborhoodGraph::search), the read-only open
 * with searchReadOnlyGraph's, as the reference does. */
NGTIndex ngt_open_index(const char *, NGTError);
NGTIndex ngt_open_index_as_read_only(const char *, NGTError);
void ngt_close_index(NGTIndex);

/* Number of objects in the index.  Replaces lib/NGT/Capi.h:376
 * (impl lib/NGT/Capi.cpp:1672-1681). */
uint32_t ngt_get_number_of_objects(NGTIndex, NGTError);

/* Graph search.  Replaces lib/NGT/Capi.h:236-256 (impl lib/NGT/Capi.cpp:534-800). */
bool ngt_search_index(NGTIndex, double *, int32_t, size_t, float, float, NGTObjectDistances, NGTError);
bool ngt_search_index_as_float(NGTIndex, float *, int32_t, size_t, float, float, NGTObjectDistances, NGTError);
bool ngt_search_index_as_uint8(NGTIndex, uint8_t *, int32_t, size_t, float, float, NGTObjectDistances, NGTError);
bool ngt_search_index_as_float16(NGTIndex, NGTFloat16 *, int32_t, size_t, float, float, NGTObjectDistances,
                                 NGTError);
bool ngt_search_index_with_query(NGTIndex, NGTQuery, NGTObjectDistances, NGTError);
void ngt_initialize_query_parameters(NGTQueryParameters *);
bool ngt_search_index_with_query_float(NGTIndex, NGTQueryFloat, NGTObjectDistances, NGTError);
bool ngt_search_index_with_query_uint8(NGTIndex, NGTQueryUint8, NGTObjectDistances, NGTError);
bool ngt_search_index_with_query_float16(NGTIndex, NGTQueryFloat16, NGTObjectDistances, NGTError);

/* Exhaustive search.  Replaces lib/NGT/Capi.h:257-262 (impl lib/NGT/Capi.cpp:817-930). */
bool ngt_linear_search_index(NGTIndex, double *, int32_t, size_t, NGTObjectDistances, NGTError);
bool ngt_linear_search_index_as_float(NGTIndex, float *, int32_t, size_t, NGTObjectDistances, NGTError);
bool ngt_linear_search_index_with_query(NGTIndex, NGTQuery, NGTObjectDistances, NGTError);

/* Results.  Replaces lib/NGT/Capi.h:234,263-267,318 (impl lib/NGT/Capi.cpp:503-512,925-960,1410-1413). */
NGTObjectDistances ngt_create_empty_results(NGTError);
int32_t ngt_get_size(NGTObjectDistances, NGTError); /* deprecated in the reference */
uint32_t ngt_get_result_size(NGTObjectDistances, NGTError);
NGTObjectDistance ngt_get_result(const NGTObjectDistances, const uint32_t, NGTError);
void ngt_destroy_results(NGTObjectDistances);

/* Errors.  Replaces lib/NGT/Capi.h:330-336 (impl lib/NGT/Capi.cpp:1456-1480). */
NGTError ngt_create_error_object();
const char *ngt_get_error_string(const NGTError);
void ngt_clear_error_string(NGTError);
void ngt_destroy_error_object(NGTError);

#ifdef __cplusplus
}
#endif
