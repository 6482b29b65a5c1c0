// C ABI: NGT's search-side C API (lib/NGT/Capi.cpp) over the GB300 engine,
// plus the batched extensions declared in include/ngtgpu.h.
//
// Error convention (lib/NGT/Capi.cpp:26-39): every entry point catches
// exceptions, writes "Capi : <function>() : ..." into the NGTError string (or
// stderr when it is NULL) and returns false / NULL / 0.  Nothing throws across
// the ABI.
#include <cfloat>
#include <climits>
#include <cstring>
#include <iostream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "engine.h"

extern "C" {
#include "../../include/ngt_capi.h"
#include "../../include/ngtgpu.h"
#include "../../include/ngtq_capi.h"
}

using ngtg::GraphEngine;
using ngtg::QBGArgs;
using ngtg::QGArgs;
using ngtg::GraphMode;
using ngtg::QueryType;
using ngtg::SearchArgs;
using ngtg::SearchOutput;

namespace {

typedef std::vector<NGTObjectDistance> Results;

void set_error(const std::stringstream& ss, NGTError error) {
  if (error != nullptr) {
    *static_cast<std::string*>(error) = ss.str();
  } else {
    std::cerr << ss.str() << std::endl;
  }
}

#define CAPI_PARAM_ERROR(error, what)                                                   \
  do {                                                                                  \
    std::stringstream ss_;                                                              \
    ss_ << "Capi : " << __FUNCTION__ << "() : parametor error: " << what;               \
    set_error(ss_, error);                                                              \
  } while (0)

#define CAPI_CATCH(error, retval)                                                       \
  catch (std::exception & err) {                                                        \
    std::stringstream ss_;                                                              \
    ss_ << "Capi : " << __FUNCTION__ << "() : Error: " << err.what();                   \
    set_error(ss_, error);                                                              \
    return retval;                                                                      \
  }

GraphEngine* engine(NGTIndex index) { return static_cast<GraphEngine*>(index); }

void fill_results(const SearchOutput& out, size_t q, NGTObjectDistances results) {
  Results& r = *static_cast<Results*>(results);
  r.clear();
  uint32_t n = out.counts[q];
  r.reserve(n);
  for (uint32_t i = 0; i < n; i++) {
    const ngtg::ObjDist& o = out.results[q * out.kmax + i];
    r.push_back(NGTObjectDistance{o.id, o.distance});
  }
}

SearchArgs make_args(size_t size, float epsilon, float radius, int64_t edge_size) {
  SearchArgs a;
  a.size = size;
  a.epsilon = epsilon;
  a.radius = radius < 0.0f ? FLT_MAX : radius;
  a.edge_size = edge_size;
  return a;
}

// The reference stores INT_MIN ("use the index default") in a size_t field.
int64_t edge_size_from_field(size_t v) {
  int e = (int)v;
  return e == INT_MIN ? -1 : (int64_t)e;
}

bool search_common(NGTIndex index, const void* query, QueryType qt, int32_t dim, size_t size, float epsilon,
                   float radius, int64_t edge_size, NGTObjectDistances results) {
  SearchArgs a = make_args(size, epsilon, radius, edge_size);
  SearchOutput out;
  engine(index)->search_one(query, qt, (size_t)dim, a, out);
  fill_results(out, 0, results);
  return true;
}

bool linear_common(NGTIndex index, const void* query, QueryType qt, int32_t dim, size_t size,
                   NGTObjectDistances results) {
  SearchOutput out;
  engine(index)->linear_search(query, qt, 1, (size_t)dim, size, out);
  fill_results(out, 0, results);
  return true;
}

}  // namespace

extern "C" {

NGTIndex ngt_open_index(const char* index_path, NGTError error) {
  try {
    if (index_path == nullptr) throw std::runtime_error("index path is NULL");
    return static_cast<NGTIndex>(new GraphEngine(index_path, GraphMode::Updatable));
  }
  CAPI_CATCH(error, nullptr)
}

NGTIndex ngt_open_index_as_read_only(const char* index_path, NGTError error) {
  try {
    if (index_path == nullptr) throw std::runtime_error("index path is NULL");
    return static_cast<NGTIndex>(new GraphEngine(index_path, GraphMode::ReadOnly));
  }
  CAPI_CATCH(error, nullptr)
}

void ngt_close_index(NGTIndex index) {
  if (index == nullptr) return;
  delete engine(index);
}

uint32_t ngt_get_number_of_objects(NGTIndex index, NGTError error) {
  if (index == nullptr) {
    CAPI_PARAM_ERROR(error, "index = " << index);
    return 0;
  }
  const auto& p = engine(index)->host().present;
  uint32_t n = 0;
  for (size_t i = 1; i < p.size(); i++) n += p[i];
  return n;
}

NGTObjectDistances ngt_create_empty_results(NGTError error) {
  try {
    return static_cast<NGTObjectDistances>(new Results());
  }
  CAPI_CATCH(error, nullptr)
}

#define SEARCH_ARGS_CHECK()                                                                                \
  if (index == nullptr || query == nullptr || results == nullptr || query_dim <= 0) {                      \
    CAPI_PARAM_ERROR(error, "index = " << index << " query = " << (const void*)query                      \
                                       << " results = " << results << " query_dim = " << query_dim);       \
    return false;                                                                                          \
  }

bool ngt_search_index(NGTIndex index, double* query, int32_t query_dim, size_t size, float epsilon, float radius,
                      NGTObjectDistances results, NGTError error) {
  SEARCH_ARGS_CHECK();
  try {
    return search_common(index, query, QueryType::Float64, query_dim, size, epsilon, radius, -1, results);
  }
  CAPI_CATCH(error, false)
}

bool ngt_search_index_as_float(NGTIndex index, float* query, int32_t query_dim, size_t size, float epsilon,
                               float radius, NGTObjectDistances results, NGTError error) {
  SEARCH_ARGS_CHECK();
  try {
    return search_common(index, query, QueryType::Float32, query_dim, size, epsilon, radius, -1, results);
  }
  CAPI_CATCH(error, false)
}

bool ngt_search_index_as_uint8(NGTIndex index, uint8_t* query, int32_t query_dim, size_t size, float epsilon,
                               float radius, NGTObjectDistances results, NGTError error) {
  SEARCH_ARGS_CHECK();
  try {
    return search_common(index, query, QueryType::Uint8, query_dim, size, epsilon, radius, -1, results);
  }
  CAPI_CATCH(error, false)
}

bool ngt_search_index_as_float16(NGTIndex index, NGTFloat16* query, int32_t query_dim, size_t size, float epsilon,
                                 float radius, NGTObjectDistances results, NGTError error) {
  SEARCH_ARGS_CHECK();
  try {
    return search_common(index, query, QueryType::Float16, query_dim, size, epsilon, radius, -1, results);
  }
  CAPI_CATCH(error, false)
}

bool ngt_search_index_with_query(NGTIndex index, NGTQuery query, NGTObjectDistances results, NGTError error) {
  if (index == nullptr || query.query == nullptr || results == nullptr) {
    CAPI_PARAM_ERROR(error, "index = " << index << " query = " << query.query << " results = " << results);
    return false;
  }
  try {
    int32_t dim = (int32_t)engine(index)->dimension();
    return search_common(index, query.query, QueryType::Float32, dim, query.size, query.epsilon, query.radius,
                         edge_size_from_field(query.edge_size), results);
  }
  CAPI_CATCH(error, false)
}

void ngt_initialize_query_parameters(NGTQueryParameters* params) {
  // lib/NGT/Capi.cpp:690-695
  params->epsilon = 0.1f;
  params->edge_size = (size_t)INT_MIN;
  params->radius = -1;
  params->size = 10;
}

#define WITH_QUERY_BODY(QT)                                                                                  \
  if (index == nullptr || query.query == nullptr || results == nullptr) {                                    \
    CAPI_PARAM_ERROR(error, "index = " << index << " query = " << (const void*)query.query                  \
                                       << " results = " << results);                                         \
    return false;                                                                                            \
  }                                                                                                          \
  try {                                                                                                      \
    int32_t dim = (int32_t)engine(index)->dimension();                                                       \
    return search_common(index, query.query, QT, dim, query.params.size, query.params.epsilon,               \
                         query.params.radius, edge_size_from_field(query.params.edge_size), results);        \
  }                                                                                                          \
  CAPI_CATCH(error, false)

bool ngt_search_index_with_query_float(NGTIndex index, NGTQueryFloat query, NGTObjectDistances results,
                                       NGTError error) {
  WITH_QUERY_BODY(QueryType::Float32)
}

bool ngt_search_index_with_query_uint8(NGTIndex index, NGTQueryUint8 query, NGTObjectDistances results,
                                       NGTError error) {
  WITH_QUERY_BODY(QueryType::Uint8)
}

bool ngt_search_index_with_query_float16(NGTIndex index, NGTQueryFloat16 query, NGTObjectDistances results,
                                         NGTError error) {
  WITH_QUERY_BODY(QueryType::Float16)
}

bool ngt_linear_search_index(NGTIndex index, double* query, int32_t query_dim, size_t size,
                             NGTObjectDistances results, NGTError error) {
  SEARCH_ARGS_CHECK();
  try {
    return linear_common(index, query, QueryType::Float64, query_dim, size, results);
  }
  CAPI_CATCH(error, false)
}

bool ngt_linear_search_index_as_float(NGTIndex index, float* query, int32_t query_dim, size_t size,
                                      NGTObjectDistances results, NGTError error) {
  SEARCH_ARGS_CHECK();
  try {
    return linear_common(index, query, QueryType::Float32, query_dim, size, results);
  }
  CAPI_CATCH(error, false)
}

bool ngt_linear_search_index_with_query(NGTIndex index, NGTQuery query, NGTObjectDistances results,
                                        NGTError error) {
  if (index == nullptr || query.query == nullptr || results == nullptr) {
    CAPI_PARAM_ERROR(error, "index = " << index << " query = " << query.query << " results = " << results);
    return false;
  }
  try {
    int32_t dim = (int32_t)engine(index)->dimension();
    return linear_common(index, query.query, QueryType::Float32, dim, query.size, results);
  }
  CAPI_CATCH(error, false)
}

int32_t ngt_get_size(NGTObjectDistances results, NGTError error) {
  if (results == nullptr) {
    CAPI_PARAM_ERROR(error, "results = " << results);
    return -1;
  }
  return (int32_t) static_cast<Results*>(results)->size();
}

uint32_t ngt_get_result_size(NGTObjectDistances results, NGTError error) {
  if (results == nullptr) {
    CAPI_PARAM_ERROR(error, "results = " << results);
    return 0;
  }
  return (uint32_t) static_cast<Results*>(results)->size();
}

NGTObjectDistance ngt_get_result(const NGTObjectDistances results, const uint32_t i, NGTError error) {
  NGTObjectDistance none = {0, 0.0f};
  if (results == nullptr) {
    CAPI_PARAM_ERROR(error, "results = " << results);
    return none;
  }
  const Results& r = *static_cast<const Results*>(results);
  if (i >= r.size()) {
    std::stringstream ss;
    ss << "Capi : " << __FUNCTION__ << "() : Error: index " << i << " out of range (size " << r.size() << ")";
    set_error(ss, error);
    return none;
  }
  return r[i];
}

void ngt_destroy_results(NGTObjectDistances results) {
  if (results == nullptr) return;
  delete static_cast<Results*>(results);
}

NGTError ngt_create_error_object() {
  try {
    return static_cast<NGTError>(new std::string());
  } catch (std::exception& err) {
    std::cerr << "Capi : " << __FUNCTION__ << "() : Error: " << err.what();
    return nullptr;
  }
}

const char* ngt_get_error_string(const NGTError error) { return static_cast<std::string*>(error)->c_str(); }

void ngt_clear_error_string(NGTError error) { *static_cast<std::string*>(error) = ""; }

void ngt_destroy_error_object(NGTError error) { delete static_cast<std::string*>(error); }

// ---------------------------------------------------------------------------
// Extensions (include/ngtgpu.h)

int32_t ngtgpu_get_dimension(NGTIndex index, NGTError error) {
  if (index == nullptr) {
    CAPI_PARAM_ERROR(error, "index = " << index);
    return -1;
  }
  return (int32_t)engine(index)->dimension();
}

static std::vector<SearchArgs> args_from(const NGTQueryParameters* params, size_t nparams) {
  std::vector<SearchArgs> a(nparams);
  for (size_t i = 0; i < nparams; i++)
    a[i] = make_args(params[i].size, params[i].epsilon, params[i].radius, edge_size_from_field(params[i].edge_size));
  return a;
}

static ngtg::Kernel check_kernel(uint32_t kernel) {
  switch (kernel) {
    case NGTGPU_KERNEL_EXACT: return ngtg::Kernel::Exact;
    case NGTGPU_KERNEL_BATCHED: return ngtg::Kernel::Fast;
    case NGTGPU_KERNEL_BATCHED_FP32: return ngtg::Kernel::FastFp32;
    case NGTGPU_KERNEL_WIDE: return ngtg::Kernel::Wide;
    default: throw std::runtime_error("unknown kernel selector " + std::to_string(kernel));
  }
}

static bool search_batch_args(NGTIndex index, const float* queries, size_t nq, int32_t dim,
                              const std::vector<SearchArgs>& a, NGTObjectDistance* results, size_t kmax,
                              uint32_t* counts, NGTGPUQueryStats* stats, ngtg::Kernel kk) {
  for (const auto& x : a)
    if ((x.refinement_expansion >= 1.0f ? x.size : engine(index)->output_size(x)) > kmax)
      throw std::runtime_error("a query asks for more results than kmax");
  SearchOutput out;
  engine(index)->search(queries, QueryType::Float32, nq, (size_t)dim, a.data(), a.size(), out, kk);
  for (size_t q = 0; q < nq; q++) {
    counts[q] = out.counts[q];
    for (uint32_t i = 0; i < out.counts[q]; i++) {
      const ngtg::ObjDist& o = out.results[q * out.kmax + i];
      results[q * kmax + i] = NGTObjectDistance{o.id, o.distance};
    }
    if (stats) std::memcpy(stats + q, &out.stats[q], sizeof(NGTGPUQueryStats));
  }
  return true;
}

bool ngtgpu_search_batch_ex_float(NGTIndex index, const float* queries, size_t nq, int32_t dim,
                                  const NGTGPUSearchParameters* params, size_t nparams, NGTObjectDistance* results,
                                  size_t kmax, uint32_t* counts, NGTGPUQueryStats* stats, uint32_t kernel,
                                  NGTError error) {
  if (index == nullptr || (nq && (queries == nullptr || results == nullptr || counts == nullptr)) ||
      params == nullptr || dim <= 0 || !(nparams == 1 || nparams == nq)) {
    CAPI_PARAM_ERROR(error, "index = " << index << " queries = " << queries << " nq = " << nq
                                       << " nparams = " << nparams << " dim = " << dim);
    return false;
  }
  try {
    ngtg::Kernel kk = check_kernel(kernel);
    std::vector<SearchArgs> a(nparams);
    for (size_t i = 0; i < nparams; i++) {
      a[i] = make_args(params[i].size, params[i].epsilon, params[i].radius, edge_size_from_field(params[i].edge_size));
      a[i].accuracy = params[i].accuracy;
      a[i].refinement_expansion = params[i].refinement_expansion;
    }
    return search_batch_args(index, queries, nq, dim, a, results, kmax, counts, stats, kk);
  }
  CAPI_CATCH(error, false)
}

bool ngtgpu_search_batch_float(NGTIndex index, const float* queries, size_t nq, int32_t dim,
                               const NGTQueryParameters* params, size_t nparams, NGTObjectDistance* results,
                               size_t kmax, uint32_t* counts, NGTGPUQueryStats* stats, uint32_t kernel,
                               NGTError error) {
  if (index == nullptr || (nq && (queries == nullptr || results == nullptr || counts == nullptr)) ||
      params == nullptr || dim <= 0 || !(nparams == 1 || nparams == nq)) {
    CAPI_PARAM_ERROR(error, "index = " << index << " queries = " << queries << " nq = " << nq
                                       << " nparams = " << nparams << " dim = " << dim);
    return false;
  }
  try {
    ngtg::Kernel kk = check_kernel(kernel);
    std::vector<SearchArgs> a = args_from(params, nparams);
    for (const auto& x : a)
      if (engine(index)->output_size(x) > kmax) throw std::runtime_error("a query asks for more results than kmax");
    SearchOutput out;
    engine(index)->search(queries, QueryType::Float32, nq, (size_t)dim, a.data(), a.size(), out, kk);
    for (size_t q = 0; q < nq; q++) {
      counts[q] = out.counts[q];
      for (uint32_t i = 0; i < out.counts[q]; i++) {
        const ngtg::ObjDist& o = out.results[q * out.kmax + i];
        results[q * kmax + i] = NGTObjectDistance{o.id, o.distance};
      }
      if (stats) std::memcpy(&stats[q], &out.stats[q], sizeof(NGTGPUQueryStats));
    }
    return true;
  }
  CAPI_CATCH(error, false)
}

size_t ngtgpu_query_row_bytes(NGTIndex index, NGTError error) {
  if (index == nullptr) {
    CAPI_PARAM_ERROR(error, "index = " << index);
    return 0;
  }
  return engine(index)->host().row_bytes();
}

bool ngtgpu_convert_queries_float(NGTIndex index, const float* queries, size_t nq, int32_t dim, void* rows_out,
                                  NGTError error) {
  if (index == nullptr || (nq && (queries == nullptr || rows_out == nullptr)) || dim <= 0) {
    CAPI_PARAM_ERROR(error, "index = " << index << " queries = " << queries << " rows = " << rows_out);
    return false;
  }
  try {
    std::vector<uint8_t> rows;
    engine(index)->convert_queries(queries, QueryType::Float32, nq, (size_t)dim, rows);
    if (!rows.empty()) std::memcpy(rows_out, rows.data(), rows.size());
    return true;
  }
  CAPI_CATCH(error, false)
}

bool ngtgpu_search_batch_device(NGTIndex index, const void* d_rows, size_t nq, const NGTQueryParameters* params,
                                size_t nparams, NGTObjectDistance* d_results, size_t kmax, uint32_t* d_counts,
                                NGTGPUQueryStats* d_stats, void* stream, uint32_t kernel, NGTError error) {
  if (index == nullptr || (nq && (d_rows == nullptr || d_results == nullptr || d_counts == nullptr ||
                                  d_stats == nullptr)) ||
      params == nullptr || !(nparams == 1 || nparams == nq)) {
    CAPI_PARAM_ERROR(error, "index = " << index << " rows = " << d_rows << " nq = " << nq << " nparams = " << nparams);
    return false;
  }
  try {
    ngtg::Kernel kk = check_kernel(kernel);
    std::vector<SearchArgs> a = args_from(params, nparams);
    GraphEngine* e = engine(index);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : e->stream();
    e->search_device(static_cast<const uint4*>(d_rows), nq, a.data(), a.size(),
                     reinterpret_cast<ngtg::ObjDist*>(d_results), d_counts,
                     reinterpret_cast<ngtg::QueryStats*>(d_stats), kmax, s, kk);
    return true;
  }
  CAPI_CATCH(error, false)
}

bool ngtgpu_linear_search_tc_device(NGTIndex index, const void* d_rows, size_t nq, size_t size, size_t candidates,
                                    NGTObjectDistance* d_results, size_t kmax, uint32_t* d_counts, uint32_t* d_status,
                                    void* stream, NGTError error) {
  if (index == nullptr ||
      (nq && (d_rows == nullptr || d_results == nullptr || d_counts == nullptr || d_status == nullptr))) {
    CAPI_PARAM_ERROR(error, "index = " << index << " rows = " << d_rows << " nq = " << nq);
    return false;
  }
  try {
    GraphEngine* e = engine(index);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : e->stream();
    e->linear_search_tc_device(static_cast<const uint4*>(d_rows), nq, size, candidates,
                               reinterpret_cast<ngtg::ObjDist*>(d_results), kmax, d_counts, d_status, s);
    return true;
  }
  CAPI_CATCH(error, false)
}

namespace {
bool tc_float_impl(NGTIndex index, const float* queries, size_t nq, int32_t dim, size_t size, size_t candidates,
                   uint32_t precision, uint32_t flags, NGTObjectDistance* results, size_t kmax, uint32_t* counts,
                   uint32_t* status, NGTError error);
}  // namespace

bool ngtgpu_linear_search_tc_float(NGTIndex index, const float* queries, size_t nq, int32_t dim, size_t size,
                                   size_t candidates, NGTObjectDistance* results, size_t kmax, uint32_t* counts,
                                   uint32_t* status, NGTError error) {
  return tc_float_impl(index, queries, nq, dim, size, candidates, NGTGPU_TC_BF16, 0, results, kmax, counts, status,
                       error);
}

bool ngtgpu_linear_search_tc_float_ex(NGTIndex index, const float* queries, size_t nq, int32_t dim, size_t size,
                                      size_t candidates, uint32_t precision, uint32_t flags,
                                      NGTObjectDistance* results, size_t kmax, uint32_t* counts, uint32_t* status,
                                      NGTError error) {
  return tc_float_impl(index, queries, nq, dim, size, candidates, precision, flags, results, kmax, counts, status,
                       error);
}

bool ngtgpu_linear_search_tc_ex(NGTIndex index, const void* d_rows, size_t nq, size_t size, size_t candidates,
                                uint32_t precision, uint32_t flags, NGTObjectDistance* d_results, size_t kmax,
                                uint32_t* d_counts, uint32_t* d_status, void* stream, NGTError error) {
  if (index == nullptr || precision > NGTGPU_TC_FP8 || (flags & ~(NGTGPU_TC_FP64_TIES | NGTGPU_TC_PAIR)) != 0 ||
      (nq && (d_rows == nullptr || d_results == nullptr || d_counts == nullptr || d_status == nullptr))) {
    CAPI_PARAM_ERROR(error, "index = " << index << " rows = " << d_rows << " nq = " << nq << " precision = "
                                       << precision << " flags = " << flags);
    return false;
  }
  try {
    GraphEngine* e = engine(index);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : e->stream();
    e->linear_search_tc_device(static_cast<const uint4*>(d_rows), nq, size, candidates,
                               reinterpret_cast<ngtg::ObjDist*>(d_results), kmax, d_counts, d_status, s,
                               precision == NGTGPU_TC_FP8, (flags & NGTGPU_TC_FP64_TIES) != 0,
                               (flags & NGTGPU_TC_PAIR) != 0);
    return true;
  }
  CAPI_CATCH(error, false)
}

namespace {
bool tc_float_impl(NGTIndex index, const float* queries, size_t nq, int32_t dim, size_t size, size_t candidates,
                   uint32_t precision, uint32_t flags, NGTObjectDistance* results, size_t kmax, uint32_t* counts,
                   uint32_t* status, NGTError error) {
  if (index == nullptr || dim <= 0 || precision > NGTGPU_TC_FP8 ||
      (flags & ~(NGTGPU_TC_FP64_TIES | NGTGPU_TC_PAIR)) != 0 ||
      (nq && (queries == nullptr || results == nullptr || counts == nullptr || status == nullptr))) {
    CAPI_PARAM_ERROR(error, "index = " << index << " queries = " << queries << " nq = " << nq << " dim = " << dim);
    return false;
  }
  try {
    GraphEngine* e = engine(index);
    e->linear_search_tc_host(queries, nq, (size_t)dim, size, candidates, reinterpret_cast<ngtg::ObjDist*>(results),
                             kmax, counts, status, precision == NGTGPU_TC_FP8, (flags & NGTGPU_TC_FP64_TIES) != 0,
                             (flags & NGTGPU_TC_PAIR) != 0);
    return true;
  }
  CAPI_CATCH(error, false)
}
}  // namespace

bool ngtgpu_tc_scores_device(NGTIndex index, const void* d_rows, size_t nq, float* d_scores, size_t ld, void* stream,
                             NGTError error) {
  if (index == nullptr || (nq && (d_rows == nullptr || d_scores == nullptr))) {
    CAPI_PARAM_ERROR(error, "index = " << index << " rows = " << d_rows << " scores = " << d_scores);
    return false;
  }
  try {
    GraphEngine* e = engine(index);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : e->stream();
    e->tc_scores_device(static_cast<const uint4*>(d_rows), nq, d_scores, ld, s);
    return true;
  }
  CAPI_CATCH(error, false)
}

bool ngtgpu_set_tc_row_range(NGTIndex index, size_t begin, size_t end, NGTError error) {
  if (index == nullptr) {
    CAPI_PARAM_ERROR(error, "index = " << index);
    return false;
  }
  try {
    engine(index)->set_tc_row_range(begin, end);
    return true;
  }
  CAPI_CATCH(error, false)
}

bool ngtgpu_coalescing_stats(NGTIndex index, uint64_t* queries, uint64_t* launches, NGTError error) {
  if (index == nullptr || queries == nullptr || launches == nullptr) {
    CAPI_PARAM_ERROR(error, "index = " << index);
    return false;
  }
  *queries = engine(index)->coalesced_queries();
  *launches = engine(index)->coalesced_launches();
  return true;
}

bool ngtgpu_set_coalescing_lanes(NGTIndex index, uint32_t lanes, NGTError error) {
  if (index == nullptr) {
    CAPI_PARAM_ERROR(error, "index = " << index);
    return false;
  }
  try {
    engine(index)->set_coalescing_lanes(lanes);
    return true;
  }
  CAPI_CATCH(error, false)
}

bool ngtgpu_tc_phase_times(NGTIndex index, float* ms3, NGTError error) {
  if (index == nullptr || ms3 == nullptr) {
    CAPI_PARAM_ERROR(error, "index = " << index << " ms = " << ms3);
    return false;
  }
  engine(index)->tc_phase_ms(ms3);
  return true;
}

bool ngtgpu_set_tc_first_rows(NGTIndex index, size_t rows, NGTError error) {
  if (index == nullptr) {
    CAPI_PARAM_ERROR(error, "index = " << index);
    return false;
  }
  engine(index)->set_tc_first_rows(rows);
  return true;
}

bool ngtgpu_set_tc_graphs(NGTIndex index, int enable, NGTError error) {
  if (index == nullptr) {
    CAPI_PARAM_ERROR(error, "index = " << index);
    return false;
  }
  try {
    engine(index)->set_tc_graphs(enable != 0);
    return true;
  }
  CAPI_CATCH(error, false)
}

bool ngtgpu_set_batched_tuning(NGTIndex index, uint32_t list_capacity, uint32_t parents, float rerank_factor,
                               NGTError error) {
  if (index == nullptr || list_capacity > 1024 || parents > 16 || rerank_factor < 0.f) {
    CAPI_PARAM_ERROR(error, "index = " << index << " list_capacity = " << list_capacity << " parents = " << parents
                                       << " rerank_factor = " << rerank_factor);
    return false;
  }
  ngtg::FastTuning t = engine(index)->tuning();
  t.list_cap = list_capacity;
  t.parents = parents;
  t.rerank_factor = rerank_factor;
  engine(index)->set_tuning(t);
  return true;
}

bool ngtgpu_set_batched_rows_in_flight(NGTIndex index, uint32_t rows, NGTError error) {
  if (index == nullptr || !(rows == 0 || rows == 2 || rows == 4 || rows == 6 || rows == 8)) {
    CAPI_PARAM_ERROR(error, "index = " << index << " rows = " << rows);
    return false;
  }
  ngtg::FastTuning t = engine(index)->tuning();
  t.rows_in_flight = rows;
  engine(index)->set_tuning(t);
  return true;
}

bool ngtgpu_set_batched_tuning_ex(NGTIndex index, const NGTGPUBatchedTuning* tuning, NGTError error) {
  if (index == nullptr || tuning == nullptr || tuning->list_capacity > 1024 || tuning->parents > 32 ||
      tuning->rerank_factor < 0.f || tuning->neighbour_capacity > 4096 ||
      !(tuning->rows_in_flight <= 2 || tuning->rows_in_flight == 4 ||
        tuning->rows_in_flight == 6 || tuning->rows_in_flight == 8) ||
      tuning->ctas_per_sm > 8 || !(tuning->cta_threads == 0 || tuning->cta_threads == 64 ||
                                   tuning->cta_threads == 128 || tuning->cta_threads == 256) || tuning->stage_kilobytes > 200 || tuning->l2_policy > 3 ||
      tuning->search_rows > 2) {
    CAPI_PARAM_ERROR(error, "index = " << index << " tuning = " << tuning);
    return false;
  }
  ngtg::FastTuning t;
  t.list_cap = tuning->list_capacity;
  t.parents = tuning->parents;
  t.rerank_factor = tuning->rerank_factor;
  t.rows_in_flight = tuning->rows_in_flight;
  t.ctas_per_sm = tuning->ctas_per_sm;
  t.nbr_cap = tuning->neighbour_capacity;
  t.cta_threads = tuning->cta_threads;
  t.stage_kb = tuning->stage_kilobytes;
  t.l2_policy = tuning->l2_policy;
  t.search_rows = tuning->search_rows;
  engine(index)->set_tuning(t);
  return true;
}

uint32_t ngtgpu_get_wide_search_rows(NGTIndex index, NGTError error) {
  if (index == nullptr) {
    CAPI_PARAM_ERROR(error, "index = " << index);
    return UINT32_MAX;
  }
  try {
    return (uint32_t)engine(index)->wide_search_rows();
  }
  CAPI_CATCH(error, UINT32_MAX)
}

uint64_t ngtgpu_kernel_launches(NGTIndex index, NGTError error) {
  if (index == nullptr) {
    CAPI_PARAM_ERROR(error, "index = " << index);
    return 0;
  }
  return engine(index)->launches();
}

// ---- quantized graph (lib/NGT/NGTQ/Capi.cpp) ---------------------------------

NGTQGIndex ngtqg_open_index(const char* index_path, NGTQGError error) {
  try {
    if (index_path == nullptr) throw std::runtime_error("index path is NULL");
    // NGTQG::Index opens the index updatable (tree seeds) plus its quantized graph
    return static_cast<NGTQGIndex>(new GraphEngine(index_path, GraphMode::Updatable, true));
  }
  CAPI_CATCH(error, nullptr)
}

void ngtqg_close_index(NGTQGIndex index) {
  if (index == nullptr) return;
  delete engine(index);
}

void ngtqg_initialize_query_parameters(NGTQGQueryParameters* parameters) {
  if (parameters == nullptr) return;
  parameters->size = 20;
  parameters->epsilon = 0.03f;
  parameters->result_expansion = 3.0f;
  parameters->radius = FLT_MAX;
}

void ngtqg_initialize_query(NGTQGQuery* query) {
  if (query == nullptr) return;
  query->query = nullptr;
  query->size = 20;
  query->epsilon = 0.03f;
  query->result_expansion = 3.0f;
  query->radius = FLT_MAX;
}

}  // extern "C"

namespace {

QGArgs qg_args(const NGTQGQueryParameters& p) {
  QGArgs a;
  a.size = p.size;
  a.epsilon = p.epsilon;
  a.result_expansion = p.result_expansion;
  a.radius = p.radius < 0.0f ? FLT_MAX : p.radius;      // ngtqg_search_index_ (Capi.cpp:110-112)
  return a;
}

bool qg_search_common(NGTQGIndex index, const void* query, QueryType qt, const NGTQGQueryParameters& p,
                      NGTObjectDistances results, NGTQGError error, const char* fn) {
  if (index == nullptr || query == nullptr || results == nullptr) {
    std::stringstream ss;
    ss << "Capi : " << fn << "() : parametor error: index = " << index << " query = " << query
       << " results = " << results;
    set_error(ss, error);
    return false;
  }
  try {
    GraphEngine* e = engine(index);
    QGArgs a = qg_args(p);
    SearchOutput out;
    e->qg_search(query, qt, 1, e->dimension(), &a, 1, out);
    fill_results(out, 0, results);
    return true;
  } catch (std::exception& err) {
    std::stringstream ss;
    ss << "Capi : " << fn << "() : Error: " << err.what();
    set_error(ss, error);
    return false;
  }
}

}  // namespace

extern "C" {

bool ngtqg_search_index(NGTQGIndex index, NGTQGQuery query, NGTObjectDistances results, NGTQGError error) {
  NGTQGQueryParameters p{query.size, query.epsilon, query.result_expansion, query.radius};
  return qg_search_common(index, query.query, QueryType::Float32, p, results, error, __FUNCTION__);
}

bool ngtqg_search_index_float(NGTQGIndex index, NGTQGQueryFloat query, NGTObjectDistances results,
                              NGTQGError error) {
  return qg_search_common(index, query.query, QueryType::Float32, query.params, results, error, __FUNCTION__);
}

bool ngtqg_search_index_uint8(NGTQGIndex index, NGTQGQueryUint8 query, NGTObjectDistances results,
                              NGTQGError error) {
  return qg_search_common(index, query.query, QueryType::Uint8, query.params, results, error, __FUNCTION__);
}

bool ngtqg_search_index_float16(NGTQGIndex index, NGTQGQueryFloat16 query, NGTObjectDistances results,
                                NGTQGError error) {
  return qg_search_common(index, query.query, QueryType::Float16, query.params, results, error, __FUNCTION__);
}

bool ngtqg_gpu_search_batch_float(NGTQGIndex index, const float* queries, size_t nq, int32_t dim,
                                  const NGTQGQueryParameters* params, size_t nparams, NGTObjectDistance* results,
                                  size_t kmax, uint32_t* counts, void* stats, NGTQGError error) {
  return ngtqg_gpu_search_batch_ex_float(index, queries, nq, dim, params, nparams, results, kmax, counts, stats,
                                         NGTGPU_KERNEL_EXACT, error);
}

bool ngtqg_gpu_search_batch_ex_float(NGTQGIndex index, const float* queries, size_t nq, int32_t dim,
                                     const NGTQGQueryParameters* params, size_t nparams, NGTObjectDistance* results,
                                     size_t kmax, uint32_t* counts, void* stats, uint32_t kernel,
                                     NGTQGError error) {
  if (kernel != NGTGPU_KERNEL_EXACT && kernel != NGTGPU_KERNEL_WIDE) {
    CAPI_PARAM_ERROR(error, "kernel = " << kernel);
    return false;
  }
  if (index == nullptr || (nq && (queries == nullptr || results == nullptr || counts == nullptr)) ||
      params == nullptr || dim <= 0 || !(nparams == 1 || nparams == nq)) {
    CAPI_PARAM_ERROR(error, "index = " << index << " queries = " << queries << " nq = " << nq
                                       << " nparams = " << nparams << " dim = " << dim);
    return false;
  }
  try {
    std::vector<QGArgs> a;
    for (size_t i = 0; i < nparams; i++) {
      a.push_back(qg_args(params[i]));
      if (a.back().size > kmax) throw std::runtime_error("a query asks for more results than kmax");
    }
    SearchOutput out;
    engine(index)->qg_search(queries, QueryType::Float32, nq, (size_t)dim, a.data(), a.size(), out,
                             kernel == NGTGPU_KERNEL_WIDE);
    for (size_t q = 0; q < nq; q++) {
      counts[q] = out.counts[q];
      for (uint32_t i = 0; i < out.counts[q]; i++) {
        const ngtg::ObjDist& o = out.results[q * out.kmax + i];
        results[q * kmax + i] = NGTObjectDistance{o.id, o.distance};
      }
      if (stats) std::memcpy(static_cast<NGTGPUQueryStats*>(stats) + q, &out.stats[q], sizeof(NGTGPUQueryStats));
    }
    return true;
  }
  CAPI_CATCH(error, false)
}

bool ngtqg_gpu_search_batch_device(NGTQGIndex index, const void* d_rows, size_t nq,
                                   const NGTQGQueryParameters* params, size_t nparams, NGTObjectDistance* d_results,
                                   size_t kmax, uint32_t* d_counts, void* d_stats, void* stream, NGTQGError error) {
  return ngtqg_gpu_search_batch_ex_device(index, d_rows, nq, params, nparams, d_results, kmax, d_counts, d_stats,
                                          stream, NGTGPU_KERNEL_EXACT, error);
}

bool ngtqg_gpu_search_batch_ex_device(NGTQGIndex index, const void* d_rows, size_t nq,
                                      const NGTQGQueryParameters* params, size_t nparams,
                                      NGTObjectDistance* d_results, size_t kmax, uint32_t* d_counts, void* d_stats,
                                      void* stream, uint32_t kernel, NGTQGError error) {
  if (kernel != NGTGPU_KERNEL_EXACT && kernel != NGTGPU_KERNEL_WIDE) {
    CAPI_PARAM_ERROR(error, "kernel = " << kernel);
    return false;
  }
  if (index == nullptr || (nq && (d_rows == nullptr || d_results == nullptr || d_counts == nullptr ||
                                  d_stats == nullptr)) ||
      params == nullptr || !(nparams == 1 || nparams == nq)) {
    CAPI_PARAM_ERROR(error, "index = " << index << " rows = " << d_rows << " nq = " << nq << " nparams = " << nparams);
    return false;
  }
  try {
    std::vector<QGArgs> a;
    for (size_t i = 0; i < nparams; i++) a.push_back(qg_args(params[i]));
    GraphEngine* e = engine(index);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : e->stream();
    if (kernel == NGTGPU_KERNEL_WIDE)
      e->qg_search_device_relaxed(static_cast<const uint4*>(d_rows), nq, a.data(), a.size(),
                                  reinterpret_cast<ngtg::ObjDist*>(d_results), d_counts,
                                  static_cast<ngtg::QueryStats*>(d_stats), kmax, s);
    else
      e->qg_search_device(static_cast<const uint4*>(d_rows), nq, a.data(), a.size(),
                          reinterpret_cast<ngtg::ObjDist*>(d_results), d_counts,
                          static_cast<ngtg::QueryStats*>(d_stats), kmax, s);
    return true;
  }
  CAPI_CATCH(error, false)
}

// ---- quantized blob graph (lib/NGT/NGTQ/Capi.cpp) ------------------------------

QBGIndex qbg_open_index(const char* index_path, bool prebuilt, QBGError error) {
  (void)prebuilt;
  try {
    if (index_path == nullptr) throw std::runtime_error("index path is NULL");
    return static_cast<QBGIndex>(new GraphEngine(index_path, true));
  }
  CAPI_CATCH(error, nullptr)
}

void qbg_close_index(QBGIndex index) {
  if (index == nullptr) return;
  delete engine(index);
}

void qbg_initialize_query_parameters(QBGQueryParameters* parameters) {
  if (parameters == nullptr) return;
  parameters->number_of_results = 20;
  parameters->epsilon = 0.1f;
  parameters->blob_epsilon = 0.0f;
  parameters->result_expansion = 3.0f;
  parameters->number_of_explored_blobs = 256;
  parameters->number_of_edges = 0;
  parameters->radius = 0;
}

void qbg_initialize_query(QBGQuery* query) {
  if (query == nullptr) return;
  query->query = nullptr;
  query->number_of_results = 20;
  query->epsilon = 0.1f;
  query->blob_epsilon = 0.0f;
  query->result_expansion = 3.0f;
  query->number_of_explored_blobs = 256;
  query->number_of_edges = 0;
  query->radius = 0;
}

uint32_t qbg_get_result_size(QBGObjectDistances results, NGTError error) {
  return ngt_get_result_size(results, error);
}

NGTObjectDistance qbg_get_result(const QBGObjectDistances results, const uint32_t idx, NGTError error) {
  return ngt_get_result(results, idx, error);
}

void qbg_destroy_results(QBGObjectDistances results) { ngt_destroy_results(results); }

size_t qbg_get_dimension(QBGIndex index, QBGError error) {
  if (index == nullptr) {
    CAPI_PARAM_ERROR(error, "index = " << index);
    return 0;
  }
  return engine(index)->qbg_genuine_dimension();
}

}  // extern "C"

namespace {

QBGArgs qbg_args(const QBGQueryParameters& p) {
  QBGArgs a;
  a.size = p.number_of_results;
  a.epsilon = p.epsilon;
  a.blob_epsilon = p.blob_epsilon;
  a.result_expansion = p.result_expansion;
  a.explored_blobs = p.number_of_explored_blobs;
  a.edges = p.number_of_edges;
  return a;
}

bool qbg_search_common(QBGIndex index, const void* query, QueryType qt, const QBGQueryParameters& p,
                       QBGObjectDistances results, QBGError error, const char* fn) {
  if (index == nullptr || query == nullptr || results == nullptr) {
    std::stringstream ss;
    ss << "Capi : " << fn << "() : parametor error: index = " << index << " query = " << query
       << " results = " << results;
    set_error(ss, error);
    return false;
  }
  try {
    GraphEngine* e = engine(index);
    QBGArgs a = qbg_args(p);
    SearchOutput out;
    e->qbg_search(query, qt, 1, e->qbg_genuine_dimension(), &a, 1, out);
    fill_results(out, 0, results);
    return true;
  } catch (std::exception& err) {
    std::stringstream ss;
    ss << "Capi : " << fn << "() : Error: " << err.what();
    set_error(ss, error);
    return false;
  }
}

}  // namespace

extern "C" {

bool qbg_search_index(QBGIndex index, QBGQuery query, QBGObjectDistances results, QBGError error) {
  QBGQueryParameters p{query.number_of_results, query.epsilon, query.blob_epsilon, query.result_expansion,
                       query.number_of_explored_blobs, query.number_of_edges, query.radius};
  return qbg_search_common(index, query.query, QueryType::Float32, p, results, error, __FUNCTION__);
}

bool qbg_search_index_float(QBGIndex index, QBGQueryFloat query, QBGObjectDistances results, QBGError error) {
  return qbg_search_common(index, query.query, QueryType::Float32, query.params, results, error, __FUNCTION__);
}

bool qbg_search_index_uint8(QBGIndex index, QBGQueryUint8 query, QBGObjectDistances results, QBGError error) {
  return qbg_search_common(index, query.query, QueryType::Uint8, query.params, results, error, __FUNCTION__);
}

bool qbg_search_index_float16(QBGIndex index, QBGQueryFloat16 query, QBGObjectDistances results,
                              QBGError error) {
  return qbg_search_common(index, query.query, QueryType::Float16, query.params, results, error, __FUNCTION__);
}

bool qbg_gpu_search_batch_float(QBGIndex index, const float* queries, size_t nq, int32_t dim,
                                const QBGQueryParameters* params, size_t nparams, NGTObjectDistance* results,
                                size_t kmax, uint32_t* counts, void* stats, QBGError error) {
  return qbg_gpu_search_batch_ex(index, queries, nq, dim, params, nparams, 0u, results, kmax, counts, stats, error);
}

bool qbg_gpu_search_batch_device(QBGIndex index, const void* d_rows, size_t nq, const QBGQueryParameters* params,
                                 size_t nparams, uint32_t flags, NGTObjectDistance* d_results, size_t kmax,
                                 uint32_t* d_counts, void* d_stats, void* stream, QBGError error) {
  if (index == nullptr || (nq && (d_rows == nullptr || d_results == nullptr || d_counts == nullptr ||
                                  d_stats == nullptr)) ||
      params == nullptr || !(nparams == 1 || nparams == nq) ||
      (flags & ~(NGTGPU_QBG_TWO_STEP | NGTGPU_QBG_REFINE)) != 0) {
    CAPI_PARAM_ERROR(error, "index = " << index << " rows = " << d_rows << " nq = " << nq << " nparams = " << nparams
                                       << " flags = " << flags);
    return false;
  }
  try {
    std::vector<QBGArgs> a;
    for (size_t i = 0; i < nparams; i++) {
      a.push_back(qbg_args(params[i]));
      a.back().two_step = (flags & NGTGPU_QBG_TWO_STEP) != 0;
      a.back().refine = (flags & NGTGPU_QBG_REFINE) != 0;
      if (GraphEngine::qbg_result_size(a.back()) > kmax)
        throw std::runtime_error("a query asks for more results than kmax");
    }
    GraphEngine* e = engine(index);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : e->stream();
    e->qbg_search_device(static_cast<const uint4*>(d_rows), nq, a.data(), a.size(),
                         reinterpret_cast<ngtg::ObjDist*>(d_results), d_counts,
                         static_cast<ngtg::QueryStats*>(d_stats), kmax, s);
    return true;
  }
  CAPI_CATCH(error, false)
}

bool qbg_gpu_search_batch_ex(QBGIndex index, const float* queries, size_t nq, int32_t dim,
                             const QBGQueryParameters* params, size_t nparams, uint32_t flags,
                             NGTObjectDistance* results, size_t kmax, uint32_t* counts, void* stats, QBGError error) {
  if (index == nullptr || (nq && (queries == nullptr || results == nullptr || counts == nullptr)) ||
      params == nullptr || dim <= 0 || !(nparams == 1 || nparams == nq) ||
      (flags & ~(NGTGPU_QBG_TWO_STEP | NGTGPU_QBG_REFINE)) != 0) {
    CAPI_PARAM_ERROR(error, "index = " << index << " queries = " << queries << " nq = " << nq
                                       << " nparams = " << nparams << " dim = " << dim << " flags = " << flags);
    return false;
  }
  try {
    std::vector<QBGArgs> a;
    for (size_t i = 0; i < nparams; i++) {
      a.push_back(qbg_args(params[i]));
      a.back().two_step = (flags & NGTGPU_QBG_TWO_STEP) != 0;
      a.back().refine = (flags & NGTGPU_QBG_REFINE) != 0;
      if (GraphEngine::qbg_result_size(a.back()) > kmax)
        throw std::runtime_error("a query asks for more results than kmax");
    }
    SearchOutput out;
    engine(index)->qbg_search(queries, QueryType::Float32, nq, (size_t)dim, a.data(), a.size(), out);
    for (size_t q = 0; q < nq; q++) {
      counts[q] = out.counts[q];
      for (uint32_t i = 0; i < out.counts[q]; i++) {
        const ngtg::ObjDist& o = out.results[q * out.kmax + i];
        results[q * kmax + i] = NGTObjectDistance{o.id, o.distance};
      }
      if (stats) std::memcpy(static_cast<NGTGPUQueryStats*>(stats) + q, &out.stats[q], sizeof(NGTGPUQueryStats));
    }
    return true;
  }
  CAPI_CATCH(error, false)
}

}  // extern "C"
