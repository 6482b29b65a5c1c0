// ORACLE -- test infrastructure only.  Runs the unmodified reference NGT
// (oracle/_ref/libngt_ref.so, built from the reference sources by the Makefile
// in this directory) through its own C API (lib/NGT/Capi.h) and dumps the
// results in binary, so tests/golden/make_golden.py can record golden vectors.
//
// usage: ref_dump <graph|linear|range|graph_acc|graph_refine|qg|qbg> <index> <queries.f32> <nq> <dim> <k> <eps> <edge_size|x> <ro|rw> <out>
//   out: nq x k uint32 ids, then nq x k float distances, then nq uint32 counts.
//   For qg the edge_size argument is the result expansion (ngtqg_search_index_float).
//   For qbg it is "expansion:explored_blobs:blob_epsilon" (qbg_search_index_float),
//   and the rows are floor(k * expansion) wide when expansion >= 1 (the C API
//   returns that many results).
//   For graph-only indexes srand(1) runs before every query, so that the
//   random seeds the reference draws are reproducible.
#include <NGT/Capi.h>
#include <NGT/Index.h>
#include <NGT/NGTQ/Capi.h>

#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

int main(int argc, char** argv) {
  if (argc != 11) {
    std::fprintf(stderr, "usage: %s <graph|linear> <index> <queries> <nq> <dim> <k> <eps> <edge|x> <ro|rw> <out>\n",
                 argv[0]);
    return 2;
  }
  std::string op = argv[1];
  const char* index_path = argv[2];
  size_t nq = std::strtoul(argv[4], nullptr, 10), dim = std::strtoul(argv[5], nullptr, 10);
  size_t k = std::strtoul(argv[6], nullptr, 10);
  float eps = std::strtof(argv[7], nullptr);
  bool has_edge = std::string(argv[8]) != "x";
  long edge = has_edge ? std::strtol(argv[8], nullptr, 10) : 0;
  bool ro = std::string(argv[9]) == "ro";
  std::vector<float> q(nq * dim);
  FILE* f = std::fopen(argv[3], "rb");
  if (!f || std::fread(q.data(), 4, q.size(), f) != q.size()) return 3;
  std::fclose(f);
  NGTError err = ngt_create_error_object();
  std::vector<uint32_t> ids(nq * k, 0), cnt(nq, 0);
  std::vector<float> ds(nq * k, 0.f);
  if (op == "qbg") {
    float expansion = 0.f, blob_eps = 0.f;
    unsigned long blobs = 0;
    if (std::sscanf(argv[8], "%f:%lu:%f", &expansion, &blobs, &blob_eps) != 3) return 2;
    size_t w = expansion >= 1.0f ? (size_t)((float)k * expansion) : k;
    ids.assign(nq * w, 0);
    ds.assign(nq * w, 0.f);
    QBGIndex qbg = qbg_open_index(index_path, true, err);
    if (!qbg) {
      std::fprintf(stderr, "open failed: %s\n", ngt_get_error_string(err));
      return 4;
    }
    NGTObjectDistances res = ngt_create_empty_results(err);
    for (size_t i = 0; i < nq; i++) {
      std::srand(1);
      QBGQueryFloat qf;
      qf.query = &q[i * dim];
      qbg_initialize_query_parameters(&qf.params);
      qf.params.number_of_results = k;
      qf.params.epsilon = eps;
      qf.params.blob_epsilon = blob_eps;
      qf.params.result_expansion = expansion;
      qf.params.number_of_explored_blobs = blobs;
      if (!qbg_search_index_float(qbg, qf, res, err)) {
        std::fprintf(stderr, "search failed: %s\n", ngt_get_error_string(err));
        return 5;
      }
      uint32_t n = ngt_get_result_size(res, err);
      cnt[i] = n;
      for (uint32_t j = 0; j < n && j < w; j++) {
        NGTObjectDistance od = ngt_get_result(res, j, err);
        ids[i * w + j] = od.id;
        ds[i * w + j] = od.distance;
      }
    }
    ngt_destroy_results(res);
    qbg_close_index(qbg);
    FILE* o = std::fopen(argv[10], "wb");
    std::fwrite(ids.data(), 4, ids.size(), o);
    std::fwrite(ds.data(), 4, ds.size(), o);
    std::fwrite(cnt.data(), 4, cnt.size(), o);
    std::fclose(o);
    return 0;
  }
  if (op == "qg") {
    NGTQGIndex qg = ngtqg_open_index(index_path, err);
    if (!qg) {
      std::fprintf(stderr, "open failed: %s\n", ngt_get_error_string(err));
      return 4;
    }
    NGTObjectDistances res = ngt_create_empty_results(err);
    for (size_t i = 0; i < nq; i++) {
      std::srand(1);
      NGTQGQueryFloat qf;
      qf.query = &q[i * dim];
      ngtqg_initialize_query_parameters(&qf.params);
      qf.params.size = k;
      qf.params.epsilon = eps;
      qf.params.result_expansion = std::strtof(argv[8], nullptr);
      if (!ngtqg_search_index_float(qg, qf, res, err)) {
        std::fprintf(stderr, "search failed: %s\n", ngt_get_error_string(err));
        return 5;
      }
      uint32_t n = ngt_get_result_size(res, err);
      cnt[i] = n;
      for (uint32_t j = 0; j < n && j < k; j++) {
        NGTObjectDistance od = ngt_get_result(res, j, err);
        ids[i * k + j] = od.id;
        ds[i * k + j] = od.distance;
      }
    }
    ngt_destroy_results(res);
    ngtqg_close_index(qg);
    FILE* o = std::fopen(argv[10], "wb");
    std::fwrite(ids.data(), 4, ids.size(), o);
    std::fwrite(ds.data(), 4, ds.size(), o);
    std::fwrite(cnt.data(), 4, cnt.size(), o);
    std::fclose(o);
    return 0;
  }
  if (op == "graph_acc" || op == "graph_refine") {
    // the C++ API's expected accuracy (SearchContainer::setExpectedAccuracy; the C API
    // ignores NGTQuery::accuracy): epsilon from the index's AccuracyTable
    // (lib/NGT/Index.h:1700-1702); or its refinement expansion (SearchQuery::
    // setRefinementExpansion: k x expansion results re-ranked over the refinement
    // objects, lib/NGT/Index.h:1146-1236); the edge argument holds the accuracy or the
    // expansion
    NGT::Index cindex(index_path, ro);
    const float acc = std::strtof(argv[8], nullptr);
    for (size_t i = 0; i < nq; i++) {
      std::srand(1);
      std::vector<float> qv(q.begin() + i * dim, q.begin() + (i + 1) * dim);
      NGT::SearchQuery sc(qv);
      sc.setSize(k);
      sc.setEpsilon(eps);
      if (op == "graph_refine") sc.setRefinementExpansion(acc);
      else sc.setExpectedAccuracy(acc);
      cindex.search(sc);
      auto& rs = sc.getWorkingResult();          // a max-heap of (distance, id)
      std::vector<NGT::ObjectDistance> v;
      while (!rs.empty()) {
        v.push_back(rs.top());
        rs.pop();
      }
      cnt[i] = (uint32_t)std::min(v.size(), k);
      for (size_t j = 0; j < cnt[i]; j++) {
        ids[i * k + j] = v[v.size() - 1 - j].id;
        ds[i * k + j] = v[v.size() - 1 - j].distance;
      }
    }
    FILE* o = std::fopen(argv[10], "wb");
    std::fwrite(ids.data(), 4, ids.size(), o);
    std::fwrite(ds.data(), 4, ds.size(), o);
    std::fwrite(cnt.data(), 4, cnt.size(), o);
    std::fclose(o);
    return 0;
  }
  NGTIndex index = ro ? ngt_open_index_as_read_only(index_path, err) : ngt_open_index(index_path, err);
  if (!index) {
    std::fprintf(stderr, "open failed: %s\n", ngt_get_error_string(err));
    return 4;
  }
  NGTObjectDistances res = ngt_create_empty_results(err);
  for (size_t i = 0; i < nq; i++) {
    bool ok;
    std::srand(1);
    if (op == "linear") {
      ok = ngt_linear_search_index_as_float(index, &q[i * dim], (int32_t)dim, k, res, err);
    } else if (op == "range") {
      // range search: results within the radius (the edge argument), at most k
      ok = ngt_search_index_as_float(index, &q[i * dim], (int32_t)dim, k, eps, std::strtof(argv[8], nullptr), res,
                                     err);
    } else if (has_edge) {
      NGTQueryFloat qf;
      qf.query = &q[i * dim];
      ngt_initialize_query_parameters(&qf.params);
      qf.params.size = k;
      qf.params.epsilon = eps;
      qf.params.edge_size = (size_t)edge;
      ok = ngt_search_index_with_query_float(index, qf, res, err);
    } else {
      ok = ngt_search_index_as_float(index, &q[i * dim], (int32_t)dim, k, eps, -1.0f, res, err);
    }
    if (!ok) {
      std::fprintf(stderr, "search failed: %s\n", ngt_get_error_string(err));
      return 5;
    }
    uint32_t n = ngt_get_result_size(res, err);
    cnt[i] = n;
    for (uint32_t j = 0; j < n && j < k; j++) {
      NGTObjectDistance od = ngt_get_result(res, j, err);
      ids[i * k + j] = od.id;
      ds[i * k + j] = od.distance;
    }
  }
  ngt_destroy_results(res);
  ngt_close_index(index);
  ngt_destroy_error_object(err);
  FILE* o = std::fopen(argv[10], "wb");
  std::fwrite(ids.data(), 4, ids.size(), o);
  std::fwrite(ds.data(), 4, ds.size(), o);
  std::fwrite(cnt.data(), 4, cnt.size(), o);
  std::fclose(o);
  return 0;
}
