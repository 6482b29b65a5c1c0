// ORACLE -- test infrastructure only.  Runs the unmodified reference QBG search
// through its C++ API (QBG::Index, lib/NGT/NGTQ/QuantizedBlobGraph.h) the way the
// reference's `qbg search` command drives it (lib/NGT/NGTQ/QbgCli.cpp:1050-1081):
// searchInOneStep or searchInTwoSteps with a refinement (result) expansion, and
// dumps the results in binary for tests/golden/make_golden.py.
//
// usage: ref_qbg_dump <one|two> <index> <queries.f32> <nq> <dim> <k> <epsilon> <blob_epsilon>
//                     <probes> <refinement_expansion> <out>
//   probes: the two-step search's probed blobs, and the one-step search's explored
//   blobs (its graph exploration size).
//   out: nq x w uint32 ids, then nq x w float distances, then nq uint32 counts, with
//   w = k when the refinement expansion is >= 1 (exact distances of the k best), else
//   w = k (the quantized distances of the k best).
#include <NGT/NGTQ/QuantizedBlobGraph.h>

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

int main(int argc, char** argv) {
  if (argc != 12) {
    std::fprintf(stderr,
                 "usage: %s <one|two> <index> <queries.f32> <nq> <dim> <k> <eps> <blob_eps> <probes> <re> <out>\n",
                 argv[0]);
    return 2;
  }
  const std::string mode = argv[1];
  const size_t nq = std::strtoul(argv[4], nullptr, 10), dim = std::strtoul(argv[5], nullptr, 10);
  const size_t k = std::strtoul(argv[6], nullptr, 10);
  const float eps = std::strtof(argv[7], nullptr), beps = std::strtof(argv[8], nullptr);
  const size_t probes = std::strtoul(argv[9], nullptr, 10);
  const float re = std::strtof(argv[10], nullptr);
  std::vector<float> q(nq * dim);
  FILE* f = std::fopen(argv[3], "rb");
  if (!f || std::fread(q.data(), 4, q.size(), f) != q.size()) return 3;
  std::fclose(f);
  QBG::Index index(argv[2], true);
  std::vector<uint32_t> ids(nq * k, 0), cnt(nq, 0);
  std::vector<float> ds(nq * k, 0.f);
  for (size_t i = 0; i < nq; i++) {
    std::srand(1);
    std::vector<float> qv(q.begin() + i * dim, q.begin() + (i + 1) * dim);
    NGT::ObjectDistances objects;
    QBG::SearchContainer sc;
    sc.setObjectVector(qv);
    sc.setResults(&objects);
    sc.setRefinementExpansion(re);
    sc.setNumOfProbes(probes);              // blobs probed by the two-step search
    sc.setGraphExplorationSize(probes);     // blobs judged at most by the one-step search
    sc.setEpsilon(eps);
    sc.setSize(k);
    sc.setBlobEpsilon(beps);
    sc.setEdgeSize(0);                      // as qbg_search_index_ (NGTQ/Capi.cpp:570): every global edge
    if (mode == "two") index.searchInTwoSteps(sc);
    else index.searchInOneStep(sc);
    if (objects.size() > k) objects.resize(k);
    cnt[i] = (uint32_t)objects.size();
    for (size_t j = 0; j < objects.size(); j++) {
      ids[i * k + j] = objects[j].id;
      ds[i * k + j] = objects[j].distance;
    }
  }
  FILE* o = std::fopen(argv[11], "wb");
  if (!o) return 4;
  std::fwrite(ids.data(), 4, ids.size(), o);
  std::fwrite(ds.data(), 4, ds.size(), o);
  std::fwrite(cnt.data(), 4, cnt.size(), o);
  std::fclose(o);
  return 0;
}
