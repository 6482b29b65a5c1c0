// ORACLE -- test infrastructure only.  Times the unmodified reference NGT
// (oracle/_ref/libngt_ref.so, built from the reference sources by the Makefile
// in this directory) on graph search, the way ngtpy's batch_search drives it
// (python/src/ngtpy.cpp:422-458): an OpenMP `schedule(dynamic)` loop over the
// queries, one NGT::SearchQuery per query through NGT::Index::search.  It only
// runs where the reference sources are (they are needed to build it), and serves
// to calibrate the oracle's speed build (the timed CPU baseline of the GPU host,
// where the reference cannot be built) against the reference itself.
//
// usage: ref_bench <index> <queries.f32> <nq> <dim> <k> <epsilon> <threads> <reps> [ids.out]
// prints one JSON line: queries/s of the fastest repetition, threads, and the
// ids of the last repetition to ids.out (nq x k uint32, 0 past a short result).
#include <NGT/Index.h>
#include <omp.h>

#include <cfloat>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <vector>

int main(int argc, char** argv) {
  if (argc != 9 && argc != 10) {
    std::fprintf(stderr, "usage: %s <index> <queries.f32> <nq> <dim> <k> <epsilon> <threads> <reps> [ids.out]\n",
                 argv[0]);
    return 2;
  }
  const size_t nq = std::strtoul(argv[3], nullptr, 10), dim = std::strtoul(argv[4], nullptr, 10);
  const size_t k = std::strtoul(argv[5], nullptr, 10);
  const float eps = std::strtof(argv[6], nullptr);
  const int threads = std::atoi(argv[7]), reps = std::atoi(argv[8]);
  std::vector<float> q(nq * dim);
  FILE* f = std::fopen(argv[2], "rb");
  if (!f || std::fread(q.data(), 4, q.size(), f) != q.size()) return 3;
  std::fclose(f);
  NGT::Index index(argv[1], true);
  std::vector<uint32_t> ids(nq * k, 0);
  double best = 1e30;
  for (int r = 0; r < reps; r++) {
    auto t0 = std::chrono::steady_clock::now();
#pragma omp parallel for schedule(dynamic) num_threads(threads)
    for (long i = 0; i < (long)nq; i++) {
      std::vector<float> qv(q.begin() + i * dim, q.begin() + (i + 1) * dim);
      NGT::SearchQuery sc(qv);
      sc.setSize(k);
      sc.setRadius(FLT_MAX);
      sc.setEpsilon(eps);
      index.search(sc);
      auto& rs = sc.getWorkingResult();          // a max-heap of (distance, id)
      std::vector<uint32_t> v;
      while (!rs.empty()) {
        v.push_back(rs.top().id);
        rs.pop();
      }
      for (size_t j = 0; j < v.size() && j < k; j++) ids[i * k + j] = v[v.size() - 1 - j];
    }
    double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (dt < best) best = dt;
  }
  if (argc == 10) {
    FILE* o = std::fopen(argv[9], "wb");
    if (!o || std::fwrite(ids.data(), 4, ids.size(), o) != ids.size()) return 4;
    std::fclose(o);
  }
  std::printf("{\"qps\": %.1f, \"threads\": %d, \"nq\": %zu}\n", nq / best, threads, nq);
  return 0;
}
