// Restatement of the glibc rand()/srand() generator that NGT uses to thin the
// seed list of a DVP-tree leaf (GraphAndTreeIndex::getSeedsFromTree,
// lib/NGT/Index.h:2197-2215) and to draw random seeds
// (GraphIndex::getRandomSeeds, lib/NGT/Index.h:1270-1302).
//
// The algorithm is glibc's published additive-feedback generator (random_r.c,
// TYPE_3: degree 31, separation 3): the state is seeded with the Park-Miller
// minimal standard LCG (16807 * x mod 2^31-1, evaluated with Schrage's method),
// 310 outputs are discarded, and each output is (s[f] += s[r]) >> 1.
// Written here from that description so seeds are reproducible per call and
// thread-safe (the reference calls the process-global rand()).
#pragma once
#include <cstdint>
#include <cmath>
#include <vector>

namespace ngtg {

class GlibcRand {
 public:
  static constexpr int32_t kRandMax = 2147483647;
  explicit GlibcRand(uint32_t seed = 1) { seed_with(seed); }

  void seed_with(uint32_t seed) {
    if (seed == 0) seed = 1;
    s_[0] = (int32_t)seed;
    int64_t word = (int32_t)seed;
    for (int i = 1; i < 31; i++) {
      int64_t hi = word / 127773;
      int64_t lo = word % 127773;
      word = 16807 * lo - 2836 * hi;
      if (word < 0) word += 2147483647;
      s_[i] = (int32_t)word;
    }
    f_ = 3;
    r_ = 0;
    for (int i = 0; i < 310; i++) next();
  }

  int32_t next() {
    uint32_t v = (uint32_t)s_[f_] + (uint32_t)s_[r_];
    s_[f_] = (int32_t)v;
    int32_t out = (int32_t)(v >> 1);
    if (++f_ == 31) f_ = 0;
    if (++r_ == 31) r_ = 0;
    return out;
  }

  // ((double)rand() + 1.0) / ((double)RAND_MAX + 2.0), the form NGT uses.
  double unit() { return ((double)next() + 1.0) / ((double)kRandMax + 2.0); }

 private:
  int32_t s_[31];
  int f_ = 3, r_ = 0;
};

// Thinning of a leaf's object list to seedSize entries, exactly as
// GraphAndTreeIndex::getSeedsFromTree does it after srand(leafID).
inline void thin_leaf_seeds(std::vector<uint32_t>& seeds, uint32_t leaf_index, size_t seed_size) {
  if (seeds.size() <= seed_size) return;
  GlibcRand rng(leaf_index);
  for (size_t i = seeds.size(); i > seed_size; i--) {
    double random = rng.unit();
    size_t idx = (size_t)std::floor((double)i * random);
    seeds[idx] = seeds[i - 1];
  }
  seeds.resize(seed_size);
}

}  // namespace ngtg
