// ORACLE -- test infrastructure only.  Opens a quantized-graph index with the
// unmodified reference (oracle/_ref/libngt_ref.so, built by the Makefile in
// this directory) and dumps the intermediate values of its QG search for a set
// of queries, so that the restatement in oracle/ngt_oracle.c can be checked
// step by step:
//   rotated query      lib/NGT/NGTQ/QuantizedGraph.h:297-304 (Rotation::mul)
//   uint8 lookup table lib/NGT/NGTQ/Quantizer.h:1731-1800  (createFloatL2DistanceLookup)
//   4-bit scan         lib/NGT/NGTQ/Quantizer.h:2331-2440  (operator() over a node's stream)
//
// usage: ref_qg_probe <index> <queries.f32> <nq> <dim> <nodes> <out>
//   out, per query: qdim floats (rotated query), M*16 bytes (LUT), float scale,
//   float totalOffset, then for node ids 1..nodes: uint32 count + count floats.
#include <NGT/NGTQ/QuantizedGraph.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

int main(int argc, char** argv) {
  if (argc != 7) {
    std::fprintf(stderr, "usage: %s <index> <queries> <nq> <dim> <nodes> <out>\n", argv[0]);
    return 2;
  }
  size_t nq = std::strtoul(argv[3], nullptr, 10), dim = std::strtoul(argv[4], nullptr, 10);
  size_t nodes = std::strtoul(argv[5], nullptr, 10);
  std::vector<float> q(nq * dim);
  FILE* f = std::fopen(argv[2], "rb");
  if (!f || std::fread(q.data(), 4, q.size(), f) != q.size()) return 3;
  std::fclose(f);
  NGTQG::Index index(argv[1]);
  NGTQ::Quantizer& quantizer = index.quantizedIndex.getQuantizer();
  NGTQ::QuantizedObjectDistance& qod = quantizer.getQuantizedObjectDistance();
  size_t qdim = quantizer.property.dimension;
  size_t m = quantizer.property.localDivisionNo;
  FILE* o = std::fopen(argv[6], "wb");
  for (size_t i = 0; i < nq; i++) {
    std::vector<float> rq(q.begin() + i * dim, q.begin() + (i + 1) * dim);
    if (qdim > rq.size()) rq.resize(qdim);
    if (qod.rotation) qod.rotation->mul(rq.data());
    NGTQ::QuantizedObjectDistance::DistanceLookupTableUint8 lut;
    qod.initialize(lut);
    qod.createDistanceLookup(rq.data(), 0, lut);
    std::fwrite(rq.data(), 4, qdim, o);
    std::fwrite(lut.localDistanceLookup, 1, m * 16, o);
    std::fwrite(&lut.scales[0], 4, 1, o);
    std::fwrite(&lut.totalOffset, 4, 1, o);
    for (size_t id = 1; id <= nodes; id++) {
      auto& ids = index.quantizedGraph.getIDs(id);
      uint32_t n = ids.size();
      std::vector<float> ds(n + 16);
      if (n > 0) qod(index.quantizedGraph.get(id), ds.data(), n, lut);
      std::fwrite(&n, 4, 1, o);
      std::fwrite(ds.data(), 4, n, o);
    }
  }
  std::fclose(o);
  return 0;
}
