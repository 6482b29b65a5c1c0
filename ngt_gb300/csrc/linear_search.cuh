// Exhaustive (linear) k-NN search with the reference's exact ordering.
//
// Reference: ObjectSpaceRepository::linearSearch (lib/NGT/ObjectSpaceRepository.h:860-922):
// every object id 1..N is compared, objects with d <= radius (or all, when the
// radius is negative) enter a bounded max-heap of `size`; ties keep the
// smaller id because the heap orders by (distance, id) and ids arrive in
// increasing order.  The result is therefore exactly the `size` smallest
// (distance, id) keys, which is what the two kernels below compute:
//   1. linear_distance_kernel: distances for a block of queries x all rows
//      (group-cooperative 16-byte loads, same comparators as the graph search);
//   2. linear_select_kernel: per query, radix select of the k-th smallest
//      distance (four 8-bit passes over the IEEE bits, which order like
//      integers for d >= 0), then the keys below it plus the lowest ids among
//      the ties, sorted by (distance, id).
#pragma once
#include <cfloat>
#include "distance.cuh"
#include "device_index.h"

namespace ngtg {

constexpr int kLinThreads = 256;
constexpr int kLinRowsPerBlock = 512;

template <ObjType OT, Metric M>
__global__ void __launch_bounds__(kLinThreads)
linear_distance_kernel(DevGraph g, const uint4* __restrict__ queries, uint32_t q0, uint32_t nqb,
                       const uint8_t* __restrict__ present, float* __restrict__ dist, uint32_t group) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint4* qv = reinterpret_cast<uint4*>(smem);
  const uint32_t rc = g.row_chunks;
  const uint32_t qi = blockIdx.y;
  const uint32_t q = q0 + qi;
  for (uint32_t i = threadIdx.x; i < rc; i += blockDim.x) qv[i] = queries[(size_t)q * rc + i];
  __syncthreads();
  const int G = (int)group;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gl = lane & (G - 1);
  const uint32_t gpw = 32 / G, ngroups = kLinThreads / G;
  const uint32_t r0 = blockIdx.x * kLinRowsPerBlock;
  const uint32_t r1 = min(g.nrows, r0 + kLinRowsPerBlock);
  for (uint32_t b = r0 + warp * gpw; b < r1; b += ngroups) {
    uint32_t r = b + (uint32_t)(lane / G);
    bool valid = r < r1;
    uint32_t row = valid ? r : 0u;
    float d = group_distance<OT, M>(qv, g.objects + (size_t)row * rc, (int)rc, gl, G);
    if (valid && gl == 0) {
      bool ok = row != 0 && present[row];
      dist[(size_t)qi * g.nrows + row] = ok ? d : __int_as_float(0x7f800000);  // +inf = excluded
    }
  }
}

}  // namespace ngtg
