// Top-k selection stage of the exhaustive search (see linear_search.cuh for
// the reference semantics).  Included by exactly one translation unit.
#pragma once
#include "linear_search.cuh"

namespace ngtg {

__device__ __forceinline__ uint32_t dist_bits(float d) { return order_bits(d); }

__global__ void __launch_bounds__(512)
linear_select_kernel(const float* __restrict__ dist, uint32_t nrows, uint32_t q0, uint32_t nqb, uint32_t k,
                     float radius, ObjDist* __restrict__ out, uint32_t* __restrict__ out_count) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint32_t* hist = reinterpret_cast<uint32_t*>(smem);             // 256
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(hist + 256 + 16);  // k
  unsigned long long* sorted = keys + k;                          // k
  __shared__ uint32_t sh_prefix, sh_need, sh_count, sh_valid, sh_warp[16];
  const uint32_t qi = blockIdx.x;
  const uint32_t q = q0 + qi;
  const float* D = dist + (size_t)qi * nrows;
  const uint32_t inf_bits = 0xff800000u;   // order_bits(+inf); NaN orders above it
  const bool use_radius = radius >= 0.0f;
  auto valid_bits = [&](uint32_t row, uint32_t& bits) -> bool {
    float d = D[row];
    bits = dist_bits(d);
    if (bits >= inf_bits) return false;            // dummy row / missing object
    if (use_radius && !(d <= radius)) return false;
    return true;
  };
  // number of valid entries
  if (threadIdx.x == 0) sh_valid = 0;
  __syncthreads();
  uint32_t cnt = 0, bits;
  for (uint32_t r = threadIdx.x; r < nrows; r += blockDim.x) cnt += valid_bits(r, bits) ? 1u : 0u;
  cnt = __reduce_add_sync(0xffffffffu, cnt);
  if ((threadIdx.x & 31) == 0) atomicAdd(&sh_valid, cnt);
  __syncthreads();
  const uint32_t kk = min(k, sh_valid);
  uint32_t prefix = 0, mask = 0, need = kk;
  if (kk > 0 && kk < sh_valid) {
    for (int shift = 24; shift >= 0; shift -= 8) {
      for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0;
      __syncthreads();
      for (uint32_t r = threadIdx.x; r < nrows; r += blockDim.x)
        if (valid_bits(r, bits) && (bits & mask) == prefix) atomicAdd(&hist[(bits >> shift) & 255u], 1u);
      __syncthreads();
      if (threadIdx.x == 0) {
        uint32_t acc = 0, b = 0;
        for (b = 0; b < 256; b++) {
          if (acc + hist[b] >= need) break;
          acc += hist[b];
        }
        sh_prefix = prefix | (b << shift);
        sh_need = need - acc;
      }
      __syncthreads();
      prefix = sh_prefix;
      need = sh_need;
      mask |= 255u << shift;
      __syncthreads();
    }
  } else {
    prefix = 0xffffffffu;   // take every valid entry
    need = 0;
  }
  // collect: bits < prefix (all of them), then the `need` lowest ids with bits == prefix
  if (threadIdx.x == 0) sh_count = 0;
  __syncthreads();
  for (uint32_t r = threadIdx.x; r < nrows; r += blockDim.x) {
    if (valid_bits(r, bits) && (bits < prefix || (prefix == 0xffffffffu))) {
      uint32_t slot = atomicAdd(&sh_count, 1u);
      if (slot < kk) keys[slot] = ((unsigned long long)bits << 32) | r;
    }
  }
  __syncthreads();
  if (need > 0) {
    // ordered scan for ties in increasing id order
    uint32_t taken = 0;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (uint32_t base = 0; base < nrows && taken < need; base += blockDim.x) {
      uint32_t r = base + threadIdx.x;
      bool tie = r < nrows && valid_bits(r, bits) && bits == prefix;
      unsigned b = __ballot_sync(0xffffffffu, tie);
      if (lane == 0) sh_warp[warp] = __popc(b);
      __syncthreads();
      uint32_t before = 0, total = 0;
      for (int w = 0; w < nw; w++) {
        if (w < warp) before += sh_warp[w];
        total += sh_warp[w];
      }
      uint32_t rank = taken + before + __popc(b & ((1u << lane) - 1u));
      if (tie && rank < need) keys[sh_count + rank] = ((unsigned long long)bits << 32) | r;
      taken += total;
      __syncthreads();
    }
  }
  __syncthreads();
  // sort the kk keys
  for (uint32_t i = threadIdx.x; i < kk; i += blockDim.x) {
    unsigned long long x = keys[i];
    uint32_t rank = 0;
    for (uint32_t j = 0; j < kk; j++) rank += keys[j] < x ? 1u : 0u;
    sorted[rank] = x;
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < kk; i += blockDim.x) {
    unsigned long long x = sorted[i];
    out[(size_t)q * k + i] = ObjDist{(uint32_t)x, order_float((uint32_t)(x >> 32))};
  }
  if (threadIdx.x == 0) out_count[q] = kk;
}

}  // namespace ngtg
