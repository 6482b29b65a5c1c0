// Two-tier exact min-queue of 64-bit (distance, id) keys for one CTA: the
// smallest `cap` keys sorted in shared memory (double-buffered for merges),
// the rest unsorted in a per-CTA global overflow tier whose keys are all larger
// than every shared-memory key.  When the shared list drains, the smallest
// `cap` overflow keys are picked by an exact radix select over the 64-bit keys,
// sorted and moved back, so pops follow the total (distance, id) order exactly.
// Only the overflow tier's capacity can make it inexact (QueueState::status).
//
// Every function is called by all threads of the CTA with the same arguments.
#pragma once
#include <cstdint>
#include "graph_exact.cuh"

namespace ngtg {

struct QueueState {
  uint32_t head, tail, cur;        // live shared entries: list[cur][head, tail)
  uint32_t ovf_n, ovf_cur;         // overflow entries, live overflow buffer
  uint32_t tmp_n;
  unsigned long long ovf_min;      // smallest overflow key (~0 when empty)
  unsigned long long evict_min;
  unsigned long long sel_prefix;
  uint32_t sel_need;
  uint32_t status;                 // 1 when the overflow tier lost keys
};

struct TierQueue {
  unsigned long long* list[2];     // shared memory, cap keys each
  uint32_t cap;                    // power of two
  unsigned long long* ovf[2];      // global memory, ocap keys each
  uint32_t ocap;
  QueueState* s;
  uint32_t* hist;                  // 256 counters in shared memory (select scratch)
};

__device__ __forceinline__ void tq_init(const TierQueue& q) {
  if (threadIdx.x == 0) {
    QueueState& s = *q.s;
    s.head = s.tail = s.cur = 0;
    s.ovf_n = 0; s.ovf_cur = 0; s.tmp_n = 0;
    s.ovf_min = ~0ull;
    s.status = 0;
  }
  __syncthreads();
}

// Moves the smallest overflow keys into the (empty) shared list.
__device__ __forceinline__ void tq_refill(const TierQueue& q) {
  QueueState& s = *q.s;
  if (!(s.head >= s.tail && s.ovf_n > 0)) return;       // uniform: read after the caller's barrier
  const uint32_t tid = threadIdx.x;
  const uint32_t r = s.ovf_n;
  unsigned long long* src = q.ovf[s.ovf_cur];
  unsigned long long* dst = q.ovf[s.ovf_cur ^ 1u];
  unsigned long long* cl = q.list[s.cur];
  __syncthreads();
  if (r <= q.cap) {
    for (uint32_t i = tid; i < r; i += blockDim.x) cl[i] = src[i];
    __syncthreads();
    bitonic_sort(cl, r, q.cap);
    if (tid == 0) { s.head = 0; s.tail = r; s.ovf_n = 0; s.ovf_min = ~0ull; }
    __syncthreads();
    return;
  }
  // exact radix select of the cap-th smallest key
  unsigned long long prefix = 0, mask = 0;
  uint32_t need = q.cap;
  for (int shift = 56; shift >= 0; shift -= 8) {
    for (uint32_t i = tid; i < 256; i += blockDim.x) q.hist[i] = 0;
    __syncthreads();
    for (uint32_t i = tid; i < r; i += blockDim.x) {
      unsigned long long k = src[i];
      if ((k & mask) == prefix) atomicAdd(&q.hist[(uint32_t)(k >> shift) & 255u], 1u);
    }
    __syncthreads();
    if (tid == 0) {
      uint32_t acc = 0, b;
      for (b = 0; b < 255; b++) {
        if (acc + q.hist[b] >= need) break;
        acc += q.hist[b];
      }
      s.sel_prefix = prefix | ((unsigned long long)b << shift);
      s.sel_need = need - acc;
    }
    __syncthreads();
    prefix = s.sel_prefix;
    need = s.sel_need;
    mask |= 255ull << shift;
    __syncthreads();
  }
  // keys <= prefix (exactly cap, keys are unique) go to shared memory
  if (tid == 0) { s.tmp_n = 0; s.head = 0; s.tail = 0; s.ovf_min = ~0ull; }
  __syncthreads();
  for (uint32_t i = tid; i < r; i += blockDim.x) {
    unsigned long long k = src[i];
    if (k <= prefix) {
      cl[atomicAdd(&s.tail, 1u)] = k;
    } else {
      dst[atomicAdd(&s.tmp_n, 1u)] = k;
      atomicMin(&s.ovf_min, k);
    }
  }
  __syncthreads();
  bitonic_sort(cl, q.cap, q.cap);
  if (tid == 0) { s.ovf_n = s.tmp_n; s.ovf_cur ^= 1u; }
  __syncthreads();
}

// Smallest key (~0 when the queue is empty).  Refills first.
__device__ __forceinline__ unsigned long long tq_top(const TierQueue& q) {
  tq_refill(q);
  const QueueState& s = *q.s;
  unsigned long long t = s.head < s.tail ? q.list[s.cur][s.head] : ~0ull;
  __syncthreads();
  return t;
}

__device__ __forceinline__ void tq_pop(const TierQueue& q) {
  if (threadIdx.x == 0) q.s->head++;
  __syncthreads();
}

// Inserts m unique keys, sorted ascending, from `keys` (shared memory).
__device__ __forceinline__ void tq_push_sorted(const TierQueue& q, const unsigned long long* keys, uint32_t m) {
  QueueState& s = *q.s;
  const uint32_t tid = threadIdx.x;
  if (m == 0) return;
  unsigned long long* cl = q.list[s.cur];
  unsigned long long* cn = q.list[s.cur ^ 1u];
  unsigned long long* ovf = q.ovf[s.ovf_cur];
  const uint32_t nold = s.tail - s.head;
  const unsigned long long* old = cl + s.head;
  // keys not below the overflow tier's minimum join the tier directly
  const uint32_t mk = s.ovf_n ? lower_bound_keys(keys, m, s.ovf_min) : m;
  const uint32_t obase = s.ovf_n;
  const uint32_t nevict = (nold + mk > q.cap) ? nold + mk - q.cap : 0u;
  __syncthreads();
  if (tid == 0) s.evict_min = ~0ull;
  __syncthreads();
  for (uint32_t i = tid; i < m - mk; i += blockDim.x) {
    uint32_t o = obase + i;
    if (o < q.ocap) ovf[o] = keys[mk + i];
  }
  for (uint32_t i = tid; i < nold; i += blockDim.x) {
    unsigned long long k = old[i];
    uint32_t pos = i + lower_bound_keys(keys, mk, k);
    if (pos < q.cap) cn[pos] = k;
    else {
      uint32_t o = obase + (m - mk) + (pos - q.cap);
      if (o < q.ocap) ovf[o] = k;
      if (pos == q.cap) s.evict_min = k;
    }
  }
  for (uint32_t i = tid; i < mk; i += blockDim.x) {
    unsigned long long k = keys[i];
    uint32_t pos = i + lower_bound_keys(old, nold, k);
    if (pos < q.cap) cn[pos] = k;
    else {
      uint32_t o = obase + (m - mk) + (pos - q.cap);
      if (o < q.ocap) ovf[o] = k;
      if (pos == q.cap) s.evict_min = k;
    }
  }
  __syncthreads();
  if (tid == 0) {
    uint32_t added = (m - mk) + nevict;
    if (added) {
      unsigned long long mn = s.evict_min;
      if (mk < m && keys[mk] < mn) mn = keys[mk];
      if (mn < s.ovf_min) s.ovf_min = mn;
      uint32_t n2 = s.ovf_n + added;
      if (n2 > q.ocap) { n2 = q.ocap; s.status = 1; }
      s.ovf_n = n2;
    }
    s.head = 0;
    s.tail = nold + mk - nevict;
    s.cur ^= 1u;
  }
  __syncthreads();
}

}  // namespace ngtg
