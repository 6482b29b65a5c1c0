// Exact-order graph search: one query per CTA, FP32 (or the object's native
// type), reproducing NGT's sequential best-first search step for step.
//
// Reference: NeighborhoodGraph::searchReadOnlyGraph (lib/NGT/Graph.cpp:716-835)
// and NeighborhoodGraph::search (lib/NGT/Graph.cpp:840-1024), seeded by
// GraphAndTreeIndex::getSeedsFromTree (lib/NGT/Index.h:2173-2220) through
// DVPTree::search in SearchLeaf mode (lib/NGT/Tree.cpp:403-559), with
// setupDistances/setupSeeds (lib/NGT/Graph.cpp:420-586).
//
// Why the results are the reference's, not just close to them:
//   * The neighbours of the expanded node are filtered against the visited set
//     in edge order and their distances computed in parallel; the result-set
//     updates (the only order-dependent step) are then replayed sequentially by
//     one warp in edge order, with the reference's push / push_pop semantics.
//   * The candidate queue only needs the set of entries <= explorationRadius:
//     the radius never grows, the loop stops at the first popped entry above it,
//     so pushing a chunk's survivors after the chunk (against the radius reached
//     at its end) leaves the pop sequence unchanged.
//   * The queue is a sorted array in shared memory, merged with each chunk's
//     sorted survivors; (distance, id) keys make the order total, like
//     ObjectDistance::operator< (lib/NGT/Common.h:2347-2360).
//   * The queue has two tiers: the best `ccap` entries sorted in shared memory
//     and an unsorted overflow tier in global memory whose entries are all
//     larger than every shared-memory entry.  When the shared list drains, the
//     overflow's live entries (<= explorationRadius) are filtered, the ccap
//     smallest picked by an exact radix select over the 64-bit keys, sorted, and
//     moved back.  Pops therefore follow the reference's order exactly.
// The only limit that can make a query inexact is the overflow tier's capacity
// (reported in QueryStats::status).  The visited set never loses entries: it
// starts as a hash table in shared memory and moves to a per-CTA bitmap in
// global memory when the table is half full.
#pragma once
#include <cfloat>
#include "distance.cuh"
#include "device_index.h"

namespace ngtg {

constexpr int kExactThreads = 128;
constexpr int kExactWarps = kExactThreads / 32;
constexpr int kExactChunk = kExactThreads;   // neighbours processed per round

struct ExactShared {
  float radius;
  uint32_t nres;
  uint32_t head, tail, cur;
  uint32_t nvisited;
  uint32_t spilled;
  uint32_t done;
  uint32_t target;
  uint32_t nnew;
  uint32_t nbatch;
  uint32_t live_old;
  uint32_t status;
  uint32_t dc;
  uint32_t expansions;
  uint32_t edges;
  uint32_t seed_leaf;
  uint32_t ovf_n;                 // entries in the global overflow tier
  uint32_t ovf_tmp;
  unsigned long long ovf_min;     // smallest key in the overflow tier (~0 when empty)
  unsigned long long evict_min;
  unsigned long long sel_prefix;
  uint32_t sel_need;
  uint32_t warp_cnt[kExactWarps];
  uint32_t hist[256];
};

struct ExactConfig {
  uint32_t kcap;     // result capacity (>= max size in the batch)
  uint32_t ccap;     // candidate-list capacity
  uint32_t hcap;     // visited hash capacity (power of two)
  uint32_t mode;     // GraphMode
  uint32_t group;    // lanes per distance (power of two <= 32)
  uint32_t bitmap_words;  // words per CTA in the spill bitmap
  uint32_t ocap;          // overflow-tier capacity per CTA (keys)
};

__device__ __forceinline__ uint32_t hash_slot(uint32_t id, uint32_t mask) {
  return (id * 0x9E3779B1u) & mask;
}

// Returns true when `id` was not in the visited set (and inserts it).
__device__ __forceinline__ bool visit_insert(uint32_t* table, uint32_t mask, uint32_t* bitmap, bool spilled,
                                             uint32_t id) {
  if (spilled) {
    uint32_t bit = 1u << (id & 31u);
    uint32_t old = atomicOr(&bitmap[id >> 5], bit);
    return (old & bit) == 0u;
  }
  uint32_t h = hash_slot(id, mask);
  // The table is kept at most half full (plus one chunk), so probing ends.
  for (uint32_t probe = 0; probe <= mask; probe++) {
    uint32_t old = atomicCAS(&table[h], 0u, id);
    if (old == 0u) return true;
    if (old == id) return false;
    h = (h + 1u) & mask;
  }
  return false;
}

// Insert key x into the sorted array res[0..n) with the reference's semantics.
// Returns the new count; updates radius when the reference would.
// Executed by one full warp.
__device__ __forceinline__ void result_insert(unsigned long long* res, uint32_t& n, float& radius,
                                              uint32_t size, uint32_t mode, unsigned long long x, int lane) {
  // Read-only search: push_pop replaces the current maximum when full
  // (ResultSet::push_pop, lib/NGT/Common.h:2421-2428).  Updatable search:
  // push, then pop the maximum if the set grew beyond `size`
  // (lib/NGT/Graph.cpp:990-1004).
  uint32_t live = n;
  bool full = n >= size;
  if (mode == (uint32_t)GraphMode::ReadOnly && full) live = n - 1;   // drop the max first
  uint32_t cnt = 0;
  for (uint32_t i = lane; i < live; i += 32) cnt += res[i] < x ? 1u : 0u;
  uint32_t p = __reduce_add_sync(0xffffffffu, cnt);
  // shift res[p..live) right by one, from the top down
  for (int hi = (int)live; hi > (int)p; hi -= 32) {
    int lo = max((int)p, hi - 32);
    int idx = lo + lane;
    unsigned long long v = 0;
    bool act = idx < hi;
    if (act) v = res[idx];
    __syncwarp();
    if (act) res[idx + 1] = v;
    __syncwarp();
  }
  if (lane == 0) res[p] = x;
  __syncwarp();
  if (mode == (uint32_t)GraphMode::ReadOnly) {
    if (full) {
      radius = key_dist(res[n - 1]);
    } else {
      n = n + 1;
    }
  } else {
    n = n + 1;
    if (n > size) n = size;          // pop the maximum (it sits at index size)
    if (n >= size) radius = key_dist(res[n - 1]);
  }
}

// Rank sort of up to kExactChunk keys (unique) by the whole CTA.
__device__ __forceinline__ void rank_sort(const unsigned long long* in, unsigned long long* out, uint32_t m) {
  for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
    unsigned long long k = in[i];
    uint32_t r = 0;
    for (uint32_t j = 0; j < m; j++) r += in[j] < k ? 1u : 0u;
    out[r] = k;
  }
}

// In-place ascending bitonic sort of a[0..n) in shared memory by the whole CTA;
// entries [n, p) are padded with ~0 where p is the next power of two (<= cap).
__device__ __forceinline__ void bitonic_sort(unsigned long long* a, uint32_t n, uint32_t cap) {
  uint32_t p = 1;
  while (p < n) p <<= 1;
  for (uint32_t i = n + threadIdx.x; i < p && i < cap; i += blockDim.x) a[i] = ~0ull;
  __syncthreads();
  for (uint32_t k = 2; k <= p; k <<= 1) {
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < p; i += blockDim.x) {
        uint32_t l = i ^ j;
        if (l > i) {
          unsigned long long x = a[i], y = a[l];
          bool up = (i & k) == 0;
          if ((x > y) == up) { a[i] = y; a[l] = x; }
        }
      }
      __syncthreads();
    }
  }
}

__device__ __forceinline__ uint32_t lower_bound_keys(const unsigned long long* a, uint32_t n, unsigned long long x) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ uint32_t upper_bound_dist(const unsigned long long* a, uint32_t n, float r) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    if (key_dist(a[mid]) <= r) lo = mid + 1; else hi = mid;
  }
  return lo;
}

template <ObjType OT, Metric M>
__global__ void __launch_bounds__(kExactThreads)
graph_search_exact_kernel(DevGraph g, const uint4* __restrict__ queries, uint32_t nq,
                          const QueryParams* __restrict__ params, const uint32_t* __restrict__ seed_list,
                          ObjDist* __restrict__ out, uint32_t* __restrict__ out_count,
                          QueryStats* __restrict__ stats, uint32_t* __restrict__ bitmaps,
                          unsigned long long* __restrict__ overflow, ExactConfig cfg) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t rc = g.row_chunks;
  // ---- shared-memory carve-up -------------------------------------------
  uint4* qv = reinterpret_cast<uint4*>(smem);
  unsigned long long* res = reinterpret_cast<unsigned long long*>(qv + rc);
  unsigned long long* cand0 = res + cfg.kcap;
  unsigned long long* cand1 = cand0 + cfg.ccap;
  unsigned long long* bkeys = cand1 + cfg.ccap;          // chunk survivors (unsorted)
  unsigned long long* bsorted = bkeys + kExactChunk;     // chunk survivors (sorted)
  uint32_t* table = reinterpret_cast<uint32_t*>(bsorted + kExactChunk);
  uint32_t* nid = table + cfg.hcap;
  float* nd = reinterpret_cast<float*>(nid + kExactChunk);
  ExactShared& s = *reinterpret_cast<ExactShared*>(nd + kExactChunk);
  uint32_t* bitmap = bitmaps + (size_t)blockIdx.x * cfg.bitmap_words;
  unsigned long long* ovf = overflow + (size_t)blockIdx.x * 2 * cfg.ocap;     // overflow tier
  unsigned long long* ovf_tmp = ovf + cfg.ocap;                                 // refill scratch
  const uint32_t hmask = cfg.hcap - 1;
  const int G = (int)cfg.group;
  const int gl = lane & (G - 1);                   // lane inside the distance group
  const int ngroups = kExactThreads / G;

  for (uint32_t q = blockIdx.x; q < nq; q += gridDim.x) {
    const QueryParams P = params[q];
    // ---- per-query initialisation ----------------------------------------
    for (uint32_t i = tid; i < rc; i += blockDim.x) qv[i] = queries[(size_t)q * rc + i];
    for (uint32_t i = tid; i < cfg.hcap; i += blockDim.x) table[i] = 0u;
    if (tid == 0) {
      s.radius = P.radius;
      s.nres = 0; s.head = 0; s.tail = 0; s.cur = 0; s.nvisited = 0; s.spilled = 0;
      s.done = 0; s.status = 0; s.dc = 0; s.expansions = 0; s.nnew = 0;
      s.ovf_n = 0; s.ovf_min = ~0ull; s.edges = 0;
    }
    __syncthreads();
    if (P.size == 0) {          // GraphIndex::search returns nothing for size 0
      if (tid == 0) { out_count[q] = 0; stats[q] = QueryStats{0, 0, 0, 0, 0}; }
      __syncthreads();
      continue;
    }
    // ---- seeds --------------------------------------------------------------
    const uint32_t* seeds = nullptr;
    uint32_t nseeds = 0;
    if (P.seed_cnt == 0xffffffffu) {
      // DVP-tree descent with radius 0 (one region per level) -- warp 0.
      if (warp == 0) {
        uint32_t node = g.root;
        int depth = 0;
        while (!(node & 0x80000000u) && depth < 64) {
          const DevInternal& in = g.internals[node];
          float d = group_distance<TreeSpace<OT, M>::ot, TreeSpace<OT, M>::m>(qv, g.pivots + (size_t)in.pivot * rc, (int)rc, lane, 32);
          uint32_t bsize = in.nchildren - 1, mid;
          for (mid = 0; mid < bsize; mid++)
            if (d < in.borders[mid]) break;
          node = in.children[mid];
          depth++;
        }
        if (lane == 0) {
          if (node & 0x80000000u) s.seed_leaf = node & 0x7fffffffu;
          else { s.seed_leaf = 0xffffffffu; s.status |= kStatusTreeError; }
        }
      }
      __syncthreads();
      if (s.seed_leaf != 0xffffffffu && s.seed_leaf < g.nleaves) {
        const uint32_t* off = g.leaf_seed_off + P.seed_off;    // this query's seed-size table
        uint32_t a = off[s.seed_leaf], b = off[s.seed_leaf + 1];
        seeds = g.leaf_seed_ids + a;
        nseeds = b - a;
      }
    } else {
      seeds = seed_list + P.seed_off;
      nseeds = P.seed_cnt;
    }
    nseeds = min(nseeds, (uint32_t)kExactChunk);
    if (nseeds == 0) {
      if (tid == 0) {
        out_count[q] = 0;
        stats[q] = QueryStats{0, 0, 0, 0, s.status | kStatusEmptySeeds};
      }
      __syncthreads();
      continue;
    }
    // setupDistances: exact distances of the seeds
    // (warp-uniform trip counts: every lane of a warp reaches the shuffles)
    for (uint32_t b = (uint32_t)(warp * (32 / G)); b < nseeds; b += ngroups) {
      uint32_t i = b + (uint32_t)(lane / G);
      bool valid = i < nseeds;
      uint32_t id = valid ? seeds[i] : 0u;
      bool inrange = id < g.nrows;
      float d = group_distance<OT, M>(qv, g.objects + (size_t)(inrange ? id : 0u) * rc, (int)rc, gl, G);
      if (valid && gl == 0) bkeys[i] = pack_key(inrange ? d : FLT_MAX, id);
    }
    __syncthreads();
    rank_sort(bkeys, bsorted, nseeds);
    __syncthreads();
    // setupSeeds: results take the leading seeds within the radius; all seeds are
    // marked visited and become candidates.
    if (tid == 0) {
      uint32_t n = 0;
      float radius = s.radius;
      for (uint32_t i = 0; i < nseeds; i++) {
        float d = key_dist(bsorted[i]);
        if (n < P.size && d <= radius) res[n++] = bsorted[i];
        else break;
      }
      if (n >= P.size) radius = key_dist(res[n - 1]);
      s.nres = n;
      s.radius = radius;
      s.dc = nseeds;
      s.tail = nseeds;
    }
    for (uint32_t i = tid; i < nseeds; i += blockDim.x) {
      cand0[i] = bsorted[i];
      visit_insert(table, hmask, bitmap, false, key_id(bsorted[i]));
    }
    if (tid == 0) s.nvisited = nseeds;
    __syncthreads();

    // ---- best-first loop -----------------------------------------------------
    uint32_t guard = 0;
    while (true) {
      if (s.head >= s.tail && s.ovf_n > 0) {
        // ---- refill the shared list from the overflow tier ----
        const float expR0 = P.coef * s.radius;
        const uint32_t r0 = s.ovf_n;
        if (tid == 0) s.ovf_tmp = 0;
        __syncthreads();
        for (uint32_t i = tid; i < r0; i += blockDim.x) {      // drop entries above the radius
          unsigned long long k = ovf[i];
          if (key_dist(k) <= expR0) ovf_tmp[atomicAdd(&s.ovf_tmp, 1u)] = k;
        }
        __syncthreads();
        const uint32_t r = s.ovf_tmp;
        unsigned long long* cl = s.cur ? cand1 : cand0;
        if (r <= cfg.ccap) {
          for (uint32_t i = tid; i < r; i += blockDim.x) cl[i] = ovf_tmp[i];
          __syncthreads();
          bitonic_sort(cl, r, cfg.ccap);
          if (tid == 0) { s.head = 0; s.tail = r; s.ovf_n = 0; s.ovf_min = ~0ull; }
        } else {
          // exact radix select of the ccap-th smallest 64-bit key
          unsigned long long prefix = 0, mask = 0;
          uint32_t need = cfg.ccap;
          for (int shift = 56; shift >= 0; shift -= 8) {
            for (uint32_t i = tid; i < 256; i += blockDim.x) s.hist[i] = 0;
            __syncthreads();
            for (uint32_t i = tid; i < r; i += blockDim.x) {
              unsigned long long k = ovf_tmp[i];
              if ((k & mask) == prefix) atomicAdd(&s.hist[(uint32_t)(k >> shift) & 255u], 1u);
            }
            __syncthreads();
            if (tid == 0) {
              uint32_t acc = 0, b;
              for (b = 0; b < 255; b++) {
                if (acc + s.hist[b] >= need) break;
                acc += s.hist[b];
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
          // keys <= prefix (exactly ccap) go to shared memory, the rest stay in the tier
          if (tid == 0) { s.ovf_n = 0; s.nnew = 0; s.ovf_min = ~0ull; }
          __syncthreads();
          for (uint32_t i = tid; i < r; i += blockDim.x) {
            unsigned long long k = ovf_tmp[i];
            if (k <= prefix) {
              cl[atomicAdd(&s.nnew, 1u)] = k;
            } else {
              ovf[atomicAdd(&s.ovf_n, 1u)] = k;
              atomicMin(&s.ovf_min, k);
            }
          }
          __syncthreads();
          bitonic_sort(cl, cfg.ccap, cfg.ccap);
          if (tid == 0) { s.head = 0; s.tail = cfg.ccap; }
        }
        __syncthreads();
      }
      if (tid == 0) {
        unsigned long long* cl = s.cur ? cand1 : cand0;
        float expR = P.coef * s.radius;
        if (s.head >= s.tail) {
          s.done = 1;
        } else {
          unsigned long long t = cl[s.head++];
          if (key_dist(t) > expR) s.done = 1;
          else { s.target = key_id(t); s.expansions++; }
        }
      }
      __syncthreads();
      if (s.done) break;
      if (++guard > g.nrows + 8) {     // cannot happen: each id is expanded at most once
        if (tid == 0) s.status |= kStatusIterationLimit;
        break;
      }
      const uint32_t target = s.target;
      const uint32_t e0 = g.offsets[target];
      const uint32_t deg = g.offsets[target + 1] - e0;
      const uint32_t nsz = min(deg, P.edge_size);
      if (tid == 0) s.edges += nsz;
      for (uint32_t c0 = 0; c0 < nsz; c0 += kExactChunk) {
        const uint32_t clen = min((uint32_t)kExactChunk, nsz - c0);
        // spill the visited set to the bitmap before it gets more than half full
        if (!s.spilled && s.nvisited + clen > (cfg.hcap >> 1)) {
          for (uint32_t i = tid; i < cfg.hcap; i += blockDim.x) {
            uint32_t id = table[i];
            if (id) atomicOr(&bitmap[id >> 5], 1u << (id & 31u));
          }
          __threadfence_block();
          __syncthreads();
          if (tid == 0) { s.spilled = 1; s.status |= kStatusVisitedSpill; }
          __syncthreads();
        }
        const bool spilled = s.spilled != 0;
        // visited filter in edge order + order-preserving compaction
        bool isnew = false;
        uint32_t id = 0;
        if ((uint32_t)tid < clen) {
          id = g.edges[e0 + c0 + tid];
          isnew = visit_insert(table, hmask, bitmap, spilled, id);
        }
        unsigned ballot = __ballot_sync(0xffffffffu, isnew);
        if (lane == 0) s.warp_cnt[warp] = __popc(ballot);
        __syncthreads();
        uint32_t base = 0;
        for (int w = 0; w < warp; w++) base += s.warp_cnt[w];
        if (isnew) nid[base + __popc(ballot & ((1u << lane) - 1u))] = id;
        __syncthreads();
        uint32_t nnew = 0;
        for (int w = 0; w < kExactWarps; w++) nnew += s.warp_cnt[w];
        // distances
        if (rc <= (uint32_t)G) {
          // one 16-byte chunk per lane per row: U rows per group in flight
          constexpr int U = 4;
          const uint4 q1 = (uint32_t)gl < rc ? qv[gl] : make_uint4(0, 0, 0, 0);
          const uint32_t step = (uint32_t)ngroups;
          for (uint32_t b = (uint32_t)(warp * (32 / G)); b < nnew; b += step * U) {
            uint4 xv[U];
            uint32_t iu[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
              iu[u] = b + u * step + (uint32_t)(lane / G);
              uint32_t v = iu[u] < nnew ? nid[iu[u]] : 0u;
              xv[u] = (uint32_t)gl < rc ? __ldg(g.objects + (size_t)v * rc + gl) : make_uint4(0, 0, 0, 0);
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
              Acc<OT, M> acc;
              if ((uint32_t)gl < rc) acc.add(q1, xv[u], gl);
              acc.reduce(G);
              float d = acc.finish();
              if (iu[u] < nnew && gl == 0) nd[iu[u]] = d;
            }
          }
        } else {
          for (uint32_t b = (uint32_t)(warp * (32 / G)); b < nnew; b += ngroups) {
            uint32_t i = b + (uint32_t)(lane / G);
            bool valid = i < nnew;
            uint32_t v = valid ? nid[i] : 0u;
            float d = group_distance<OT, M>(qv, g.objects + (size_t)v * rc, (int)rc, gl, G);
            if (valid && gl == 0) nd[i] = d;
          }
        }
        __syncthreads();
        // sequential replay of the result-set updates (warp 0)
        if (warp == 0) {
          float radius = s.radius;
          uint32_t n = s.nres;
          for (uint32_t b = 0; b < nnew; b += 32) {
            uint32_t i = b + lane;
            // a neighbour joins when within the exploration radius and the radius
            // of that moment (both only shrink; with epsilon < 0 the first is
            // the tighter one)
            float d = i < nnew ? nd[i] : FLT_MAX;
            float lim = fminf(radius, P.coef * radius);
            unsigned m = __ballot_sync(0xffffffffu, i < nnew && d <= lim);
            while (m) {
              int src = __ffs(m) - 1;
              float dj = __shfl_sync(0xffffffffu, d, src);
              uint32_t idj = nid[b + src];
              if (dj <= radius && dj <= P.coef * radius)
                result_insert(res, n, radius, P.size, cfg.mode, pack_key(dj, idj), lane);
              m &= (src == 31) ? 0u : ~((2u << src) - 1u);
              lim = fminf(radius, P.coef * radius);
              m &= __ballot_sync(0xffffffffu, i < nnew && d <= lim);
            }
          }
          if (lane == 0) {
            s.radius = radius;
            s.nres = n;
            s.dc += nnew;
            s.nvisited += nnew;
          }
        }
        __syncthreads();
        // chunk survivors within the exploration radius become candidates
        const float expR = P.coef * s.radius;
        {
          bool keep = (uint32_t)tid < nnew && nd[tid] <= expR;
          unsigned kb = __ballot_sync(0xffffffffu, keep);
          if (lane == 0) s.warp_cnt[warp] = __popc(kb);
          __syncthreads();
          uint32_t kbase = 0;
          for (int w = 0; w < warp; w++) kbase += s.warp_cnt[w];
          if (keep) bkeys[kbase + __popc(kb & ((1u << lane) - 1u))] = pack_key(nd[tid], nid[tid]);
          __syncthreads();
        }
        uint32_t m = 0;
        for (int w = 0; w < kExactWarps; w++) m += s.warp_cnt[w];
        rank_sort(bkeys, bsorted, m);
        unsigned long long* cl = s.cur ? cand1 : cand0;
        unsigned long long* cn = s.cur ? cand0 : cand1;
        if (tid == 0) {
          // entries above the exploration radius can never be expanded again
          s.live_old = upper_bound_dist(cl + s.head, s.tail - s.head, expR);
        }
        __syncthreads();
        const uint32_t nold = s.live_old;
        const unsigned long long* old = cl + s.head;
        // survivors not below the overflow tier's minimum join the tier directly
        const uint32_t mk = s.ovf_n ? lower_bound_keys(bsorted, m, s.ovf_min) : m;
        const uint32_t obase = s.ovf_n;
        const uint32_t nevict = (nold + mk > cfg.ccap) ? nold + mk - cfg.ccap : 0u;
        if (tid == 0) s.evict_min = ~0ull;
        __syncthreads();
        for (uint32_t i = tid; i < m - mk; i += blockDim.x) {
          uint32_t o = obase + i;
          if (o < cfg.ocap) ovf[o] = bsorted[mk + i];
        }
        for (uint32_t i = tid; i < nold; i += blockDim.x) {
          unsigned long long k = old[i];
          uint32_t pos = i + lower_bound_keys(bsorted, mk, k);
          if (pos < cfg.ccap) cn[pos] = k;
          else {
            uint32_t o = obase + (m - mk) + (pos - cfg.ccap);
            if (o < cfg.ocap) ovf[o] = k;
            if (pos == cfg.ccap) s.evict_min = k;
          }
        }
        for (uint32_t i = tid; i < mk; i += blockDim.x) {
          unsigned long long k = bsorted[i];
          uint32_t pos = i + lower_bound_keys(old, nold, k);
          if (pos < cfg.ccap) cn[pos] = k;
          else {
            uint32_t o = obase + (m - mk) + (pos - cfg.ccap);
            if (o < cfg.ocap) ovf[o] = k;
            if (pos == cfg.ccap) s.evict_min = k;
          }
        }
        __syncthreads();
        if (tid == 0) {
          uint32_t added = (m - mk) + nevict;
          if (added) {
            unsigned long long mn = s.evict_min;
            if (mk < m && bsorted[mk] < mn) mn = bsorted[mk];
            if (mn < s.ovf_min) s.ovf_min = mn;
            uint32_t n2 = s.ovf_n + added;
            if (n2 > cfg.ocap) { n2 = cfg.ocap; s.status |= kStatusCandidateOverflow; }
            s.ovf_n = n2;
          }
          s.head = 0;
          s.tail = nold + mk - nevict;
          s.cur ^= 1u;
        }
        __syncthreads();
      }
      // every thread is done with this expansion's target before thread 0 pops the next one
      __syncthreads();
    }
    // ---- results ---------------------------------------------------------------
    __syncthreads();
    {
      uint32_t n = s.nres;
      if (n > P.size_out) n = P.size_out;       // RESULT_DEFINED_RANGE: cut back to sizeBackup
      for (uint32_t i = tid; i < n; i += blockDim.x) {
        unsigned long long k = res[i];
        out[P.out_off + i] = ObjDist{key_id(k), key_dist(k)};
      }
      if (tid == 0) {
        out_count[q] = n;
        stats[q] = QueryStats{s.dc, s.expansions, s.nvisited, s.edges, s.status};
      }
    }
    if (s.spilled) {                         // leave the bitmap clean for the next query
      for (uint32_t i = tid; i < cfg.bitmap_words; i += blockDim.x) bitmap[i] = 0u;
      __threadfence();
    }
    __syncthreads();
  }
}

inline size_t exact_smem_bytes(uint32_t row_chunks, const ExactConfig& c) {
  return (size_t)row_chunks * 16 + (size_t)c.kcap * 8 + (size_t)c.ccap * 16 + (size_t)kExactChunk * 16 +
         (size_t)c.hcap * 4 + (size_t)kExactChunk * 8 + sizeof(ExactShared) + 16;
}

}  // namespace ngtg
