// Batched graph search: one warp per query inside a persistent kernel fed by a
// device work counter, search distances on a compact copy of the objects
// (bf16 for float objects), and an exact re-rank of the best candidates with
// the full-precision rows.
//
// Algorithm (the reference's best-first search, lib/NGT/Graph.cpp:716-835,
// with its order relaxed for parallelism):
//   * one sorted list of L (distance, id) keys per query holds candidates and
//     results together; bit 31 of the id word marks an entry as expanded;
//   * each iteration expands the P best unexpanded entries whose distance is
//     within explorationRadius = (1+epsilon) * r_k (r_k: the size-th best
//     distance so far, or the caller's radius), the reference's stopping rule;
//     the search ends when no such entry remains;
//   * the neighbours of the P parents (at most edge_size each, in edge order)
//     pass a per-query visited bitmap (one bit per object, in global memory,
//     cleared after the query) and their distances are computed by groups of
//     lanes with 16-byte loads; keys below the list's worst are sorted and
//     merged into the list;
//   * finally the best R = ceil(size * rerank_factor) entries are re-ranked with
//     the exact comparator over the full-precision rows, so every returned
//     distance is the reference comparator's value for that id.
//   * candidates that do not fit in the list (or are pushed out of it) go to a
//     per-warp spill tier in global memory, all larger than every list key;
//     when every list entry is expanded, the spill entries still within the
//     exploration limit come back (the smallest first, by an exact radix
//     select), so the candidate set is as unbounded as the reference's queue.
// Differences from the reference that can change which ids are found (and are
// why this kernel is checked by recall, not by id equality): P > 1 expands
// slightly more nodes per step, an expanded node reads at most nbr_cap / P
// neighbours, and the search distances are bf16 (exact for integer coordinates
// <= 256).
#pragma once
#include <cuda_bf16.h>
#include <cfloat>
#include "distance.cuh"
#include "device_index.h"

namespace ngtg {

constexpr int kFastWarps = 4;
constexpr int kFastThreads = 32 * kFastWarps;
constexpr uint32_t kExpandedBit = 0x80000000u;

struct FastConfig {
  uint32_t list_cap;       // L: power of two, 64..1024
  uint32_t nbr_cap;        // neighbour ids handled per iteration (power of two)
  uint32_t parents;        // P
  uint32_t sgroup;         // lanes per search distance (power of two <= 32)
  uint32_t ngroup;         // lanes per full-precision distance
  uint32_t search_chunks;  // 16-byte chunks per search row
  uint32_t rerank_x16;     // rerank factor * 16
  uint32_t bitmap_words;
  uint32_t max_iters;
  uint32_t spill_cap;      // keys per warp slot in the global spill tier
};

struct FastWarpSmem {
  uint32_t q;              // current query
  uint32_t n;              // list length
  uint32_t cur;            // active list buffer
  uint32_t nparents;
  uint32_t parents[16];
  uint32_t pexcl[16];
  uint32_t pbase[16];
  uint32_t seed_leaf;
};

__device__ __forceinline__ uint32_t key_rawid(unsigned long long k) { return (uint32_t)k & 0x7fffffffu; }
__device__ __forceinline__ bool key_expanded(unsigned long long k) { return ((uint32_t)k & kExpandedBit) != 0; }

// Ascending bitonic sort of a[0..n) (smem) by one warp; pads to the next power of two with ~0.
__device__ __forceinline__ void warp_bitonic_sort(unsigned long long* a, uint32_t n, int lane) {
  if (n <= 1) return;
  uint32_t p = 1;
  while (p < n) p <<= 1;
  for (uint32_t i = n + lane; i < p; i += 32) a[i] = ~0ull;
  __syncwarp();
  for (uint32_t k = 2; k <= p; k <<= 1) {
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = lane; i < p; i += 32) {
        uint32_t l = i ^ j;
        if (l > i) {
          unsigned long long x = a[i], y = a[l];
          bool up = (i & k) == 0;
          if ((x > y) == up) { a[i] = y; a[l] = x; }
        }
      }
      __syncwarp();
    }
  }
}

// Ascending sort of a[0..n), n <= 32, in registers (one key per lane, shuffle
// bitonic network), written back to a.
__device__ __forceinline__ void warp_sort32(unsigned long long* a, uint32_t n, int lane) {
  unsigned long long x = (uint32_t)lane < n ? a[lane] : ~0ull;
#pragma unroll
  for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      unsigned long long y = __shfl_xor_sync(0xffffffffu, x, j);
      bool lower = (lane & j) == 0;
      bool up = (lane & k) == 0;
      // keep the smaller key in the lower lane of an ascending pair
      bool take_min = lower == up;
      x = take_min ? (y < x ? y : x) : (y > x ? y : x);
    }
  }
  __syncwarp();
  if ((uint32_t)lane < n) a[lane] = x;
  __syncwarp();
}

// Ascending sort of a[0..n), n <= 32 * J, in registers: element e = j * 32 + lane
// sits in k[j] of `lane`; bitonic network with compare-exchanges inside a lane for
// strides >= 32 and shuffles below.  Written back to a.
template <int J>
__device__ __forceinline__ void warp_sort_reg(unsigned long long* a, uint32_t n, int lane) {
  unsigned long long k[J];
#pragma unroll
  for (int j = 0; j < J; j++) {
    const uint32_t e = (uint32_t)(j * 32 + lane);
    k[j] = e < n ? a[e] : ~0ull;
  }
#pragma unroll
  for (int size = 2; size <= 32 * J; size <<= 1) {
#pragma unroll
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      if (stride >= 32) {
        const int js = stride >> 5;
#pragma unroll
        for (int j = 0; j < J; j++) {
          if ((j & js) == 0) {
            const uint32_t e = (uint32_t)(j * 32 + lane);
            const bool up = (e & (uint32_t)size) == 0;
            unsigned long long x = k[j], y = k[j + js];
            if ((x > y) == up) { k[j] = y; k[j + js] = x; }
          }
        }
      } else {
#pragma unroll
        for (int j = 0; j < J; j++) {
          const uint32_t e = (uint32_t)(j * 32 + lane);
          const bool up = (e & (uint32_t)size) == 0;
          const bool lower = (lane & stride) == 0;
          unsigned long long y = __shfl_xor_sync(0xffffffffu, k[j], stride);
          k[j] = (lower == up) ? (y < k[j] ? y : k[j]) : (y > k[j] ? y : k[j]);
        }
      }
    }
  }
  __syncwarp();
#pragma unroll
  for (int j = 0; j < J; j++) {
    const uint32_t e = (uint32_t)(j * 32 + lane);
    if (e < n) a[e] = k[j];
  }
  __syncwarp();
}

// Number of entries of the sorted a[0..n) that are < x (ignoring the expanded bit of a's entries
// is not needed: keys are ordered by distance first, the bit only reorders exact distance ties).
__device__ __forceinline__ uint32_t warp_lower_bound(const unsigned long long* a, uint32_t n, unsigned long long x) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// L2 over float-typed rows with the packed fp32 instructions of sm_100-class
// GPUs (two lanes of IEEE fma per instruction, the same rounding as the scalar
// form): sum of (x - q)^2 accumulated in a float2.
template <ObjType ST, Metric M>
struct PackedL2 {
  static constexpr bool kOn = (M == Metric::L2 || M == Metric::InnerProduct) &&
                              (ST == ObjType::Bfloat16 || ST == ObjType::Float || ST == ObjType::Float16);
  static constexpr int P = ObjTraits<ST>::kPerChunk;
  // the query chunk negated and unpacked once per query
  __device__ __forceinline__ static void prepare(const uint4& q, float2 (&nq)[P / 2]) {
    float a[P];
    unpack<ST>(q, a);
#pragma unroll
    for (int i = 0; i < P; i += 2) nq[i / 2] = make_float2(-a[i], -a[i + 1]);
  }
  __device__ __forceinline__ static float2 add(float2 acc, const float2 (&nq)[P / 2], const uint4& x) {
    float b[P];
    unpack<ST>(x, b);
#pragma unroll
    for (int i = 0; i < P; i += 2) {
      float2 dlt = __fadd2_rn(make_float2(b[i], b[i + 1]), nq[i / 2]);
      acc = __ffma2_rn(dlt, dlt, acc);
    }
    return acc;
  }
};

// U: rows per lane group in flight in the distance loop; MINB: CTAs per SM the
// register allocation is sized for.
template <ObjType ST, ObjType OT, Metric M, int U = 4, int MINB = 5>
__global__ void __launch_bounds__(kFastThreads, MINB)
graph_search_fast_kernel(DevGraph g, const uint4* __restrict__ srows, const uint4* __restrict__ queries, uint32_t nq,
                         const QueryParams* __restrict__ params, const uint32_t* __restrict__ seed_list,
                         ObjDist* __restrict__ out, uint32_t* __restrict__ out_count, QueryStats* __restrict__ stats,
                         uint32_t* __restrict__ bitmaps, uint32_t* __restrict__ work,
                         unsigned long long* __restrict__ spills, FastConfig cfg) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t rc = g.row_chunks, sc = cfg.search_chunks;
  const uint32_t L = cfg.list_cap, NB = cfg.nbr_cap;
  // per-warp carve-up
  const size_t per_warp = (size_t)rc * 16 + (size_t)sc * 16 + (size_t)L * 8 + (size_t)NB * 16 + sizeof(FastWarpSmem);
  unsigned char* base = smem + warp * ((per_warp + 15) & ~(size_t)15);
  uint4* qn = reinterpret_cast<uint4*>(base);                  // query, object type
  uint4* qs = qn + rc;                                          // query, search type
  unsigned long long* list = reinterpret_cast<unsigned long long*>(qs + sc);
  unsigned long long* nkey = list + L;                          // NB keys
  uint32_t* nid = reinterpret_cast<uint32_t*>(nkey + NB);       // NB ids
  float* nd = reinterpret_cast<float*>(nid + NB);                // NB search distances
  FastWarpSmem& w = *reinterpret_cast<FastWarpSmem*>(nd + NB);
  const uint32_t slot = blockIdx.x * kFastWarps + warp;
  uint32_t* bitmap = bitmaps + (size_t)slot * cfg.bitmap_words;
  // spill tier: candidates that do not fit in the list, all larger than every list key
  unsigned long long* spill = spills + (size_t)slot * 2 * cfg.spill_cap;
  unsigned long long* spill_tmp = spill + cfg.spill_cap;
  const int SG = (int)cfg.sgroup, NG = (int)cfg.ngroup;
  const int sgl = lane & (SG - 1), ngl = lane & (NG - 1);

  while (true) {
    if (lane == 0) w.q = atomicAdd(work, 1u);
    __syncwarp();
    const uint32_t q = w.q;
    if (q >= nq) break;
    const QueryParams P = params[q];
    for (uint32_t i = lane; i < rc; i += 32) qn[i] = queries[(size_t)q * rc + i];
    __syncwarp();
    if constexpr (ST != OT) {
      // float object rows -> bf16 search rows (round to nearest even)
      const float* qf = reinterpret_cast<const float*>(qn);
      uint32_t* qb = reinterpret_cast<uint32_t*>(qs);
      for (uint32_t i = lane; i < sc * 4; i += 32) {
        uint32_t lo = __bfloat16_as_ushort(__float2bfloat16_rn(qf[2 * i]));
        uint32_t hi = __bfloat16_as_ushort(__float2bfloat16_rn(qf[2 * i + 1]));
        qb[i] = lo | (hi << 16);
      }
    } else {
      for (uint32_t i = lane; i < sc; i += 32) qs[i] = qn[i];
    }
    __syncwarp();
    uint32_t dc = 0, expansions = 0, edges_read = 0, status = 0, visited = 0;
    uint32_t n = 0;
    uint32_t scan0 = 0;        // no unexpanded entry before this position
    uint32_t spill_n = 0;
    unsigned long long spill_min = ~0ull;
    bool refill = false;
    if (P.size == 0) {
      if (lane == 0) { out_count[q] = 0; stats[q] = QueryStats{0, 0, 0, 0, 0}; }
      __syncwarp();
      continue;
    }
    // ---- seeds -------------------------------------------------------------------
    const uint32_t* seeds = nullptr;
    uint32_t nseeds = 0;
    if (P.seed_cnt == 0xffffffffu) {
      uint32_t node = g.root;
      int depth = 0;
      while (!(node & 0x80000000u) && depth < 64) {
        const DevInternal& in = g.internals[node];
        float d = group_distance<TreeSpace<OT, M>::ot, TreeSpace<OT, M>::m>(qn, g.pivots + (size_t)in.pivot * rc, (int)rc, lane, 32);
        uint32_t bsize = in.nchildren - 1, mid;
        for (mid = 0; mid < bsize; mid++)
          if (d < in.borders[mid]) break;
        node = in.children[mid];
        depth++;
      }
      if (node & 0x80000000u) {
        uint32_t leaf = node & 0x7fffffffu;
        if (leaf < g.nleaves) {
          const uint32_t* off = g.leaf_seed_off + P.seed_off;
          seeds = g.leaf_seed_ids + off[leaf];
          nseeds = off[leaf + 1] - off[leaf];
        }
      } else {
        status |= kStatusTreeError;
      }
    } else {
      seeds = seed_list + P.seed_off;
      nseeds = P.seed_cnt;
    }
    nseeds = min(nseeds, NB);
    // seeds are marked visited and become the first candidates
    uint32_t m = 0;
    for (uint32_t b = 0; b < nseeds; b += 32) {
      uint32_t i = b + lane;
      bool fresh = false;
      uint32_t id = 0;
      if (i < nseeds) {
        id = seeds[i];
        if (id < g.nrows) {
          uint32_t bit = 1u << (id & 31u);
          fresh = (atomicOr(&bitmap[id >> 5], bit) & bit) == 0u;
        }
      }
      unsigned bal = __ballot_sync(0xffffffffu, fresh);
      if (fresh) nid[m + __popc(bal & ((1u << lane) - 1u))] = id;
      m += __popc(bal);
    }
    __syncwarp();
    for (uint32_t b = 0; b < m; b += 32 / SG) {     // warp-uniform trip count
      uint32_t i = b + (uint32_t)(lane / SG);
      bool valid = i < m;
      uint32_t id = valid ? nid[i] : 0u;
      float d = group_distance<ST, M>(qs, srows + (size_t)id * sc, (int)sc, sgl, SG);
      if (valid && sgl == 0) nkey[i] = pack_key(d, id);
    }
    __syncwarp();
    dc += m;
    visited += m;
    warp_bitonic_sort(nkey, m, lane);
    n = min(m, L);
    for (uint32_t i = lane; i < n; i += 32) list[i] = nkey[i];
    __syncwarp();
    if (nseeds == 0) status |= kStatusEmptySeeds;

    // ---- best-first iterations ----------------------------------------------------------
    const float user_radius = P.radius;
    for (uint32_t it = 0; it < cfg.max_iters; it++) {
      float rk = (n >= P.size) ? fminf(key_dist(list[P.size - 1]), user_radius) : user_radius;
      const float limit = P.coef * rk;
      // pick up to `parents` unexpanded entries within the limit, in list order
      uint32_t np = 0;
      bool stop = false;
      if (refill) {
        // ---- every list entry is expanded: refill from the spill tier ----
        // keep the first `size` entries (the results so far), drop the other expanded ones
        n = min(n, P.size);
        const uint32_t room = L - n;
        uint32_t r = 0;
        for (uint32_t b = 0; b < spill_n; b += 32) {           // live spill entries -> spill_tmp
          uint32_t i = b + lane;
          unsigned long long k = i < spill_n ? spill[i] : ~0ull;
          bool live = i < spill_n && key_dist(k) <= limit;
          unsigned bal = __ballot_sync(0xffffffffu, live);
          if (live) spill_tmp[r + __popc(bal & ((1u << lane) - 1u))] = k;
          r += __popc(bal);
        }
        __syncwarp();
        unsigned long long thr = ~0ull;                           // take keys <= thr
        if (r > room) {
          // exact radix select of the room-th smallest key
          unsigned long long prefix = 0, mask = 0;
          uint32_t need = room;
          for (int shift = 56; shift >= 0; shift -= 8) {
            uint32_t* hist = reinterpret_cast<uint32_t*>(nd);     // nd is idle during a refill
            for (uint32_t i = lane; i < 256; i += 32) hist[i] = 0;
            __syncwarp();
            for (uint32_t i = lane; i < r; i += 32) {
              unsigned long long k = spill_tmp[i];
              if ((k & mask) == prefix) atomicAdd(&hist[(uint32_t)(k >> shift) & 255u], 1u);
            }
            __syncwarp();
            uint32_t acc = 0, bsel = 255;
            for (uint32_t b = 0; b < 256; b++) {
              uint32_t h = hist[b];
              if (acc + h >= need) { bsel = b; break; }
              acc += h;
            }
            prefix |= (unsigned long long)bsel << shift;
            need -= acc;
            mask |= 255ull << shift;
            __syncwarp();
          }
          thr = prefix;
        }
        // entries <= thr go behind the kept results (all larger than them); the rest stay
        uint32_t moved = 0, stay = 0;
        unsigned long long smin = ~0ull;
        for (uint32_t b = 0; b < r; b += 32) {
          uint32_t i = b + lane;
          unsigned long long k = i < r ? spill_tmp[i] : ~0ull;
          bool take = i < r && k <= thr;
          bool keep = i < r && k > thr;
          unsigned bt = __ballot_sync(0xffffffffu, take), bk = __ballot_sync(0xffffffffu, keep);
          if (take) nkey[moved + __popc(bt & ((1u << lane) - 1u))] = k;
          if (keep) { spill[stay + __popc(bk & ((1u << lane) - 1u))] = k; smin = k < smin ? k : smin; }
          moved += __popc(bt);
          stay += __popc(bk);
        }
        for (int off = 16; off > 0; off >>= 1) {
          unsigned long long o = __shfl_xor_sync(0xffffffffu, smin, off);
          smin = o < smin ? o : smin;
        }
        __syncwarp();
        warp_bitonic_sort(nkey, moved, lane);
        for (uint32_t i = lane; i < moved; i += 32) list[n + i] = nkey[i];
        __syncwarp();
        scan0 = n;
        n += moved;
        spill_n = stay;
        spill_min = smin;
        refill = false;
      }
      for (uint32_t b = scan0 & ~31u; b < n && !stop && np < cfg.parents; b += 32) {
        uint32_t i = b + lane;
        unsigned long long k = i < n ? list[i] : ~0ull;
        unsigned ball = __ballot_sync(0xffffffffu, i < n && !key_expanded(k));
        while (ball && np < cfg.parents) {
          int j = __ffs(ball) - 1;
          unsigned long long kj = __shfl_sync(0xffffffffu, k, j);
          if (key_dist(kj) > limit) { stop = true; break; }
          if (lane == j) list[i] = k | kExpandedBit;
          if (lane == 0) w.parents[np] = key_rawid(kj);
          np++;
          scan0 = b + (uint32_t)j + 1;
          ball &= ball - 1;
        }
      }
      __syncwarp();
      if (np == 0) {
        // the list is exhausted (not stopped by the radius): continue from the spill tier
        if (!stop && spill_n > 0 && key_dist(spill_min) <= limit) {
          scan0 = n;
          refill = true;
          continue;
        }
        break;
      }
      expansions += np;
      // gather unvisited neighbours of the parents, in edge order.  All edge
      // loads are issued before any visited-bit atomic, and all atomics before
      // any compaction, so the gather costs a few memory round trips, not one
      // per 32 edges.
      const uint32_t per_parent = min(P.edge_size, NB / np);
      uint32_t pe0 = 0, pne = 0;
      if ((uint32_t)lane < np) {
        const uint32_t v = w.parents[lane];
        const uint32_t a = g.offsets[v];
        pe0 = a;
        pne = min(g.offsets[v + 1] - a, per_parent);
      }
      uint32_t incl = pne;
#pragma unroll
      for (int off = 1; off < 16; off <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += t;
      }
      const uint32_t total = __shfl_sync(0xffffffffu, incl, np - 1);
      // parent of edge slot t: the last parent whose exclusive prefix is <= t
      if ((uint32_t)lane < np) {
        w.pexcl[lane] = incl - pne;
        w.pbase[lane] = pe0;
      }
      __syncwarp();
      edges_read += total;
      uint32_t cnt = 0;
      constexpr int J = 12;     // 384 edge slots per round: four parents of an ONNG node in one pass
      for (uint32_t base0 = 0; base0 < total; base0 += 32 * J) {
        uint32_t ids[J];
        bool fresh[J];
#pragma unroll
        for (int j = 0; j < J; j++) {
          uint32_t t = base0 + lane + 32 * j;
          ids[j] = 0;
          if (t < total) {
            uint32_t p2 = 0;
            for (uint32_t c = 1; c < np; c++)
              if (t >= w.pexcl[c]) p2 = c;
            ids[j] = __ldg(g.edges + w.pbase[p2] + (t - w.pexcl[p2]));
          }
        }
#pragma unroll
        for (int j = 0; j < J; j++) {
          uint32_t t = base0 + lane + 32 * j;
          fresh[j] = false;
          if (t < total) {
            uint32_t bit = 1u << (ids[j] & 31u);
            fresh[j] = (atomicOr(&bitmap[ids[j] >> 5], bit) & bit) == 0u;
          }
        }
#pragma unroll
        for (int j = 0; j < J; j++) {
          unsigned bal = __ballot_sync(0xffffffffu, fresh[j]);
          if (fresh[j]) nid[cnt + __popc(bal & ((1u << lane) - 1u))] = ids[j];
          cnt += __popc(bal);
        }
      }
      __syncwarp();
      visited += cnt;
      dc += cnt;
      // distances of the new neighbours: keys below the list's worst are merged,
      // the others (still within the exploration limit) join the spill tier
      const unsigned long long worst = (n >= L) ? (list[L - 1] & ~(unsigned long long)kExpandedBit) : ~0ull;
      float rk2 = (n >= P.size) ? fminf(key_dist(list[P.size - 1]), user_radius) : user_radius;
      const float insert_limit = P.coef * rk2;
      uint32_t kept = 0;
      const uint32_t gpw = 32 / SG;
      unsigned long long smin = spill_min;
      // distances are parked in nd[] by the group leaders and placed 32 at a time below
      auto place = [&](uint32_t i, float d, uint32_t) {
        if (i < cnt && sgl == 0) nd[i] = d;
      };
      if (sc <= (uint32_t)SG * 2) {
        // at most two 16-byte chunks per lane per row; U rows per group in flight
        const uint32_t c0 = (uint32_t)sgl, c1 = (uint32_t)sgl + (uint32_t)SG;
        const uint4 zero = make_uint4(0, 0, 0, 0);
        const uint4 q0 = c0 < sc ? qs[c0] : zero, q1 = c1 < sc ? qs[c1] : zero;
        float2 nq0[PackedL2<ST, M>::P / 2], nq1[PackedL2<ST, M>::P / 2];
        if constexpr (PackedL2<ST, M>::kOn) {
          PackedL2<ST, M>::prepare(q0, nq0);
          PackedL2<ST, M>::prepare(q1, nq1);
        }
        for (uint32_t b = 0; b < cnt; b += gpw * U) {
          uint4 x0[U], x1[U];
          uint32_t idu[U];
#pragma unroll
          for (int u = 0; u < U; u++) {
            uint32_t i = b + u * gpw + (uint32_t)(lane / SG);
            idu[u] = i < cnt ? nid[i] : 0u;
            const uint4* row = srows + (size_t)idu[u] * sc;
            x0[u] = c0 < sc ? __ldg(row + c0) : zero;
            x1[u] = c1 < sc ? __ldg(row + c1) : zero;
          }
#pragma unroll
          for (int u = 0; u < U; u++) {
            float d;
            if constexpr (PackedL2<ST, M>::kOn) {
              float2 acc = make_float2(0.f, 0.f);
              if (c0 < sc) acc = PackedL2<ST, M>::add(acc, nq0, x0[u]);
              if (c1 < sc) acc = PackedL2<ST, M>::add(acc, nq1, x1[u]);
              float v = acc.x + acc.y;
#pragma unroll
              for (int off = 16; off > 0; off >>= 1)
                if (off < SG) v += __shfl_xor_sync(0xffffffffu, v, off);
              d = sqrtf(v);
            } else {
              Acc<ST, M> acc;
              if (c0 < sc) acc.add(q0, x0[u], (int)c0);
              if (c1 < sc) acc.add(q1, x1[u], (int)c1);
              acc.reduce(SG);
              d = acc.finish();
            }
            place(b + u * gpw + (uint32_t)(lane / SG), d, idu[u]);
          }
        }
      } else {
        for (uint32_t b = 0; b < cnt; b += gpw) {
          uint32_t i = b + (uint32_t)(lane / SG);
          uint32_t id = i < cnt ? nid[i] : 0u;
          float d = group_distance<ST, M>(qs, srows + (size_t)id * sc, (int)sc, sgl, SG);
          place(i, d, id);
        }
      }
      __syncwarp();
      // placement: keys below the list's worst are merged, the others still within
      // the exploration limit join the spill tier (one entry per lane per step)
      for (uint32_t b = 0; b < cnt; b += 32) {
        uint32_t i = b + lane;
        float d = i < cnt ? nd[i] : 0.f;
        unsigned long long key = i < cnt ? pack_key(d, nid[i]) : ~0ull;
        bool live = i < cnt && d <= insert_limit;
        bool keep = live && key < worst;
        bool spl = live && key >= worst;
        unsigned bal = __ballot_sync(0xffffffffu, keep), bs = __ballot_sync(0xffffffffu, spl);
        if (keep) nkey[kept + __popc(bal & ((1u << lane) - 1u))] = key;
        if (spl) {
          uint32_t o = spill_n + __popc(bs & ((1u << lane) - 1u));
          if (o < cfg.spill_cap) spill[o] = key;
          smin = key < smin ? key : smin;
        }
        kept += __popc(bal);
        spill_n += __popc(bs);
      }
      for (int off = 16; off > 0; off >>= 1) {
        unsigned long long o = __shfl_xor_sync(0xffffffffu, smin, off);
        smin = o < smin ? o : smin;
      }
      spill_min = smin;
      if (spill_n > cfg.spill_cap) { spill_n = cfg.spill_cap; status |= kStatusCandidateOverflow; }
      __syncwarp();
      if (kept == 0) continue;
      if (kept <= 32) warp_sort32(nkey, kept, lane);
      else if (kept <= 64) warp_sort_reg<2>(nkey, kept, lane);
      else if (kept <= 128) warp_sort_reg<4>(nkey, kept, lane);
      else warp_bitonic_sort(nkey, kept, lane);
      // In-place merge of nkey[0..kept) into list[0..n), keeping the first L.
      // 1. merged positions of the new keys (list entries compare without their
      //    expanded bit), parked in nid (no longer needed)
      for (uint32_t i = lane; i < kept; i += 32) {
        unsigned long long k = nkey[i];
        uint32_t lo = 0, hi = n;
        while (lo < hi) {
          uint32_t mid = (lo + hi) >> 1;
          if ((list[mid] & ~(unsigned long long)kExpandedBit) < k) lo = mid + 1; else hi = mid;
        }
        nid[i] = i + lo;
      }
      __syncwarp();
      const uint32_t first_new = nid[0];
      // 2. list entries move right (never left): chunks from the top down, each
      //    read completely before any of it is written; unexpanded entries pushed
      //    past the end join the spill tier
      unsigned long long emin = ~0ull;
      for (int hi = (int)n; hi > (int)first_new; hi -= 32) {
        int idx = hi - 32 + lane;
        if (idx < (int)first_new) idx = -1;          // below the first insertion: unchanged
        unsigned long long k = 0;
        uint32_t pos = 0xffffffffu;
        if (idx >= 0) {
          k = list[idx];
          pos = (uint32_t)idx + warp_lower_bound(nkey, kept, k & ~(unsigned long long)kExpandedBit);
        }
        __syncwarp();
        if (idx >= 0 && pos < L) list[pos] = k;
        bool ev = idx >= 0 && pos >= L && !key_expanded(k);
        unsigned be = __ballot_sync(0xffffffffu, ev);
        if (ev) {
          uint32_t o = spill_n + __popc(be & ((1u << lane) - 1u));
          if (o < cfg.spill_cap) spill[o] = k;
          emin = k < emin ? k : emin;
        }
        spill_n += __popc(be);
        __syncwarp();
      }
      // 3. the new keys (those pushed past the end join the spill tier)
      for (uint32_t b = 0; b < kept; b += 32) {
        uint32_t i = b + lane;
        bool in = i < kept && nid[i] < L;
        bool ev = i < kept && nid[i] >= L;
        if (in) list[nid[i]] = nkey[i];
        unsigned be = __ballot_sync(0xffffffffu, ev);
        if (ev) {
          uint32_t o = spill_n + __popc(be & ((1u << lane) - 1u));
          if (o < cfg.spill_cap) spill[o] = nkey[i];
          emin = nkey[i] < emin ? nkey[i] : emin;
        }
        spill_n += __popc(be);
      }
      for (int off = 16; off > 0; off >>= 1) {
        unsigned long long o = __shfl_xor_sync(0xffffffffu, emin, off);
        emin = o < emin ? o : emin;
      }
      if (emin < spill_min) spill_min = emin;
      if (spill_n > cfg.spill_cap) { spill_n = cfg.spill_cap; status |= kStatusCandidateOverflow; }
      __syncwarp();
      n = min(n + kept, L);
      if (first_new < scan0) scan0 = first_new;
    }

    // ---- exact re-rank of the best entries with the full-precision rows -------------------
    uint32_t R = min(n, max(P.size, (uint32_t)((P.size * cfg.rerank_x16 + 15) / 16)));
    const uint32_t gpn = 32 / NG;
    for (uint32_t b = 0; b < R; b += gpn) {
      uint32_t i = b + (uint32_t)(lane / NG);
      bool valid = i < R;
      uint32_t id = valid ? key_rawid(list[i]) : 0u;
      float d = group_distance<OT, M>(qn, g.objects + (size_t)id * rc, (int)rc, ngl, NG);
      if (valid && ngl == 0) nkey[i] = pack_key(d, id);
    }
    __syncwarp();
    warp_bitonic_sort(nkey, R, lane);
    uint32_t nout = 0;
    for (uint32_t b = 0; b < R && nout < P.size_out; b += 32) {
      uint32_t i = b + lane;
      bool ok = i < R && key_dist(nkey[i]) <= user_radius;
      unsigned bal = __ballot_sync(0xffffffffu, ok);
      uint32_t pos = nout + __popc(bal & ((1u << lane) - 1u));
      if (ok && pos < P.size_out) out[P.out_off + pos] = ObjDist{key_id(nkey[i]), key_dist(nkey[i])};
      nout = min(P.size_out, nout + __popc(bal));
    }
    if (lane == 0) {
      out_count[q] = nout;
      stats[q] = QueryStats{dc, expansions, visited, edges_read, status};
    }
    // clear this slot's visited bitmap for the next query
    uint4* bm4 = reinterpret_cast<uint4*>(bitmap);
    for (uint32_t i = lane; i < cfg.bitmap_words / 4; i += 32) bm4[i] = make_uint4(0, 0, 0, 0);
    __syncwarp();
  }
}

inline size_t fast_smem_per_warp(uint32_t row_chunks, const FastConfig& c) {
  size_t per = (size_t)row_chunks * 16 + (size_t)c.search_chunks * 16 + (size_t)c.list_cap * 8 +
               (size_t)c.nbr_cap * 16 + sizeof(FastWarpSmem);
  return (per + 15) & ~(size_t)15;
}

}  // namespace ngtg
