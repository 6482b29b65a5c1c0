// Relaxed-order quantized-graph search: the batched form of NGTQG's search
// (lib/NGT/NGTQ/QuantizedGraph.h:283-447), one query per 128-thread CTA over a
// work counter.  The query is rotated and its uint8 distance table built exactly
// as qg_search_kernel does, so every quantized distance equals the reference's;
// what is relaxed is the order of expansion, as in the CTA-per-query graph kernel:
//   * one sorted candidate list of (distance, id) keys (seeds with exact L2, then
//     quantized distances), an expanded flag per entry kept beside it;
//   * per step, up to P unexpanded entries within (1 + epsilon) x r_k (r_k: the
//     size-th entry's distance, or the radius) are expanded together: the 16-
//     neighbour code blocks of all of them are scanned by the four warps at once
//     (two blocks per warp iteration, both loaded before either is scored; the
//     reference's 4-bit lookups and saturating sums);
//   * the neighbours within the limit are checked against the per-CTA visited
//     bitmap afterwards, eight atomics in flight per thread, and the fresh ones
//     sorted and merged into the list (each key's place is its rank in the other
//     list), which keeps the L best;
//   * the search stops when no unexpanded entry is within the limit; the first
//     `size` entries within the radius are the result set, re-ranked by exact L2
//     (cut at the radius, truncated to k) when the result expansion is >= 1.
// Results are a superset walk of the reference's (recall at a given epsilon at
// least the exact-order kernel's in the tests); returned distances are exact
// whenever the re-rank runs.
#pragma once
#include <cfloat>
#include "graph_wide.cuh"
#include "qg_search.cuh"

namespace ngtg {

constexpr uint32_t kQGWideThreads = 128;
constexpr uint32_t kQGWideWarps = kQGWideThreads / 32;

struct QGWideConfig {
  uint32_t list_cap;      // L: power of two, > the largest result-set size
  uint32_t nbr_cap;       // NB: power of two, >= 16 x the code blocks of the largest node
  uint32_t parents;       // P: 1..32
  uint32_t group;         // lanes per exact distance (power of two <= 32)
  uint32_t bitmap_words;  // per CTA, multiple of 4
  uint32_t max_iters;
};

struct QGWideShared {
  uint32_t q, n, cur, np, nblk, cnt, pend, status, dc, expansions, edges, visited, seed_leaf;
  float lut_min, lut_scale, limit;
  float wmin[kQGWideWarps], wmax[kQGWideWarps];
  uint32_t parents[32], pdeg[32], poff[32], pblk[33];
};

// bytes of the work region (new keys, ids, distances), which also holds the float
// table while it is built
__host__ __device__ inline size_t qg_wide_work_bytes(uint32_t nbr_cap, uint32_t m) {
  const size_t work = (size_t)nbr_cap * 16, flut = (size_t)m * 64;
  return work > flut ? work : flut;
}

inline size_t qg_wide_smem_bytes(uint32_t row_chunks, uint32_t dim, uint32_t m, const QGWideConfig& c) {
  size_t b = (size_t)row_chunks * 16;                    // query row
  b += ((size_t)dim * 4 + 15) / 16 * 16;                 // rotated query
  b += ((size_t)m * 16 + 15) / 16 * 16;                  // uint8 table
  b += (size_t)c.list_cap * 16;                          // two list buffers
  b += ((size_t)c.list_cap * 2 + 15) / 16 * 16;          // their expanded flags
  b += qg_wide_work_bytes(c.nbr_cap, m);
  b += sizeof(QGWideShared) + 16;
  return b;
}

// first index i in a[0..n) with a[i] >= k (a ascending)
__device__ __forceinline__ uint32_t qgw_lower_bound(const unsigned long long* a, uint32_t n, unsigned long long k) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (a[mid] < k) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// BPI: code blocks each warp loads before scoring them (2 or 4)
template <int SPL, int BPI>
__global__ void __launch_bounds__(kQGWideThreads, SPL <= 4 && BPI == 2 ? 6 : 4)
qg_wide_kernel(DevGraph g, DevQG qg, const uint4* __restrict__ queries, uint32_t nq,
               const QGParams* __restrict__ params, const uint32_t* __restrict__ seed_list,
               ObjDist* __restrict__ out, uint32_t* __restrict__ out_count, QueryStats* __restrict__ stats,
               uint32_t* __restrict__ bitmaps, uint32_t* __restrict__ work, QGWideConfig cfg) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t rc = g.row_chunks, D = qg.dim, M = qg.m, LD = qg.ld;
  const uint32_t L = cfg.list_cap, NB = cfg.nbr_cap;
  uint4* qv = reinterpret_cast<uint4*>(smem);
  float* rq = reinterpret_cast<float*>(qv + rc);
  uint8_t* lut = reinterpret_cast<uint8_t*>(rq + (D + 3) / 4 * 4);
  unsigned long long* lists = reinterpret_cast<unsigned long long*>(lut + ((size_t)M * 16 + 15) / 16 * 16);
  uint8_t* lexp = reinterpret_cast<uint8_t*>(lists + 2 * (size_t)L);
  unsigned long long* nkey = reinterpret_cast<unsigned long long*>(lexp + ((size_t)L * 2 + 15) / 16 * 16);
  uint32_t* nid = reinterpret_cast<uint32_t*>(nkey + NB);
  float* nd = reinterpret_cast<float*>(nid + NB);
  float* flut = reinterpret_cast<float*>(nkey);          // only while the table is built
  QGWideShared& s =
      *reinterpret_cast<QGWideShared*>(reinterpret_cast<unsigned char*>(nkey) + qg_wide_work_bytes(NB, M));
  uint32_t* bitmap = bitmaps + (size_t)blockIdx.x * cfg.bitmap_words;
  const int G = (int)cfg.group;
  const int gl = lane & (G - 1);
  const int ngroups = (int)kQGWideThreads / G;
  const float* qf = reinterpret_cast<const float*>(qv);
  const uint32_t qlen = rc * 4;

  while (true) {
    if (tid == 0) s.q = atomicAdd(work, 1u);
    __syncthreads();
    const uint32_t q = s.q;
    if (q >= nq) break;
    const QGParams P = params[q];
    for (uint32_t i = tid; i < rc; i += blockDim.x) qv[i] = queries[(size_t)q * rc + i];
    if (tid == 0) {
      s.n = 0; s.cur = 0; s.status = 0; s.dc = 0; s.expansions = 0; s.edges = 0; s.visited = 0;
    }
    __syncthreads();
    if (P.size == 0 || P.k == 0) {
      if (tid == 0) { out_count[q] = 0; stats[q] = QueryStats{0, 0, 0, 0, 0}; }
      __syncthreads();
      continue;
    }
    // ---- rotation and distance table (the exact-order kernel's arithmetic) -------
    for (uint32_t c = tid; c < D; c += blockDim.x) {
      float acc = 0.f;
      if (qg.rotation == nullptr) {
        acc = c < qlen ? qf[c] : 0.f;
      } else if (D <= 48) {
        for (uint32_t p = 0; p < D; p++)
          acc = __fmaf_rn(qg.rotation[(size_t)p * D + c], p < qlen ? qf[p] : 0.f, acc);
      } else {
        for (uint32_t p0 = 0; p0 < D; p0 += 8) {
          const uint32_t p1 = min(p0 + 8u, D);
          float t = __fmul_rn(qg.rotation[(size_t)p0 * D + c], p0 < qlen ? qf[p0] : 0.f);
          for (uint32_t p = p0 + 1; p < p1; p++)
            t = __fmaf_rn(qg.rotation[(size_t)p * D + c], p < qlen ? qf[p] : 0.f, t);
          acc = __fadd_rn(acc, t);
        }
      }
      rq[c] = acc;
    }
    __syncthreads();
    {
      float lmin = FLT_MAX, lmax = -FLT_MAX;
      for (uint32_t e = tid; e < M * 16; e += blockDim.x) {
        const uint32_t sv = e >> 4, c = e & 15u;
        float v = 0.f;
        for (uint32_t d = 0; d < LD; d++) {
          const float rsv = __fsub_rn(rq[sv * LD + d], qg.gcentroid[sv * LD + d]);
          const float sub = __fsub_rn(rsv, qg.lcentroids[((size_t)sv * 16 + c) * LD + d]);
          v = d == 0 ? __fmul_rn(sub, sub) : __fmaf_rn(sub, sub, v);
        }
        flut[e] = v;
        lmin = fminf(lmin, v);
        lmax = fmaxf(lmax, v);
      }
      for (int off = 16; off > 0; off >>= 1) {
        lmin = fminf(lmin, __shfl_xor_sync(0xffffffffu, lmin, off));
        lmax = fmaxf(lmax, __shfl_xor_sync(0xffffffffu, lmax, off));
      }
      if (lane == 0) { s.wmin[warp] = lmin; s.wmax[warp] = lmax; }
      __syncthreads();
      if (tid == 0) {
        float mn = s.wmin[0], mx = s.wmax[0];
        for (uint32_t w = 1; w < kQGWideWarps; w++) { mn = fminf(mn, s.wmin[w]); mx = fmaxf(mx, s.wmax[w]); }
        s.lut_min = mn;
        s.lut_scale = __double2float_rn(__ddiv_rn((double)__fsub_rn(mx, mn), 255.0));
      }
      __syncthreads();
      const float mn = s.lut_min, scale = s.lut_scale;
      for (uint32_t e = tid; e < M * 16; e += blockDim.x)
        lut[e] = (uint8_t)(int)rintf(__fdiv_rn(__fsub_rn(flut[e], mn), scale));
      __syncthreads();
    }
    uint32_t Lr[SPL][4];
#pragma unroll
    for (int j = 0; j < SPL; j++) {
      const uint32_t sv = (uint32_t)lane + 32u * (uint32_t)j;
      const uint4 t = sv < M ? reinterpret_cast<const uint4*>(lut)[sv] : make_uint4(0, 0, 0, 0);
      Lr[j][0] = t.x; Lr[j][1] = t.y; Lr[j][2] = t.z; Lr[j][3] = t.w;
    }
    const float lscale = s.lut_scale, loffset = __fmul_rn(s.lut_min, (float)M);
    // ---- seeds: tree leaf or explicit list, exact L2, marked visited --------------
    const uint32_t* seeds = nullptr;
    uint32_t nseeds = 0;
    if (P.seed_cnt == 0xffffffffu) {
      if (warp == 0) {
        uint32_t node = g.root;
        int depth = 0;
        while (!(node & 0x80000000u) && depth < 64) {
          const DevInternal& in = g.internals[node];
          float d = group_distance<ObjType::Float, Metric::L2>(qv, g.pivots + (size_t)in.pivot * rc, (int)rc, lane,
                                                               32);
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
        const uint32_t* off = g.leaf_seed_off + P.seed_off;
        seeds = g.leaf_seed_ids + off[s.seed_leaf];
        nseeds = off[s.seed_leaf + 1] - off[s.seed_leaf];
      }
    } else {
      seeds = seed_list + P.seed_off;
      nseeds = P.seed_cnt;
    }
    nseeds = min(nseeds, NB);
    if (tid == 0) s.cnt = 0;
    __syncthreads();
    for (uint32_t i = tid; i < nseeds; i += blockDim.x) {
      const uint32_t id = seeds[i];
      if (id < g.nrows) {
        const uint32_t bit = 1u << (id & 31u);
        if ((atomicOr(&bitmap[id >> 5], bit) & bit) == 0u) nid[atomicAdd(&s.cnt, 1u)] = id;
      }
    }
    __syncthreads();
    {
      const uint32_t m = s.cnt;
      for (uint32_t b = (uint32_t)(warp * (32 / G)); b < m; b += (uint32_t)ngroups) {
        const uint32_t i = b + (uint32_t)(lane / G);
        const bool valid = i < m;
        const uint32_t id = valid ? nid[i] : 0u;
        const float d = group_distance<ObjType::Float, Metric::L2>(qv, g.objects + (size_t)id * rc, (int)rc, gl, G);
        if (valid && gl == 0) nkey[i] = pack_key(d, id);
      }
      __syncthreads();
      cta_bitonic_sort(nkey, m, NB);
      const uint32_t n0 = min(m, L);
      for (uint32_t i = tid; i < n0; i += blockDim.x) {
        lists[i] = nkey[i];
        lexp[i] = 0;
      }
      if (tid == 0) {
        s.n = n0;
        s.dc = m;
        s.visited = m;
        if (m == 0) s.status |= kStatusEmptySeeds;
      }
      __syncthreads();
    }
    const float user_radius = P.radius;
    // ---- relaxed best-first steps ---------------------------------------------------
    uint32_t it = 0;
    for (; it < cfg.max_iters; it++) {
      // control (warp 0): the first P unexpanded entries within the limit whose code
      // blocks fit the neighbour slots
      if (warp == 0) {
        const uint32_t n = s.n;
        const unsigned long long* list = lists + (size_t)s.cur * L;
        uint8_t* flags = lexp + (size_t)s.cur * L;
        const float rk = n >= P.size ? fminf(key_dist(list[P.size - 1]), user_radius) : user_radius;
        const float limit = __fmul_rn(P.coef, rk);
        uint32_t np = 0, nblk = 0;
        bool full = false;
        for (uint32_t b = 0; b < n && !full; b += 32) {
          const uint32_t i = b + (uint32_t)lane;
          const unsigned long long k = i < n ? list[i] : ~0ull;
          const bool beyond = i < n && key_dist(k) > limit;
          unsigned bal = __ballot_sync(0xffffffffu, i < n && !beyond && flags[i] == 0);
          while (bal) {
            const int src = __ffs(bal) - 1;
            bal &= bal - 1;
            const uint32_t p = key_id(__shfl_sync(0xffffffffu, k, src));
            const bool has = p < qg.nnodes;
            const uint32_t e0 = has ? qg.offsets[p] : 0u;
            uint32_t dg = has ? qg.offsets[p + 1] - e0 : 0u;
            if (np == 0) dg = min(dg, NB);                 // a node beyond the slots keeps its first NB
            const uint32_t nb = (dg + 15) / 16;
            if (np > 0 && (nblk + nb) * 16 > NB) { full = true; break; }
            if (lane == 0) {
              s.parents[np] = p;
              s.pdeg[np] = dg;
              s.poff[np] = e0;
              s.pblk[np] = nblk;
              flags[b + (uint32_t)src] = 1;
            }
            np++;
            nblk += nb;
            if (np == cfg.parents) { full = true; break; }
          }
          if (__any_sync(0xffffffffu, beyond)) break;     // the list is sorted: nothing later qualifies
        }
        if (lane == 0) {
          s.np = np;
          s.nblk = nblk;
          s.pblk[np] = nblk;
          s.limit = limit;
          s.expansions += np;
          s.cnt = 0;
          s.pend = 0;
          uint32_t e = 0;
          for (uint32_t j = 0; j < np; j++) e += s.pdeg[j];
          s.edges += e;
          s.dc += e;
        }
      }
      __syncthreads();
      const uint32_t np = s.np;
      if (np == 0) break;
      // scan: BPI 16-neighbour blocks per warp iteration (all their code words and ids
      // loaded before any is scored); the neighbours within the limit are kept
      // as pending (distance bits << 32 | id) in the key buffer
      {
        const uint32_t nblk = s.nblk;
        const float limit = s.limit;
        unsigned long long* pend = nkey;
        for (uint32_t b0 = (uint32_t)warp * BPI; b0 < nblk; b0 += (uint32_t)BPI * kQGWideWarps) {
          uint2 w[BPI][SPL];
          uint32_t idv[BPI], pj[BPI], lbk[BPI];
          bool on[BPI];
#pragma unroll
          for (int u = 0; u < BPI; u++) {
            const uint32_t bi = b0 + (uint32_t)u;
            on[u] = bi < nblk;
            uint32_t j = 0;
            if (on[u])
              while (j + 1 < np && s.pblk[j + 1] <= bi) j++;
            pj[u] = j;
            lbk[u] = on[u] ? bi - s.pblk[j] : 0u;
            if (on[u]) {
              const uint32_t p = s.parents[j];
              qg_block_words<SPL>(qg.codes + (size_t)qg.code_off16[p] * 16 + (size_t)lbk[u] * 8 * qg.ma, qg.ma,
                                  lane, w[u]);
              const uint32_t e = lbk[u] * 16u + (uint32_t)lane;
              idv[u] = (lane < 16 && e < s.pdeg[j]) ? qg.ids[s.poff[j] + e] : 0u;
            } else {
#pragma unroll
              for (int x = 0; x < SPL; x++) w[u][x] = make_uint2(0u, 0u);
              idv[u] = 0u;
            }
          }
#pragma unroll
          for (int u = 0; u < BPI; u++) {
            if (!on[u]) continue;                          // uniform over the warp
            int o;
            const float d = qg_block_distance_words<SPL>(w[u], Lr, M, lscale, loffset, lane, &o);
            const uint32_t id = __shfl_sync(0xffffffffu, idv[u], o >= 0 ? o : 0);
            const bool keep = o >= 0 && lbk[u] * 16u + (uint32_t)o < s.pdeg[pj[u]] && d <= limit && id < g.nrows;
            const unsigned bal = __ballot_sync(0xffffffffu, keep);
            uint32_t base = 0;
            if (lane == 0 && bal) base = atomicAdd(&s.pend, (uint32_t)__popc(bal));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (keep)
              pend[base + (uint32_t)__popc(bal & ((1u << lane) - 1u))] =
                  ((unsigned long long)__float_as_uint(d) << 32) | id;
          }
        }
      }
      __syncthreads();
      // visited bits of the pending neighbours, eight atomics in flight per thread; the
      // fresh ones (ids and distances) are compacted into nid / nd
      {
        const uint32_t npend = s.pend;
        const unsigned long long* pend = nkey;
        for (uint32_t b = 0; b < npend; b += 8u * kQGWideThreads) {
          uint32_t old[8], bit[8];
          unsigned long long kv[8];
#pragma unroll
          for (int r = 0; r < 8; r++) {
            const uint32_t i = b + (uint32_t)r * kQGWideThreads + (uint32_t)tid;
            kv[r] = i < npend ? pend[i] : 0ull;
            const uint32_t id = (uint32_t)kv[r];
            bit[r] = 1u << (id & 31u);
            old[r] = i < npend ? atomicOr(&bitmap[id >> 5], bit[r]) : bit[r];
          }
#pragma unroll
          for (int r = 0; r < 8; r++) {
            const bool fresh = (old[r] & bit[r]) == 0u;
            const unsigned bal = __ballot_sync(0xffffffffu, fresh);
            uint32_t base = 0;
            if (lane == 0 && bal) base = atomicAdd(&s.cnt, (uint32_t)__popc(bal));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (fresh) {
              const uint32_t pos = base + (uint32_t)__popc(bal & ((1u << lane) - 1u));
              nid[pos] = (uint32_t)kv[r];
              nd[pos] = __uint_as_float((uint32_t)(kv[r] >> 32));
            }
          }
        }
      }
      __syncthreads();
      // merge the new keys into the list (keeps the L best)
      const uint32_t m = s.cnt;
      if (m > 0) {
        for (uint32_t i = tid; i < m; i += blockDim.x) nkey[i] = pack_key(nd[i], nid[i]);
        __syncthreads();
        cta_bitonic_sort(nkey, m, NB);
        const uint32_t n = s.n, cur = s.cur;
        const unsigned long long* ol = lists + (size_t)cur * L;
        const uint8_t* of = lexp + (size_t)cur * L;
        unsigned long long* nl = lists + (size_t)(cur ^ 1u) * L;
        uint8_t* nf = lexp + (size_t)(cur ^ 1u) * L;
        for (uint32_t i = tid; i < n; i += blockDim.x) {
          const unsigned long long k = ol[i];
          const uint32_t pos = i + qgw_lower_bound(nkey, m, k);
          if (pos < L) {
            nl[pos] = k;
            nf[pos] = of[i];
          }
        }
        for (uint32_t i = tid; i < m; i += blockDim.x) {
          const unsigned long long k = nkey[i];
          const uint32_t pos = i + qgw_lower_bound(ol, n, k);
          if (pos < L) {
            nl[pos] = k;
            nf[pos] = 0;
          }
        }
        __syncthreads();
        if (tid == 0) {
          s.n = min(L, n + m);
          s.cur = cur ^ 1u;
          s.visited += m;
        }
      }
      __syncthreads();
    }
    if (it == cfg.max_iters && tid == 0) s.status |= kStatusIterationLimit;
    // ---- results --------------------------------------------------------------------
    __syncthreads();
    const unsigned long long* list = lists + (size_t)s.cur * L;
    if (tid == 0) {
      uint32_t r = min(s.n, P.size);
      while (r > 0 && key_dist(list[r - 1]) > user_radius) r--;
      s.cnt = r;
    }
    __syncthreads();
    uint32_t n = s.cnt;
    if (P.rerank) {
      for (uint32_t b = (uint32_t)(warp * (32 / G)); b < n; b += (uint32_t)ngroups) {
        const uint32_t i = b + (uint32_t)(lane / G);
        const bool valid = i < n;
        const uint32_t id = valid ? key_id(list[i]) : 0u;
        const float d = group_distance<ObjType::Float, Metric::L2>(qv, g.objects + (size_t)id * rc, (int)rc, gl, G);
        if (valid && gl == 0) nkey[i] = pack_key(d, id);
      }
      __syncthreads();
      cta_bitonic_sort(nkey, n, NB);
      if (tid == 0) {
        uint32_t keep = n;
        if (P.radius < FLT_MAX) {
          keep = 0;
          while (keep < n && key_dist(nkey[keep]) < P.radius) keep++;
        }
        s.cnt = min(keep, P.k);
      }
      __syncthreads();
      n = s.cnt;
      for (uint32_t i = tid; i < n; i += blockDim.x) out[P.out_off + i] = ObjDist{key_id(nkey[i]), key_dist(nkey[i])};
    } else {
      for (uint32_t i = tid; i < n; i += blockDim.x) out[P.out_off + i] = ObjDist{key_id(list[i]), key_dist(list[i])};
    }
    if (tid == 0) {
      out_count[q] = n;
      stats[q] = QueryStats{s.dc, s.expansions, s.visited, s.edges, s.status};
    }
    // a clean bitmap for the next query
    uint4* bm4 = reinterpret_cast<uint4*>(bitmap);
    for (uint32_t i = tid; i < cfg.bitmap_words / 4; i += blockDim.x) bm4[i] = make_uint4(0, 0, 0, 0);
    __syncthreads();
  }
}

}  // namespace ngtg
