// Batched graph search with one query per CTA ("wide"): the same relaxed
// best-first search as graph_fast.cuh (sorted candidate list with expanded
// bits, P parents per iteration within (1+epsilon) x r_k, spill tier, exact
// re-rank of the best candidates), with every phase of an iteration spread
// over the CTA so that one query moves many rows at once:
//   * the P parents' edge slots are read, filtered against the query's
//     visited bitmap and compacted by all threads of the CTA (128 or 256);
//   * the new neighbours' search rows (bf16 or 8-bit copies of float objects, or
//     the objects themselves) are copied into a shared-memory stage with 16-byte
//     cp.async in two halves, the next half in flight while the current one is
//     scored, several rows per lane group at once;
//   * every survivor's place in the list is its rank among the new keys (counted
//     when there are at most T of them, else after a CTA bitonic sort) plus its
//     rank in the list; keys land in a second list buffer.
// One warp (warp 0) owns the control decisions (parent selection, the refill
// from the spill tier), exactly as the warp-per-query kernel makes them.
// Per-query latency is set by a few memory round trips per iteration instead of
// one per 16 rows, which is what a lightly loaded server needs.
#pragma once
#include <cuda_bf16.h>
#include <cfloat>
#include <type_traits>
#include "distance.cuh"
#include "device_index.h"
#include "graph_fast.cuh"

namespace ngtg {

constexpr int kWideMaxThreads = 256;
constexpr int kWideMaxWarps = kWideMaxThreads / 32;

struct WideConfig {
  uint32_t list_cap;       // L: power of two
  uint32_t nbr_cap;        // neighbour slots per iteration (power of two >= L)
  uint32_t parents;        // P (<= 32)
  uint32_t stage_rows;     // search rows staged in shared memory per round
  uint32_t sgroup;         // lanes per search distance (power of two <= 32)
  uint32_t ngroup;         // lanes per full-precision distance
  uint32_t search_chunks;  // 16-byte chunks per search row
  uint32_t rerank_x16;
  uint32_t bitmap_words;   // per CTA, multiple of 4
  uint32_t max_iters;
  uint32_t spill_cap;
  uint32_t l2_policy;      // 0: default caching; 1: visited bitmap kept in L2 (evict_last);
                           // 2: as 1, and staged rows streamed through L2 (evict_first)
  uint32_t score_rows;     // rows per lane group scored at once (1, 2 or 4)
  // 8-bit search rows of float objects: code = rint((x - sq_offset) / s), the query
  // mapped the same way in 1/256 steps; distance = sqrt(sum) * sq_out (s / 256)
  uint32_t sq8, dim;
  float sq_offset, sq_in, sq_out;   // sq_in = 256 / s
};

struct WideShared {
  uint32_t q, n, cur, np, total, cnt, kept, scan0, spill_n, stop, done, refill, first_new;
  uint32_t status, dc, expansions, edges, visited;
  unsigned long long spill_min, worst;
  float limit, insert_limit;
  uint32_t parents[32], pexcl[32], pbase[32];
  unsigned long long wmin[kWideMaxWarps];
};

// 16-byte chunks of the row stage, which also holds the NB candidate keys
__host__ __device__ inline size_t wide_stage_chunks(uint32_t search_chunks, uint32_t stage_rows, uint32_t nbr_cap) {
  const size_t rows = (size_t)stage_rows * search_chunks, keys = ((size_t)nbr_cap * 8 + 15) / 16;
  return rows > keys ? rows : keys;
}

inline size_t wide_smem_bytes(uint32_t row_chunks, const WideConfig& c) {
  size_t b = (size_t)row_chunks * 16 + (size_t)c.search_chunks * (c.sq8 ? 64 : 16);
  b += (size_t)c.list_cap * 16;                                   // list, double-buffered
  b += (size_t)c.nbr_cap * 8;                                     // nid, nd
  b += wide_stage_chunks(c.search_chunks, c.stage_rows, c.nbr_cap) * 16;   // row staging / nkey
  b += sizeof(WideShared) + 16;
  return b;
}

__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async16_hint(void* smem_dst, const void* gmem_src, uint64_t policy) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;\n" ::"r"(d), "l"(gmem_src), "l"(policy)
               : "memory");
}
// atomicOr on a visited-bitmap word, with an L2 eviction-priority hint when `hint`
__device__ __forceinline__ uint32_t visit_or(uint32_t* word, uint32_t bit, bool hint, uint64_t policy) {
  if (!hint) return atomicOr(word, bit);
  uint32_t old;
  asm volatile("atom.global.or.L2::cache_hint.b32 %0, [%1], %2, %3;\n"
               : "=r"(old) : "l"(word), "r"(bit), "l"(policy) : "memory");
  return old;
}
__device__ __forceinline__ void store_zero16(uint4* p, bool hint, uint64_t policy) {
  if (!hint) { *p = make_uint4(0, 0, 0, 0); return; }
  asm volatile("st.global.L2::cache_hint.v4.u32 [%0], {%1, %1, %1, %1}, %2;\n" ::"l"(p), "r"(0u), "l"(policy)
               : "memory");
}
__device__ __forceinline__ uint64_t l2_policy_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;\n" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;\n" : "=l"(p));
  return p;
}

// CTA-wide ascending bitonic sort of a[0..n) (shared memory), padded with ~0 to
// the next power of two (<= cap).
__device__ __forceinline__ void cta_bitonic_sort(unsigned long long* a, uint32_t n, uint32_t cap) {
  if (n <= 1) return;
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

// (row - query)^2 of one 16-byte row chunk, two float lanes at a time, against the
// query chunk prepared once per query: bf16 / fp32 rows through PackedL2, 8-bit
// rows of float objects (Sq8) by placing each code in the mantissa of 2^23
// (2^23 + 256 c, one byte permute) and adding the negated 2^23 + rint(256 q'),
// so that the difference 256 (c - q') is exact.
template <ObjType ST, ObjType OT, Metric M>
struct WideDot {
  typedef PackedL2<ST, M> PL;
  static constexpr bool kSq8 = ST == ObjType::Uint8 && OT == ObjType::Float && M == Metric::L2;
  static constexpr bool kOn = kSq8 || PL::kOn;
  static constexpr int NQ = kSq8 ? 8 : (PL::P / 2 > 0 ? PL::P / 2 : 1);
  // query chunk c: qs holds the search-type query (4 uint4 of floats per chunk for Sq8)
  __device__ __forceinline__ static void prepare(const uint4* qs, uint32_t c, float2 (&nq)[NQ]) {
    if constexpr (kSq8) {
      const float2* f = reinterpret_cast<const float2*>(qs + 4 * (size_t)c);
#pragma unroll
      for (int i = 0; i < 8; i++) nq[i] = f[i];
    } else if constexpr (PL::kOn) {
      PL::prepare(qs[c], nq);
    }
  }
  __device__ __forceinline__ static void zero(float2 (&nq)[NQ]) {
#pragma unroll
    for (int i = 0; i < NQ; i++) nq[i] = make_float2(0.f, 0.f);
  }
  __device__ __forceinline__ static float2 add(float2 acc, const float2 (&nq)[NQ], const uint4& x) {
    if constexpr (kSq8) {
      const uint32_t w[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const float a = __uint_as_float(__byte_perm(w[i], 0x4B000000u, 0x7504u));
        const float b = __uint_as_float(__byte_perm(w[i], 0x4B000000u, 0x7514u));
        const float c = __uint_as_float(__byte_perm(w[i], 0x4B000000u, 0x7524u));
        const float d = __uint_as_float(__byte_perm(w[i], 0x4B000000u, 0x7534u));
        const float2 d0 = __fadd2_rn(make_float2(a, b), nq[2 * i]);
        const float2 d1 = __fadd2_rn(make_float2(c, d), nq[2 * i + 1]);
        acc = __ffma2_rn(d0, d0, acc);
        acc = __ffma2_rn(d1, d1, acc);
      }
      return acc;
    } else if constexpr (PL::kOn) {
      return PL::add(acc, nq, x);
    } else {
      return acc;
    }
  }
};

// T: threads per CTA (64, 128 or 256), one query per CTA.
template <ObjType ST, ObjType OT, Metric M, int T>
__global__ void __launch_bounds__(T, T == 64 ? 10 : T == 128 ? 6 : 2)
graph_search_wide_kernel(DevGraph g, const uint4* __restrict__ srows, const uint4* __restrict__ queries,
                         uint32_t nq, const QueryParams* __restrict__ params, const uint32_t* __restrict__ seed_list,
                         ObjDist* __restrict__ out, uint32_t* __restrict__ out_count, QueryStats* __restrict__ stats,
                         uint32_t* __restrict__ bitmaps, uint32_t* __restrict__ work,
                         unsigned long long* __restrict__ spills, WideConfig cfg) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t rc = g.row_chunks, sc = cfg.search_chunks;
  const uint32_t L = cfg.list_cap, NB = cfg.nbr_cap, SR = cfg.stage_rows;
  uint4* qn = reinterpret_cast<uint4*>(smem);
  typedef WideDot<ST, OT, M> Dot;
  uint4* qs = qn + rc;                                                           // sc (x 4 for Sq8) chunks
  unsigned long long* lists = reinterpret_cast<unsigned long long*>(qs + (Dot::kSq8 ? 4 * sc : sc));   // 2 x L
  uint32_t* nid = reinterpret_cast<uint32_t*>(lists + 2 * (size_t)L);
  float* nd = reinterpret_cast<float*>(nid + NB);
  uint4* stage = reinterpret_cast<uint4*>(nd + NB);
  // the candidate keys share the row stage: rows are staged only inside a score
  // phase, keys are built after it and consumed before the next one
  unsigned long long* nkey = reinterpret_cast<unsigned long long*>(stage);
  WideShared& s = *reinterpret_cast<WideShared*>(stage + wide_stage_chunks(sc, SR, NB));
  uint32_t* bitmap = bitmaps + (size_t)blockIdx.x * cfg.bitmap_words;
  unsigned long long* spill = spills + (size_t)blockIdx.x * 2 * cfg.spill_cap;
  unsigned long long* spill_tmp = spill + cfg.spill_cap;
  const int SG = (int)cfg.sgroup, NG = (int)cfg.ngroup;
  const int sgl = lane & (SG - 1), ngl = lane & (NG - 1);
  const bool keep_visited = cfg.l2_policy >= 1, stream_rows = cfg.l2_policy >= 2;
  const uint64_t pol_keep = keep_visited ? l2_policy_evict_last() : 0ull;
  const uint64_t pol_stream = stream_rows ? l2_policy_evict_first() : 0ull;

  // distances of nid[0..cnt) into nd[], rows staged through shared memory
  // distances of nid[0..cnt) into nd[]: rows staged through shared memory in two
  // halves, the next half's copies in flight while the current half is scored
  const uint32_t SRH = SR / 2;
  // each thread copies chunk (tid % sc) of every (T / sc)-th row when sc divides T
  const bool rows_split = ((uint32_t)T % sc) == 0;
  const uint32_t my_chunk = (uint32_t)tid % sc, my_row = (uint32_t)tid / sc, row_step = (uint32_t)T / sc;
  auto issue = [&](uint32_t r0, uint32_t nr, uint4* buf) {
    if (rows_split) {
      if (stream_rows) {
        for (uint32_t i = my_row; i < nr; i += row_step)
          cp_async16_hint(buf + (size_t)i * sc + my_chunk, srows + (size_t)nid[r0 + i] * sc + my_chunk, pol_stream);
      } else {
        for (uint32_t i = my_row; i < nr; i += row_step)
          cp_async16(buf + (size_t)i * sc + my_chunk, srows + (size_t)nid[r0 + i] * sc + my_chunk);
      }
    } else {
      for (uint32_t idx = tid; idx < nr * sc; idx += blockDim.x) {
        const uint32_t i = idx / sc, c = idx - i * sc;
        cp_async16(buf + idx, srows + (size_t)nid[r0 + i] * sc + c);
      }
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  };
  auto score = [&](uint32_t cnt) {
    if (cnt == 0) return;
    // the query chunks this lane reads (c = sgl + j * SG), negated and unpacked once
    // the host sets sgroup so that every lane reads at most two chunks (one for 8-bit rows)
    constexpr int kQC = Dot::kSq8 ? 1 : 2;
    float2 nqc[kQC][Dot::NQ];
    if constexpr (Dot::kOn) {
#pragma unroll
      for (int j = 0; j < kQC; j++) {
        const uint32_t c = (uint32_t)sgl + (uint32_t)(j * SG);
        if (c < sc) Dot::prepare(qs, c, nqc[j]);
        else Dot::zero(nqc[j]);
      }
    }
    uint4* buf[2] = {stage, stage + (size_t)SRH * sc};
    issue(0, min(SRH, cnt), buf[0]);
    if (cnt > SRH) issue(SRH, min(SRH, cnt - SRH), buf[1]);
    uint32_t h = 0;
    for (uint32_t r0 = 0; r0 < cnt; r0 += SRH, h ^= 1u) {
      const uint32_t nr = min(SRH, cnt - r0);
      if (r0 + SRH < cnt) {
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");   // this half landed
      } else {
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
      }
      __syncthreads();
      const uint4* stg = buf[h];
      const uint32_t gpb = (uint32_t)T / SG;
      const uint32_t gi = (uint32_t)(tid / SG);
      if (Dot::kOn && sc <= (uint32_t)(kQC * SG)) {
        // KR rows per lane group at once: their shared-memory loads first, then 2 x KR
        // independent accumulations (one per chunk) and interleaved shuffle reductions
        auto rows_at_once = [&](auto kr_tag) {
          constexpr int KR = decltype(kr_tag)::value;
          for (uint32_t b = 0; b < nr; b += gpb * KR) {    // uniform trip count per warp
            uint4 x[KR][kQC];
#pragma unroll
            for (int u = 0; u < KR; u++) {
              const uint32_t i = b + (uint32_t)u * gpb + gi;
              const uint4* row = stg + (size_t)(i < nr ? i : 0u) * sc;
#pragma unroll
              for (int j = 0; j < kQC; j++) {
                const uint32_t c = (uint32_t)sgl + (uint32_t)(j * SG);
                x[u][j] = c < sc ? row[c] : make_uint4(0, 0, 0, 0);
              }
            }
            float v[KR];
#pragma unroll
            for (int u = 0; u < KR; u++) {
              float2 acc[kQC];
#pragma unroll
              for (int j = 0; j < kQC; j++) {
                acc[j] = make_float2(0.f, 0.f);
                if ((uint32_t)sgl + (uint32_t)(j * SG) < sc) acc[j] = Dot::add(acc[j], nqc[j], x[u][j]);
              }
              float t = acc[0].x + acc[0].y;
#pragma unroll
              for (int j = 1; j < kQC; j++) t += acc[j].x + acc[j].y;
              v[u] = t;
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1)
              if (off < SG) {
#pragma unroll
                for (int u = 0; u < KR; u++) v[u] += __shfl_xor_sync(0xffffffffu, v[u], off);
              }
#pragma unroll
            for (int u = 0; u < KR; u++) {
              const uint32_t i = b + (uint32_t)u * gpb + gi;
              if (i < nr && sgl == 0) nd[r0 + i] = Dot::kSq8 ? sqrtf(v[u]) * cfg.sq_out : sqrtf(v[u]);
            }
          }
        };
        const uint32_t kr = min(cfg.score_rows, (nr + gpb - 1) / gpb);   // uniform
        if (kr >= 4) rows_at_once(std::integral_constant<int, 4>{});
        else if (kr >= 2) rows_at_once(std::integral_constant<int, 2>{});
        else rows_at_once(std::integral_constant<int, 1>{});
      } else {
        for (uint32_t b = 0; b < nr; b += gpb) {          // uniform trip count per warp
          const uint32_t i = b + gi;
          const bool valid = i < nr;
          const uint4* row = stg + (size_t)(valid ? i : 0u) * sc;
          float d;
          if constexpr (Dot::kOn) {
            float2 acc = make_float2(0.f, 0.f);
            for (uint32_t c = (uint32_t)sgl; c < sc; c += (uint32_t)SG) {
              float2 nq[Dot::NQ];
              Dot::prepare(qs, c, nq);
              acc = Dot::add(acc, nq, row[c]);
            }
            float v = acc.x + acc.y;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1)
              if (off < SG) v += __shfl_xor_sync(0xffffffffu, v, off);
            d = Dot::kSq8 ? sqrtf(v) * cfg.sq_out : sqrtf(v);
          } else {
            Acc<ST, M> acc;
            for (uint32_t c = (uint32_t)sgl; c < sc; c += (uint32_t)SG) acc.add(qs[c], row[c], (int)c);
            acc.reduce(SG);
            d = acc.finish();
          }
          if (valid && sgl == 0) nd[r0 + i] = d;
        }
      }
      __syncthreads();                                   // the half is free again
      if (r0 + 2 * SRH < cnt) issue(r0 + 2 * SRH, min(SRH, cnt - (r0 + 2 * SRH)), buf[h]);
    }
  };

  while (true) {
    if (tid == 0) s.q = atomicAdd(work, 1u);
    __syncthreads();
    const uint32_t q = s.q;
    if (q >= nq) break;
    const QueryParams P = params[q];
    for (uint32_t i = tid; i < rc; i += blockDim.x) qn[i] = queries[(size_t)q * rc + i];
    __syncthreads();
    if constexpr (Dot::kSq8) {
      // 16 negated values per row chunk: -(2^23 + rint(256 (q - offset) / s)), 0 past dim
      const float* qf = reinterpret_cast<const float*>(qn);
      float* qv = reinterpret_cast<float*>(qs);
      for (uint32_t i = tid; i < sc * 16; i += blockDim.x) {
        float v = 0.f;
        if (i < cfg.dim) v = fminf(fmaxf(rintf((qf[i] - cfg.sq_offset) * cfg.sq_in), -8388607.f), 8388607.f);
        qv[i] = -(8388608.f + v);
      }
    } else if constexpr (ST != OT) {
      const float* qf = reinterpret_cast<const float*>(qn);
      uint32_t* qb = reinterpret_cast<uint32_t*>(qs);
      for (uint32_t i = tid; i < sc * 4; i += blockDim.x) {
        uint32_t lo = __bfloat16_as_ushort(__float2bfloat16_rn(qf[2 * i]));
        uint32_t hi = __bfloat16_as_ushort(__float2bfloat16_rn(qf[2 * i + 1]));
        qb[i] = lo | (hi << 16);
      }
    } else {
      for (uint32_t i = tid; i < sc; i += blockDim.x) qs[i] = qn[i];
    }
    if (tid == 0) {
      s.n = 0; s.cur = 0; s.scan0 = 0; s.spill_n = 0; s.spill_min = ~0ull; s.refill = 0; s.done = 0;
      s.status = 0; s.dc = 0; s.expansions = 0; s.edges = 0; s.visited = 0;
    }
    __syncthreads();
    if (P.size == 0) {
      if (tid == 0) { out_count[q] = 0; stats[q] = QueryStats{0, 0, 0, 0, 0}; }
      __syncthreads();
      continue;
    }
    // ---- seeds (warp 0): tree leaf or explicit list, marked visited, compacted ----
    if (warp == 0) {
      const uint32_t* seeds = nullptr;
      uint32_t nseeds = 0, st = 0;
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
          st |= kStatusTreeError;
        }
      } else {
        seeds = seed_list + P.seed_off;
        nseeds = P.seed_cnt;
      }
      nseeds = min(nseeds, NB);
      if (nseeds == 0) st |= kStatusEmptySeeds;
      uint32_t m = 0;
      for (uint32_t b = 0; b < nseeds; b += 32) {
        uint32_t i = b + lane;
        bool fresh = false;
        uint32_t id = 0;
        if (i < nseeds) {
          id = seeds[i];
          if (id < g.nrows) {
            uint32_t bit = 1u << (id & 31u);
            fresh = (visit_or(&bitmap[id >> 5], bit, keep_visited, pol_keep) & bit) == 0u;
          }
        }
        unsigned bal = __ballot_sync(0xffffffffu, fresh);
        if (fresh) nid[m + __popc(bal & ((1u << lane) - 1u))] = id;
        m += __popc(bal);
      }
      if (lane == 0) { s.cnt = m; s.status |= st; s.dc = m; s.visited = m; }
    }
    __syncthreads();
    {
      const uint32_t m = s.cnt;
      score(m);
      for (uint32_t i = tid; i < m; i += blockDim.x) nkey[i] = pack_key(nd[i], nid[i]);
      __syncthreads();
      cta_bitonic_sort(nkey, m, NB);
      const uint32_t n0 = min(m, L);
      for (uint32_t i = tid; i < n0; i += blockDim.x) lists[i] = nkey[i];
      if (tid == 0) s.n = n0;
      __syncthreads();
    }
    const float user_radius = P.radius;

    // ---- best-first iterations ---------------------------------------------------------
    for (uint32_t it = 0; it < cfg.max_iters; it++) {
      // control (warp 0): refill from the spill tier when flagged, then pick parents
      if (warp == 0) {
        unsigned long long* list = lists + (size_t)s.cur * L;
        uint32_t n = s.n, scan0 = s.scan0, spill_n = s.spill_n;
        unsigned long long spill_min = s.spill_min;
        bool refill = s.refill != 0;
        float rk = (n >= P.size) ? fminf(key_dist(list[P.size - 1]), user_radius) : user_radius;
        const float limit = P.coef * rk;
        if (refill) {
          n = min(n, P.size);
          const uint32_t room = L - n;
          uint32_t r = 0;
          for (uint32_t b = 0; b < spill_n; b += 32) {
            uint32_t i = b + lane;
            unsigned long long k = i < spill_n ? spill[i] : ~0ull;
            bool live = i < spill_n && key_dist(k) <= limit;
            unsigned bal = __ballot_sync(0xffffffffu, live);
            if (live) spill_tmp[r + __popc(bal & ((1u << lane) - 1u))] = k;
            r += __popc(bal);
          }
          __syncwarp();
          unsigned long long thr = ~0ull;
          if (r > room) {
            unsigned long long prefix = 0, mask = 0;
            uint32_t need = room;
            uint32_t* hist = reinterpret_cast<uint32_t*>(nd);
            for (int shift = 56; shift >= 0; shift -= 8) {
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
        uint32_t np = 0;
        bool stop = false;
        for (uint32_t b = scan0 & ~31u; b < n && !stop && np < cfg.parents; b += 32) {
          uint32_t i = b + lane;
          unsigned long long k = i < n ? list[i] : ~0ull;
          unsigned ball = __ballot_sync(0xffffffffu, i < n && !key_expanded(k));
          while (ball && np < cfg.parents) {
            int j = __ffs(ball) - 1;
            unsigned long long kj = __shfl_sync(0xffffffffu, k, j);
            if (key_dist(kj) > limit) { stop = true; break; }
            if (lane == j) list[i] = k | kExpandedBit;
            if (lane == 0) s.parents[np] = key_rawid(kj);
            np++;
            scan0 = b + (uint32_t)j + 1;
            ball &= ball - 1;
          }
        }
        __syncwarp();
        uint32_t done = 0, next_refill = 0;
        if (np == 0) {
          if (!stop && spill_n > 0 && key_dist(spill_min) <= limit) {
            scan0 = n;
            next_refill = 1;
          } else {
            done = 1;
          }
        } else {
          // edge slots of the parents
          const uint32_t per_parent = min(P.edge_size, NB / np);
          uint32_t pe0 = 0, pne = 0;
          if ((uint32_t)lane < np) {
            const uint32_t v = s.parents[lane];
            const uint32_t a = g.offsets[v];
            pe0 = a;
            pne = min(g.offsets[v + 1] - a, per_parent);
          }
          uint32_t incl = pne;
#pragma unroll
          for (int off = 1; off < 32; off <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off) incl += t;
          }
          const uint32_t total = __shfl_sync(0xffffffffu, incl, np - 1);
          if ((uint32_t)lane < np) {
            s.pexcl[lane] = incl - pne;
            s.pbase[lane] = pe0;
          }
          if (lane == 0) { s.total = total; s.edges += total; s.expansions += np; }
        }
        if (lane == 0) {
          s.n = n; s.scan0 = scan0; s.spill_n = spill_n; s.spill_min = spill_min;
          s.refill = next_refill; s.done = done; s.np = np; s.limit = limit;
          s.cnt = 0; s.kept = 0;              // counters of this step's gather and placement
        }
      }
      __syncthreads();
      const uint32_t done = s.done, refill_next = s.refill, np = s.np, total = s.total;
      __syncthreads();              // everyone has read the decision before warp 0 writes the next one
      if (done) break;
      if (refill_next) continue;
      // ---- gather: unvisited neighbours of the parents ----------------------------------
      // Every thread takes up to kGatherSlots edge slots (t = base + j*T + tid): all
      // edge loads, then all visited-bit atomics, then one CTA scan of the per-thread
      // counts places the new ids (their order does not matter to this search).
      constexpr int kGatherSlots = 8;
      for (uint32_t base0 = 0; base0 < total; base0 += kGatherSlots * (uint32_t)T) {
        uint32_t ids[kGatherSlots];
        uint32_t fm = 0, p2 = 0;
#pragma unroll
        for (int j = 0; j < kGatherSlots; j++) {
          const uint32_t t = base0 + (uint32_t)j * (uint32_t)T + (uint32_t)tid;
          ids[j] = 0;
          if (t < total) {
            while (p2 + 1 < np && t >= s.pexcl[p2 + 1]) p2++;       // slots increase with j
            ids[j] = __ldg(g.edges + s.pbase[p2] + (t - s.pexcl[p2]));
          }
        }
#pragma unroll
        for (int j = 0; j < kGatherSlots; j++) {
          const uint32_t t = base0 + (uint32_t)j * (uint32_t)T + (uint32_t)tid;
          if (t < total) {
            const uint32_t bit = 1u << (ids[j] & 31u);
            if ((visit_or(&bitmap[ids[j] >> 5], bit, keep_visited, pol_keep) & bit) == 0u) fm |= 1u << j;
          }
        }
        // places in nid: a warp scan of the per-thread counts and one counter
        // increment per warp (the order of the new ids does not matter to this search)
        const uint32_t c = (uint32_t)__popc(fm);
        uint32_t incl = c;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
          uint32_t v = __shfl_up_sync(0xffffffffu, incl, off);
          if (lane >= off) incl += v;
        }
        uint32_t wbase = 0;
        if (lane == 31 && incl) wbase = atomicAdd(&s.cnt, incl);
        wbase = __shfl_sync(0xffffffffu, wbase, 31);
        uint32_t pos = wbase + incl - c;
#pragma unroll
        for (int j = 0; j < kGatherSlots; j++)
          if (fm & (1u << j)) nid[pos++] = ids[j];
      }
      __syncthreads();
      const uint32_t cnt = s.cnt;
      if (tid == 0) { s.dc += cnt; s.visited += cnt; }
      // ---- distances ------------------------------------------------------------------------
      score(cnt);
      // ---- placement: below the list's worst -> merged; else within the limit -> spill ---
      const unsigned long long* list = lists + (size_t)s.cur * L;
      const uint32_t n = s.n;
      const unsigned long long worst = (n >= L) ? (list[L - 1] & ~(unsigned long long)kExpandedBit) : ~0ull;
      const float rk2 = (n >= P.size) ? fminf(key_dist(list[P.size - 1]), user_radius) : user_radius;
      const float insert_limit = P.coef * rk2;
      // kept keys are appended through one counter increment per warp and round
      // (their order does not matter: they are ranked or sorted before the merge)
      unsigned long long smin = ~0ull;
      for (uint32_t base0 = 0; base0 < cnt; base0 += blockDim.x) {
        const uint32_t i = base0 + tid;
        unsigned long long key = ~0ull;
        bool live = false;
        if (i < cnt) {
          key = pack_key(nd[i], nid[i]);
          live = nd[i] <= insert_limit;
        }
        const bool keep = live && key < worst;
        const bool spl = live && key >= worst;
        const unsigned kb = __ballot_sync(0xffffffffu, keep);
        uint32_t kbase = 0;
        if (lane == 0 && kb) kbase = atomicAdd(&s.kept, (uint32_t)__popc(kb));
        kbase = __shfl_sync(0xffffffffu, kbase, 0);
        if (keep) nkey[kbase + __popc(kb & ((1u << lane) - 1u))] = key;
        if (spl) {
          const uint32_t o = atomicAdd(&s.spill_n, 1u);
          if (o < cfg.spill_cap) spill[o] = key;
          smin = key < smin ? key : smin;
        }
      }
      for (int off = 16; off > 0; off >>= 1) {
        unsigned long long o = __shfl_xor_sync(0xffffffffu, smin, off);
        smin = o < smin ? o : smin;
      }
      if (lane == 0) s.wmin[warp] = smin;
      __syncthreads();
      const uint32_t kept = s.kept;
      if (tid == 0) {
        unsigned long long mn = s.spill_min;
        for (int w = 0; w < T / 32; w++) mn = s.wmin[w] < mn ? s.wmin[w] : mn;
        s.spill_min = mn;
        if (s.spill_n > cfg.spill_cap) { s.spill_n = cfg.spill_cap; s.status |= kStatusCandidateOverflow; }
        s.first_new = 0xffffffffu;
      }
      __syncthreads();
      if (kept == 0) continue;
      // ---- merge into the other list buffer (entries compare without the expanded bit) ---
      // Every key's place is its rank among the new keys plus its rank among the list's:
      // up to T new keys are ranked by counting (no sort, no barrier), more are sorted
      // first and ranked by binary search.
      const bool by_count = kept <= (uint32_t)T;
      if (!by_count) cta_bitonic_sort(nkey, kept, NB);
      auto rank_new = [&](unsigned long long x, uint32_t j_hint) -> uint32_t {
        if (!by_count) return j_hint;
        uint32_t r = 0;
        for (uint32_t t = 0; t < kept; t++) r += nkey[t] < x ? 1u : 0u;
        return r;
      };
      unsigned long long* dst = lists + (size_t)(s.cur ^ 1u) * L;
      for (uint32_t i = tid; i < n; i += blockDim.x) {
        const unsigned long long k = list[i];
        const unsigned long long km = k & ~(unsigned long long)kExpandedBit;
        const uint32_t pos = i + (by_count ? rank_new(km, 0u) : warp_lower_bound(nkey, kept, km));
        if (pos < L) dst[pos] = k;
        else if (!key_expanded(k)) {
          const uint32_t o = atomicAdd(&s.spill_n, 1u);
          if (o < cfg.spill_cap) spill[o] = k;
          atomicMin(&s.spill_min, k);
        }
      }
      for (uint32_t j = tid; j < kept; j += blockDim.x) {
        const unsigned long long k = nkey[j];
        uint32_t lo = 0, hi = n;
        while (lo < hi) {
          uint32_t mid = (lo + hi) >> 1;
          if ((list[mid] & ~(unsigned long long)kExpandedBit) < k) lo = mid + 1; else hi = mid;
        }
        const uint32_t pos = rank_new(k, j) + lo;
        if (pos < L) {
          dst[pos] = k;
          atomicMin(&s.first_new, pos);
        } else {
          const uint32_t o = atomicAdd(&s.spill_n, 1u);
          if (o < cfg.spill_cap) spill[o] = k;
          atomicMin(&s.spill_min, k);
        }
      }
      __syncthreads();
      if (tid == 0) {
        s.cur ^= 1u;
        s.n = min(n + kept, L);
        if (s.first_new < s.scan0) s.scan0 = s.first_new;
        if (s.spill_n > cfg.spill_cap) { s.spill_n = cfg.spill_cap; s.status |= kStatusCandidateOverflow; }
      }
      __syncthreads();
    }
    // ---- exact re-rank of the best entries with the full-precision rows --------------------
    {
      const unsigned long long* list = lists + (size_t)s.cur * L;
      const uint32_t n = s.n;
      const uint32_t R = min(n, max(P.size, (uint32_t)((P.size * cfg.rerank_x16 + 15) / 16)));
      const uint32_t gpb = (uint32_t)T / NG;
      for (uint32_t b = 0; b < R; b += gpb) {
        const uint32_t i = b + (uint32_t)(tid / NG);
        const bool valid = i < R;
        const uint32_t id = valid ? key_rawid(list[i]) : 0u;
        float d = group_distance<OT, M>(qn, g.objects + (size_t)id * rc, (int)rc, ngl, NG);
        if (valid && ngl == 0) nkey[i] = pack_key(d, id);
      }
      __syncthreads();
      cta_bitonic_sort(nkey, R, NB);
      if (warp == 0) {
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
          stats[q] = QueryStats{s.dc, s.expansions, s.visited, s.edges, s.status};
        }
      }
    }
    uint4* bm4 = reinterpret_cast<uint4*>(bitmap);
    for (uint32_t i = tid; i < cfg.bitmap_words / 4; i += blockDim.x) store_zero16(bm4 + i, keep_visited, pol_keep);
    __syncthreads();
  }
}

}  // namespace ngtg
