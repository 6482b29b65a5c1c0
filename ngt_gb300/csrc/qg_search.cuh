// Quantized-graph search (NGTQG): one query per CTA, reproducing
// NGTQG::Index::searchQuantizedGraph (lib/NGT/NGTQ/QuantizedGraph.h:283-447)
// step for step, so that results equal the reference's.
//
// Per query:
//   1. the query is rotated (Rotation::mul, lib/NGT/NGTQ/Quantizer.h:117-160)
//      and its uint8 distance table built (createFloatL2DistanceLookup,
//      lib/NGT/NGTQ/Quantizer.h:1731-1810): squared L2 of each subvector to each
//      of the 16 local centroids, one global offset (the minimum) and scale
//      ((max - min) / 255), entries rounded to nearest even.  The rotation sums
//      in the order of the x86-64 OpenBLAS sgemv the reference links (one FMA
//      chain for dimensions <= 48, else blocks of 8 columns).
//   2. seeds come from the DVP tree (getSeedsFromTree, thinned to the requested
//      size) with exact L2 distances, as setupDistances(L2Float) / setupSeeds do.
//   3. best-first loop: each expanded node's neighbours are scored by the 4-bit
//      scan of its code stream (lib/NGT/NGTQ/Quantizer.h:2331-2440): every lane
//      keeps the 16-entry tables of ceil(m/32) subspaces in registers and looks
//      up four neighbours per byte_perm pair, the per-lane sums of 16 neighbours
//      are reduce-scattered over the warp; distance = sqrt(sum * scale + offset)
//      with the multiply-add fused.
//   4. a neighbour enters the visited set only when it is within the
//      exploration radius, then joins the results (updatable-search semantics:
//      push, pop the maximum when over size, radius = maximum) when within the
//      radius; the result size is size x result expansion.
//   5. with result expansion >= 1 the results are re-ranked by exact L2, cut at
//      the radius (kept when distance < radius) and truncated to the size.
// Order independence inside one expanded node follows the exact graph kernel:
// the radius never grows, so marking visited against the radius at the start
// of a chunk, replaying the result updates in edge order with the reference's
// conditions and pushing candidates against the radius at the end of the chunk
// gives the reference's pop sequence.
#pragma once
#include <cfloat>
#include "graph_exact.cuh"

namespace ngtg {

struct QGShared {
  float radius;
  uint32_t nres;
  uint32_t head, tail, cur;
  uint32_t nvisited;
  uint32_t spilled;
  uint32_t done;
  uint32_t target;
  uint32_t nnew;
  uint32_t live_old;
  uint32_t status;
  uint32_t dc;
  uint32_t expansions;
  uint32_t edges;
  uint32_t seed_leaf;
  uint32_t ovf_n;
  uint32_t ovf_tmp;
  unsigned long long ovf_min;
  unsigned long long evict_min;
  unsigned long long sel_prefix;
  uint32_t sel_need;
  float lut_min, lut_scale, lut_offset;
  float wmin[kExactWarps], wmax[kExactWarps];
  uint32_t warp_cnt[kExactWarps];
  uint32_t hist[256];
};

// Four table lookups per byte_perm triple: nibble i of w (neighbour i) selects
// entry i of the subspace's 16-byte table held in L[0..3].  Adds the entries of
// neighbours 0,2 / 1,3 of each half-word into a[0] / a[1] (low half-word) and
// a[2] / a[3] (high half-word) as two 16-bit lanes.
__device__ __forceinline__ void qg_lookup8(uint32_t w, const uint32_t (&L)[4], uint32_t* a) {
  const uint32_t sel = ((w >> 1) & 0x44444444u) | 0x32103210u;   // bit 3 of a code picks the upper 8 entries
  uint32_t v = __byte_perm(__byte_perm(L[0], L[1], w), __byte_perm(L[2], L[3], w), sel);
  a[0] += __byte_perm(v, 0u, 0x4240u);
  a[1] += __byte_perm(v, 0u, 0x4341u);
  const uint32_t wh = w >> 16, selh = sel >> 16;
  v = __byte_perm(__byte_perm(L[0], L[1], wh), __byte_perm(L[2], L[3], wh), selh);
  a[2] += __byte_perm(v, 0u, 0x4240u);
  a[3] += __byte_perm(v, 0u, 0x4341u);
}

// The code words of one 16-neighbour block this lane reads (subspaces lane + 32j).
template <int SPL>
__device__ __forceinline__ void qg_block_words(const uint8_t* __restrict__ blk, uint32_t ma, int lane,
                                               uint2 (&w)[SPL]) {
#pragma unroll
  for (int j = 0; j < SPL; j++) {
    const uint32_t s = (uint32_t)lane + 32u * (uint32_t)j;
    w[j] = s < ma ? *reinterpret_cast<const uint2*>(blk + 8u * s) : make_uint2(0u, 0u);
  }
}

// Quantized distances of the 16 neighbours of one code block, by one warp, from the
// words qg_block_words loaded.  Returns, in lanes whose bits 1..0 select it, one
// neighbour's distance: *obj receives the neighbour (0..15) the lane holds, or -1.
template <int SPL>
__device__ __forceinline__ float qg_block_distance_words(const uint2 (&w)[SPL], const uint32_t (&L)[SPL][4],
                                                         uint32_t m, float scale, float offset, int lane, int* obj) {
  uint32_t acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int j = 0; j < SPL; j++) {
    qg_lookup8(w[j].x, L[j], acc);
    qg_lookup8(w[j].y, L[j], acc + 4);
  }
  uint32_t sum;
  int o;
  if (m <= 256) {
    // every 16-bit lane stays below 65536: reduce-scatter the packed pairs
    // (register r = 2*group + parity holds neighbours 4g+p and 4g+2+p)
    uint32_t r4[4], r2[2];
    {
      const bool b = (lane & 16) != 0;
#pragma unroll
      for (int i = 0; i < 4; i++) {
        uint32_t send = b ? acc[i] : acc[i + 4], keep = b ? acc[i + 4] : acc[i];
        r4[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
      }
    }
    {
      const bool b = (lane & 8) != 0;
#pragma unroll
      for (int i = 0; i < 2; i++) {
        uint32_t send = b ? r4[i] : r4[i + 2], keep = b ? r4[i + 2] : r4[i];
        r2[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
      }
    }
    const bool b4 = (lane & 4) != 0;
    uint32_t r1 = (b4 ? r2[1] : r2[0]) + __shfl_xor_sync(0xffffffffu, b4 ? r2[0] : r2[1], 4);
    r1 += __shfl_xor_sync(0xffffffffu, r1, 2);
    r1 += __shfl_xor_sync(0xffffffffu, r1, 1);
    const int r = ((lane >> 2) & 1) | (((lane >> 3) & 1) << 1) | (((lane >> 4) & 1) << 2);
    const int g = r >> 1, par = r & 1;
    const int sub = lane & 3;
    o = sub == 0 ? 4 * g + par : sub == 1 ? 4 * g + 2 + par : -1;
    sum = sub == 0 ? (r1 & 0xFFFFu) : (r1 >> 16);
  } else {
    // wide sums: per-neighbour 32-bit values; even and odd subspaces (lane
    // parity) saturate separately at 65535 like the reference's 16-bit lanes
    uint32_t u[16];
#pragma unroll
    for (int g = 0; g < 4; g++) {
      u[4 * g + 0] = acc[2 * g] & 0xFFFFu;
      u[4 * g + 2] = acc[2 * g] >> 16;
      u[4 * g + 1] = acc[2 * g + 1] & 0xFFFFu;
      u[4 * g + 3] = acc[2 * g + 1] >> 16;
    }
    uint32_t r8[8], r4[4], r2[2];
    {
      const bool b = (lane & 16) != 0;
#pragma unroll
      for (int i = 0; i < 8; i++) {
        uint32_t send = b ? u[i] : u[i + 8], keep = b ? u[i + 8] : u[i];
        r8[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
      }
    }
    {
      const bool b = (lane & 8) != 0;
#pragma unroll
      for (int i = 0; i < 4; i++) {
        uint32_t send = b ? r8[i] : r8[i + 4], keep = b ? r8[i + 4] : r8[i];
        r4[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
      }
    }
    {
      const bool b = (lane & 4) != 0;
#pragma unroll
      for (int i = 0; i < 2; i++) {
        uint32_t send = b ? r4[i] : r4[i + 2], keep = b ? r4[i + 2] : r4[i];
        r2[i] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
      }
    }
    const bool b2 = (lane & 2) != 0;
    uint32_t r1 = (b2 ? r2[1] : r2[0]) + __shfl_xor_sync(0xffffffffu, b2 ? r2[0] : r2[1], 2);
    r1 = min(r1, 65535u);
    sum = r1 + __shfl_xor_sync(0xffffffffu, r1, 1);
    o = (lane & 1) ? -1 : ((lane >> 1) & 15);
  }
  *obj = o;
  return __fsqrt_rn(__fmaf_rn(__uint2float_rn(sum), scale, offset));
}

// Quantized distances of the 16 neighbours of one code block, by one warp.
template <int SPL>
__device__ __forceinline__ float qg_block_distance(const uint8_t* __restrict__ blk, const uint32_t (&L)[SPL][4],
                                                   uint32_t m, uint32_t ma, float scale, float offset, int lane,
                                                   int* obj) {
  uint2 w[SPL];
  qg_block_words<SPL>(blk, ma, lane, w);
  return qg_block_distance_words<SPL>(w, L, m, scale, offset, lane, obj);
}

inline size_t qg_smem_bytes(uint32_t row_chunks, uint32_t dim, uint32_t m, const ExactConfig& c) {
  size_t b = (size_t)row_chunks * 16;
  b += ((size_t)dim * 4 + 15) / 16 * 16;                 // rotated query
  b += (size_t)m * 16 * 4;                               // float table
  b += ((size_t)m * 16 + 15) / 16 * 16;                  // uint8 table
  b += (size_t)c.kcap * 8 + (size_t)c.ccap * 16 + (size_t)kExactChunk * 16;
  b += (size_t)c.hcap * 4 + (size_t)kExactChunk * 12;
  b += sizeof(QGShared) + 16;
  return b;
}

template <int SPL>
__global__ void __launch_bounds__(kExactThreads)
qg_search_kernel(DevGraph g, DevQG qg, const uint4* __restrict__ queries, uint32_t nq,
                 const QGParams* __restrict__ params, const uint32_t* __restrict__ seed_list,
                 ObjDist* __restrict__ out, uint32_t* __restrict__ out_count, QueryStats* __restrict__ stats,
                 uint32_t* __restrict__ bitmaps, unsigned long long* __restrict__ overflow, ExactConfig cfg) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t rc = g.row_chunks;
  const uint32_t D = qg.dim, M = qg.m, LD = qg.ld;
  // ---- shared-memory carve-up -------------------------------------------
  uint4* qv = reinterpret_cast<uint4*>(smem);
  float* rq = reinterpret_cast<float*>(qv + rc);
  float* flut = rq + (D + 3) / 4 * 4;
  uint8_t* lut = reinterpret_cast<uint8_t*>(flut + (size_t)M * 16);
  unsigned long long* res = reinterpret_cast<unsigned long long*>(lut + ((size_t)M * 16 + 15) / 16 * 16);
  unsigned long long* cand0 = res + cfg.kcap;
  unsigned long long* cand1 = cand0 + cfg.ccap;
  unsigned long long* bkeys = cand1 + cfg.ccap;
  unsigned long long* bsorted = bkeys + kExactChunk;
  uint32_t* table = reinterpret_cast<uint32_t*>(bsorted + kExactChunk);
  uint32_t* nid = table + cfg.hcap;
  float* nd = reinterpret_cast<float*>(nid + kExactChunk);
  float* qd = nd + kExactChunk;
  QGShared& s = *reinterpret_cast<QGShared*>(qd + kExactChunk);
  uint32_t* bitmap = bitmaps + (size_t)blockIdx.x * cfg.bitmap_words;
  unsigned long long* ovf = overflow + (size_t)blockIdx.x * 2 * cfg.ocap;
  unsigned long long* ovf_tmp = ovf + cfg.ocap;
  const uint32_t hmask = cfg.hcap - 1;
  const int G = (int)cfg.group;
  const int gl = lane & (G - 1);
  const int ngroups = kExactThreads / G;
  const float* qf = reinterpret_cast<const float*>(qv);
  const uint32_t qlen = rc * 4;                      // floats in the padded query row

  for (uint32_t q = blockIdx.x; q < nq; q += gridDim.x) {
    const QGParams P = params[q];
    for (uint32_t i = tid; i < rc; i += blockDim.x) qv[i] = queries[(size_t)q * rc + i];
    for (uint32_t i = tid; i < cfg.hcap; i += blockDim.x) table[i] = 0u;
    if (tid == 0) {
      s.radius = P.radius;
      s.nres = 0; s.head = 0; s.tail = 0; s.cur = 0; s.nvisited = 0; s.spilled = 0;
      s.done = 0; s.status = 0; s.dc = 0; s.expansions = 0; s.nnew = 0;
      s.ovf_n = 0; s.ovf_min = ~0ull; s.edges = 0;
    }
    __syncthreads();
    if (P.size == 0 || P.k == 0) {
      if (tid == 0) { out_count[q] = 0; stats[q] = QueryStats{0, 0, 0, 0, 0}; }
      __syncthreads();
      continue;
    }
    // ---- rotation and distance table ---------------------------------------
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
        for (int w = 1; w < kExactWarps; w++) { mn = fminf(mn, s.wmin[w]); mx = fmaxf(mx, s.wmax[w]); }
        s.lut_min = mn;
        s.lut_scale = __double2float_rn(__ddiv_rn((double)__fsub_rn(mx, mn), 255.0));
        s.lut_offset = __fmul_rn(mn, (float)M);
      }
      __syncthreads();
      const float mn = s.lut_min, scale = s.lut_scale;
      for (uint32_t e = tid; e < M * 16; e += blockDim.x)
        lut[e] = (uint8_t)(int)rintf(__fdiv_rn(__fsub_rn(flut[e], mn), scale));
      __syncthreads();
    }
    uint32_t L[SPL][4];
#pragma unroll
    for (int j = 0; j < SPL; j++) {
      const uint32_t sv = (uint32_t)lane + 32u * (uint32_t)j;
      const uint4 t = sv < M ? reinterpret_cast<const uint4*>(lut)[sv] : make_uint4(0, 0, 0, 0);
      L[j][0] = t.x; L[j][1] = t.y; L[j][2] = t.z; L[j][3] = t.w;
    }
    const float lscale = s.lut_scale, loffset = s.lut_offset;
    // ---- seeds --------------------------------------------------------------
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
    for (uint32_t b = (uint32_t)(warp * (32 / G)); b < nseeds; b += ngroups) {
      uint32_t i = b + (uint32_t)(lane / G);
      bool valid = i < nseeds;
      uint32_t id = valid ? seeds[i] : 0u;
      bool inrange = id < g.nrows;
      float d = group_distance<ObjType::Float, Metric::L2>(qv, g.objects + (size_t)(inrange ? id : 0u) * rc,
                                                           (int)rc, gl, G);
      if (valid && gl == 0) bkeys[i] = pack_key(inrange ? d : FLT_MAX, id);
    }
    __syncthreads();
    rank_sort(bkeys, bsorted, nseeds);
    __syncthreads();
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
        const float expR0 = __fmul_rn(P.coef, s.radius);
        const uint32_t r0 = s.ovf_n;
        if (tid == 0) s.ovf_tmp = 0;
        __syncthreads();
        for (uint32_t i = tid; i < r0; i += blockDim.x) {
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
        float expR = __fmul_rn(P.coef, s.radius);
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
      if (++guard > g.nrows + 8) {
        if (tid == 0) s.status |= kStatusIterationLimit;
        break;
      }
      const uint32_t target = s.target;
      const bool has_node = target < qg.nnodes;       // nodes beyond the quantized graph have no edges
      const uint32_t e0 = has_node ? qg.offsets[target] : 0u;
      const uint32_t deg = has_node ? qg.offsets[target + 1] - e0 : 0u;
      const uint8_t* stream = qg.codes + (has_node ? (size_t)qg.code_off16[target] * 16 : 0);
      if (tid == 0) { s.edges += deg; s.dc += deg; }
      for (uint32_t c0 = 0; c0 < deg; c0 += kExactChunk) {
        const uint32_t clen = min((uint32_t)kExactChunk, deg - c0);
        // quantized distances of the chunk: one 16-neighbour block per warp at a time
        const uint32_t nblk = (clen + 15) / 16;
        for (uint32_t bi = (uint32_t)warp; bi < nblk; bi += kExactWarps) {
          const uint8_t* blk = stream + (size_t)(c0 / 16 + bi) * 8 * qg.ma;
          int o;
          float d = qg_block_distance<SPL>(blk, L, M, qg.ma, lscale, loffset, lane, &o);
          if (o >= 0 && bi * 16 + (uint32_t)o < clen) qd[bi * 16 + o] = d;
        }
        if (!s.spilled && s.nvisited + clen > (cfg.hcap >> 1)) {
          for (uint32_t i = tid; i < cfg.hcap; i += blockDim.x) {
            uint32_t id = table[i];
            if (id) atomicOr(&bitmap[id >> 5], 1u << (id & 31u));
          }
          __threadfence_block();
          __syncthreads();
          if (tid == 0) { s.spilled = 1; s.status |= kStatusVisitedSpill; }
        }
        __syncthreads();
        const bool spilled = s.spilled != 0;
        // within the exploration radius and not visited yet: new, in edge order
        const float expR0 = __fmul_rn(P.coef, s.radius);
        bool isnew = false;
        uint32_t id = 0;
        float dq = 0.f;
        if ((uint32_t)tid < clen) {
          dq = qd[tid];
          id = qg.ids[e0 + c0 + tid];
          if (dq <= expR0) isnew = visit_insert(table, hmask, bitmap, spilled, id);
        }
        unsigned ballot = __ballot_sync(0xffffffffu, isnew);
        if (lane == 0) s.warp_cnt[warp] = __popc(ballot);
        __syncthreads();
        uint32_t base = 0;
        for (int w = 0; w < warp; w++) base += s.warp_cnt[w];
        if (isnew) {
          const uint32_t pos = base + __popc(ballot & ((1u << lane) - 1u));
          nid[pos] = id;
          nd[pos] = dq;
        }
        __syncthreads();
        uint32_t nnew = 0;
        for (int w = 0; w < kExactWarps; w++) nnew += s.warp_cnt[w];
        // sequential replay of the result-set updates (warp 0): a neighbour joins
        // when within both the exploration radius and the radius of that moment
        if (warp == 0) {
          float radius = s.radius;
          uint32_t n = s.nres;
          for (uint32_t b = 0; b < nnew; b += 32) {
            uint32_t i = b + lane;
            float d = i < nnew ? nd[i] : FLT_MAX;
            float lim = fminf(radius, __fmul_rn(P.coef, radius));
            unsigned m = __ballot_sync(0xffffffffu, i < nnew && d <= lim);
            while (m) {
              int src = __ffs(m) - 1;
              float dj = __shfl_sync(0xffffffffu, d, src);
              uint32_t idj = nid[b + src];
              if (dj <= radius && dj <= __fmul_rn(P.coef, radius))
                result_insert(res, n, radius, P.size, (uint32_t)GraphMode::Updatable, pack_key(dj, idj), lane);
              m &= (src == 31) ? 0u : ~((2u << src) - 1u);
              lim = fminf(radius, __fmul_rn(P.coef, radius));
              m &= __ballot_sync(0xffffffffu, i < nnew && d <= lim);
            }
          }
          if (lane == 0) {
            s.radius = radius;
            s.nres = n;
            s.nvisited += nnew;
          }
        }
        __syncthreads();
        const float expR = __fmul_rn(P.coef, s.radius);
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
        if (tid == 0) s.live_old = upper_bound_dist(cl + s.head, s.tail - s.head, expR);
        __syncthreads();
        const uint32_t nold = s.live_old;
        const unsigned long long* old = cl + s.head;
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
      __syncthreads();
    }
    // ---- results ---------------------------------------------------------------
    __syncthreads();
    uint32_t n = s.nres;
    if (P.rerank) {
      // exact L2 of every result, sorted by (distance, id); kept while distance <
      // radius (upper_bound at (0, radius)); at most k
      for (uint32_t b = (uint32_t)(warp * (32 / G)); b < n; b += ngroups) {
        uint32_t i = b + (uint32_t)(lane / G);
        bool valid = i < n;
        uint32_t id = valid ? key_id(res[i]) : 0u;
        float d = group_distance<ObjType::Float, Metric::L2>(qv, g.objects + (size_t)id * rc, (int)rc, gl, G);
        if (valid && gl == 0) cand0[i] = pack_key(d, id);
      }
      __syncthreads();
      bitonic_sort(cand0, n, cfg.ccap);
      if (tid == 0) {
        uint32_t keep = n;
        if (P.radius < FLT_MAX) {
          keep = 0;
          while (keep < n && key_dist(cand0[keep]) < P.radius) keep++;
        }
        s.nnew = min(keep, P.k);
      }
      __syncthreads();
      n = s.nnew;
      for (uint32_t i = tid; i < n; i += blockDim.x) {
        unsigned long long k = cand0[i];
        out[P.out_off + i] = ObjDist{key_id(k), key_dist(k)};
      }
    } else {
      for (uint32_t i = tid; i < n; i += blockDim.x) {
        unsigned long long k = res[i];
        out[P.out_off + i] = ObjDist{key_id(k), key_dist(k)};
      }
    }
    if (tid == 0) {
      out_count[q] = n;
      stats[q] = QueryStats{s.dc, s.expansions, s.nvisited, s.edges, s.status};
    }
    if (s.spilled) {
      for (uint32_t i = tid; i < cfg.bitmap_words; i += blockDim.x) bitmap[i] = 0u;
      __threadfence();
    }
    __syncthreads();
  }
}

}  // namespace ngtg
