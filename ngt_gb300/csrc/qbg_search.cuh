// Quantized-blob-graph search (QBG): one query per CTA, reproducing
// QBG::Index::searchInOneStep (lib/NGT/NGTQ/QuantizedBlobGraph.h:1332-1594) as
// the C API (qbg_search_index_, lib/NGT/NGTQ/Capi.cpp:549-574) drives it, so
// that results equal the reference's.
//
// The index has a global NGT index over the blob centroids (graph + DVP tree)
// and, per blob (= global node), the 4-bit codes of its objects quantized
// against the rotated codebook centroid of the blob's subspace id.
//   1. seeds: the global tree's leaf (thinned to the result size) with exact L2
//      distances; the nearest is the current blob, the others are "discarded"
//      (waiting) blobs; all are untraced graph nodes.
//   2. while the nearest untraced node is within blob_coef x d(current blob),
//      it is expanded: its unvisited neighbours get exact L2 distances, become
//      untraced, and either replace the current blob (strictly nearer; the first
//      such neighbour in edge order) or wait.
//   3. otherwise the current blob is judged (QuantizedBlobGraph.h:1033-1080):
//      its LUT is built for the blob's subspace id (the rotated query minus that
//      centroid, as in the QG table) and its objects scanned; when the scan's
//      minimum is below the radius every object within the radius joins the
//      result set (kept to its size, radius = its maximum when full).  The search
//      stops when the minimum exceeds radius x (1 + epsilon), after
//      number_of_explored_blobs judgements, or when no blob waits; else the
//      nearest waiting blob becomes current.
// Results carry the quantized distances, number_of_results x result_expansion
// of them when the expansion is >= 1 (the C API never sets refinement).
// Both queues are exact two-tier min-queues (tier_queue.cuh).
#pragma once
#include <cfloat>
#include "qg_search.cuh"
#include "tier_queue.cuh"

namespace ngtg {

struct QBGShared {
  float radius, expR;
  uint32_t nres, rcur;
  unsigned long long current;       // (distance, id) of the current blob
  uint32_t done;
  uint32_t exploration;
  uint32_t nblobs, expansions, dc, status;
  uint32_t seed_leaf;
  uint32_t nnew, nacc;
  uint32_t lut_sid;
  float lut_min, lut_scale, lut_offset;
  float bmin;
  float wmin[kExactWarps], wmax[kExactWarps];
  uint32_t warp_cnt[kExactWarps];
  QueueState uq, dq;
  uint32_t hist[256];
};

struct QBGConfig {
  uint32_t rcap;          // result capacity (>= the largest result size), power of two
  uint32_t qcap;          // shared entries per queue (power of two)
  uint32_t ocap;          // overflow keys per queue and buffer
  uint32_t bitmap_words;  // visited bitmap words per CTA (global nodes)
  uint32_t blob_cap;      // distance scratch per CTA (largest blob, rounded up to 16)
  uint32_t group;         // lanes per exact distance (power of two <= 32)
};

inline size_t qbg_smem_bytes(uint32_t row_chunks, uint32_t dim, uint32_t m, const QBGConfig& c) {
  size_t b = (size_t)row_chunks * 16;
  b += ((size_t)dim * 4 + 15) / 16 * 16;
  b += (size_t)m * 16 * 4;
  b += ((size_t)m * 16 + 15) / 16 * 16;
  b += (size_t)c.rcap * 16;                            // results, double-buffered
  b += (size_t)c.qcap * 32;                            // two queues x two buffers
  b += (size_t)kExactChunk * 8 * 3;                    // keys, sorted keys, queue batch
  b += (size_t)kExactChunk * 8;                        // nid + nd
  b += sizeof(QBGShared) + 16;
  return b;
}

// Builds the uint8 LUT of the rotated query against codebook centroid `gc`
// (same arithmetic as the QG table) into lut[] and the scale / offset in s.
__device__ __forceinline__ void qbg_build_lut(const float* rq, const float* __restrict__ gc,
                                              const float* __restrict__ lc, float* flut, uint8_t* lut, uint32_t M,
                                              uint32_t LD, QBGShared& s) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  float lmin = FLT_MAX, lmax = -FLT_MAX;
  for (uint32_t e = tid; e < M * 16; e += blockDim.x) {
    const uint32_t sv = e >> 4, c = e & 15u;
    float v = 0.f;
    for (uint32_t d = 0; d < LD; d++) {
      const float rsv = __fsub_rn(rq[sv * LD + d], gc[sv * LD + d]);
      const float sub = __fsub_rn(rsv, lc[((size_t)sv * 16 + c) * LD + d]);
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

// Merges m sorted keys into the sorted result set (double-buffered), keeping the
// `size` smallest.
__device__ __forceinline__ void qbg_merge_results(unsigned long long* const* resb, QBGShared& s,
                                                  const unsigned long long* keys, uint32_t m, uint32_t size) {
  const uint32_t tid = threadIdx.x;
  const unsigned long long* old = resb[s.rcur];
  unsigned long long* dst = resb[s.rcur ^ 1u];
  const uint32_t nold = s.nres;
  for (uint32_t i = tid; i < nold; i += blockDim.x) {
    uint32_t pos = i + lower_bound_keys(keys, m, old[i]);
    if (pos < size) dst[pos] = old[i];
  }
  for (uint32_t i = tid; i < m; i += blockDim.x) {
    uint32_t pos = i + lower_bound_keys(old, nold, keys[i]);
    if (pos < size) dst[pos] = keys[i];
  }
  __syncthreads();
  if (tid == 0) {
    s.nres = min(nold + m, size);
    s.rcur ^= 1u;
  }
  __syncthreads();
}

// Rotation::mul of the query (the OpenBLAS sgemv order: one FMA chain for D <= 48,
// else blocks of 8 columns), the query zero-padded to D.
__device__ __forceinline__ void qbg_rotate(const DevQG& qb, const float* qf, uint32_t qlen, float* rq) {
  const uint32_t D = qb.dim;
  for (uint32_t c = threadIdx.x; c < D; c += blockDim.x) {
    float acc = 0.f;
    if (qb.rotation == nullptr) {
      acc = c < qlen ? qf[c] : 0.f;
    } else if (D <= 48) {
      for (uint32_t p = 0; p < D; p++) acc = __fmaf_rn(qb.rotation[(size_t)p * D + c], p < qlen ? qf[p] : 0.f, acc);
    } else {
      for (uint32_t p0 = 0; p0 < D; p0 += 8) {
        const uint32_t p1 = min(p0 + 8u, D);
        float t = __fmul_rn(qb.rotation[(size_t)p0 * D + c], p0 < qlen ? qf[p0] : 0.f);
        for (uint32_t p = p0 + 1; p < p1; p++) t = __fmaf_rn(qb.rotation[(size_t)p * D + c], p < qlen ? qf[p] : 0.f, t);
        acc = __fadd_rn(acc, t);
      }
    }
    rq[c] = acc;
  }
}

// judge (lib/NGT/NGTQ/QuantizedBlobGraph.h:1033-1080) of one blob by the whole CTA:
// the blob's LUT (rebuilt only when its subspace id differs from the last one),
// the scan of its codes into bdist, its minimum into s.bmin; when that minimum is
// below the radius, every object within the radius joins the result set (kept to
// `size`), and the radius becomes the set's maximum once it is full.
template <int SPL>
__device__ __forceinline__ void qbg_judge_blob(const DevQG& qb, const uint32_t* __restrict__ blob_sid, uint32_t blob,
                                               const float* rq, float* flut, uint8_t* lut, QBGShared& s,
                                               float* bdist, unsigned long long* const* resb,
                                               unsigned long long* bkeys, unsigned long long* bsorted,
                                               uint32_t size) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t M = qb.m, LD = qb.ld, D = qb.dim;
  if (tid == 0) s.bmin = FLT_MAX;
  __syncthreads();
  if (blob >= qb.nnodes) return;
  const uint32_t a = qb.offsets[blob];
  const uint32_t n = qb.offsets[blob + 1] - a;
  const uint32_t sid = blob_sid[blob];
  if (sid != s.lut_sid) {
    qbg_build_lut(rq, qb.gcentroid + (size_t)sid * D, qb.lcentroids, flut, lut, M, LD, s);
    if (tid == 0) s.lut_sid = sid;
  }
  uint32_t L[SPL][4];
#pragma unroll
  for (int j = 0; j < SPL; j++) {
    const uint32_t sv = (uint32_t)lane + 32u * (uint32_t)j;
    const uint4 v = sv < M ? reinterpret_cast<const uint4*>(lut)[sv] : make_uint4(0, 0, 0, 0);
    L[j][0] = v.x; L[j][1] = v.y; L[j][2] = v.z; L[j][3] = v.w;
  }
  const float lscale = s.lut_scale, loffset = s.lut_offset;
  const uint8_t* stream = qb.codes + (size_t)qb.code_off16[blob] * 16;
  const uint32_t nblk = (n + 15) / 16;
  float wmin = FLT_MAX;
  for (uint32_t bi = (uint32_t)warp; bi < nblk; bi += kExactWarps) {
    int o;
    float d = qg_block_distance<SPL>(stream + (size_t)bi * 8 * qb.ma, L, M, qb.ma, lscale, loffset, lane, &o);
    if (o >= 0 && bi * 16 + (uint32_t)o < n) {
      bdist[bi * 16 + o] = d;
      wmin = fminf(wmin, d);
    }
  }
  for (int off = 16; off > 0; off >>= 1) wmin = fminf(wmin, __shfl_xor_sync(0xffffffffu, wmin, off));
  if (lane == 0) s.wmin[warp] = wmin;
  __threadfence_block();
  __syncthreads();
  if (tid == 0) {
    float mn = s.wmin[0];
    for (int w = 1; w < kExactWarps; w++) mn = fminf(mn, s.wmin[w]);
    s.bmin = mn;
    s.nblobs++;
    s.dc += n;
  }
  __syncthreads();
  const float radius0 = s.radius;
  if (s.bmin < radius0) {
    for (uint32_t c0 = 0; c0 < n; c0 += kExactChunk) {
      const uint32_t clen = min((uint32_t)kExactChunk, n - c0);
      bool acc = false;
      float d = 0.f;
      if ((uint32_t)tid < clen) {
        d = bdist[c0 + tid];
        acc = d <= radius0;
      }
      unsigned ballot = __ballot_sync(0xffffffffu, acc);
      if (lane == 0) s.warp_cnt[warp] = __popc(ballot);
      __syncthreads();
      uint32_t base = 0, m = 0;
      for (int w = 0; w < kExactWarps; w++) {
        if (w < warp) base += s.warp_cnt[w];
        m += s.warp_cnt[w];
      }
      if (acc) bkeys[base + __popc(ballot & ((1u << lane) - 1u))] = pack_key(d, qb.ids[a + c0 + tid]);
      __syncthreads();
      rank_sort(bkeys, bsorted, m);
      __syncthreads();
      qbg_merge_results(resb, s, bsorted, m, size);
    }
    if (tid == 0 && s.nres >= size) s.radius = key_dist(resb[s.rcur][s.nres - 1]);
    __syncthreads();
  }
}

template <int SPL>
__global__ void __launch_bounds__(kExactThreads)
qbg_search_kernel(DevGraph g, DevQG qb, const uint32_t* __restrict__ blob_sid, const uint4* __restrict__ queries,
                  uint32_t nq, const QBGParams* __restrict__ params, const uint32_t* __restrict__ seed_list,
                  ObjDist* __restrict__ out, uint32_t* __restrict__ out_count, QueryStats* __restrict__ stats,
                  uint32_t* __restrict__ bitmaps, unsigned long long* __restrict__ overflow,
                  float* __restrict__ blob_dist, QBGConfig cfg) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t rc = g.row_chunks;
  const uint32_t D = qb.dim, M = qb.m, LD = qb.ld;
  uint4* qv = reinterpret_cast<uint4*>(smem);
  float* rq = reinterpret_cast<float*>(qv + rc);
  float* flut = rq + (D + 3) / 4 * 4;
  uint8_t* lut = reinterpret_cast<uint8_t*>(flut + (size_t)M * 16);
  unsigned long long* res0 = reinterpret_cast<unsigned long long*>(lut + ((size_t)M * 16 + 15) / 16 * 16);
  unsigned long long* res1 = res0 + cfg.rcap;
  unsigned long long* uq0 = res1 + cfg.rcap;
  unsigned long long* uq1 = uq0 + cfg.qcap;
  unsigned long long* dq0 = uq1 + cfg.qcap;
  unsigned long long* dq1 = dq0 + cfg.qcap;
  unsigned long long* bkeys = dq1 + cfg.qcap;
  unsigned long long* bsorted = bkeys + kExactChunk;
  unsigned long long* batch = bsorted + kExactChunk;
  uint32_t* nid = reinterpret_cast<uint32_t*>(batch + kExactChunk);
  float* nd = reinterpret_cast<float*>(nid + kExactChunk);
  QBGShared& s = *reinterpret_cast<QBGShared*>(nd + kExactChunk);
  unsigned long long* resb[2] = {res0, res1};
  uint32_t* bitmap = bitmaps + (size_t)blockIdx.x * cfg.bitmap_words;
  unsigned long long* ovf = overflow + (size_t)blockIdx.x * 4 * cfg.ocap;
  float* bdist = blob_dist + (size_t)blockIdx.x * cfg.blob_cap;
  const TierQueue uq{{uq0, uq1}, cfg.qcap, {ovf, ovf + cfg.ocap}, cfg.ocap, &s.uq, s.hist};
  const TierQueue dq{{dq0, dq1}, cfg.qcap, {ovf + 2 * (size_t)cfg.ocap, ovf + 3 * (size_t)cfg.ocap}, cfg.ocap,
                     &s.dq, s.hist};
  const int G = (int)cfg.group;
  const int gl = lane & (G - 1);
  const int ngroups = kExactThreads / G;
  const float* qf = reinterpret_cast<const float*>(qv);
  const uint32_t qlen = rc * 4;

  for (uint32_t q = blockIdx.x; q < nq; q += gridDim.x) {
    const QBGParams P = params[q];
    for (uint32_t i = tid; i < rc; i += blockDim.x) qv[i] = queries[(size_t)q * rc + i];
    if (tid == 0) {
      s.radius = FLT_MAX;
      s.nres = 0; s.rcur = 0; s.done = 0; s.exploration = 1;
      s.nblobs = 0; s.expansions = 0; s.dc = 0; s.status = 0;
      s.lut_sid = 0xffffffffu;
    }
    tq_init(uq);
    tq_init(dq);
    if (P.size == 0) {
      if (tid == 0) { out_count[q] = 0; stats[q] = QueryStats{0, 0, 0, 0, 0}; }
      __syncthreads();
      continue;
    }
    // ---- rotation (Rotation::mul, the OpenBLAS sgemv order) ------------------
    qbg_rotate(qb, qf, qlen, rq);
    // ---- seeds: tree leaf of the global index, else the fixed random list ---
    const uint32_t* seeds = nullptr;
    uint32_t nseeds = 0;
    if (tid == 0) s.seed_leaf = 0xffffffffu;
    __syncthreads();
    if (warp == 0 && P.seed_cnt == 0xffffffffu) {
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
    if (P.seed_cnt == 0xffffffffu && s.seed_leaf != 0xffffffffu && s.seed_leaf < g.nleaves) {
      const uint32_t* off = g.leaf_seed_off + P.seed_off;
      uint32_t a = off[s.seed_leaf], b = off[s.seed_leaf + 1];
      seeds = g.leaf_seed_ids + a;
      nseeds = b - a;
    }
    if (nseeds == 0) {
      seeds = seed_list + P.fb_off;
      nseeds = P.fb_cnt;
    }
    nseeds = min(nseeds, (uint32_t)kExactChunk);
    if (nseeds == 0) {
      if (tid == 0) { out_count[q] = 0; stats[q] = QueryStats{0, 0, 0, 0, s.status | kStatusEmptySeeds}; }
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
    for (uint32_t i = tid; i < nseeds; i += blockDim.x) {
      uint32_t id = key_id(bsorted[i]);
      atomicOr(&bitmap[id >> 5], 1u << (id & 31u));
    }
    if (tid == 0) {
      s.current = bsorted[0];
      s.expR = __fmul_rn(P.bcoef, key_dist(bsorted[0]));
      s.dc = nseeds;
    }
    __syncthreads();
    tq_push_sorted(uq, bsorted, nseeds);
    tq_push_sorted(dq, bsorted + 1, nseeds - 1);

    // ---- main loop ------------------------------------------------------------
    uint32_t guard = 0;
    while (true) {
      if (++guard > 4u * g.nrows + 64u) {            // each node is traced / judged at most once
        if (tid == 0) s.status |= kStatusIterationLimit;
        break;
      }
      const unsigned long long t = tq_top(uq);
      if (t == ~0ull || key_dist(t) > s.expR) {
        // ---- judge the current blob ----
        const uint32_t blob = key_id(s.current);
        if (tid == 0) s.exploration++;
        qbg_judge_blob<SPL>(qb, blob_sid, blob, rq, flut, lut, s, bdist, resb, bkeys, bsorted, P.size);
        // ---- stop, or take the nearest waiting blob ----
        if (s.bmin > __fmul_rn(s.radius, P.coef) || s.exploration > P.explored) break;
        const unsigned long long nxt = tq_top(dq);
        if (nxt == ~0ull) break;
        tq_pop(dq);
        if (tid == 0) {
          s.current = nxt;
          s.expR = __fmul_rn(P.bcoef, key_dist(nxt));
        }
        __syncthreads();
        continue;
      }
      // ---- expand the nearest untraced node of the global graph ----
      tq_pop(uq);
      const uint32_t target = key_id(t);
      const uint32_t e0 = g.offsets[target];
      const uint32_t deg = g.offsets[target + 1] - e0;
      const uint32_t nsz = min(deg, P.edge_size);
      if (tid == 0) s.expansions++;
      for (uint32_t c0 = 0; c0 < nsz; c0 += kExactChunk) {
        const uint32_t clen = min((uint32_t)kExactChunk, nsz - c0);
        bool isnew = false;
        uint32_t id = 0;
        if ((uint32_t)tid < clen) {
          id = g.edges[e0 + c0 + tid];
          const uint32_t bit = 1u << (id & 31u);
          isnew = (atomicOr(&bitmap[id >> 5], bit) & bit) == 0u;
        }
        unsigned ballot = __ballot_sync(0xffffffffu, isnew);
        if (lane == 0) s.warp_cnt[warp] = __popc(ballot);
        __syncthreads();
        uint32_t base = 0, nnew = 0;
        for (int w = 0; w < kExactWarps; w++) {
          if (w < warp) base += s.warp_cnt[w];
          nnew += s.warp_cnt[w];
        }
        if (isnew) nid[base + __popc(ballot & ((1u << lane) - 1u))] = id;
        __syncthreads();
        for (uint32_t b = (uint32_t)(warp * (32 / G)); b < nnew; b += ngroups) {
          uint32_t i = b + (uint32_t)(lane / G);
          bool valid = i < nnew;
          uint32_t v = valid ? nid[i] : 0u;
          float d = group_distance<ObjType::Float, Metric::L2>(qv, g.objects + (size_t)v * rc, (int)rc, gl, G);
          if (valid && gl == 0) nd[i] = d;
        }
        __syncthreads();
        if (nnew == 0) continue;
        // the first neighbour (edge order) strictly nearer than the current blob
        // replaces it; everything else waits
        if (warp == 0) {
          float best = FLT_MAX;
          uint32_t bi = 0xffffffffu;
          for (uint32_t i = lane; i < nnew; i += 32) {
            if (nd[i] < best) { best = nd[i]; bi = i; }
          }
          for (int off = 16; off > 0; off >>= 1) {
            float ob = __shfl_xor_sync(0xffffffffu, best, off);
            uint32_t oi = __shfl_xor_sync(0xffffffffu, bi, off);
            if (ob < best || (ob == best && oi < bi)) { best = ob; bi = oi; }
          }
          if (lane == 0) s.nacc = (best < key_dist(s.current)) ? bi : 0xffffffffu;
        }
        __syncthreads();
        const uint32_t rep = s.nacc;
        for (uint32_t i = tid; i < nnew; i += blockDim.x) bkeys[i] = pack_key(nd[i], nid[i]);
        __syncthreads();
        rank_sort(bkeys, bsorted, nnew);
        __syncthreads();
        tq_push_sorted(uq, bsorted, nnew);
        // waiting blobs: the new nodes except the replacement, plus the old current
        uint32_t nw = 0;
        {
          const unsigned long long repk = rep != 0xffffffffu ? pack_key(nd[rep], nid[rep]) : ~0ull;
          const unsigned long long oldc = s.current;
          // bsorted without repk, with oldc inserted in order (when replaced)
          for (uint32_t i = tid; i < nnew; i += blockDim.x) {
            unsigned long long k = bsorted[i];
            if (k == repk) continue;
            uint32_t pos = i - (repk != ~0ull && repk < k ? 1u : 0u) + (rep != 0xffffffffu && oldc < k ? 1u : 0u);
            batch[pos] = k;
          }
          if (tid == 0 && rep != 0xffffffffu) {
            uint32_t pos = lower_bound_keys(bsorted, nnew, oldc);
            pos -= (repk < oldc) ? 1u : 0u;
            batch[pos] = oldc;
          }
          nw = nnew;                                // -1 replacement +1 old current, or all new
        }
        __syncthreads();
        tq_push_sorted(dq, batch, nw);
        if (tid == 0 && rep != 0xffffffffu) {
          s.current = pack_key(nd[rep], nid[rep]);
          s.expR = __fmul_rn(P.bcoef, nd[rep]);
        }
        if (tid == 0) s.dc += nnew;
        __syncthreads();
      }
      __syncthreads();
    }
    // ---- results: ascending (distance, id), quantized distances ----------------
    __syncthreads();
    const uint32_t n = s.nres;
    const unsigned long long* res = resb[s.rcur];
    for (uint32_t i = tid; i < n; i += blockDim.x) out[P.out_off + i] = ObjDist{key_id(res[i]), key_dist(res[i])};
    if (tid == 0) {
      uint32_t st = s.status | (s.uq.status || s.dq.status ? kStatusCandidateOverflow : 0u);
      out_count[q] = n;
      stats[q] = QueryStats{s.dc, s.expansions, s.nblobs, 0, st};
    }
    // leave the visited bitmap clean for the next query
    for (uint32_t i = tid; i < cfg.bitmap_words; i += blockDim.x) bitmap[i] = 0u;
    __threadfence();
    __syncthreads();
  }
}

// Shared memory of qbg_scan_kernel: query row, rotated query, float and uint8
// tables, the double-buffered result set, the chunk keys, the shared state.
inline size_t qbg_scan_smem_bytes(uint32_t row_chunks, uint32_t dim, uint32_t m, uint32_t rcap) {
  size_t b = (size_t)row_chunks * 16;
  b += ((size_t)dim * 4 + 15) / 16 * 16;
  b += (size_t)m * 16 * 4;
  b += ((size_t)m * 16 + 15) / 16 * 16;
  b += (size_t)rcap * 16;
  b += (size_t)kExactChunk * 16;
  b += sizeof(QBGShared) + 16;
  return b;
}

// The blob phase of searchInTwoSteps (lib/NGT/NGTQ/QuantizedBlobGraph.h:1240-1306):
// one query per CTA; its probed blobs (blobs[q * bstride ..], bcount[q] of them,
// nearest first, from the global index's graph search) are judged in that order
// with a result set of P.size.  Results: the quantized distances, ascending.
template <int SPL>
__global__ void __launch_bounds__(kExactThreads)
qbg_scan_kernel(DevQG qb, const uint32_t* __restrict__ blob_sid, const uint4* __restrict__ queries,
                uint32_t row_chunks, uint32_t nq, const QBGParams* __restrict__ params,
                const ObjDist* __restrict__ blobs, const uint32_t* __restrict__ bcount, uint32_t bstride,
                ObjDist* __restrict__ out, uint32_t* __restrict__ out_count, QueryStats* __restrict__ stats,
                float* __restrict__ blob_dist, uint32_t blob_cap, uint32_t rcap) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x;
  const uint32_t rc = row_chunks;
  const uint32_t D = qb.dim, M = qb.m;
  uint4* qv = reinterpret_cast<uint4*>(smem);
  float* rq = reinterpret_cast<float*>(qv + rc);
  float* flut = rq + (D + 3) / 4 * 4;
  uint8_t* lut = reinterpret_cast<uint8_t*>(flut + (size_t)M * 16);
  unsigned long long* res0 = reinterpret_cast<unsigned long long*>(lut + ((size_t)M * 16 + 15) / 16 * 16);
  unsigned long long* res1 = res0 + rcap;
  unsigned long long* bkeys = res1 + rcap;
  unsigned long long* bsorted = bkeys + kExactChunk;
  QBGShared& s = *reinterpret_cast<QBGShared*>(bsorted + kExactChunk);
  unsigned long long* resb[2] = {res0, res1};
  float* bdist = blob_dist + (size_t)blockIdx.x * blob_cap;
  const float* qf = reinterpret_cast<const float*>(qv);
  for (uint32_t q = blockIdx.x; q < nq; q += gridDim.x) {
    const QBGParams P = params[q];
    for (uint32_t i = tid; i < rc; i += blockDim.x) qv[i] = queries[(size_t)q * rc + i];
    if (tid == 0) {
      s.radius = FLT_MAX;
      s.nres = 0; s.rcur = 0;
      s.nblobs = 0; s.expansions = 0; s.dc = 0; s.status = 0;
      s.lut_sid = 0xffffffffu;
    }
    __syncthreads();
    const uint32_t nb = P.size == 0 ? 0u : bcount[q];
    if (nb > 0) qbg_rotate(qb, qf, rc * 4, rq);
    __syncthreads();
    for (uint32_t b = 0; b < nb; b++)
      qbg_judge_blob<SPL>(qb, blob_sid, blobs[(size_t)q * bstride + b].id, rq, flut, lut, s, bdist, resb, bkeys,
                          bsorted, P.size);
    __syncthreads();
    const uint32_t n = s.nres;
    const unsigned long long* res = resb[s.rcur];
    for (uint32_t i = tid; i < n; i += blockDim.x) out[P.out_off + i] = ObjDist{key_id(res[i]), key_dist(res[i])};
    if (tid == 0) {
      out_count[q] = n;
      stats[q] = QueryStats{s.dc, 0, s.nblobs, 0, s.status};
    }
    __syncthreads();
  }
}

// refineDistances (lib/NGT/NGTQ/QuantizedBlobGraph.h:1136-1185): per query (one CTA)
// the cand_count[q] candidates at cand[q * cstride ..] get their exact L2 distances
// over the object list (rows of `orc` 16-byte chunks, row 0 unused; the float query
// cast element-wise to the row type, as setObject does), are sorted by (distance,
// id) and the first min(exact[q], n) written to out[q * kmax ..].
// M: the comparator (L2 for QBG; the index's distance for a graph index's refinement
// objects, lib/NGT/Index.h:1146-1236).
template <ObjType OT, Metric M = Metric::L2>
__global__ void __launch_bounds__(256)
qbg_refine_kernel(const ObjDist* __restrict__ cand, const uint32_t* __restrict__ cand_count, uint32_t cstride,
                  const float* __restrict__ qrows, uint32_t qdim, const uint4* __restrict__ olist, uint32_t orc,
                  uint32_t odim, uint32_t nrows, const uint32_t* __restrict__ exact, uint32_t nq, uint32_t P,
                  ObjDist* __restrict__ out, uint32_t kmax, uint32_t* __restrict__ out_count) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint4* qv = reinterpret_cast<uint4*>(smem);                                        // orc chunks
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(qv + orc);          // P
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t G = 1;
  while (G < orc && G < 32) G <<= 1;
  const uint32_t gl = lane & (G - 1), gpw = 32 / G, ngroups = blockDim.x / G;
  for (uint32_t q = blockIdx.x; q < nq; q += gridDim.x) {
    const uint32_t n = min(cand_count[q], P);
    if constexpr (OT == ObjType::Uint8) {
      uint8_t* qb = reinterpret_cast<uint8_t*>(qv);
      for (uint32_t i = threadIdx.x; i < orc * 16; i += blockDim.x)
        qb[i] = i < odim && i < qdim ? (uint8_t)__float2int_rz(qrows[(size_t)q * qdim + i]) : (uint8_t)0;
    } else {
      float* qb = reinterpret_cast<float*>(qv);
      for (uint32_t i = threadIdx.x; i < orc * 4; i += blockDim.x)
        qb[i] = i < odim && i < qdim ? qrows[(size_t)q * qdim + i] : 0.f;
    }
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) keys[i] = ~0ull;
    __syncthreads();
    for (uint32_t b = warp * gpw; b < n; b += ngroups) {
      const uint32_t i = b + lane / G;
      const bool valid = i < n;
      const uint32_t id = valid ? cand[(size_t)q * cstride + i].id : 0u;
      const bool inrange = id > 0 && id < nrows;
      const float d = group_distance<OT, M>(qv, olist + (size_t)(inrange ? id : 0u) * orc, (int)orc, (int)gl,
                                            (int)G);
      if (valid && gl == 0) keys[i] = pack_key(inrange ? d : FLT_MAX, id);
    }
    __syncthreads();
    for (uint32_t k2 = 2; k2 <= P; k2 <<= 1) {
      for (uint32_t j = k2 >> 1; j > 0; j >>= 1) {
        for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
          const uint32_t l = i ^ j;
          if (l > i) {
            const unsigned long long x = keys[i], y = keys[l];
            const bool up = (i & k2) == 0;
            if ((x > y) == up) {
              keys[i] = y;
              keys[l] = x;
            }
          }
        }
        __syncthreads();
      }
    }
    const uint32_t m = min(exact[q], n);
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x)
      out[(size_t)q * kmax + i] = ObjDist{key_id(keys[i]), key_dist(keys[i])};
    if (threadIdx.x == 0) out_count[q] = m;
    __syncthreads();
  }
}

}  // namespace ngtg
