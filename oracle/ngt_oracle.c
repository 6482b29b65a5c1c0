/*
 * ORACLE -- test infrastructure only.  A plain-C, single-threaded-per-query
 * restatement of NGT's search path, used by tests/ to check the CUDA library
 * and by bench.py as the timed CPU baseline (OpenMP over queries, the pattern
 * of ngtpy.Index.batch_search, python/src/ngtpy.cpp:422-458).  Nothing in the
 * product links or calls this file.
 *
 * Restated from the reference (file:line in the NGT source tree):
 *   comparators       lib/NGT/PrimitiveComparatorNoArch.h:30-390 (scalar forms;
 *                     double accumulation, exact for integer-valued data)
 *   linear search     lib/NGT/ObjectSpaceRepository.h:860-922
 *   graph search      lib/NGT/Graph.cpp:716-835 (read-only) and 840-1024 (updatable),
 *                     setupDistances/setupSeeds lib/NGT/Graph.cpp:420-586,
 *                     getEdgeSize lib/NGT/Graph.h:991-1010
 *   result heap       ResultSet push / pop / push_pop lib/NGT/Common.h:2412-2431
 *                     (libstdc++ pop_heap on Linux: push_pop replaces the top)
 *   tree seeds        DVPTree::search SearchLeaf lib/NGT/Tree.cpp:403-559,
 *                     getSeedsFromTree thinning lib/NGT/Index.h:2173-2220
 *   glibc rand()      random_r TYPE_3 (degree 31, separation 3) as published
 *   query conversion  ObjectRepository::setObject lib/NGT/ObjectRepository.h:238-282,
 *                     ObjectSpace::normalize lib/NGT/ObjectSpace.h:356-384
 *   qsint8 objects    ObjectSpace::quantizeSymmetrically lib/NGT/ObjectSpace.h:432-441
 *                     (query codes), PrimitiveComparator::compareL2(qsint8)
 *                     lib/NGT/PrimitiveComparatorX86.h:341-431 (the squared sum,
 *                     no square root, in the x86 build), the updatable search's
 *                     result-size rule for quantized objects lib/NGT/Graph.cpp:845-852
 */
#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

enum { OT_FLOAT = 0, OT_UINT8 = 1, OT_HALF = 2, OT_QSINT8 = 3 };
enum {
  M_L1 = 0, M_L2 = 1, M_HAMMING = 2, M_ANGLE = 3, M_COSINE = 4, M_NANGLE = 5, M_NCOSINE = 6,
  M_JACCARD = 7, M_NL2 = 9, M_IP = 10, M_POINCARE = 100, M_LORENTZ = 101
};

typedef struct {
  int otype, metric;
  uint32_t nrows, dpad;
  const void *objects;
  const uint8_t *present;
  const uint32_t *offsets, *edges;
  int has_tree;
  uint32_t root, ninternals, nleaves;
  const uint32_t *in_pivot, *in_nchildren, *in_children; /* children: [ninternals][5] */
  const float *in_borders;                               /* [ninternals][4] */
  const void *pivots;
  const uint32_t *leaf_first, *leaf_count, *leaf_ids;
  int seed_size, seed_type, epsilon_type, edge_size_for_search, dyn_base, dyn_rate;
} OracleIndex;

/* ---------------- glibc rand() ---------------- */
typedef struct { int32_t s[31]; int f, r; } grand_t;

static int32_t grand_next(grand_t *g) {
  uint32_t v = (uint32_t)g->s[g->f] + (uint32_t)g->s[g->r];
  g->s[g->f] = (int32_t)v;
  if (++g->f == 31) g->f = 0;
  if (++g->r == 31) g->r = 0;
  return (int32_t)(v >> 1);
}

static void grand_seed(grand_t *g, uint32_t seed) {
  if (seed == 0) seed = 1;
  int64_t w = (int32_t)seed;
  g->s[0] = (int32_t)seed;
  for (int i = 1; i < 31; i++) {
    int64_t hi = w / 127773, lo = w % 127773;
    w = 16807 * lo - 2836 * hi;
    if (w < 0) w += 2147483647;
    g->s[i] = (int32_t)w;
  }
  g->f = 3;
  g->r = 0;
  for (int i = 0; i < 310; i++) grand_next(g);
}

void oracle_rand_sequence(uint32_t seed, size_t n, int32_t *out) {
  grand_t g;
  grand_seed(&g, seed);
  for (size_t i = 0; i < n; i++) out[i] = grand_next(&g);
}

/* ---------------- element access ---------------- */
static double half_to_double(uint16_t h) {
  uint32_t sign = (h >> 15) & 1, exp = (h >> 10) & 31, man = h & 1023;
  double v;
  if (exp == 0) v = ldexp((double)man, -24);
  else if (exp == 31) v = man ? NAN : INFINITY;
  else v = ldexp((double)(man | 1024), (int)exp - 25);
  return sign ? -v : v;
}

static inline double elem(const void *row, int ot, size_t i) {
  switch (ot) {
    case OT_FLOAT: return ((const float *)row)[i];
    case OT_UINT8: return ((const uint8_t *)row)[i];
    case OT_QSINT8: return ((const int8_t *)row)[i];
    default: return half_to_double(((const uint16_t *)row)[i]);
  }
}

static size_t elem_size(int ot) { return ot == OT_FLOAT ? 4 : (ot == OT_UINT8 || ot == OT_QSINT8) ? 1 : 2; }

/* ---------------- comparators ---------------- */
static float compare(int ot, int metric, const void *a, const void *b, size_t n) {
  if (ot == OT_QSINT8 && (metric == M_IP || metric == M_NCOSINE)) {
    /* the signed query codes against the stored codes shifted to unsigned (code + 127):
     * 127*127*n (inner product) or 127*255*n (normalized cosine) minus their integer dot
     * product over the n padded elements (PrimitiveComparator::InnerProductQsint8 and
     * NormalizedCosineSimilarityQsint8, lib/NGT/PrimitiveComparator.h:376-404) */
    int64_t s = 0;
    for (size_t i = 0; i < n; i++) s += (int64_t)((const int8_t *)a)[i] * (int64_t)((const uint8_t *)b)[i];
    double c = metric == M_IP ? 127.0 * 127.0 * (double)n : 127.0 * 255.0 * (double)n;
    return (float)(c - (double)s);
  }
  switch (metric) {
    case M_L2:
    case M_IP: {
      double d = 0.0;
      for (size_t i = 0; i < n; i++) {
        double x = elem(a, ot, i) - elem(b, ot, i);
        d += x * x;
      }
      if (ot == OT_QSINT8) return (float)d;     /* squared sum of the codes' differences */
      return (float)sqrt(d);
    }
    case M_L1: {
      double d = 0.0;
      for (size_t i = 0; i < n; i++) d += fabs(elem(a, ot, i) - elem(b, ot, i));
      return (float)d;
    }
    case M_HAMMING:
    case M_JACCARD: {
      const uint8_t *x = (const uint8_t *)a, *y = (const uint8_t *)b;
      size_t nb = n * elem_size(ot);
      uint64_t c = 0, u = 0;
      for (size_t i = 0; i < nb; i++) {
        if (metric == M_HAMMING) c += (uint64_t)__builtin_popcount((unsigned)(x[i] ^ y[i]));
        else {
          c += (uint64_t)__builtin_popcount((unsigned)(x[i] & y[i]));
          u += (uint64_t)__builtin_popcount((unsigned)(x[i] | y[i]));
        }
      }
      if (metric == M_HAMMING) return (float)(double)c;
      return (float)(1.0 - (double)c / (double)u);
    }
    case M_NCOSINE:
    case M_NANGLE:
    case M_NL2: {
      double s = 0.0;
      for (size_t i = 0; i < n; i++) s += (double)(float)elem(a, ot, i) * (double)(float)elem(b, ot, i);
      if (metric == M_NCOSINE) { double v = 1.0 - s; return (float)(v < 0.0 ? -v : v); }
      if (metric == M_NL2) { double v = 2.0 - 2.0 * s; return (float)(v < 0.0 ? 0.0 : sqrt(v)); }
      if (s >= 1.0) return 0.0f;
      if (s <= -1.0) return (float)acos(-1.0);
      return (float)acos(s);
    }
    case M_COSINE:
    case M_ANGLE: {
      double na = 0, nb = 0, s = 0;
      for (size_t i = 0; i < n; i++) {
        double x = elem(a, ot, i), y = elem(b, ot, i);
        na += x * x; nb += y * y; s += x * y;
      }
      double c = s / sqrt(na * nb);
      if (metric == M_COSINE) { double v = 1.0 - c; return (float)(v < 0.0 ? -v : v); }
      if (c >= 1.0) return 0.0f;
      if (c <= -1.0) return (float)acos(-1.0);
      return (float)acos(c);
    }
    case M_POINCARE: {
      double a2 = 0, b2 = 0, l2 = 0;
      for (size_t i = 0; i < n; i++) {
        double x = elem(a, ot, i), y = elem(b, ot, i);
        a2 += x * x; b2 += y * y; l2 += (x - y) * (x - y);
      }
      double c2 = sqrt(l2);
      return (float)acosh(1 + 2.0 * c2 * c2 / (1.0 - a2) / (1.0 - b2));
    }
    case M_LORENTZ: {
      double s = elem(a, ot, 0) * elem(b, ot, 0);
      for (size_t i = 1; i < n; i++) s -= elem(a, ot, i) * elem(b, ot, i);
      return (float)acosh(s);
    }
  }
  return NAN;
}

float oracle_distance(int ot, int metric, const void *a, const void *b, size_t n) {
  return compare(ot, metric, a, b, n);
}

static const void *row_ptr(const OracleIndex *ix, const void *base, size_t r) {
  return (const uint8_t *)base + r * (size_t)ix->dpad * elem_size(ix->otype);
}

/* ---------------- (distance, id) order and heaps ---------------- */
typedef struct { uint32_t id; float d; } od_t;

static inline int od_less(od_t a, od_t b) { return a.d == b.d ? a.id < b.id : a.d < b.d; }

/* max-heap (ResultSet) */
static void maxheap_push(od_t *h, size_t *n, od_t x) {
  size_t i = (*n)++;
  h[i] = x;
  while (i > 0) {
    size_t p = (i - 1) / 2;
    if (!od_less(h[p], h[i])) break;
    od_t t = h[p]; h[p] = h[i]; h[i] = t;
    i = p;
  }
}
static void maxheap_siftdown(od_t *h, size_t n, size_t i) {
  for (;;) {
    size_t l = 2 * i + 1, r = l + 1, m = i;
    if (l < n && od_less(h[m], h[l])) m = l;
    if (r < n && od_less(h[m], h[r])) m = r;
    if (m == i) break;
    od_t t = h[m]; h[m] = h[i]; h[i] = t;
    i = m;
  }
}
static void maxheap_pop(od_t *h, size_t *n) {
  h[0] = h[--(*n)];
  maxheap_siftdown(h, *n, 0);
}
/* push_pop as the reference executes it on Linux: the new element replaces the
 * current top, whatever their order (pop_heap without the preceding push_heap). */
static void maxheap_replace_top(od_t *h, size_t n, od_t x) {
  h[0] = x;
  maxheap_siftdown(h, n, 0);
}

/* min-heap (UncheckedSet) with growth */
typedef struct { od_t *a; size_t n, cap; } minheap_t;
static void minheap_push(minheap_t *m, od_t x) {
  if (m->n == m->cap) {
    m->cap = m->cap ? m->cap * 2 : 256;
    m->a = (od_t *)realloc(m->a, m->cap * sizeof(od_t));
  }
  size_t i = m->n++;
  m->a[i] = x;
  while (i > 0) {
    size_t p = (i - 1) / 2;
    if (!od_less(m->a[i], m->a[p])) break;
    od_t t = m->a[p]; m->a[p] = m->a[i]; m->a[i] = t;
    i = p;
  }
}
static od_t minheap_pop(minheap_t *m) {
  od_t top = m->a[0];
  m->a[0] = m->a[--m->n];
  size_t i = 0;
  for (;;) {
    size_t l = 2 * i + 1, r = l + 1, s = i;
    if (l < m->n && od_less(m->a[l], m->a[s])) s = l;
    if (r < m->n && od_less(m->a[r], m->a[s])) s = r;
    if (s == i) break;
    od_t t = m->a[s]; m->a[s] = m->a[i]; m->a[i] = t;
    i = s;
  }
  return top;
}

static int od_cmp(const void *x, const void *y) {
  od_t a = *(const od_t *)x, b = *(const od_t *)y;
  return od_less(a, b) ? -1 : od_less(b, a) ? 1 : 0;
}

/* heap -> ascending array (ObjectDistances::moveFrom) */
static size_t heap_to_sorted(od_t *h, size_t n, uint32_t *ids, float *ds) {
  qsort(h, n, sizeof(od_t), od_cmp);
  for (size_t i = 0; i < n; i++) { ids[i] = h[i].id; ds[i] = h[i].d; }
  return n;
}

/* ---------------- linear search ---------------- */
static size_t linear_one(const OracleIndex *ix, const void *q, size_t k, uint32_t *ids, float *ds) {
  od_t *h = (od_t *)malloc((k + 1) * sizeof(od_t));
  size_t n = 0;
  for (uint32_t r = 1; r < ix->nrows; r++) {
    if (!ix->present[r]) continue;
    float d = compare(ix->otype, ix->metric, q, row_ptr(ix, ix->objects, r), ix->dpad);
    od_t x = {r, d};
    maxheap_push(h, &n, x);
    if (n > k) maxheap_pop(h, &n);
  }
  size_t m = heap_to_sorted(h, n, ids, ds);
  free(h);
  return m;
}

void oracle_linear_search(const OracleIndex *ix, const void *qrows, size_t nq, size_t k, uint32_t *out_ids,
                          float *out_d, uint32_t *out_n, int nthreads) {
  size_t rb = (size_t)ix->dpad * elem_size(ix->otype);
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
  for (long q = 0; q < (long)nq; q++) {
    out_n[q] = k ? (uint32_t)linear_one(ix, (const uint8_t *)qrows + q * rb, k, out_ids + q * k, out_d + q * k) : 0;
  }
}

/* ---------------- seeds ---------------- */
/* The tree's comparator (ObjectSpace::getComparator, lib/NGT/Tree.cpp:403-491): the
 * search comparator, except for scalar-quantized inner-product and normalized-cosine
 * indexes, whose comparator is the squared L2 over unsigned bytes (ComparatorL2Quint8Quint8,
 * lib/NGT/ObjectSpaceRepository.h:514-533, 727-745), the query's signed codes read as
 * unsigned. */
static float tree_compare(const OracleIndex *ix, const void *q, const void *pivot) {
  if (ix->otype == OT_QSINT8 && (ix->metric == M_IP || ix->metric == M_NCOSINE)) {
    int64_t s = 0;
    for (size_t i = 0; i < ix->dpad; i++) {
      int64_t x = (int64_t)((const uint8_t *)q)[i] - (int64_t)((const uint8_t *)pivot)[i];
      s += x * x;
    }
    return (float)(double)s;
  }
  return compare(ix->otype, ix->metric, q, pivot, ix->dpad);
}

static size_t tree_seeds(const OracleIndex *ix, const void *q, size_t size, uint32_t *seeds, uint32_t *ndc) {
  uint32_t node = ix->root;
  while (!(node & 0x80000000u)) {
    float d = tree_compare(ix, q, row_ptr(ix, ix->pivots, ix->in_pivot[node]));
    (*ndc)++;
    uint32_t bsize = ix->in_nchildren[node] - 1, mid;
    for (mid = 0; mid < bsize; mid++)
      if (d < ix->in_borders[(size_t)node * 4 + mid]) break;
    node = ix->in_children[(size_t)node * 5 + mid];
  }
  uint32_t leaf = node & 0x7fffffffu;
  size_t cnt = ix->leaf_count[leaf];
  for (size_t i = 0; i < cnt; i++) seeds[i] = ix->leaf_ids[ix->leaf_first[leaf] + i];
  if (ix->seed_type == 4) return cnt; /* AllLeafNodes */
  size_t seed_size = ix->seed_size == 0 ? size : (size_t)ix->seed_size;
  if (seed_size > size) seed_size = size;
  if (cnt > seed_size) {
    grand_t g;
    grand_seed(&g, leaf);
    for (size_t i = cnt; i > seed_size; i--) {
      double random = ((double)grand_next(&g) + 1.0) / ((double)2147483647 + 2.0);
      size_t idx = (size_t)floor((double)i * random);
      seeds[idx] = seeds[i - 1];
    }
    cnt = seed_size;
  }
  return cnt;
}

/* GraphIndex::getSeedsFromGraph / getRandomSeeds (lib/NGT/Index.h:1270-1302,1658-1679),
 * with the generator freshly seeded with 1 for every query. */
static size_t graph_seeds(const OracleIndex *ix, uint32_t *seeds) {
  size_t n = ix->nrows ? ix->nrows - 1 : 0;
  size_t ss = (size_t)ix->seed_size < n ? (size_t)ix->seed_size : n;
  size_t cnt = 0;
  if (ix->seed_type == 2) {
    for (size_t i = 1; i <= ss; i++) seeds[cnt++] = (uint32_t)i;
    return cnt;
  }
  if (ix->seed_type == 3) { seeds[0] = 1; return 1; }
  grand_t g;
  grand_seed(&g, 1);
  size_t empty = 0;
  while (cnt < ss) {
    double r = ((double)grand_next(&g) + 1.0) / ((double)2147483647 + 2.0);
    size_t idx = (size_t)floor((double)n * r) + 1;
    if (!ix->present[idx]) { if (++empty > n) break; continue; }
    int dup = 0;
    for (size_t i = 0; i < cnt; i++) dup |= seeds[i] == idx;
    if (dup) continue;
    seeds[cnt++] = (uint32_t)idx;
  }
  return cnt;
}

static size_t edge_size_for(const OracleIndex *ix, int64_t edge_size, float coef) {
  int64_t e = edge_size == -1 ? ix->edge_size_for_search : edge_size;
  if (e == 0) return INT_MAX;
  if (e > 0) return (size_t)e;
  double add = pow(10, ((double)coef - 1.0) * (double)(float)ix->dyn_rate);
  return add >= (double)INT_MAX ? (size_t)INT_MAX : (size_t)(ix->dyn_base + add);
}

/* ---------------- graph search ---------------- */
static size_t graph_one(const OracleIndex *ix, const void *q, size_t k, size_t kout, float epsilon, float radius0,
                        int64_t edge_size, int mode, uint32_t *ids, float *ds, uint32_t *dc_out,
                        const uint32_t *given_seeds, size_t ngiven) {
  float coef = epsilon + 1.0f;
  if (coef == 0.0f) coef = 1.1f;
  size_t size = k, size_backup = 0;
  /* EpsilonType ResultSize, and the updatable search over quantized objects with
   * EpsilonType None (lib/NGT/Graph.cpp:845-852) */
  if (ix->epsilon_type == 2 || (mode != 0 && ix->epsilon_type == 0 && ix->otype == OT_QSINT8)) {
    size_backup = k;
    size = (size_t)roundf(coef * (float)k);
  }
  float radius = radius0 < 0.0f ? FLT_MAX : radius0;
  size_t esz = edge_size_for(ix, edge_size, coef);
  float expcoef = size_backup ? 1.0f : coef;
  uint32_t dc = 0;
  uint32_t *seeds = (uint32_t *)malloc(sizeof(uint32_t) * (65536 + ngiven));
  size_t ns;
  if (ix->has_tree) ns = tree_seeds(ix, q, size, seeds, &dc), dc = 0;
  else if (given_seeds) { memcpy(seeds, given_seeds, ngiven * sizeof(uint32_t)); ns = ngiven; }
  else ns = graph_seeds(ix, seeds);
  if (k == 0 || ns == 0) { free(seeds); *dc_out = 0; return 0; }
  od_t *sd = (od_t *)malloc(ns * sizeof(od_t));
  for (size_t i = 0; i < ns; i++) {
    sd[i].id = seeds[i];
    sd[i].d = compare(ix->otype, ix->metric, q, row_ptr(ix, ix->objects, seeds[i]), ix->dpad);
  }
  dc += (uint32_t)ns;
  qsort(sd, ns, sizeof(od_t), od_cmp);
  od_t *res = (od_t *)malloc((size + 2) * sizeof(od_t));
  size_t nres = 0;
  for (size_t i = 0; i < ns; i++) {
    if (nres < size && sd[i].d <= radius) maxheap_push(res, &nres, sd[i]);
    else break;
  }
  if (nres >= size) radius = res[0].d;
  uint64_t *visited = (uint64_t *)calloc((ix->nrows + 63) / 64, 8);   /* vector<bool> */
  minheap_t cand = {0, 0, 0};
  for (size_t i = 0; i < ns; i++) {
    visited[sd[i].id >> 6] |= 1ull << (sd[i].id & 63);
    minheap_push(&cand, sd[i]);
  }
  float expR = expcoef * radius;
  while (cand.n) {
    od_t t = minheap_pop(&cand);
    if (t.d > expR) break;
    uint32_t e0 = ix->offsets[t.id], deg = ix->offsets[t.id + 1] - e0;
    size_t nsz = deg < esz ? deg : esz;
    for (size_t j = 0; j < nsz; j++) {
      uint32_t v = ix->edges[e0 + j];
      if (visited[v >> 6] & (1ull << (v & 63))) continue;
      visited[v >> 6] |= 1ull << (v & 63);
      float d = compare(ix->otype, ix->metric, q, row_ptr(ix, ix->objects, v), ix->dpad);
      dc++;
      if (d <= expR) {
        od_t x = {v, d};
        minheap_push(&cand, x);
        if (d <= radius) {
          if (mode == 0) {          /* read-only: push_pop when full */
            if (nres >= size) {
              maxheap_replace_top(res, nres, x);
              radius = res[0].d;
              expR = expcoef * radius;
            } else {
              maxheap_push(res, &nres, x);
            }
          } else {                  /* updatable: push, pop when over, radius = top */
            maxheap_push(res, &nres, x);
            if (nres >= size) {
              if (res[0].d >= d) {
                if (nres > size) maxheap_pop(res, &nres);
                radius = res[0].d;
                expR = expcoef * radius;
              }
            }
          }
        }
      }
    }
  }
  /* Only the read-only search cuts the expanded result set back to sizeBackup
   * (lib/NGT/Graph.cpp:821-828); the updatable search returns it as is. */
  if (size_backup && mode == 0) while (nres > size_backup) maxheap_pop(res, &nres);
  qsort(res, nres, sizeof(od_t), od_cmp);
  size_t n = nres;
  for (size_t i = 0; i < n && i < kout; i++) { ids[i] = res[i].id; ds[i] = res[i].d; }
  free(res); free(sd); free(seeds); free(visited); free(cand.a);
  *dc_out = dc;
  return n;
}

/* out arrays are nq x kout (kout >= the largest result count).  seed_list/seed_off/seed_cnt are used for graph-only indexes. */
void oracle_graph_search(const OracleIndex *ix, const void *qrows, size_t nq, size_t k, size_t kout, float epsilon,
                         float radius, int64_t edge_size, int mode, uint32_t *out_ids, float *out_d, uint32_t *out_n,
                         uint32_t *out_dc, const uint32_t *seed_list, const uint32_t *seed_off,
                         const uint32_t *seed_cnt, int nthreads) {
  size_t rb = (size_t)ix->dpad * elem_size(ix->otype);
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
  for (long q = 0; q < (long)nq; q++) {
    const uint32_t *gs = seed_list ? seed_list + seed_off[q] : NULL;
    size_t ng = seed_list ? seed_cnt[q] : 0;
    uint32_t dc = 0;
    out_n[q] = (uint32_t)graph_one(ix, (const uint8_t *)qrows + q * rb, k, kout, epsilon, radius, edge_size, mode,
                                   out_ids + q * kout, out_d + q * kout, &dc, gs, ng);
    if (out_dc) out_dc[q] = dc;
  }
}

/* float -> IEEE half, round to nearest even (half.hpp's default rounding). */
static uint16_t float_to_half(float f) {
  uint32_t x;
  memcpy(&x, &f, 4);
  uint32_t sign = (x >> 16) & 0x8000u;
  int32_t exp = (int32_t)((x >> 23) & 0xff) - 127 + 15;
  uint32_t man = x & 0x7fffffu;
  if (((x >> 23) & 0xff) == 0xff) return (uint16_t)(sign | 0x7c00u | (man ? 0x200u : 0));
  if (exp >= 31) return (uint16_t)(sign | 0x7c00u);
  if (exp <= 0) {
    if (exp < -10) return (uint16_t)sign;
    man |= 0x800000u;
    uint32_t shift = (uint32_t)(14 - exp);
    uint32_t h = man >> shift, rem = man & ((1u << shift) - 1), half = 1u << (shift - 1);
    if (rem > half || (rem == half && (h & 1u))) h++;
    return (uint16_t)(sign | h);
  }
  uint32_t h = ((uint32_t)exp << 10) | (man >> 13), rem = man & 0x1fffu;
  if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
  return (uint16_t)(sign | h);
}

/* Query conversion: cast to the object type, normalise (float sum, sqrt,
 * divide, in the object type) for the normalised metrics. */
/* qsint8 query codes: round(v / scale x 127.5) clamped to [-127, 127], the division in
 * float and the product and rounding in double (lib/NGT/ObjectSpace.h:432-441); under a
 * normalized distance the float query is normalized first (ObjectSpaceRepository::
 * allocateNormalizedObject, lib/NGT/ObjectSpaceRepository.h:1120-1160). */
void oracle_prepare_qsint8(uint32_t dpad, const float *q, size_t nq, size_t dim, float scale, int normalize,
                           int8_t *rows) {
  memset(rows, 0, nq * dpad);
  for (size_t i = 0; i < nq; i++) {
    float s = 1.0f;
    if (normalize) {
      volatile float sum = 0.0f;
      for (size_t j = 0; j < dim; j++) { float p = q[i * dim + j] * q[i * dim + j]; sum = sum + p; }
      s = (float)sqrt((double)sum);
    }
    for (size_t j = 0; j < dim; j++) {
      float fv = normalize ? q[i * dim + j] / s : q[i * dim + j];
      fv = (float)round((double)(fv / scale) * 127.5);
      fv = fv < -127.0f ? -127.0f : fv;
      fv = fv > 127.0f ? 127.0f : fv;
      rows[i * dpad + j] = (int8_t)fv;
    }
  }
}

void oracle_prepare_queries(int ot, int metric, uint32_t dpad, const float *q, size_t nq, size_t dim, void *rows) {
  size_t rb = (size_t)dpad * elem_size(ot);
  memset(rows, 0, nq * rb);
  int norm = metric == M_NCOSINE || metric == M_NANGLE || metric == M_NL2;
  for (size_t i = 0; i < nq; i++) {
    uint8_t *dst = (uint8_t *)rows + i * rb;
    const float *src = q + i * dim;
    if (ot == OT_FLOAT) {
      float *o = (float *)dst;
      for (size_t j = 0; j < dim; j++) o[j] = src[j];
      if (norm) {
        volatile float sum = 0.0f;
        for (size_t j = 0; j < dim; j++) { float p = o[j] * o[j]; sum = sum + p; }
        float s = (float)sqrt((double)sum);
        for (size_t j = 0; j < dim; j++) o[j] = o[j] / s;
      }
    } else if (ot == OT_UINT8) {
      for (size_t j = 0; j < dim; j++) dst[j] = (uint8_t)(int)src[j];
    } else {
      uint16_t *o = (uint16_t *)dst;
      for (size_t j = 0; j < dim; j++) o[j] = float_to_half(src[j]);
    }
  }
}

/* Parses the body of an NGT graph file (Repository<GraphNode>: '+'/'-' markers,
 * uint32 counts, (uint32 id, float distance) pairs).  With edges == NULL only
 * the edge total is returned; otherwise offsets[nrows+1] and edges are filled.
 * Returns -1 on a malformed buffer. */
int64_t oracle_parse_graph(const uint8_t *buf, size_t len, size_t nrows, uint32_t *offsets, uint32_t *edges) {
  if (len < 8) return -1;
  uint64_t n;
  memcpy(&n, buf, 8);
  size_t pos = 8;
  int64_t total = 0;
  for (uint64_t i = 0; i < n; i++) {
    if (pos >= len) return -1;
    uint8_t t = buf[pos++];
    if (offsets && i < nrows) offsets[i] = (uint32_t)total;
    if (t == '-') continue;
    if (t != '+' || pos + 4 > len) return -1;
    uint32_t cnt;
    memcpy(&cnt, buf + pos, 4);
    pos += 4;
    if (pos + (size_t)cnt * 8 > len) return -1;
    if (edges)
      for (uint32_t e = 0; e < cnt; e++) memcpy(&edges[total + e], buf + pos + (size_t)e * 8, 4);
    pos += (size_t)cnt * 8;
    total += cnt;
  }
  if (offsets)
    for (uint64_t i = n; i <= nrows; i++) offsets[i] = (uint32_t)total;
  return total;
}

/* ---------------- quantized graph (QG) ----------------
 * NGTQG::Index::searchQuantizedGraph (lib/NGT/NGTQ/QuantizedGraph.h:283-447) over the
 * quantized graph written by `qbg build-qg`: every node stores its first <= E graph
 * edges and the 4-bit codes of those neighbours (QuantizedGraphRepository,
 * lib/NGT/NGTQ/QuantizedGraph.h:67-257). */
typedef struct {
  uint32_t dim;              /* quantizer dimension (queries are zero-padded to it) */
  uint32_t m;                /* subspaces (LocalDivisionNo), one codebook each */
  uint32_t ld;               /* dimensions per subspace */
  uint32_t ma;               /* m rounded up to even: subspaces per code block */
  const float *rotation;     /* dim x dim, element [p * dim + c]; NULL = none */
  const float *gcentroid;    /* dim (the single global centroid) */
  const float *lcentroids;   /* [m][16][ld] */
  uint32_t nnodes;
  const uint32_t *offsets;   /* nnodes + 1 */
  const uint32_t *ids;       /* neighbour ids */
  const uint64_t *code_off;  /* byte offset of each node's code stream in codes */
  const uint8_t *codes;
  const uint32_t *sid;       /* QBG: per blob, the codebook centroid of its LUT (NULL: centroid 0) */
  const void *olist;         /* QBG: the object list (qbg_dir/obj), rows of olist_dim; row 0 unused */
  uint32_t olist_dim;
  int olist_type;            /* OT_UINT8 or OT_FLOAT */
  uint32_t olist_n;          /* rows including row 0 */
} OracleQG;

/* Rotation::mul (lib/NGT/NGTQ/Quantizer.h:117-160), y[c] = sum_p R[p][c] x[p].  The
 * reference hands it to BLAS sgemv('N'); the summation order here is the one the x86-64
 * OpenBLAS build the reference links uses: one FMA chain over p for dimensions <= 48,
 * else blocks of 8 columns (first product, then FMAs, the block total added to y[c]).
 * It equals that sgemv bit for bit at every multiple of 16 from 16 to 768, with one
 * thread or eight (tests/test_oracle_rotation.py), and QG/QBG pseudo-dimensions are
 * always multiples of 16 (lib/NGT/NGTQ/QuantizedGraph.h:640-657). */
void oracle_rotate(const float *R, const float *x, float *y, size_t d) {
  for (size_t c = 0; c < d; c++) {
    float acc = 0.0f;
    if (d <= 48) {
      for (size_t p = 0; p < d; p++) acc = fmaf(R[p * d + c], x[p], acc);
    } else {
      for (size_t p0 = 0; p0 < d; p0 += 8) {
        size_t p1 = p0 + 8 < d ? p0 + 8 : d;
        float t = R[p0 * d + c] * x[p0];
        for (size_t p = p0 + 1; p < p1; p++) t = fmaf(R[p * d + c], x[p], t);
        acc = acc + t;
      }
    }
    y[c] = acc;
  }
}

void oracle_qg_rotate(const OracleQG *qg, const float *x, float *y) {
  if (!qg->rotation) { memcpy(y, x, qg->dim * sizeof(float)); return; }
  oracle_rotate(qg->rotation, x, y, qg->dim);
}

/* createFloatL2DistanceLookup for the uint8 table (lib/NGT/NGTQ/Quantizer.h:1731-1810,
 * NGTQ_TOTAL_SCALE_OFFSET_COMPRESSION): squared L2 of the rotated query's subvector (minus
 * the global centroid) to each of the 16 local centroids, summed in float (first term a
 * product, then FMAs: the contraction of the reference's mul + add); one offset (the
 * table's minimum) and one scale ((max - min) / 255.0) for the whole table; entries
 * (v - offset) / scale rounded to nearest even. */
static void qg_lut_centroid(const OracleQG *qg, const float *rq, const float *gc, uint8_t *lut, float *scale_out,
                            float *offset_out);

void oracle_qg_lut(const OracleQG *qg, const float *rq, uint8_t *lut, float *scale_out, float *offset_out) {
  qg_lut_centroid(qg, rq, qg->gcentroid, lut, scale_out, offset_out);
}

static void qg_lut_centroid(const OracleQG *qg, const float *rq, const float *gc, uint8_t *lut, float *scale_out,
                            float *offset_out) {
  size_t m = qg->m, ld = qg->ld;
  float *fl = (float *)malloc(m * 16 * sizeof(float));
  float mn = FLT_MAX, mx = -FLT_MAX;
  for (size_t s = 0; s < m; s++) {
    for (size_t c = 0; c < 16; c++) {
      float v = 0.0f;
      for (size_t d = 0; d < ld; d++) {
        float rsv = rq[s * ld + d] - gc[s * ld + d];
        float sub = rsv - qg->lcentroids[(s * 16 + c) * ld + d];
        v = d == 0 ? sub * sub : fmaf(sub, sub, v);
      }
      fl[s * 16 + c] = v;
      if (v < mn) mn = v;
      if (v > mx) mx = v;
    }
  }
  float scale = (float)((double)(mx - mn) / 255.0);
  for (size_t i = 0; i < m * 16; i++) lut[i] = (uint8_t)(int32_t)nearbyintf((fl[i] - mn) / scale);
  *scale_out = scale;
  *offset_out = mn * (float)m;
  free(fl);
}

/* The 4-bit scan of one node's neighbours (lib/NGT/NGTQ/Quantizer.h:2331-2440): neighbour
 * o of block o / 16 has its code for subspace s in byte (o / 16) * 8 * ma + 8 * s + (o % 16) / 2,
 * low nibble for even o (QuantizedObjectProcessingStream, lib/NGT/NGTQ/Quantizer.h:1040-1120).
 * Even and odd subspaces sum in separate saturating 16-bit lanes; the distance is
 * sqrt(sum * scale + offset) with the multiply-add fused. */
float oracle_qg_scan(const OracleQG *qg, const uint8_t *lut, float scale, float offset, uint32_t node, float *ds) {
  uint32_t a = qg->offsets[node], n = qg->offsets[node + 1] - a;
  const uint8_t *st = qg->codes + qg->code_off[node];
  for (uint32_t o = 0; o < n; o++) {
    const uint8_t *blk = st + (size_t)(o / 16) * 8 * qg->ma;
    uint32_t oo = o % 16, se = 0, so = 0;
    for (uint32_t s = 0; s < qg->m; s++) {
      uint8_t b = blk[8 * s + oo / 2];
      uint32_t code = (oo & 1) ? (uint32_t)(b >> 4) : (uint32_t)(b & 15);
      if (s & 1) so += lut[s * 16 + code]; else se += lut[s * 16 + code];
    }
    if (se > 65535) se = 65535;
    if (so > 65535) so = 65535;
    ds[o] = sqrtf(fmaf((float)(se + so), scale, offset));
  }
  float mn = FLT_MAX;                 /* the scan's minimum (NGTQBG_MIN) */
  for (uint32_t o = 0; o < n; o++) mn = ds[o] < mn ? ds[o] : mn;
  return mn;
}

static size_t qg_one(const OracleIndex *ix, const OracleQG *qg, const float *qf, size_t qdim, const void *q,
                     size_t k, float epsilon, float expansion, float radius0, uint32_t *ids, float *ds,
                     uint32_t *dc_out, const uint32_t *given_seeds, size_t ngiven) {
  *dc_out = 0;
  if (k == 0) return 0;
  float coef = epsilon + 1.0f;
  if (coef == 0.0f) coef = 1.1f;                     /* NGT_EXPLORATION_COEFFICIENT */
  float radius = radius0 < 0.0f ? FLT_MAX : radius0;
  const float specified = radius;
  size_t size = k;
  if (expansion > 1.0f) size = (size_t)((float)k * expansion);
  /* seeds: the tree leaf of the query (getSeedsFromTree, thinned to k), else graph seeds */
  uint32_t *seeds = (uint32_t *)malloc(sizeof(uint32_t) * (65536 + ngiven));
  uint32_t tdc = 0;
  size_t ns = 0;
  if (ix->has_tree) ns = tree_seeds(ix, q, k, seeds, &tdc);
  if (ns == 0) {
    if (given_seeds) { memcpy(seeds, given_seeds, ngiven * sizeof(uint32_t)); ns = ngiven; }
    else ns = graph_seeds(ix, seeds);
  }
  /* the lookup table of the rotated query */
  float *rq = (float *)calloc(qg->dim > qdim ? qg->dim : qdim, sizeof(float));
  memcpy(rq, qf, qdim * sizeof(float));
  float *rot = (float *)malloc(qg->dim * sizeof(float));
  oracle_qg_rotate(qg, rq, rot);
  uint8_t *lut = (uint8_t *)malloc((size_t)qg->m * 16);
  float scale, offset;
  oracle_qg_lut(qg, rot, lut, &scale, &offset);
  /* setupDistances with L2Float::compare, setupSeeds (lib/NGT/Graph.cpp:533-558) */
  od_t *sd = (od_t *)malloc((ns + 1) * sizeof(od_t));
  for (size_t i = 0; i < ns; i++) {
    sd[i].id = seeds[i];
    sd[i].d = compare(ix->otype, ix->metric, q, row_ptr(ix, ix->objects, seeds[i]), ix->dpad);
  }
  qsort(sd, ns, sizeof(od_t), od_cmp);
  od_t *res = (od_t *)malloc((size + 2) * sizeof(od_t));
  size_t nres = 0;
  for (size_t i = 0; i < ns; i++) {
    if (nres < size && sd[i].d <= radius) maxheap_push(res, &nres, sd[i]);
    else break;
  }
  if (nres >= size && nres > 0) radius = res[0].d;
  uint64_t *visited = (uint64_t *)calloc((ix->nrows + 63) / 64 + 1, 8);
  minheap_t cand = {0, 0, 0};
  for (size_t i = 0; i < ns; i++) {
    visited[sd[i].id >> 6] |= 1ull << (sd[i].id & 63);
    minheap_push(&cand, sd[i]);
  }
  float expR = coef * radius;
  float *qd = (float *)malloc(sizeof(float) * 65536);
  uint32_t dc = 0;
  while (cand.n) {
    od_t t = minheap_pop(&cand);
    if (t.d > expR) break;
    if (t.id >= qg->nnodes) continue;
    uint32_t a = qg->offsets[t.id], n = qg->offsets[t.id + 1] - a;
    oracle_qg_scan(qg, lut, scale, offset, t.id, qd);
    dc += n;
    for (uint32_t j = 0; j < n; j++) {
      float d = qd[j];
      uint32_t v = qg->ids[a + j];
      if (d <= expR) {
        if (visited[v >> 6] & (1ull << (v & 63))) continue;
        visited[v >> 6] |= 1ull << (v & 63);
        od_t x = {v, d};
        minheap_push(&cand, x);
        if (d <= radius) {
          maxheap_push(res, &nres, x);
          if (nres >= size) {
            if (nres > size) maxheap_pop(res, &nres);
            radius = res[0].d;
            expR = coef * radius;
          }
        }
      }
    }
  }
  qsort(res, nres, sizeof(od_t), od_cmp);
  if (expansion >= 1.0f) {
    /* exact re-rank, then the radius cut (upper_bound at (0, radius): d < radius) and k */
    for (size_t i = 0; i < nres; i++)
      res[i].d = compare(ix->otype, ix->metric, q, row_ptr(ix, ix->objects, res[i].id), ix->dpad);
    qsort(res, nres, sizeof(od_t), od_cmp);
    if (specified < FLT_MAX) {
      size_t keep = 0;
      while (keep < nres && res[keep].d < specified) keep++;
      nres = keep;
    }
    if (nres > k) nres = k;
  }
  for (size_t i = 0; i < nres; i++) { ids[i] = res[i].id; ds[i] = res[i].d; }
  free(qd); free(visited); free(cand.a); free(res); free(sd); free(lut); free(rot); free(rq); free(seeds);
  *dc_out = dc;
  return nres;
}

/* qf: nq x qdim float queries (as given); qrows: the same prepared as index rows.
 * Out arrays are nq x k (a QG search returns at most k results). */
void oracle_qg_search(const OracleIndex *ix, const OracleQG *qg, const float *qf, size_t qdim, const void *qrows,
                      size_t nq, size_t k, float epsilon, float expansion, float radius, uint32_t *out_ids,
                      float *out_d, uint32_t *out_n, uint32_t *out_dc, const uint32_t *seed_list,
                      const uint32_t *seed_off, const uint32_t *seed_cnt, int nthreads) {
  size_t rb = (size_t)ix->dpad * elem_size(ix->otype);
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
  for (long q = 0; q < (long)nq; q++) {
    const uint32_t *gs = seed_list ? seed_list + seed_off[q] : NULL;
    size_t ng = seed_list ? seed_cnt[q] : 0;
    uint32_t dc = 0;
    out_n[q] = (uint32_t)qg_one(ix, qg, qf + q * qdim, qdim, (const uint8_t *)qrows + q * rb, k, epsilon,
                                expansion, radius, out_ids + q * k, out_d + q * k, &dc, gs, ng);
    if (out_dc) out_dc[q] = dc;
  }
}

/* ---------------- quantized blob graph (QBG) ----------------
 * QBG::Index::searchInOneStep (lib/NGT/NGTQ/QuantizedBlobGraph.h:1332-1594) as the C API
 * (qbg_search_index_, lib/NGT/NGTQ/Capi.cpp:549-574) drives it: the result size is
 * number_of_results x result_expansion (>= 1), no refinement (the C API leaves
 * refinementExpansion at 0), so the distances returned are the quantized ones.
 * ix is the global index (blob centroids, their graph and tree); qg the blobs. */
static size_t qbg_one(const OracleIndex *ix, const OracleQG *qg, const float *qf, size_t qdim, const void *q,
                      size_t size, size_t seed_size, float epsilon, float blob_epsilon, size_t explored,
                      int64_t edge_size, uint32_t *ids, float *ds, uint32_t *blobs_out) {
  *blobs_out = 0;
  if (size == 0) return 0;
  float coef = epsilon + 1.0f;
  if (coef == 0.0f) coef = 1.1f;
  float bcoef = blob_epsilon + 1.0f;
  size_t esz = edge_size_for(ix, edge_size, coef);
  /* seeds: getSeedsFromTree over the global graph with the container's size (the result
   * size before a refinement expansion, QuantizedBlobGraph.h:1336-1345), else 20 random */
  uint32_t *seeds = (uint32_t *)malloc(sizeof(uint32_t) * 65536);
  uint32_t tdc = 0;
  size_t ns = 0;
  if (ix->has_tree) ns = tree_seeds(ix, q, seed_size, seeds, &tdc);
  if (ns == 0) {
    OracleIndex tmp = *ix;
    tmp.seed_size = 20;
    tmp.seed_type = 1;
    ns = graph_seeds(&tmp, seeds);
  }
  od_t *sd = (od_t *)malloc((ns + 1) * sizeof(od_t));
  for (size_t i = 0; i < ns; i++) {
    sd[i].id = seeds[i];
    sd[i].d = compare(ix->otype, ix->metric, q, row_ptr(ix, ix->objects, seeds[i]), ix->dpad);
  }
  qsort(sd, ns, sizeof(od_t), od_cmp);
  uint64_t *checked = (uint64_t *)calloc((ix->nrows + 63) / 64 + 1, 8);
  minheap_t untraced = {0, 0, 0}, discarded = {0, 0, 0};
  od_t current = sd[0];
  float expR = bcoef * current.d;
  for (size_t i = 0; i < ns; i++) {
    minheap_push(&untraced, sd[i]);
    checked[sd[i].id >> 6] |= 1ull << (sd[i].id & 63);
    if (i > 0) minheap_push(&discarded, sd[i]);
  }
  /* rotated query (the query zero-padded to the quantizer dimension) */
  float *rq = (float *)calloc(qg->dim > qdim ? qg->dim : qdim, sizeof(float));
  memcpy(rq, qf, qdim * sizeof(float));
  float *rot = (float *)malloc(qg->dim * sizeof(float));
  oracle_qg_rotate(qg, rq, rot);
  uint8_t *lut = (uint8_t *)malloc((size_t)qg->m * 16);
  float *bd = (float *)malloc(sizeof(float) * 65536);
  od_t *res = (od_t *)malloc((size + 2) * sizeof(od_t));
  size_t nres = 0;
  float radius = FLT_MAX;
  size_t exploration = 1;
  uint32_t nblobs = 0;
  for (;;) {
    if (untraced.n == 0 || untraced.a[0].d > expR) {
      exploration++;
      /* judge the current blob (lib/NGT/NGTQ/QuantizedBlobGraph.h:1033-1080) */
      uint32_t blob = current.id;
      float bmin = FLT_MAX;
      if (blob < qg->nnodes) {
        uint32_t a = qg->offsets[blob], n = qg->offsets[blob + 1] - a;
        float scale, offset;
        uint32_t c = qg->sid ? qg->sid[blob] : 0;
        qg_lut_centroid(qg, rot, qg->gcentroid + (size_t)c * qg->dim, lut, &scale, &offset);
        bmin = n ? oracle_qg_scan(qg, lut, scale, offset, blob, bd) : FLT_MAX;
        nblobs++;
        if (bmin < radius) {
          for (uint32_t i = 0; i < n; i++) {
            if (bd[i] <= radius) {
              od_t x = {qg->ids[a + i], bd[i]};
              maxheap_push(res, &nres, x);
              if (nres > size) maxheap_pop(res, &nres);
            }
          }
          if (nres >= size) radius = res[0].d;
        }
      }
      if (bmin > radius * coef) break;
      if (exploration > explored) break;
      if (discarded.n == 0) break;
      current = minheap_pop(&discarded);
      expR = bcoef * current.d;
      continue;
    }
    od_t t = minheap_pop(&untraced);
    uint32_t e0 = ix->offsets[t.id], deg = ix->offsets[t.id + 1] - e0;
    size_t nsz = deg < esz ? deg : esz;
    for (size_t j = 0; j < nsz; j++) {
      uint32_t v = ix->edges[e0 + j];
      if (checked[v >> 6] & (1ull << (v & 63))) continue;
      checked[v >> 6] |= 1ull << (v & 63);
      od_t r = {v, compare(ix->otype, ix->metric, q, row_ptr(ix, ix->objects, v), ix->dpad)};
      minheap_push(&untraced, r);
      if (r.d < current.d) {
        minheap_push(&discarded, current);
        current = r;
        expR = bcoef * current.d;
      } else {
        minheap_push(&discarded, r);
      }
    }
  }
  qsort(res, nres, sizeof(od_t), od_cmp);
  for (size_t i = 0; i < nres; i++) { ids[i] = res[i].id; ds[i] = res[i].d; }
  free(res); free(bd); free(lut); free(rot); free(rq); free(untraced.a); free(discarded.a); free(checked);
  free(sd); free(seeds);
  *blobs_out = nblobs;
  return nres;
}

/* searchInTwoSteps (lib/NGT/NGTQ/QuantizedBlobGraph.h:1190-1330): the `probes` blobs
 * nearest the query by the read-only graph search of the global index (epsilon =
 * blob_epsilon as (1 + blob_epsilon) - 1, the index's edge size), then every probed
 * blob judged in that order with a result set of `size` (judge,
 * QuantizedBlobGraph.h:1033-1080: skipped when its minimum is not below the radius). */
static size_t qbg_two(const OracleIndex *ix, const OracleQG *qg, const float *qf, size_t qdim, const void *q,
                      size_t size, size_t probes, float blob_epsilon, uint32_t *ids, float *ds,
                      uint32_t *blobs_out) {
  *blobs_out = 0;
  if (size == 0 || probes == 0) return 0;
  uint32_t *bid = (uint32_t *)malloc(sizeof(uint32_t) * (probes + 1));
  float *bdist = (float *)malloc(sizeof(float) * (probes + 1));
  uint32_t dc = 0;
  const float geps = (blob_epsilon + 1.0f) - 1.0f;
  size_t nb = graph_one(ix, q, probes, probes, geps, FLT_MAX, -1, 0, bid, bdist, &dc, NULL, 0);
  float *rq = (float *)calloc(qg->dim > qdim ? qg->dim : qdim, sizeof(float));
  memcpy(rq, qf, qdim * sizeof(float));
  float *rot = (float *)malloc(qg->dim * sizeof(float));
  oracle_qg_rotate(qg, rq, rot);
  uint8_t *lut = (uint8_t *)malloc((size_t)qg->m * 16);
  float *bd = (float *)malloc(sizeof(float) * 65536);
  od_t *res = (od_t *)malloc((size + 2) * sizeof(od_t));
  size_t nres = 0;
  float radius = FLT_MAX;
  uint32_t judged = 0;
  for (size_t b = 0; b < nb; b++) {
    uint32_t blob = bid[b];
    if (blob >= qg->nnodes) continue;
    uint32_t a = qg->offsets[blob], n = qg->offsets[blob + 1] - a;
    float scale, offset;
    uint32_t c = qg->sid ? qg->sid[blob] : 0;
    qg_lut_centroid(qg, rot, qg->gcentroid + (size_t)c * qg->dim, lut, &scale, &offset);
    float bmin = n ? oracle_qg_scan(qg, lut, scale, offset, blob, bd) : FLT_MAX;
    judged++;
    if (bmin >= radius) continue;
    for (uint32_t i = 0; i < n; i++) {
      if (bd[i] <= radius) {
        od_t x = {qg->ids[a + i], bd[i]};
        maxheap_push(res, &nres, x);
        if (nres > size) maxheap_pop(res, &nres);
      }
    }
    if (nres >= size) radius = res[0].d;
  }
  qsort(res, nres, sizeof(od_t), od_cmp);
  for (size_t i = 0; i < nres; i++) { ids[i] = res[i].id; ds[i] = res[i].d; }
  free(res); free(bd); free(lut); free(rot); free(rq); free(bid); free(bdist);
  *blobs_out = judged;
  return nres;
}

/* refineDistances (lib/NGT/NGTQ/QuantizedBlobGraph.h:1136-1185): the results' exact
 * distances to the query over the object list (its comparator: L2 over uint8 or float
 * rows; a float query is cast element-wise to the row type, as setObject does,
 * lib/NGT/ObjectRepository.h:237-246), then the `exact` best by (distance, id). */
static size_t qbg_refine(const OracleQG *qg, const float *qf, size_t qdim, uint32_t *ids, float *ds, size_t n,
                         size_t exact) {
  size_t d = qg->olist_dim;
  size_t es = qg->olist_type == OT_FLOAT ? 4 : 1;
  uint8_t *qv = (uint8_t *)calloc(d, es);
  for (size_t i = 0; i < d && i < qdim; i++) {
    if (qg->olist_type == OT_FLOAT) ((float *)qv)[i] = qf[i];
    else qv[i] = (uint8_t)qf[i];
  }
  od_t *r = (od_t *)malloc((n + 1) * sizeof(od_t));
  for (size_t i = 0; i < n; i++) {
    r[i].id = ids[i];
    r[i].d = ids[i] < qg->olist_n
                 ? compare(qg->olist_type, M_L2, qv, (const uint8_t *)qg->olist + (size_t)ids[i] * d * es, d)
                 : FLT_MAX;
  }
  qsort(r, n, sizeof(od_t), od_cmp);
  size_t m = n < exact ? n : exact;
  for (size_t i = 0; i < m; i++) { ids[i] = r[i].id; ds[i] = r[i].d; }
  free(r); free(qv);
  return m;
}

/* qf: nq x qdim float queries; qrows: the same prepared as global-index rows.  kout >= size.
 * two_step: searchInTwoSteps with `explored` probes, else searchInOneStep.  exact > 0:
 * refinement to the `exact` best by exact distance (needs the object list). */
void oracle_qbg_search(const OracleIndex *ix, const OracleQG *qg, const float *qf, size_t qdim, const void *qrows,
                       size_t nq, size_t size, size_t kout, float epsilon, float blob_epsilon, size_t explored,
                       int64_t edge_size, int two_step, size_t exact, uint32_t *out_ids, float *out_d,
                       uint32_t *out_n, uint32_t *out_blobs, int nthreads) {
  size_t rb = (size_t)ix->dpad * elem_size(ix->otype);
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
  for (long q = 0; q < (long)nq; q++) {
    uint32_t nb = 0;
    size_t n;
    if (two_step)
      n = qbg_two(ix, qg, qf + q * qdim, qdim, (const uint8_t *)qrows + q * rb, size, explored, blob_epsilon,
                  out_ids + q * kout, out_d + q * kout, &nb);
    else
      n = qbg_one(ix, qg, qf + q * qdim, qdim, (const uint8_t *)qrows + q * rb, size, exact > 0 ? exact : size,
                  epsilon, blob_epsilon, explored, edge_size, out_ids + q * kout, out_d + q * kout, &nb);
    if (exact > 0 && qg->olist) n = qbg_refine(qg, qf + q * qdim, qdim, out_ids + q * kout, out_d + q * kout, n, exact);
    out_n[q] = (uint32_t)n;
    if (out_blobs) out_blobs[q] = nb;
  }
}

/* ---------------- ONNG construction (`ngt reconstruct-graph -m S`) ----------------
 * GraphOptimizer::execute (lib/NGT/GraphOptimizer.h:268-367) with shortcut reduction:
 *   GraphReconstructor::reconstructGraph (lib/NGT/GraphReconstructor.h:645-813) and
 *   GraphReconstructor::adjustPathsEffectively (lib/NGT/GraphReconstructor.h:200-409).
 * Graphs are CSR over node slots 0..n-1 (slot 0 and removed objects absent); edges
 * (id, distance).  The result is written into out_off (n+1) / out_ids / out_d, which
 * must hold the input's edges plus n x incoming.  Returns the number of edges, or -1
 * when an output buffer is too small. */
typedef struct { uint32_t id; float d; } edge_t;
typedef struct { edge_t *e; size_t n, cap; } elist_t;

static void el_push(elist_t *l, edge_t x) {
  if (l->n == l->cap) {
    l->cap = l->cap ? 2 * l->cap : 8;
    l->e = (edge_t *)realloc(l->e, l->cap * sizeof(edge_t));
  }
  l->e[l->n++] = x;
}
static int edge_cmp(const void *a, const void *b) {      /* ObjectDistance::operator< */
  const edge_t *x = (const edge_t *)a, *y = (const edge_t *)b;
  if (x->d != y->d) return x->d < y->d ? -1 : 1;
  return x->id < y->id ? -1 : (x->id > y->id);
}
/* GraphReconstructor::insert / hasEdge keep a node sorted by id (edgeComp) */
static size_t el_lower_id(const elist_t *l, uint32_t id) {
  size_t lo = 0, hi = l->n;
  while (lo < hi) {
    size_t mid = (lo + hi) / 2;
    if ((l->e[mid].id & 0x7FFFFFFFu) < (id & 0x7FFFFFFFu)) lo = mid + 1; else hi = mid;
  }
  return lo;
}
static int el_has(const elist_t *l, uint32_t id) {
  size_t i = el_lower_id(l, id);
  return i < l->n && l->e[i].id == id;
}
typedef struct { uint32_t rank, path, dst; } cand_t;
static int cand_cmp_desc(const void *a, const void *b) {   /* std::greater over (rank, (path, dst)) */
  const cand_t *x = (const cand_t *)a, *y = (const cand_t *)b;
  if (x->rank != y->rank) return x->rank > y->rank ? -1 : 1;
  if (x->path != y->path) return x->path > y->path ? -1 : 1;
  return x->dst > y->dst ? -1 : (x->dst < y->dst);
}

int64_t oracle_onng(uint64_t n, const uint8_t *present, const uint64_t *off, const uint32_t *ids, const float *ds,
                    int64_t outgoing, int64_t incoming, int64_t max_edges, int64_t min_edges, uint64_t *out_off,
                    uint32_t *out_ids, float *out_d, uint64_t out_cap) {
  elist_t *g = (elist_t *)calloc(n, sizeof(elist_t));       /* outGraph */
  for (uint64_t id = 1; id < n; id++) {
    if (!present[id]) continue;
    uint64_t cnt = off[id + 1] - off[id];
    /* a node with fewer edges than `outgoing` keeps its whole list (the warning path) */
    uint64_t keep = outgoing == 0 ? 0 : (cnt < (uint64_t)outgoing ? cnt : (uint64_t)outgoing);
    for (uint64_t e = 0; e < keep; e++) el_push(&g[id], (edge_t){ids[off[id] + e], ds[off[id] + e]});
  }
  if (max_edges == 0) max_edges = outgoing > incoming ? outgoing : incoming;
  for (uint64_t id = 1; id < n; id++) {                    /* reverse edges */
    uint64_t cnt = present[id] ? off[id + 1] - off[id] : 0;
    uint64_t rsize = (uint64_t)incoming < cnt ? (uint64_t)incoming : cnt;
    for (uint64_t i = 0; i < rsize; i++) {
      uint32_t to = ids[off[id] + i];
      float d = ds[off[id] + i];
      if (to >= n || !present[to]) continue;
      elist_t *l = &g[to];
      if ((int64_t)l->n >= max_edges) {
        edge_t b = l->e[l->n - 1];
        if (b.d > d || (b.d == d && b.id > to)) {
          edge_t x = {(uint32_t)id, d};
          size_t pos = 0;
          while (pos < l->n && edge_cmp(&l->e[pos], &x) < 0) pos++;
          el_push(l, x);
          memmove(l->e + pos + 1, l->e + pos, (l->n - 1 - pos) * sizeof(edge_t));
          l->e[pos] = x;
          l->n = (size_t)max_edges;
        }
      } else {
        el_push(l, (edge_t){(uint32_t)id, d});
        if ((int64_t)l->n >= max_edges) qsort(l->e, l->n, sizeof(edge_t), edge_cmp);
      }
    }
  }
  for (uint64_t id = 1; id < n; id++) {                    /* sort, drop repeated ids */
    elist_t *l = &g[id];
    if (!l->n) continue;
    qsort(l->e, l->n, sizeof(edge_t), edge_cmp);
    size_t w = 0;
    uint32_t prev = 0;
    for (size_t r = 0; r < l->n; r++) {
      if (l->e[r].id == prev) continue;
      prev = l->e[r].id;
      l->e[w++] = l->e[r];
    }
    l->n = w;
  }
  /* adjustPathsEffectively: tmp = the reconstructed graph, out = empty */
  elist_t *tmp = g;
  elist_t *out = (elist_t *)calloc(n, sizeof(elist_t));
  cand_t **cand = (cand_t **)calloc(n, sizeof(cand_t *));
  size_t *ncand = (size_t *)calloc(n, sizeof(size_t));
  for (uint64_t id = 1; id < n; id++) {
    const elist_t *src = &tmp[id];
    size_t cap = 0;
    for (size_t s = 0; s < src->n; s++) {
      const elist_t *pn = &tmp[src->e[s].id];
      for (size_t p = 0; p < pn->n; p++) {
        uint32_t dst = pn->e[p].id;
        size_t r;                                          /* dst's rank in src (the neighbour map) */
        for (r = src->n; r > 0; r--)
          if (src->e[r - 1].id == dst) break;
        if (r == 0) continue;
        r--;
        if (src->e[s].d < src->e[r].d && pn->e[p].d < src->e[r].d) {
          if (ncand[id] == cap) {
            cap = cap ? 2 * cap : 16;
            cand[id] = (cand_t *)realloc(cand[id], cap * sizeof(cand_t));
          }
          cand[id][ncand[id]++] = (cand_t){(uint32_t)r, src->e[s].id, dst};
        }
      }
    }
    if (ncand[id]) qsort(cand[id], ncand[id], sizeof(cand_t), cand_cmp_desc);
  }
  uint32_t *active = (uint32_t *)malloc(n * sizeof(uint32_t));
  size_t nact = 0;
  for (uint64_t id = 1; id < n; id++) active[nact++] = (uint32_t)id;
  for (size_t rank = 0; nact; rank++) {
    size_t w = 0;
    for (size_t a = 0; a < nact; a++) {
      uint32_t id = active[a];
      const elist_t *src = &tmp[id];
      if (rank >= src->n) continue;                       /* finished: leaves the list */
      active[w++] = id;
      if (!present[id]) continue;                         /* getNode throws: skipped */
      uint32_t dst = src->e[rank].id;
      if (ncand[id] > 0 && (int64_t)(out[id].n + src->n - rank) > min_edges) {
        int exist = 0;
        while (ncand[id] > 0 && cand[id][ncand[id] - 1].dst == dst) {
          cand_t c = cand[id][--ncand[id]];
          if (el_has(&out[id], c.path) && el_has(&out[c.path], c.dst)) {
            exist = 1;
            while (ncand[id] > 0 && cand[id][ncand[id] - 1].dst == dst) ncand[id]--;
            break;
          }
        }
        if (exist) continue;
      }
      elist_t *l = &out[id];
      size_t pos = el_lower_id(l, dst);
      el_push(l, src->e[rank]);
      memmove(l->e + pos + 1, l->e + pos, (l->n - 1 - pos) * sizeof(edge_t));
      l->e[pos] = src->e[rank];
    }
    nact = w;
  }
  uint64_t total = 0;
  int64_t ret = 0;
  out_off[0] = 0;
  for (uint64_t id = 0; id < n; id++) {
    elist_t *l = &out[id];
    if (l->n) qsort(l->e, l->n, sizeof(edge_t), edge_cmp);
    if (total + l->n > out_cap) ret = -1;
    for (size_t e = 0; e < l->n && ret == 0; e++) {
      out_ids[total + e] = l->e[e].id;
      out_d[total + e] = l->e[e].d;
    }
    total += l->n;
    out_off[id + 1] = total;
  }
  for (uint64_t id = 0; id < n; id++) { free(g[id].e); free(out[id].e); free(cand[id]); }
  free(g); free(out); free(cand); free(ncand); free(active);
  return ret < 0 ? -1 : (int64_t)total;
}
