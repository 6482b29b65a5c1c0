/* A native caller of the drop-in C API: `threads` POSIX threads call
 * ngt_search_index_as_float one query at a time over a query file, the way the
 * reference's own C++ callers loop over queries (ngtpy's batch_search runs one
 * NGT::Index::search per query under `#pragma omp parallel for`,
 * python/src/ngtpy.cpp:422-458).  The library coalesces the calls that meet on the
 * GPU.  Prints one JSON line: wall-clock queries/s, the median one-thread latency and
 * the coalescing counters; writes every query's ids (nq x k uint32, 0 past a short
 * result) to ids_out.
 *
 * usage: capi_loop <index> <queries.f32> <nq> <dim> <k> <epsilon> <threads> <lanes> <ids_out>
 */
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "ngt_capi.h"
#include "ngtgpu.h"

typedef struct {
  NGTIndex index;
  const float *queries;
  size_t nq, dim, k, first, stride;
  float epsilon;
  uint32_t *ids;
  int failed;
} Work;

static double now_s(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

static int search_one(NGTIndex index, const float *q, size_t dim, size_t k, float eps, uint32_t *ids,
                      NGTObjectDistances res, NGTError err) {
  if (!ngt_search_index_as_float(index, (float *)q, (int32_t)dim, k, eps, -1.0f, res, err)) {
    fprintf(stderr, "search failed: %s\n", ngt_get_error_string(err));
    return 0;
  }
  uint32_t n = ngt_get_result_size(res, err);
  for (uint32_t i = 0; i < n && i < k; i++) ids[i] = ngt_get_result(res, i, err).id;
  return 1;
}

static void *worker(void *arg) {
  Work *w = (Work *)arg;
  NGTError err = ngt_create_error_object();
  NGTObjectDistances res = ngt_create_empty_results(err);
  for (size_t j = w->first; j < w->nq; j += w->stride)
    if (!search_one(w->index, w->queries + j * w->dim, w->dim, w->k, w->epsilon, w->ids + j * w->k, res, err)) {
      w->failed = 1;
      break;
    }
  ngt_destroy_results(res);
  ngt_destroy_error_object(err);
  return NULL;
}

static int cmp_double(const void *a, const void *b) {
  double x = *(const double *)a, y = *(const double *)b;
  return x < y ? -1 : x > y;
}

int main(int argc, char **argv) {
  if (argc != 10) {
    fprintf(stderr, "usage: %s <index> <queries.f32> <nq> <dim> <k> <epsilon> <threads> <lanes> <ids_out>\n",
            argv[0]);
    return 2;
  }
  const size_t nq = strtoul(argv[3], NULL, 10), dim = strtoul(argv[4], NULL, 10), k = strtoul(argv[5], NULL, 10);
  const float eps = strtof(argv[6], NULL);
  const int threads = atoi(argv[7]);
  const uint32_t lanes = (uint32_t)strtoul(argv[8], NULL, 10);
  if (nq == 0 || dim == 0 || k == 0 || threads < 1 || threads > 1024) return 2;
  float *q = (float *)malloc(nq * dim * sizeof(float));
  uint32_t *ids = (uint32_t *)calloc(nq * k, sizeof(uint32_t));
  FILE *f = fopen(argv[2], "rb");
  if (!q || !ids || !f || fread(q, sizeof(float), nq * dim, f) != nq * dim) return 3;
  fclose(f);
  NGTError err = ngt_create_error_object();
  NGTIndex index = ngt_open_index_as_read_only(argv[1], err);
  if (!index) {
    fprintf(stderr, "open failed: %s\n", ngt_get_error_string(err));
    return 4;
  }
  if (lanes && !ngtgpu_set_coalescing_lanes(index, lanes, err)) {
    fprintf(stderr, "lanes: %s\n", ngt_get_error_string(err));
    return 4;
  }
  NGTObjectDistances res = ngt_create_empty_results(err);
  uint32_t *scratch = (uint32_t *)calloc(k, sizeof(uint32_t));
  /* warm-up (kernels loaded, lanes' scratch allocated), then the one-thread latency */
  for (size_t j = 0; j < 32 && j < nq; j++)
    if (!search_one(index, q + j * dim, dim, k, eps, scratch, res, err)) return 5;
  double lat[50];
  size_t nl = nq < 50 ? nq : 50;
  for (size_t j = 0; j < nl; j++) {
    double t0 = now_s();
    if (!search_one(index, q + j * dim, dim, k, eps, scratch, res, err)) return 5;
    lat[j] = now_s() - t0;
  }
  qsort(lat, nl, sizeof(double), cmp_double);
  uint64_t q0 = 0, l0 = 0, q1 = 0, l1 = 0;
  ngtgpu_coalescing_stats(index, &q0, &l0, err);
  Work *w = (Work *)calloc((size_t)threads, sizeof(Work));
  pthread_t *th = (pthread_t *)calloc((size_t)threads, sizeof(pthread_t));
  double t0 = now_s();
  for (int t = 0; t < threads; t++) {
    w[t] = (Work){index, q, nq, dim, k, (size_t)t, (size_t)threads, eps, ids, 0};
    pthread_create(&th[t], NULL, worker, &w[t]);
  }
  int failed = 0;
  for (int t = 0; t < threads; t++) {
    pthread_join(th[t], NULL);
    failed |= w[t].failed;
  }
  double wall = now_s() - t0;
  if (failed) return 5;
  ngtgpu_coalescing_stats(index, &q1, &l1, err);
  FILE *o = fopen(argv[9], "wb");
  if (!o || fwrite(ids, sizeof(uint32_t), nq * k, o) != nq * k) return 6;
  fclose(o);
  printf("{\"qps\": %.1f, \"threads\": %d, \"lanes\": %u, \"queries\": %zu, \"one_thread_latency_ms\": %.3f, "
         "\"queries_per_launch\": %.2f}\n",
         (double)nq / wall, threads, lanes, nq, 1e3 * lat[nl / 2],
         (double)(q1 - q0) / (double)(l1 > l0 ? l1 - l0 : 1));
  ngt_destroy_results(res);
  ngt_close_index(index);
  ngt_destroy_error_object(err);
  free(scratch);
  free(w);
  free(th);
  free(ids);
  free(q);
  return 0;
}
