/*
 * TEST INFRASTRUCTURE ONLY: the CPU oracle for the exact k-NN path.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this file's library, and only as the checker or as the timed CPU baseline.
 * The product (vecsearch_gb300) never calls it: it has no CPU fallback.
 *
 * What it restates (reference paths are relative to the vecsearch project):
 *   - include/vecsearch/distance.h:30-73   l2_sq / dot / distance(). The x86
 *     build of the reference runs the AVX2 branch: two 8-wide accumulators
 *     (acc0 takes dims i..i+7, acc1 dims i+8..i+15 of every 16-dim step, one
 *     fused multiply-add each), an 8-wide tail step into acc0, the hsum256
 *     tree of distance.h:18-27 applied to acc0+acc1, then the scalar tail
 *     (d mod 8 dims). gcc -O3 -march=native compiles that tail as one 4-wide
 *     step (four separately rounded products added in order) when at least
 *     four dims remain, and fused multiply-adds for the rest; this was
 *     measured against the compiled reference. The same operations in the same
 *     order are written here with fmaf(), so results are bit-identical to the
 *     x86/AVX2 reference on any host with IEEE fmaf (x86 and aarch64 alike).
 *   - src/brute_force.cpp:17-66   distances4(): per query the same order.
 *   - src/brute_force.cpp:116-170 search_batch(): threads split the rows,
 *     tiles of ~256 KB, query blocks of 4, a bounded heap per (thread, query),
 *     then a merge ordered by (dist, id). The heap here is keyed on
 *     (dist, id); the reference's heap compares dist only, so the two can
 *     differ only when two rows have bit-equal distances at the k-th place and
 *     one of them is evicted. Everywhere else the output is identical.
 *   - src/hnsw.cpp:336-354 search_exact(): the exact scan over a byte mask
 *     (the HNSW index's exact_below route), ordered by (dist, id).
 *
 * Parity is pinned: tests/golden/ holds outputs of the reference itself
 * (compiled from its sources by oracle/build_ref.py) and tests check this
 * restatement against them bit for bit.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define VSO_NONE 0xFFFFFFFFu

/* dot(a, b) in the reference's AVX2 order (distance.h:54-69, hsum256 at :18-27). */
static float vso_dot(const float* a, const float* b, size_t d) {
  float acc[16];
  size_t i = 0;
  for (int j = 0; j < 16; ++j) acc[j] = 0.f;
  for (; i + 16 <= d; i += 16)
    for (int j = 0; j < 16; ++j) acc[j] = fmaf(a[i + j], b[i + j], acc[j]);
  for (; i + 8 <= d; i += 8)
    for (int j = 0; j < 8; ++j) acc[j] = fmaf(a[i + j], b[i + j], acc[j]);
  float v[8];
  for (int j = 0; j < 8; ++j) v[j] = acc[j] + acc[8 + j];
  const float lo0 = v[0] + v[4], lo1 = v[1] + v[5], lo2 = v[2] + v[6], lo3 = v[3] + v[7];
  float r = (lo0 + lo1) + (lo2 + lo3);
  /* gcc vectorises the first four tail steps as separate products added in order */
  if (d - i >= 4)
    for (size_t e = i + 4; i < e; ++i) r = r + a[i] * b[i];
  for (; i < d; ++i) r = fmaf(a[i], b[i], r);
  return r;
}

/* l2_sq(a, b) in the reference's AVX2 order (distance.h:30-52). */
static float vso_l2(const float* a, const float* b, size_t d) {
  float acc[16];
  size_t i = 0;
  for (int j = 0; j < 16; ++j) acc[j] = 0.f;
  for (; i + 16 <= d; i += 16)
    for (int j = 0; j < 16; ++j) {
      const float e = a[i + j] - b[i + j];
      acc[j] = fmaf(e, e, acc[j]);
    }
  for (; i + 8 <= d; i += 8)
    for (int j = 0; j < 8; ++j) {
      const float e = a[i + j] - b[i + j];
      acc[j] = fmaf(e, e, acc[j]);
    }
  float v[8];
  for (int j = 0; j < 8; ++j) v[j] = acc[j] + acc[8 + j];
  const float lo0 = v[0] + v[4], lo1 = v[1] + v[5], lo2 = v[2] + v[6], lo3 = v[3] + v[7];
  float r = (lo0 + lo1) + (lo2 + lo3);
  if (d - i >= 4)
    for (size_t e4 = i + 4; i < e4; ++i) {
      const float e = a[i] - b[i];
      r = r + e * e;
    }
  for (; i < d; ++i) {
    const float e = a[i] - b[i];
    r = fmaf(e, e, r);
  }
  return r;
}

/* distance() of distance.h:71-73: metric 0 = L2, 1 = inner product (1 - dot). */
float vso_distance(int metric, const float* q, const float* x, size_t d) {
  return metric == 0 ? vso_l2(q, x, d) : 1.0f - vso_dot(q, x, d);
}

typedef struct {
  float d;
  uint32_t i;
} vso_nb;

static int vso_less(vso_nb a, vso_nb b) { return a.d < b.d || (a.d == b.d && a.i < b.i); }

/* Bounded max-heap on (dist, id) in h[0..n): keeps the k smallest (brute_force.cpp:77-86). */
static void vso_push(vso_nb* h, size_t* n, size_t k, vso_nb c) {
  if (*n < k) {
    size_t j = (*n)++;
    h[j] = c;
    while (j > 0) {
      size_t p = (j - 1) / 2;
      if (!vso_less(h[p], h[j])) break;
      vso_nb t = h[p];
      h[p] = h[j];
      h[j] = t;
      j = p;
    }
  } else if (vso_less(c, h[0])) {
    size_t j = 0;
    h[0] = c;
    for (;;) {
      size_t l = 2 * j + 1, r = l + 1, m = j;
      if (l < k && vso_less(h[m], h[l])) m = l;
      if (r < k && vso_less(h[m], h[r])) m = r;
      if (m == j) break;
      vso_nb t = h[m];
      h[m] = h[j];
      h[j] = t;
      j = m;
    }
  }
}

static int vso_cmp(const void* a, const void* b) {
  const vso_nb x = *(const vso_nb*)a, y = *(const vso_nb*)b;
  return vso_less(x, y) ? -1 : vso_less(y, x) ? 1 : 0;
}

typedef struct {
  const float* data;
  const float* queries;
  const uint8_t* allowed; /* NULL, or one byte per row (search_exact's mask) */
  size_t n, d, nq, k;
  int metric;
  size_t lo, hi;
  vso_nb* heaps; /* nq x k for this thread */
  size_t* sizes; /* nq */
} vso_job;

/* One thread's share of search_batch (brute_force.cpp:125-143): tiles of rows,
 * query blocks of 4, each distance pushed into the (thread, query) heap. */
static void* vso_scan(void* arg) {
  vso_job* j = (vso_job*)arg;
  const size_t d = j->d;
  const size_t tile = (size_t)((256u << 10) / (d * sizeof(float) + 1)) > 16
                          ? (size_t)((256u << 10) / (d * sizeof(float) + 1))
                          : 16;
  for (size_t b0 = j->lo; b0 < j->hi; b0 += tile) {
    const size_t b1 = b0 + tile < j->hi ? b0 + tile : j->hi;
    for (size_t q0 = 0; q0 < j->nq; q0 += 4) {
      const size_t nb = j->nq - q0 < 4 ? j->nq - q0 : 4;
      for (size_t i = b0; i < b1; ++i) {
        if (j->allowed && !j->allowed[i]) continue;
        const float* x = j->data + i * d;
        for (size_t t = 0; t < nb; ++t) {
          vso_nb c = {vso_distance(j->metric, j->queries + (q0 + t) * d, x, d), (uint32_t)i};
          vso_push(j->heaps + (q0 + t) * j->k, &j->sizes[q0 + t], j->k, c);
        }
      }
    }
  }
  return NULL;
}

/* BruteForceIndex::search_batch (brute_force.cpp:116-170), optionally restricted to
 * rows with allowed[row] != 0 (hnsw.cpp:336-354). Output nq x k, nearest first,
 * missing = (VSO_NONE, +inf). Returns 0, or -1 when memory runs out. */
int vso_search(const float* data, size_t n, size_t d, int metric, const float* queries, size_t nq,
               size_t k, const uint8_t* allowed, int num_threads, uint32_t* out_ids, float* out_dists) {
  if (nq == 0 || k == 0) return 0;
  size_t nt = num_threads < 1 ? 1 : (size_t)num_threads;
  if (nt > n) nt = n;
  if (nt == 0) nt = 1;
  vso_nb* heaps = (vso_nb*)malloc(nt * nq * k * sizeof(vso_nb));
  size_t* sizes = (size_t*)calloc(nt * nq, sizeof(size_t));
  vso_job* jobs = (vso_job*)calloc(nt, sizeof(vso_job));
  pthread_t* th = (pthread_t*)calloc(nt, sizeof(pthread_t));
  vso_nb* all = (vso_nb*)malloc(nt * k * sizeof(vso_nb));
  if (!heaps || !sizes || !jobs || !th || !all) {
    free(heaps), free(sizes), free(jobs), free(th), free(all);
    return -1;
  }
  for (size_t t = 0; t < nt; ++t) {
    vso_job j = {data, queries, allowed, n, d, nq, k, metric, n * t / nt, n * (t + 1) / nt,
                 heaps + t * nq * k, sizes + t * nq};
    jobs[t] = j;
  }
  size_t started = 1;
  for (size_t t = 1; t < nt; ++t, ++started)
    if (pthread_create(&th[t], NULL, vso_scan, &jobs[t]) != 0) break;
  vso_scan(&jobs[0]);
  for (size_t t = started; t < nt; ++t) vso_scan(&jobs[t]); /* threads that failed to start */
  for (size_t t = 1; t < started; ++t) pthread_join(th[t], NULL);

  for (size_t q = 0; q < nq; ++q) {
    size_t m = 0;
    for (size_t t = 0; t < nt; ++t) {
      memcpy(all + m, heaps + (t * nq + q) * k, sizes[t * nq + q] * sizeof(vso_nb));
      m += sizes[t * nq + q];
    }
    qsort(all, m, sizeof(vso_nb), vso_cmp);
    for (size_t j = 0; j < k; ++j) {
      out_ids[q * k + j] = j < m ? all[j].i : VSO_NONE;
      out_dists[q * k + j] = j < m ? all[j].d : INFINITY;
    }
  }
  free(heaps), free(sizes), free(jobs), free(th), free(all);
  return 0;
}

/* Distances of the listed (query, row) pairs, for tolerance checks. */
void vso_pair_distances(const float* data, size_t d, int metric, const float* queries, size_t nq,
                        const uint32_t* ids, size_t k, float* out) {
  for (size_t q = 0; q < nq; ++q)
    for (size_t j = 0; j < k; ++j) {
      const uint32_t id = ids[q * k + j];
      out[q * k + j] = id == VSO_NONE ? INFINITY : vso_distance(metric, queries + q * d, data + (size_t)id * d, d);
    }
}
