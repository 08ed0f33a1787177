/* matgen_native.c -- the heavy part of the Chung-Lu generator of matgen.py in C (bit-identical to the numpy code).
 *
 * Given the cumulative endpoint distribution, draws 2m endpoints (splitmix64 uniforms, right-sided search), drops
 * self-loops, merges duplicate edges (radix sort of lo*n + hi), draws the edge weights U(0,1], forms the weighted
 * degrees in numpy.bincount's summation order, scales by D^-1/2 on both sides and builds the symmetric CSR with
 * sorted columns.  Used by matgen.chung_lu for large graphs; matgen's numpy path is the same algorithm.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static inline uint64_t sm64(uint64_t seed, uint64_t i) {
  uint64_t z = seed + i * 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

/* the (i+1)-th uniform in [0, 1) of matgen.uniform_01(seed, .) */
static inline double u01(uint64_t seed, uint64_t i) {
  return (double)(sm64(seed, i + 1) >> 11) * (1.0 / 9007199254740992.0);
}

typedef struct {
  long long n, nnz;
  int32_t *rowptr, *colidx;
  double *vals;
} CLGraph;

static void radix_sort_u64(uint64_t *a, uint64_t *tmp, size_t count, int bits) {
  size_t *cnt = (size_t *)malloc(sizeof(size_t) * 65537);
  if (!cnt) return;
  for (int shift = 0; shift < bits; shift += 16) {
    memset(cnt, 0, sizeof(size_t) * 65537);
    for (size_t i = 0; i < count; ++i) cnt[((a[i] >> shift) & 0xFFFF) + 1]++;
    for (int d = 0; d < 65536; ++d) cnt[d + 1] += cnt[d];
    for (size_t i = 0; i < count; ++i) tmp[cnt[(a[i] >> shift) & 0xFFFF]++] = a[i];
    memcpy(a, tmp, count * sizeof(uint64_t));
  }
  free(cnt);
}

/* Returns the number of nonzeros (or -1 on allocation failure); the graph is kept until chung_lu_fetch. */
long long chung_lu_build(long long n, const double *cdf, long long m, unsigned long long seed,
                         unsigned long long weight_seed, void **handle) {
  *handle = NULL;
  uint64_t *keys = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)m);
  uint64_t *tmp = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)m);
  if (!keys || !tmp) {
    free(keys);
    free(tmp);
    return -1;
  }
  /* Right-sided search of u in cdf (the first i with cdf[i] > u), narrowed by a bucket index: for u in
   * [b/T, (b+1)/T) the answer lies in [start[b], start[b+1]], start[b] = first i with cdf[i] > b/T (T a power of
   * two, so b/T and floor(u T) are exact). */
  const long long T = 1LL << 22;
  long long *start = (long long *)malloc(sizeof(long long) * (size_t)(T + 1));
  if (!start) {
    free(keys);
    free(tmp);
    return -1;
  }
  {
    long long i = 0;
    for (long long b = 0; b <= T; ++b) {
      const double x = (double)b / (double)T;
      while (i < n && cdf[i] <= x) ++i;
      start[b] = i;
    }
  }
  /* endpoints a = draws 0..m-1, b = draws m..2m-1; self-loops marked, compacted below */
#pragma omp parallel for schedule(static)
  for (long long k = 0; k < m; ++k) {
    long long e[2];
    for (int s = 0; s < 2; ++s) {
      const double u = u01(seed, (uint64_t)(k + s * m));
      const long long bkt = (long long)(u * (double)T);
      long long lo = start[bkt], hi = bkt < T ? start[bkt + 1] : n;
      while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (cdf[mid] <= u) lo = mid + 1;
        else hi = mid;
      }
      e[s] = lo < n - 1 ? lo : n - 1;
    }
    const uint64_t a = (uint64_t)(e[0] < e[1] ? e[0] : e[1]), b = (uint64_t)(e[0] < e[1] ? e[1] : e[0]);
    keys[k] = (e[0] == e[1]) ? UINT64_MAX : a * (uint64_t)n + b;
  }
  free(start);
  size_t cnt = 0;
  for (long long k = 0; k < m; ++k)
    if (keys[k] != UINT64_MAX) keys[cnt++] = keys[k];
  int bits = 1;
  while (bits < 64 && ((uint64_t)n * (uint64_t)n) >> bits) ++bits;
  radix_sort_u64(keys, tmp, cnt, bits);
  size_t nu = 0;
  for (size_t i = 0; i < cnt; ++i)
    if (i == 0 || keys[i] != keys[i - 1]) keys[nu++] = keys[i];
  free(tmp);
  double *wt = (double *)malloc(sizeof(double) * (nu ? nu : 1));
  double *deg = (double *)calloc((size_t)n, sizeof(double));
  int32_t *rowptr = (int32_t *)calloc((size_t)n + 1, sizeof(int32_t));
  int32_t *lower = (int32_t *)calloc((size_t)n, sizeof(int32_t));
  if (!wt || !deg || !rowptr || !lower) {
    free(keys); free(wt); free(deg); free(rowptr); free(lower);
    return -1;
  }
  for (size_t k = 0; k < nu; ++k) wt[k] = 1.0 - u01(weight_seed, k);
  /* numpy.bincount(concat(lo, hi), weights=concat(wt, wt)): all lo entries in key order, then all hi entries */
  for (size_t k = 0; k < nu; ++k) deg[keys[k] / (uint64_t)n] += wt[k];
  for (size_t k = 0; k < nu; ++k) deg[keys[k] % (uint64_t)n] += wt[k];
  for (long long i = 0; i < n; ++i) deg[i] = deg[i] > 0.0 ? 1.0 / sqrt(deg[i]) : 0.0; /* now D^-1/2 */
  for (size_t k = 0; k < nu; ++k) {
    rowptr[keys[k] / (uint64_t)n + 1]++;
    rowptr[keys[k] % (uint64_t)n + 1]++;
    lower[keys[k] % (uint64_t)n]++;
  }
  for (long long i = 0; i < n; ++i) rowptr[i + 1] += rowptr[i];
  const long long nnz = 2 * (long long)nu;
  int32_t *colidx = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nnz ? nnz : 1));
  double *vals = (double *)malloc(sizeof(double) * (size_t)(nnz ? nnz : 1));
  int32_t *cur = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
  if (!colidx || !vals || !cur) {
    free(keys); free(wt); free(deg); free(rowptr); free(lower); free(colidx); free(vals); free(cur);
    return -1;
  }
  /* row r: columns below r (edges (lo, r), lo ascending) first, then columns above r (edges (r, hi)) */
  for (long long i = 0; i < n; ++i) cur[i] = rowptr[i];
  for (size_t k = 0; k < nu; ++k) {
    const long long lo = (long long)(keys[k] / (uint64_t)n), hi = (long long)(keys[k] % (uint64_t)n);
    const int32_t p = cur[hi]++;
    colidx[p] = (int32_t)lo;
    vals[p] = wt[k] * deg[hi] * deg[lo];
  }
  for (long long i = 0; i < n; ++i) cur[i] = rowptr[i] + lower[i];
  for (size_t k = 0; k < nu; ++k) {
    const long long lo = (long long)(keys[k] / (uint64_t)n), hi = (long long)(keys[k] % (uint64_t)n);
    const int32_t p = cur[lo]++;
    colidx[p] = (int32_t)hi;
    vals[p] = wt[k] * deg[lo] * deg[hi];
  }
  free(keys); free(wt); free(deg); free(lower); free(cur);
  CLGraph *g = (CLGraph *)malloc(sizeof(CLGraph));
  if (!g) {
    free(rowptr); free(colidx); free(vals);
    return -1;
  }
  g->n = n;
  g->nnz = nnz;
  g->rowptr = rowptr;
  g->colidx = colidx;
  g->vals = vals;
  *handle = g;
  return nnz;
}

void chung_lu_fetch(void *handle, int32_t *rowptr, int32_t *colidx, double *vals) {
  CLGraph *g = (CLGraph *)handle;
  if (!g) return;
  memcpy(rowptr, g->rowptr, sizeof(int32_t) * (size_t)(g->n + 1));
  memcpy(colidx, g->colidx, sizeof(int32_t) * (size_t)g->nnz);
  memcpy(vals, g->vals, sizeof(double) * (size_t)g->nnz);
  free(g->rowptr);
  free(g->colidx);
  free(g->vals);
  free(g);
}
