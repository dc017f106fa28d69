/*
 * inputs.c -- seeded host-side input generators (see include/bale_inputs.h).
 *
 * All generators are counter-based: element i depends only on (seed, i), so
 * the large ones split their index range over host threads and still give
 * the same buffers for any thread count.
 */
#define _GNU_SOURCE
#include "bale_inputs.h"

#include <math.h>
#include <pthread.h>
#include <sched.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define GOLDEN 0x9E3779B97F4A7C15ULL

static inline uint64_t sm64_mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

/* SplitMix64 (Steele, Lea & Flood 2014; Vigna's public-domain constants):
 * the state advances by GOLDEN per output, so output i is mix(seed + (i+1)*GOLDEN). */
uint64_t bale_splitmix64(uint64_t seed, uint64_t i) { return sm64_mix(seed + (i + 1) * GOLDEN); }

static inline uint64_t mulhi64(uint64_t a, uint64_t b) {
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
}

/* ------------------------------------------------------------------------ */
/* host thread pool: a blocking parallel-for over [0,n)                      */
/* ------------------------------------------------------------------------ */
static int g_host_threads = 0;

void bale_set_host_threads(int nthreads) { g_host_threads = nthreads; }

static int host_threads(void) {
  if (g_host_threads > 0) return g_host_threads;
  cpu_set_t set;
  if (sched_getaffinity(0, sizeof(set), &set) == 0 && CPU_COUNT(&set) > 0) return CPU_COUNT(&set);
  long c = sysconf(_SC_NPROCESSORS_ONLN);
  return c > 0 ? (int)c : 1;
}

typedef void (*range_fn)(void *ctx, int64_t lo, int64_t hi, int tid);
typedef struct {
  range_fn fn;
  void *ctx;
  int64_t lo, hi;
  int tid;
} par_task_t;

static void *par_entry(void *p) {
  par_task_t *t = (par_task_t *)p;
  t->fn(t->ctx, t->lo, t->hi, t->tid);
  return NULL;
}

/* Runs fn over nthreads contiguous slices of [0,n); returns the slice count. */
static int par_for(int64_t n, int64_t min_per_thread, range_fn fn, void *ctx) {
  int nt = host_threads();
  if (nt > 128) nt = 128;
  if (min_per_thread < 1) min_per_thread = 1;
  if (n / min_per_thread < nt) nt = (int)(n / min_per_thread);
  if (nt < 1) nt = 1;
  pthread_t th[128];
  par_task_t tasks[128];
  int ok[128];
  for (int t = 0; t < nt; t++) {
    tasks[t] = (par_task_t){fn, ctx, n * t / nt, n * (t + 1) / nt, t};
    ok[t] = 0;
  }
  for (int t = 1; t < nt; t++) ok[t] = pthread_create(&th[t], NULL, par_entry, &tasks[t]) == 0;
  par_entry(&tasks[0]);
  for (int t = 1; t < nt; t++) {
    if (ok[t]) pthread_join(th[t], NULL);
    else par_entry(&tasks[t]); /* could not spawn: run the slice here */
  }
  return nt;
}

/* ------------------------------------------------------------------------ */
/* uniform indices and random values                                          */
/* ------------------------------------------------------------------------ */
typedef struct {
  int64_t *out;
  uint64_t range, seed;
  int packed;
} uni_ctx_t;

static void uni_body(void *p, int64_t lo, int64_t hi, int tid) {
  (void)tid;
  uni_ctx_t *c = (uni_ctx_t *)p;
  for (int64_t i = lo; i < hi; i++) {
    uint64_t v = c->range ? mulhi64(bale_splitmix64(c->seed, (uint64_t)i), c->range)
                          : bale_splitmix64(c->seed, (uint64_t)i);
    c->out[i] = c->packed ? (int64_t)(v << 16) : (int64_t)v;
  }
}

int bale_gen_uniform(int64_t *out, int64_t n, int64_t range, uint64_t seed, int packed) {
  if (n < 0 || range <= 0 || (n > 0 && !out)) return BALE_EINVAL;
  if (packed && range > ((int64_t)1 << 47)) return BALE_EINVAL;
  uni_ctx_t c = {out, (uint64_t)range, seed, packed};
  par_for(n, 1 << 16, uni_body, &c);
  return BALE_OK;
}

int bale_gen_values(int64_t *out, int64_t n, uint64_t seed) {
  if (n < 0 || (n > 0 && !out)) return BALE_EINVAL;
  uni_ctx_t c = {out, 0, seed, 0};
  par_for(n, 1 << 16, uni_body, &c);
  return BALE_OK;
}

int bale_gen_negative_table(int64_t *out, int64_t n) {
  if (n < 0 || (n > 0 && !out)) return BALE_EINVAL;
  for (int64_t i = 0; i < n; i++) out[i] = -(i + 1);
  return BALE_OK;
}

/* ------------------------------------------------------------------------ */
/* keyed permutation of [0,range): balanced Feistel network on 2h bits      */
/* (2^(2h) >= range) with cycle walking back into [0,range).                 */
/* ------------------------------------------------------------------------ */
static inline uint64_t feistel(uint64_t x, int h, uint64_t key) {
  uint64_t mask = (h >= 32) ? 0xFFFFFFFFULL : ((1ULL << h) - 1);
  uint64_t L = x >> h, R = x & mask;
  for (int round = 0; round < 4; round++) {
    uint64_t f = sm64_mix(R ^ sm64_mix(key + (uint64_t)(round + 1) * GOLDEN)) & mask;
    uint64_t nl = R;
    R = L ^ f;
    L = nl;
  }
  return (L << h) | R;
}

int64_t bale_keyed_perm(int64_t r, int64_t range, uint64_t key) {
  if (range <= 1) return 0;
  int bits = 64 - __builtin_clzll((uint64_t)(range - 1));
  int h = (bits + 1) / 2;
  uint64_t x = (uint64_t)r;
  do {
    x = feistel(x, h, key);
  } while (x >= (uint64_t)range);
  return (int64_t)x;
}

/* ------------------------------------------------------------------------ */
/* Zipf by rejection-inversion (W. Hormann, G. Derflinger, "Rejection-       */
/* inversion to generate variates from monotone discrete distributions",   */
/* ACM TOMACS 6(3), 1996).  H is an antiderivative of h(x) = x^-s.          */
/* ------------------------------------------------------------------------ */
typedef struct {
  double s, hx1, hn, sv;
  int64_t N;
} zipf_t;

static double log1p_over_x(double x) { return fabs(x) > 1e-8 ? log1p(x) / x : 1.0 - x * (0.5 - x / 3.0); }
static double expm1_over_x(double x) { return fabs(x) > 1e-8 ? expm1(x) / x : 1.0 + x * (0.5 + x / 6.0); }
static double zipf_H(const zipf_t *z, double x) {
  double lx = log(x);
  return expm1_over_x((1.0 - z->s) * lx) * lx;
}
static double zipf_h(const zipf_t *z, double x) { return exp(-z->s * log(x)); }
static double zipf_Hinv(const zipf_t *z, double u) {
  double t = u * (1.0 - z->s);
  if (t < -1.0) t = -1.0;
  return exp(log1p_over_x(t) * u);
}
static void zipf_init(zipf_t *z, int64_t N, double s) {
  z->s = s;
  z->N = N;
  z->hx1 = zipf_H(z, 1.5) - 1.0;
  z->hn = zipf_H(z, (double)N + 0.5);
  z->sv = 2.0 - zipf_Hinv(z, zipf_H(z, 2.5) - zipf_h(z, 2.0));
}
/* rank k in [1,N]; attempt t of sample i draws output (i*64 + t%64) of a
 * stream whose seed also depends on t/64, so every sample is independent. */
static int64_t zipf_sample(const zipf_t *z, uint64_t seed, uint64_t i) {
  for (uint64_t t = 0;; t++) {
    uint64_t s2 = t < 64 ? seed : sm64_mix(seed + t / 64);
    uint64_t r = bale_splitmix64(s2, i * 64 + (t % 64));
    double U = (double)(r >> 11) * (1.0 / 9007199254740992.0);
    double u = z->hn + U * (z->hx1 - z->hn);
    double x = zipf_Hinv(z, u);
    int64_t k = (int64_t)(x + 0.5);
    if (k < 1) k = 1;
    else if (k > z->N) k = z->N;
    if ((double)k - x <= z->sv || u >= zipf_H(z, (double)k + 0.5) - zipf_h(z, (double)k)) return k;
  }
}

typedef struct {
  int64_t *out;
  zipf_t z;
  uint64_t seed_rank, seed_perm;
  int packed;
} zipf_ctx_t;

static void zipf_body(void *p, int64_t lo, int64_t hi, int tid) {
  (void)tid;
  zipf_ctx_t *c = (zipf_ctx_t *)p;
  for (int64_t i = lo; i < hi; i++) {
    int64_t rank = zipf_sample(&c->z, c->seed_rank, (uint64_t)i) - 1;
    int64_t v = bale_keyed_perm(rank, c->z.N, c->seed_perm);
    c->out[i] = c->packed ? (int64_t)((uint64_t)v << 16) : v;
  }
}

int bale_gen_zipf(int64_t *out, int64_t n, int64_t range, double s, uint64_t seed_rank,
                  uint64_t seed_perm, int packed) {
  if (n < 0 || range <= 0 || !(s > 0.0) || fabs(s - 1.0) < 1e-12 || (n > 0 && !out))
    return BALE_EINVAL;
  zipf_ctx_t c;
  c.out = out;
  zipf_init(&c.z, range, s);
  c.seed_rank = seed_rank;
  c.seed_perm = seed_perm;
  c.packed = packed;
  par_for(n, 1 << 14, zipf_body, &c);
  return BALE_OK;
}

/* ------------------------------------------------------------------------ */
/* matrices                                                                  */
/* ------------------------------------------------------------------------ */
sparsemat_t *bale_make_matrix(int64_t numrows, int64_t numcols, int64_t nnz) {
  if (numrows < 0 || numcols < 0 || nnz < 0) return NULL;
  sparsemat_t *m = (sparsemat_t *)calloc(1, sizeof(sparsemat_t));
  if (!m) return NULL;
  m->local = 0;
  m->numrows = m->lnumrows = numrows;
  m->numcols = numcols;
  m->nnz = m->lnnz = nnz;
  m->loffset = (int64_t *)calloc((size_t)numrows + 1, sizeof(int64_t));
  m->lnonzero = (int64_t *)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(int64_t));
  if (!m->loffset || !m->lnonzero) {
    free(m->loffset);
    free(m->lnonzero);
    free(m);
    return NULL;
  }
  m->offset = m->loffset;
  m->nonzero = m->lnonzero;
  return m;
}

void bale_free_matrix(sparsemat_t *m) {
  if (!m) return;
  free(m->loffset);
  free(m->lnonzero);
  free(m);
}

static int cmp_i64(const void *a, const void *b) {
  int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
  return (x > y) - (x < y);
}

static void sort_row(int64_t *v, int64_t len) {
  if (len <= 32) {
    for (int64_t i = 1; i < len; i++) {
      int64_t x = v[i], j = i - 1;
      while (j >= 0 && v[j] > x) {
        v[j + 1] = v[j];
        j--;
      }
      v[j + 1] = x;
    }
  } else {
    qsort(v, (size_t)len, sizeof(int64_t), cmp_i64);
  }
}

/* ---------------- parallel LSD radix sort of uint64 keys ---------------- */
#define RADIX_BITS 11
#define RADIX_SIZE (1 << RADIX_BITS)

typedef struct {
  uint64_t *src, *dst;
  int64_t n;
  int shift, nt;
  int64_t (*hist)[RADIX_SIZE];
} radix_ctx_t;

static void radix_count(void *p, int64_t lo, int64_t hi, int tid) {
  radix_ctx_t *c = (radix_ctx_t *)p;
  int64_t *h = c->hist[tid];
  memset(h, 0, sizeof(int64_t) * RADIX_SIZE);
  for (int64_t i = lo; i < hi; i++) h[(c->src[i] >> c->shift) & (RADIX_SIZE - 1)]++;
}

static void radix_scatter(void *p, int64_t lo, int64_t hi, int tid) {
  radix_ctx_t *c = (radix_ctx_t *)p;
  int64_t *h = c->hist[tid];
  for (int64_t i = lo; i < hi; i++) {
    uint64_t k = c->src[i];
    c->dst[h[(k >> c->shift) & (RADIX_SIZE - 1)]++] = k;
  }
}

/* Sorts keys[0,n) on their low `bits` bits; tmp has room for n keys.
 * Returns the buffer that holds the sorted keys (keys or tmp). */
static uint64_t *radix_sort_u64(uint64_t *keys, uint64_t *tmp, int64_t n, int bits) {
  int nt = host_threads();
  if (nt > 128) nt = 128;
  if (n / (1 << 16) < nt) nt = (int)(n / (1 << 16));
  if (nt < 1) nt = 1;
  int64_t(*hist)[RADIX_SIZE] = malloc(sizeof(int64_t) * RADIX_SIZE * (size_t)nt);
  uint64_t *src = keys, *dst = tmp;
  int saved = g_host_threads;
  g_host_threads = nt; /* both phases must cut [0,n) into the same slices */
  for (int shift = 0; shift < bits; shift += RADIX_BITS) {
    radix_ctx_t c = {src, dst, n, shift, nt, hist};
    par_for(n, 1, radix_count, &c);
    int64_t pos = 0;
    for (int d = 0; d < RADIX_SIZE; d++)
      for (int t = 0; t < nt; t++) {
        int64_t cnt = hist[t][d];
        hist[t][d] = pos;
        pos += cnt;
      }
    par_for(n, 1, radix_scatter, &c);
    uint64_t *x = src;
    src = dst;
    dst = x;
  }
  g_host_threads = saved;
  free(hist);
  return src;
}

/* ---------------- R-MAT ---------------- */
typedef struct {
  uint64_t *keys;
  int scale;
  uint32_t ta, tab, tabc;
  uint64_t seed;
} rmat_ctx_t;

static void rmat_body(void *p, int64_t lo, int64_t hi, int tid) {
  (void)tid;
  rmat_ctx_t *c = (rmat_ctx_t *)p;
  const int S = c->scale;
  const uint64_t draws = (uint64_t)(S + 1) / 2; /* two 32-bit levels per draw */
  for (int64_t e = lo; e < hi; e++) {
    uint64_t u = 0, v = 0, r = 0;
    for (int l = 0; l < S; l++) {
      if ((l & 1) == 0) r = bale_splitmix64(c->seed, (uint64_t)e * draws + (uint64_t)(l >> 1));
      uint32_t x = (l & 1) ? (uint32_t)(r >> 32) : (uint32_t)r;
      uint64_t ub, vb;
      if (x < c->ta) { ub = 0; vb = 0; }
      else if (x < c->tab) { ub = 0; vb = 1; }
      else if (x < c->tabc) { ub = 1; vb = 0; }
      else { ub = 1; vb = 1; }
      u = (u << 1) | ub;
      v = (v << 1) | vb;
    }
    if (u == v) c->keys[e] = UINT64_MAX; /* self loop: dropped */
    else c->keys[e] = u < v ? (u << S) | v : (v << S) | u;
  }
}

typedef struct {
  sparsemat_t *L;
} rowsort_ctx_t;

static void rowsort_body(void *p, int64_t lo, int64_t hi, int tid) {
  (void)tid;
  sparsemat_t *L = ((rowsort_ctx_t *)p)->L;
  for (int64_t i = lo; i < hi; i++)
    sort_row(L->lnonzero + L->loffset[i], L->loffset[i + 1] - L->loffset[i]);
}

static uint32_t prob_threshold(double p) {
  if (p <= 0.0) return 0;
  if (p >= 1.0) return UINT32_MAX;
  return (uint32_t)llround(p * 4294967296.0);
}

sparsemat_t *bale_gen_rmat(int64_t scale, int64_t edgefactor, double a, double b, double c,
                           uint64_t seed) {
  if (scale < 1 || scale > 31 || edgefactor < 1 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
    return NULL;
  const int S = (int)scale;
  const int64_t n = (int64_t)1 << S;
  const int64_t m = edgefactor * n;
  uint64_t *keys = (uint64_t *)malloc((size_t)m * sizeof(uint64_t));
  uint64_t *tmp = (uint64_t *)malloc((size_t)m * sizeof(uint64_t));
  int64_t *deg = (int64_t *)calloc((size_t)n, sizeof(int64_t));
  int64_t *newid = (int64_t *)malloc((size_t)n * sizeof(int64_t));
  if (!keys || !tmp || !deg || !newid) {
    free(keys); free(tmp); free(deg); free(newid);
    return NULL;
  }
  rmat_ctx_t rc = {keys, S, prob_threshold(a), prob_threshold(a + b), prob_threshold(a + b + c), seed};
  par_for(m, 1 << 14, rmat_body, &rc);

  /* sort undirected pairs (self loops carry all-ones keys and sort last) */
  uint64_t *sorted = radix_sort_u64(keys, tmp, m, 2 * S + 1 > 64 ? 64 : 2 * S + 1);
  const uint64_t mask = ((uint64_t)1 << S) - 1;
  int64_t nu = 0;
  for (int64_t e = 0; e < m; e++) {
    uint64_t k = sorted[e];
    if (k == UINT64_MAX || (k >> (2 * S)) != 0) break;
    if (nu > 0 && sorted[nu - 1] == k) continue;
    sorted[nu++] = k;
  }
  for (int64_t e = 0; e < nu; e++) {
    deg[sorted[e] >> S]++;
    deg[sorted[e] & mask]++;
  }
  /* relabel by descending degree, ties by ascending original id (counting sort) */
  int64_t maxdeg = 0;
  for (int64_t v = 0; v < n; v++) if (deg[v] > maxdeg) maxdeg = deg[v];
  int64_t *start = (int64_t *)calloc((size_t)maxdeg + 2, sizeof(int64_t));
  if (!start) {
    free(keys); free(tmp); free(deg); free(newid);
    return NULL;
  }
  for (int64_t v = 0; v < n; v++) start[maxdeg - deg[v] + 1]++;
  for (int64_t d = 0; d <= maxdeg; d++) start[d + 1] += start[d];
  for (int64_t v = 0; v < n; v++) newid[v] = start[maxdeg - deg[v]]++;
  free(start);

  sparsemat_t *L = bale_make_matrix(n, n, nu);
  if (!L) {
    free(keys); free(tmp); free(deg); free(newid);
    return NULL;
  }
  int64_t *off = L->loffset;
  for (int64_t e = 0; e < nu; e++) {
    int64_t x = newid[sorted[e] >> S], y = newid[sorted[e] & mask];
    off[(x > y ? x : y) + 1]++;
  }
  for (int64_t i = 0; i < n; i++) off[i + 1] += off[i];
  int64_t *fill = deg; /* reuse as per-row cursor */
  memcpy(fill, off, (size_t)n * sizeof(int64_t));
  for (int64_t e = 0; e < nu; e++) {
    int64_t x = newid[sorted[e] >> S], y = newid[sorted[e] & mask];
    int64_t row = x > y ? x : y, col = x > y ? y : x;
    L->lnonzero[fill[row]++] = col;
  }
  rowsort_ctx_t sc = {L};
  par_for(n, 1 << 12, rowsort_body, &sc);
  free(keys); free(tmp); free(deg); free(newid);
  return L;
}

/* ---------------- Erdos-Renyi (lower triangle) ---------------- */
/* Batagelj & Brandes, "Efficient generation of large random networks",
 * Phys. Rev. E 71 (2005), algorithm G(n,p) with geometric skips, producing
 * the strictly lower triangle row by row with ascending columns. */
sparsemat_t *bale_gen_erdos_renyi(int64_t n, double p, uint64_t seed) {
  if (n < 0 || p < 0.0 || p > 1.0) return NULL;
  int64_t cap = (int64_t)(p * (double)n * (double)(n - 1) / 2.0 * 1.05) + 1024;
  if (p >= 1.0) cap = n * (n - 1) / 2 + 1;
  int64_t *cols = (int64_t *)malloc((size_t)cap * sizeof(int64_t));
  int64_t *off = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
  if (!cols || !off) { free(cols); free(off); return NULL; }
  int64_t nnz = 0;
  if (p > 0.0 && n > 1) {
    const double lq = log1p(-p);
    int64_t v = 1, w = -1;
    uint64_t draw = 0;
    while (v < n) {
      int64_t skip;
      if (p >= 1.0) skip = 0;
      else {
        double u = (double)(bale_splitmix64(seed, draw++) >> 11) * (1.0 / 9007199254740992.0);
        double g = floor(log1p(-u) / lq);
        skip = g > 9.0e18 ? INT64_MAX / 4 : (int64_t)g;
      }
      w += 1 + skip;
      while (w >= v && v < n) {
        w -= v;
        off[v + 1] = nnz; /* close row v */
        v++;
      }
      if (v < n) {
        if (nnz == cap) {
          cap = cap * 2;
          int64_t *nc = (int64_t *)realloc(cols, (size_t)cap * sizeof(int64_t));
          if (!nc) { free(cols); free(off); return NULL; }
          cols = nc;
        }
        cols[nnz++] = w;
        off[v + 1] = nnz;
      }
    }
  }
  /* rows never touched keep the running total */
  for (int64_t i = 1; i <= n; i++) if (off[i] < off[i - 1]) off[i] = off[i - 1];
  off[n] = nnz;
  sparsemat_t *L = bale_make_matrix(n, n, nnz);
  if (!L) { free(cols); free(off); return NULL; }
  memcpy(L->loffset, off, (size_t)(n + 1) * sizeof(int64_t));
  if (nnz) memcpy(L->lnonzero, cols, (size_t)nnz * sizeof(int64_t));
  free(cols);
  free(off);
  return L;
}

/* ---------------- Kronecker products of stars ---------------- */
/* K_{1,m} adjacency with the reference's optional loop (spmat/spmat_utils.upc:969-998):
 * mode 1 puts a loop on the centre (row 0 starts with column 0), mode 2 on
 * the last outer vertex (row m gains column m). */
static sparsemat_t *star_graph(int64_t m, int mode) {
  sparsemat_t *G = bale_make_matrix(m + 1, m + 1, 2 * m + (mode > 0 ? 1 : 0));
  if (!G) return NULL;
  int64_t pos = 0;
  if (mode == 1) G->lnonzero[pos++] = 0;
  for (int64_t i = 1; i <= m; i++) G->lnonzero[pos++] = i;
  G->loffset[1] = pos;
  for (int64_t i = 1; i <= m; i++) {
    G->lnonzero[pos++] = 0;
    if (mode == 2 && i == m) G->lnonzero[pos++] = m;
    G->loffset[i + 1] = pos;
  }
  return G;
}

/* Full Kronecker product of two local pattern matrices: row rB*nC + rC holds
 * cB*numcolsC + cC for every cB in row rB of B and cC in row rC of C, in that
 * nesting order (spmat/spmat_utils.upc:921-960). */
static sparsemat_t *kron_full(const sparsemat_t *B, const sparsemat_t *C) {
  int64_t n = B->numrows * C->numrows;
  sparsemat_t *A = bale_make_matrix(n, B->numcols * C->numcols, B->nnz * C->nnz);
  if (!A) return NULL;
  int64_t pos = 0;
  for (int64_t rb = 0; rb < B->numrows; rb++)
    for (int64_t rc = 0; rc < C->numrows; rc++) {
      for (int64_t j = B->loffset[rb]; j < B->loffset[rb + 1]; j++)
        for (int64_t k = C->loffset[rc]; k < C->loffset[rc + 1]; k++)
          A->lnonzero[pos++] = B->lnonzero[j] * C->numcols + C->lnonzero[k];
      A->loffset[rb * C->numrows + rc + 1] = pos;
    }
  return A;
}

/* Left-to-right product of the stars of one half-list
 * (spmat/spmat_utils.upc:1007-1033). */
static sparsemat_t *stars_product(const int64_t *m, int64_t M, int mode) {
  if (M < 1) return NULL;
  sparsemat_t *acc = star_graph(m[0], mode);
  for (int64_t i = 1; i < M && acc; i++) {
    sparsemat_t *s = star_graph(m[i], mode);
    sparsemat_t *next = s ? kron_full(acc, s) : NULL;
    bale_free_matrix(s);
    bale_free_matrix(acc);
    acc = next;
  }
  return acc;
}

sparsemat_t *bale_gen_kronecker(int mode, const int64_t *specs, int64_t nspecs) {
  if (mode < 0 || mode > 2 || nspecs < 2 || !specs) return NULL;
  int64_t half = nspecs / 2;
  sparsemat_t *B = stars_product(specs, half, mode);
  sparsemat_t *C = stars_product(specs + half, nspecs - half, mode);
  if (!B || !C) { bale_free_matrix(B); bale_free_matrix(C); return NULL; }
  /* strictly lower part of B (x) C: within each (row of B, row of C) block
   * the C columns ascend, so the block's scan stops at the first column that
   * is not below the row (spmat/spmat_utils.upc:840-858 with lower = 1). */
  int64_t n = B->numrows * C->numrows;
  int64_t cap = 0;
  for (int64_t row = 0; row < n; row++) {
    int64_t rb = row / C->numrows, rc = row % C->numrows;
    cap += (B->loffset[rb + 1] - B->loffset[rb]) * (C->loffset[rc + 1] - C->loffset[rc]);
  }
  sparsemat_t *A = bale_make_matrix(n, n, cap);
  if (!A) { bale_free_matrix(B); bale_free_matrix(C); return NULL; }
  int64_t pos = 0;
  for (int64_t row = 0; row < n; row++) {
    int64_t rb = row / C->numrows, rc = row % C->numrows;
    for (int64_t j = B->loffset[rb]; j < B->loffset[rb + 1]; j++) {
      int64_t bcol = B->lnonzero[j];
      for (int64_t k = C->loffset[rc]; k < C->loffset[rc + 1]; k++) {
        int64_t col = bcol * C->numcols + C->lnonzero[k];
        if (col < row) A->lnonzero[pos++] = col;
        else break;
      }
    }
    A->loffset[row + 1] = pos;
  }
  A->nnz = A->lnnz = pos;
  bale_free_matrix(B);
  bale_free_matrix(C);
  return A;
}

int64_t bale_kronecker_triangles(int mode, const int64_t *specs, int64_t nspecs) {
  double ans;
  if (mode == 0) return 0;
  if (mode == 1) {
    double a = 1.0, x = 1.0;
    for (int64_t i = 0; i < nspecs; i++) {
      a *= (double)(3 * specs[i] + 1);
      x *= (double)(specs[i] + 1);
    }
    ans = a / 6.0 - 0.5 * x + 1.0 / 3.0;
  } else if (mode == 2) {
    ans = pow(4.0, (double)nspecs) / 6.0 - pow(2.0, (double)(nspecs - 1)) + 1.0 / 3.0;
  } else {
    return -1;
  }
  return (int64_t)llround(ans);
}
