/*
 * bale_oracle.c -- CPU restatement of bale's histo / ig / triangles kernels.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker and the timed CPU baseline.
 * The shipped GPU library never links, loads or calls this code.
 * Each routine restates one reference routine at a single processing element
 * (THREADS == 1, so the cyclic distribution index i -> (i / THREADS, i % THREADS)
 * is the identity) and cites the reference file:line it follows.  Parity of
 * this restatement with the reference itself is pinned by tests/golden/.
 */
#define _GNU_SOURCE
#include "bale_oracle.h"

#include <pthread.h>
#include <stdio.h>
#include <sys/stat.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* apps/histo_src/histo_agi.upc:61-66: lgp_atomic_add(counts, index[i], 1),
 * which at one PE is shmem_long_add(&counts[index[i]], 1, 0)
 * (libgetput/libgetput.upc:48-53). */
void orc_histo_agi(const int64_t *index, int64_t n, int64_t *counts) {
  for (int64_t i = 0; i < n; i++) counts[index[i]] += 1;
}

/* apps/histo_src/histo_exstack.upc:64-76: the owner PE (pckindx & 0xffff,
 * always 0 here) pops col = pckindx >> 16 and does lcounts[col]++. */
void orc_histo_exstack(const int64_t *pckindx, int64_t n, int64_t *lcounts) {
  for (int64_t i = 0; i < n; i++) lcounts[pckindx[i] >> 16]++;
}

/* A one-PE exstack (exstack/exstack.upc:163-340 at THREADS == 1): a send
 * buffer of cap packages headed by its 64-bit count, an exchange that copies
 * the used part into the receive buffer (lgp_memput to itself) and clears the
 * send count, and FIFO pops from the receive buffer.  It keeps the reference's
 * data movement -- every package copied into a buffer, across and out again
 * -- so the buffered variants below time the exstack machinery at one PE. */
typedef struct {
  int64_t cap, pkg;
  char *snd, *rcv, *push, *fifo;
} orc_ex1_t;

static int ex1_init(orc_ex1_t *x, int64_t cap, int64_t pkg) {
  x->cap = cap;
  x->pkg = pkg;
  x->snd = malloc((size_t)(8 + cap * pkg));
  x->rcv = malloc((size_t)(8 + cap * pkg));
  if (!x->snd || !x->rcv) {
    free(x->snd);
    free(x->rcv);
    return -1;
  }
  *(uint64_t *)x->snd = 0;
  *(uint64_t *)x->rcv = 0;
  x->push = x->snd + 8;
  x->fifo = x->rcv + 8;
  return 0;
}

static void ex1_free(orc_ex1_t *x) {
  free(x->snd);
  free(x->rcv);
}

/* exstack_push (:163-175): 0 when the buffer is full. */
static int ex1_push(orc_ex1_t *x, const void *item) {
  uint64_t *ct = (uint64_t *)x->snd;
  if ((int64_t)*ct >= x->cap) return 0;
  memcpy(x->push, item, (size_t)x->pkg);
  x->push += x->pkg;
  (*ct)++;
  return 1;
}

/* exstack_exchange (:185-220). */
static void ex1_exchange(orc_ex1_t *x) {
  uint64_t ct = *(uint64_t *)x->snd;
  if (ct) memcpy(x->rcv, x->snd, (size_t)(8 + (int64_t)ct * x->pkg));
  else *(uint64_t *)x->rcv = 0;
  *(uint64_t *)x->snd = 0;
  x->push = x->snd + 8;
  x->fifo = x->rcv + 8;
}

/* exstack_pop / exstack_pop_thread (:231-288): 0 when the receive buffer is empty. */
static int ex1_pop(orc_ex1_t *x, void *item) {
  uint64_t *ct = (uint64_t *)x->rcv;
  if (*ct == 0) return 0;
  memcpy(item, x->fifo, (size_t)x->pkg);
  x->fifo += x->pkg;
  (*ct)--;
  return 1;
}

/* apps/histo_src/histo_exstack.upc:52-86 with buf_cnt-package buffers: push
 * col = pckindx[i] >> 16 to PE pckindx[i] & 0xffff (0) until the buffer is
 * full, exchange, pull and count; exstack_proceed (exstack.upc:129-152) ends
 * the loop once every index has been pushed.  -1 if the buffers cannot be had. */
int orc_histo_exstack_buffered(const int64_t *pckindx, int64_t n, int64_t *lcounts, int64_t buf_cnt) {
  orc_ex1_t x;
  if (buf_cnt < 1 || ex1_init(&x, buf_cnt, 8) != 0) return -1;
  int64_t i = 0, col;
  while (i < n) {  /* exstack_proceed(ex, i == T) at one PE */
    for (; i < n; i++) {
      col = pckindx[i] >> 16;
      if (!ex1_push(&x, &col)) break;
    }
    ex1_exchange(&x);
    while (ex1_pop(&x, &col)) lcounts[col]++;
  }
  ex1_free(&x);
  return 0;
}

/* apps/ig_src/ig_exstack.upc:54-102 with buf_cnt-package buffers: push the
 * requests' local indices, exchange, answer each popped request with
 * ltable[idx] pushed back, exchange, and retrace the round's requests in
 * order from the replies. */
int orc_ig_exstack_buffered(int64_t *tgt, const int64_t *pckindx, int64_t n, const int64_t *ltable,
                            int64_t buf_cnt) {
  orc_ex1_t x;
  if (buf_cnt < 1 || ex1_init(&x, buf_cnt, 8) != 0) return -1;
  int64_t i = 0, idx;
  while (i < n) {  /* exstack_proceed(ex, i == l_num_req) at one PE */
    const int64_t i0 = i;
    for (; i < n; i++) {
      idx = pckindx[i] >> 16;
      if (!ex1_push(&x, &idx)) break;
    }
    ex1_exchange(&x);
    while (ex1_pop(&x, &idx)) {
      idx = ltable[idx];
      ex1_push(&x, &idx);  /* as many replies as requests: room is certain */
    }
    ex1_exchange(&x);
    for (int64_t j = i0; j < i; j++) {
      ex1_pop(&x, &idx);
      tgt[j] = idx;
    }
  }
  ex1_free(&x);
  return 0;
}

/* apps/triangle_src/triangle_exstack.upc:95-168 (alg 0) with bufsiz-package
 * buffers of the reference's {int32 w, int32 vj} packages: for each nonzero
 * (i,j), push every w of row i before j to row j's owner; when the buffer is
 * full, exchange and let the owner scan row j for each popped w (:61-82),
 * then retry the push.  Rows i = row0, row0 + row_step, ... only (a bounded
 * sample when row_step > 1).  Returns the count, or -1 without buffers;
 * *pushed gets the packages pushed. */
int64_t orc_triangle_exstack_push_buffered(const int64_t *offset, const int64_t *nonzero, int64_t numrows,
                                           int64_t bufsiz, int64_t row0, int64_t row_step, int64_t *pushed) {
  typedef struct {
    int32_t w, vj;
  } pkg_t;
  orc_ex1_t x;
  if (bufsiz < 1 || row_step < 1 || ex1_init(&x, bufsiz, (int64_t)sizeof(pkg_t)) != 0) return -1;
  int64_t cnt = 0, np = 0;
  pkg_t pkg;
  for (int64_t i = row0; i < numrows; i += row_step) {
    for (int64_t k = offset[i]; k < offset[i + 1]; k++) {
      const int64_t j = nonzero[k];
      pkg.vj = (int32_t)j;
      for (int64_t kk = offset[i]; kk < offset[i + 1]; kk++) {
        pkg.w = (int32_t)nonzero[kk];
        if (pkg.w == j) break;
        np++;
        while (!ex1_push(&x, &pkg)) {  /* full: exchange, process, push again */
          ex1_exchange(&x);
          pkg_t q;
          while (ex1_pop(&x, &q))
            for (int64_t t = offset[q.vj]; t < offset[q.vj + 1]; t++) {
              if (q.w == nonzero[t]) { cnt++; break; }
              if (q.w < nonzero[t]) break;
            }
        }
      }
    }
  }
  ex1_exchange(&x);
  pkg_t q;
  while (ex1_pop(&x, &q))
    for (int64_t t = offset[q.vj]; t < offset[q.vj + 1]; t++) {
      if (q.w == nonzero[t]) { cnt++; break; }
      if (q.w < nonzero[t]) break;
    }
  ex1_free(&x);
  if (pushed) *pushed = np;
  return cnt;
}

/* apps/triangle_src/triangle_agi.upc:69-99 (alg 0) over rows i = row0,
 * row0 + row_step, ... only: a bounded sample of the AGI loop at one PE. */
static int64_t tri_agi_rows(const int64_t *off, const int64_t *col, int64_t r0, int64_t r1, int64_t *pulled);

int64_t orc_triangle_agi_sampled(const int64_t *offset, const int64_t *nonzero, int64_t numrows, int64_t row0,
                                 int64_t row_step) {
  if (row_step < 1) return -1;
  int64_t cnt = 0;
  for (int64_t i = row0; i < numrows; i += row_step) cnt += tri_agi_rows(offset, nonzero, i, i + 1, NULL);
  return cnt;
}

/* apps/ig_src/ig_agi.upc:61-64: tgt[i] = lgp_get_int64(table, index[i]). */
void orc_ig_agi(int64_t *tgt, const int64_t *index, int64_t n, const int64_t *table) {
  for (int64_t i = 0; i < n; i++) tgt[i] = table[index[i]];
}

/* apps/ig_src/ig_exstack.upc:69-94: request l_indx = pckindx >> 16 from PE
 * pckindx & 0xffff, the owner answers ltable[l_indx], the requester retraces
 * its requests in order.  With one PE the reply for request j is ltable[j's idx]. */
void orc_ig_exstack(int64_t *tgt, const int64_t *pckindx, int64_t n, const int64_t *ltable) {
  for (int64_t j = 0; j < n; j++) tgt[j] = ltable[pckindx[j] >> 16];
}

/* apps/triangle_src/triangle_agi.upc:69-99 (alg 0).  For each nonzero L[i][j]
 * after the first of row i, walk row j and advance a cursor through row i
 * (both rows ascending), counting equal columns.  pulled counts 2 offset
 * reads per (i,j) and one read per row-j element, as the reference does. */
static int64_t tri_agi_rows(const int64_t *off, const int64_t *col, int64_t r0, int64_t r1,
                            int64_t *pulled) {
  int64_t cnt = 0, np = 0;
  for (int64_t i = r0; i < r1; i++) {
    for (int64_t k = off[i] + 1; k < off[i + 1]; k++) {
      int64_t j = col[k];
      int64_t start = off[i];
      int64_t kbegin = off[j], kend = off[j + 1];
      np += 2;
      for (int64_t kk = kbegin; kk < kend; kk++) {
        int64_t w = col[kk];
        np++;
        for (int64_t ii = start; ii < off[i + 1]; ii++) {
          if (w == col[ii]) { cnt++; start = ii + 1; break; }
          if (w < col[ii]) { start = ii; break; }
        }
      }
    }
  }
  if (pulled) *pulled += np;
  return cnt;
}

int64_t orc_triangle_agi(const int64_t *offset, const int64_t *nonzero, int64_t numrows,
                         int64_t *pulled) {
  if (pulled) *pulled = 0;
  return tri_agi_rows(offset, nonzero, 0, numrows, pulled);
}

/* apps/triangle_src/triangle_exstack.upc:108-133 (push side, alg 0): for each
 * nonzero (i,j), every w in row i before the column j itself is pushed to
 * the owner of row j; :61-82 (pop side): the owner scans row j, which is
 * ascending, for w and stops at the first column >= w. */
int64_t orc_triangle_exstack_push(const int64_t *offset, const int64_t *nonzero,
                                  int64_t numrows, int64_t *pushed) {
  int64_t cnt = 0, np = 0;
  for (int64_t i = 0; i < numrows; i++) {
    for (int64_t k = offset[i]; k < offset[i + 1]; k++) {
      int64_t j = nonzero[k];
      for (int64_t kk = offset[i]; kk < offset[i + 1]; kk++) {
        int64_t w = nonzero[kk];
        if (w == j) break;
        np++;
        for (int64_t t = offset[j]; t < offset[j + 1]; t++) {
          if (w == nonzero[t]) { cnt++; break; }
          if (w < nonzero[t]) break;
        }
      }
    }
  }
  if (pushed) *pushed = np;
  return cnt;
}

/* apps/triangle_src/triangle.upc:325-361: column counts by fetch-and-inc,
 * then pulls = sum deg(i)*cc(i) and pushes = sum C(deg(i),2) for alg 0. */
void orc_triangle_work(const int64_t *offset, const int64_t *nonzero, int64_t numrows,
                       int64_t *pulls, int64_t *pushes) {
  int64_t *cc = calloc((size_t)(numrows > 0 ? numrows : 1), sizeof(int64_t));
  for (int64_t k = 0; k < offset[numrows]; k++) cc[nonzero[k]]++;
  int64_t pl = 0, ps = 0;
  for (int64_t i = 0; i < numrows; i++) {
    int64_t deg = offset[i + 1] - offset[i];
    pl += deg * cc[i];
    ps += deg * (deg - 1) / 2;
  }
  free(cc);
  *pulls = pl;
  *pushes = ps;
}

/* spmat/spmat_utils.upc:377-409 (is_lower_triangular, unit_diagonal = 0)
 * tightened to STRICTLY lower, plus ascending columns within each row
 * (the "tidy" property the merge scans need) and consistent offsets. */
int orc_is_strict_lower_tidy(const int64_t *offset, const int64_t *nonzero, int64_t numrows) {
  if (offset[0] != 0) return 0;
  for (int64_t i = 0; i < numrows; i++) {
    if (offset[i + 1] < offset[i]) return 0;
    for (int64_t k = offset[i]; k < offset[i + 1]; k++) {
      if (nonzero[k] < 0 || nonzero[k] >= i) return 0;
      if (k > offset[i] && nonzero[k] <= nonzero[k - 1]) return 0;
    }
  }
  return 1;
}

/* ------------------------------------------------------------------------ */
/* Multi-threaded variants (CPU baseline).                                   */
/* ------------------------------------------------------------------------ */
int orc_num_cpus(void) {
  cpu_set_t set;
  if (sched_getaffinity(0, sizeof(set), &set) == 0) {
    int c = CPU_COUNT(&set);
    if (c > 0) return c;
  }
  long n = sysconf(_SC_NPROCESSORS_ONLN);
  return n > 0 ? (int)n : 1;
}

typedef struct {
  int kind;
  int64_t lo, hi;
  const int64_t *a;
  const int64_t *b;
  int64_t *out;
  int64_t result;
  int64_t *next_row; /* shared cursor for dynamic row scheduling */
  int64_t numrows;
} orc_job_t;

enum { JOB_HISTO = 0, JOB_IG = 1, JOB_TRI = 2 };

static void *orc_worker(void *p) {
  orc_job_t *job = (orc_job_t *)p;
  if (job->kind == JOB_HISTO) {
    for (int64_t i = job->lo; i < job->hi; i++)
      __atomic_fetch_add(&job->out[job->a[i]], 1, __ATOMIC_RELAXED);
  } else if (job->kind == JOB_IG) {
    for (int64_t i = job->lo; i < job->hi; i++) job->out[i] = job->b[job->a[i]];
  } else {
    const int64_t chunk = 256;
    int64_t cnt = 0;
    for (;;) {
      int64_t r0 = __atomic_fetch_add(job->next_row, chunk, __ATOMIC_RELAXED);
      if (r0 >= job->numrows) break;
      int64_t r1 = r0 + chunk < job->numrows ? r0 + chunk : job->numrows;
      cnt += tri_agi_rows(job->a, job->b, r0, r1, NULL);
    }
    job->result = cnt;
  }
  return NULL;
}

static int64_t orc_run(int kind, int nthreads, int64_t n, const int64_t *a, const int64_t *b,
                       int64_t *out) {
  if (nthreads <= 0) nthreads = orc_num_cpus();
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  orc_job_t jobs[256];
  int64_t next_row = 0;
  for (int t = 0; t < nthreads; t++) {
    jobs[t].kind = kind;
    jobs[t].lo = n * t / nthreads;
    jobs[t].hi = n * (t + 1) / nthreads;
    jobs[t].a = a;
    jobs[t].b = b;
    jobs[t].out = out;
    jobs[t].result = 0;
    jobs[t].next_row = &next_row;
    jobs[t].numrows = n;
  }
  int started = 0;
  for (int t = 1; t < nthreads; t++) {
    if (pthread_create(&th[t], NULL, orc_worker, &jobs[t]) != 0) break;
    started = t;
  }
  /* threads that failed to start: their ranges run on the calling thread */
  for (int t = started + 1; t < nthreads; t++) orc_worker(&jobs[t]);
  orc_worker(&jobs[0]);
  for (int t = 1; t <= started; t++) pthread_join(th[t], NULL);
  int64_t total = 0;
  for (int t = 0; t < nthreads; t++) total += jobs[t].result;
  return total;
}

/* apps/triangle_src/triangle_agi.upc:100-136 (alg 1): for every nonzero
 * L[i][j] (the first of each row included), walk U's row j from its end
 * downwards while its columns are at least the smallest column of U's row
 * i, and advance a cursor down U's row i (both rows ascending), counting
 * equal columns: the sum over L's nonzeros of |U_i and U_j|.  pulled counts
 * 2 per (i,j) and one per row-j element read, as the reference does; like
 * the reference, an empty U row i reads the next stored column as its
 * "smallest" (only the tally can change).  Returns -1 for a NULL U. */
int64_t orc_triangle_agi_alg1(const int64_t *loff, const int64_t *lcol, int64_t n, const int64_t *uoff,
                              const int64_t *ucol, int64_t unnz, int64_t *pulled) {
  if (!uoff) return -1;
  int64_t cnt = 0, np = 0;
  for (int64_t i = 0; i < n; i++) {
    for (int64_t k = loff[i]; k < loff[i + 1]; k++) {
      const int64_t j = lcol[k];
      int64_t start = uoff[i + 1] - 1;
      const int64_t smallest = uoff[i] < unnz ? ucol[uoff[i]] : 0;
      np += 2;
      for (int64_t kk = uoff[j + 1] - 1; kk >= uoff[j]; kk--) {
        const int64_t w = ucol[kk];
        np++;
        if (w < smallest) break;
        for (int64_t ii = start; ii >= uoff[i]; ii--) {
          if (w == ucol[ii]) {
            cnt++;
            start = ii - 1;
            break;
          }
          if (w > ucol[ii]) {
            start = ii;
            break;
          }
        }
      }
    }
  }
  if (pulled) *pulled = np;
  return cnt;
}

/* Input generation (not a reference routine; see bale_oracle.h). */
typedef struct {
  int64_t *out;
  int64_t lo, hi;
  uint64_t range, seed;
} orc_gen_t;

static uint64_t orc_splitmix64(uint64_t seed, uint64_t i) {
  uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

static void *orc_gen_worker(void *p) {
  orc_gen_t *g = (orc_gen_t *)p;
  for (int64_t i = g->lo; i < g->hi; i++) {
    uint64_t v = orc_splitmix64(g->seed, (uint64_t)i);
    g->out[i] = g->range ? (int64_t)(uint64_t)(((unsigned __int128)v * g->range) >> 64) : (int64_t)v;
  }
  return NULL;
}

static void orc_gen(int64_t *out, int64_t n, uint64_t range, uint64_t seed, int nthreads) {
  if (nthreads <= 0) nthreads = orc_num_cpus();
  if (nthreads > 256) nthreads = 256;
  if (n < (int64_t)nthreads * 4096) nthreads = 1;
  pthread_t th[256];
  orc_gen_t g[256];
  int started = 0;
  for (int t = 0; t < nthreads; t++) g[t] = (orc_gen_t){out, n * t / nthreads, n * (t + 1) / nthreads, range, seed};
  for (int t = 1; t < nthreads; t++) {
    if (pthread_create(&th[t], NULL, orc_gen_worker, &g[t]) != 0) break;
    started = t;
  }
  for (int t = started + 1; t < nthreads; t++) orc_gen_worker(&g[t]);
  orc_gen_worker(&g[0]);
  for (int t = 1; t <= started; t++) pthread_join(th[t], NULL);
}

void orc_gen_uniform(int64_t *out, int64_t n, int64_t range, uint64_t seed, int nthreads) {
  if (range > 0) orc_gen(out, n, (uint64_t)range, seed, nthreads);
}

void orc_gen_values(int64_t *out, int64_t n, uint64_t seed, int nthreads) { orc_gen(out, n, 0, seed, nthreads); }

void orc_histo_agi_mt(const int64_t *index, int64_t n, int64_t *counts, int nthreads) {
  orc_run(JOB_HISTO, nthreads, n, index, NULL, counts);
}

void orc_ig_agi_mt(int64_t *tgt, const int64_t *index, int64_t n, const int64_t *table,
                   int nthreads) {
  orc_run(JOB_IG, nthreads, n, index, table, tgt);
}

int64_t orc_triangle_agi_mt(const int64_t *offset, const int64_t *nonzero, int64_t numrows,
                            int nthreads) {
  return orc_run(JOB_TRI, nthreads, numrows, offset, nonzero, NULL);
}

/* ------------------------------------------------------------------------ */
/* spmat: transpose, permute, random permutation                              */
/* ------------------------------------------------------------------------ */

/* transpose_matrix_agi (spmat/spmat_agi.upc:180-235) at THREADS = 1: column
 * counts, their prefix sums, then every nonzero of A appended to its column's
 * row of At in A's row order (so At's rows come out ascending). */
int orc_transpose(const int64_t *offset, const int64_t *nonzero, int64_t numrows, int64_t numcols,
                  int64_t *toffset, int64_t *tnonzero) {
  const int64_t nnz = offset[numrows];
  for (int64_t c = 0; c <= numcols; c++) toffset[c] = 0;
  for (int64_t k = 0; k < nnz; k++) {
    if (nonzero[k] < 0 || nonzero[k] >= numcols) return -1;
    toffset[nonzero[k] + 1]++;
  }
  for (int64_t c = 0; c < numcols; c++) toffset[c + 1] += toffset[c];
  int64_t *fill = (int64_t *)malloc((size_t)(numcols > 0 ? numcols : 1) * sizeof(int64_t));
  if (!fill) return -1;
  memcpy(fill, toffset, (size_t)numcols * sizeof(int64_t));
  for (int64_t r = 0; r < numrows; r++)
    for (int64_t k = offset[r]; k < offset[r + 1]; k++) tnonzero[fill[nonzero[k]]++] = r;
  free(fill);
  return 0;
}

/* permute_matrix_agi (spmat/spmat_agi.upc:119-173) at THREADS = 1: rperm is
 * the inverse of rperminv; row i of Ap is row rperm[i] of A with every column
 * mapped through cperminv, in the row's own order. */
void orc_permute(const int64_t *offset, const int64_t *nonzero, int64_t numrows, const int64_t *rperminv,
                 const int64_t *cperminv, int64_t *poffset, int64_t *pnonzero) {
  int64_t *rperm = (int64_t *)malloc((size_t)(numrows > 0 ? numrows : 1) * sizeof(int64_t));
  if (!rperm) return;
  for (int64_t i = 0; i < numrows; i++) rperm[rperminv[i]] = i;
  int64_t pos = 0;
  poffset[0] = 0;
  for (int64_t i = 0; i < numrows; i++) {
    const int64_t row = rperm[i];
    for (int64_t k = offset[row]; k < offset[row + 1]; k++) pnonzero[pos++] = cperminv[nonzero[k]];
    poffset[i + 1] = pos;
  }
  free(rperm);
}

/* The random permutations draw from the C library's drand48 stream and
 * reseed it only when seed != 0 (spmat_agi.upc:61, spmat_exstack.upc:92:
 * `if (seed != 0) srand48(seed)`).  With seed 0 they continue from the state
 * the caller left, and with any seed they leave the stream just past their
 * last draw, where a later lrand48() or seed-0 call picks it up.  These two
 * read and write that state: seed48 installs a state and returns the
 * previous one, so a second call puts it back untouched. */
static uint64_t libc_drand48_state(void) {
  unsigned short probe[3] = {0, 0, 0};
  const unsigned short *prev = seed48(probe);
  unsigned short keep[3] = {prev[0], prev[1], prev[2]};
  seed48(keep);
  return (uint64_t)keep[0] | (uint64_t)keep[1] << 16 | (uint64_t)keep[2] << 32;
}

static void set_libc_drand48_state(uint64_t x) {
  unsigned short s[3] = {(unsigned short)(x & 0xffff), (unsigned short)(x >> 16 & 0xffff),
                         (unsigned short)(x >> 32 & 0xffff)};
  seed48(s);
}

/* The reference's seed is an int: only the low 32 bits count, for the test
 * against 0 as for srand48. */
static int continues_stream(int64_t seed) { return ((uint64_t)seed & 0xffffffffull) == 0; }

static uint64_t drand48_start(int64_t seed) {
  return continues_stream(seed) ? libc_drand48_state() : ((((uint64_t)seed & 0xffffffffull) << 16) | 0x330eull);
}

/* rand_permp_agi (spmat/spmat_agi.upc:56-107) at THREADS = 1.
 * The drand48 family is the 48-bit linear congruential generator POSIX
 * specifies: srand48(s) sets X = (s & 0xffffffff) << 16 | 0x330e, and each
 * lrand48() steps X = (0x5deece66d X + 0xb) mod 2^48 and returns X >> 17.
 * Seed 0 continues the C library's stream (drand48_start above). */
int orc_rand_perm(int64_t n, int64_t seed, int64_t *perm) {
  const int64_t m = 2 * n;
  int64_t *target = (int64_t *)malloc((size_t)(m > 0 ? m : 1) * sizeof(int64_t));
  if (!target) return -1;
  for (int64_t i = 0; i < m; i++) target[i] = -1;
  uint64_t x = drand48_start(seed);
  int64_t i = 0;
  while (i < n) {
    x = (0x5deece66dull * x + 0xbull) & ((1ull << 48) - 1);
    const int64_t r = (int64_t)(x >> 17) % m;
    if (target[r] == -1) target[r] = i++;
  }
  set_libc_drand48_state(x); /* where the reference leaves the C library's stream */
  int64_t pos = 0;
  for (int64_t s = 0; s < m; s++)
    if (target[s] != -1) perm[pos++] = target[s];
  free(target);
  return 0;
}

/* rand_permp_exstack (spmat/spmat_exstack.upc:62-190) at THREADS = 1 (seed 0
 * continues the C library's drand48 stream); rand_permp (spmat/spmat_utils.upc:63-74) is this with
 * buf_cnt = 1024.  Darts wait in a list, initially 0..n-1.  Each round
 * throws the pending darts in list order into a buffer of buf_cnt packages
 * {slot = lrand48() % 2n, dart}; the draw that finds the buffer full is lost
 * (exstack_push returns 0 and the loop breaks before the dart advances).
 * The buffer is then popped in push order: a free slot takes the dart, a
 * taken one sends it back, and the returned darts, popped in the order they
 * were sent, are written backwards in front of the unthrown rest of the list.
 * The permutation is the darts in slot order. */
int orc_rand_perm_exstack(int64_t n, int64_t seed, int64_t buf_cnt, int64_t *perm) {
  if (buf_cnt < 1) return -1;
  const int64_t m = 2 * n;
  int64_t *target = (int64_t *)malloc((size_t)(m > 0 ? m : 1) * sizeof(int64_t));
  int64_t *list = (int64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  int64_t *slot = (int64_t *)malloc((size_t)buf_cnt * sizeof(int64_t));
  int64_t *dart = (int64_t *)malloc((size_t)buf_cnt * sizeof(int64_t));
  int rc = -1;
  if (!target || !list || !slot || !dart) goto done;
  for (int64_t i = 0; i < m; i++) target[i] = -1;
  for (int64_t i = 0; i < n; i++) list[i] = i;
  uint64_t x = drand48_start(seed);
  int64_t iend = 0;
  while (iend != n) {
    int64_t i = iend, cnt = 0;
    while (i < n) {
      x = (0x5deece66dull * x + 0xbull) & ((1ull << 48) - 1);
      const int64_t r = (int64_t)(x >> 17) % m;
      if (cnt == buf_cnt) break;
      slot[cnt] = r;
      dart[cnt++] = list[i++];
    }
    iend = i;
    int64_t back = 0;
    for (int64_t k = 0; k < cnt; k++) {
      if (target[slot[k]] == -1) target[slot[k]] = dart[k];
      else dart[back++] = dart[k];  /* back <= k: the returned darts, in order */
    }
    for (int64_t k = 0; k < back; k++) list[--iend] = dart[k];
  }
  set_libc_drand48_state(x); /* where the reference leaves the C library's stream */
  int64_t pos = 0;
  for (int64_t s = 0; s < m; s++)
    if (target[s] != -1) perm[pos++] = target[s];
  rc = 0;
done:
  free(target);
  free(list);
  free(slot);
  free(dart);
  return rc;
}

/* write_sparse_matrix_agi (spmat/spmat_agi.upc:286-335) at THREADS = 1: the
 * directory, its "metadata" file (write_sparse_matrix_metadata,
 * spmat/spmat_utils.upc:196-206: numrows, numcols, nnz and the writer count,
 * one "%ld" per line), "rowcnt_0" (write_rowcounts, spmat_agi.upc:250-277:
 * each row's length as a binary int64) and "nonzero_0" (the rows' columns as
 * binary int64, row after row). */
int orc_write_dataset(const char *dirname, const int64_t *offset, const int64_t *nonzero, int64_t numrows,
                      int64_t numcols) {
  char fname[4096];
  mkdir(dirname, 0770);
  snprintf(fname, sizeof fname, "%s/metadata", dirname);
  FILE *fp = fopen(fname, "w");
  if (!fp) return -1;
  fprintf(fp, "%ld\n%ld\n%ld\n%ld\n", (long)numrows, (long)numcols, (long)offset[numrows], 1L);
  fclose(fp);
  snprintf(fname, sizeof fname, "%s/rowcnt_0", dirname);
  if (!(fp = fopen(fname, "wb"))) return -1;
  for (int64_t i = 0; i < numrows; i++) {
    const int64_t rc = offset[i + 1] - offset[i];
    if (fwrite(&rc, sizeof rc, 1, fp) != 1) { fclose(fp); return -1; }
  }
  fclose(fp);
  snprintf(fname, sizeof fname, "%s/nonzero_0", dirname);
  if (!(fp = fopen(fname, "wb"))) return -1;
  const size_t nnz = (size_t)offset[numrows];
  const int ok = nnz == 0 || fwrite(nonzero, sizeof(int64_t), nnz, fp) == nnz;
  fclose(fp);
  return ok ? 0 : -1;
}

/* read_matrix_mm_to_dist (spmat/spmat_utils.upc:217-370) at THREADS = 1: the
 * banner's three words (matrix, coordinate, pattern or integer), the sizes,
 * then fscanf of "row col" (or "row col value") pairs, 1-based; row counts,
 * their prefix sums, and the columns appended to their rows in file order. */
int orc_read_mm(const char *path, int64_t *dims, int64_t *offset, int64_t *nonzero) {
  FILE *fp = fopen(path, "r");
  if (!fp) return -1;
  char object[64], format[64], field[64];
  int64_t nr, nc, nnz, row, col, val, pos = 0;
  int rc = -1;
  if (fscanf(fp, "%%%%MatrixMarket %63s %63s %63s\n", object, format, field) != 3) goto done;
  if (strcmp(object, "matrix") || strcmp(format, "coordinate")) goto done;
  const int integer = !strcmp(field, "integer");
  if (!integer && strcmp(field, "pattern")) goto done;
  if (fscanf(fp, "%ld %ld %ld\n", &nr, &nc, &nnz) != 3) goto done;
  if (!offset) {
    dims[0] = nr;
    dims[1] = nc;
    dims[2] = nnz;
    rc = 0;
    goto done;
  }
  int64_t *rows = (int64_t *)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(int64_t));
  int64_t *cols = (int64_t *)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(int64_t));
  if (!rows || !cols) { free(rows); free(cols); goto done; }
  for (int64_t i = 0; i <= nr; i++) offset[i] = 0;
  for (;;) {
    const int got = integer ? fscanf(fp, "%ld %ld %ld\n", &row, &col, &val) : fscanf(fp, "%ld %ld\n", &row, &col);
    if (got != (integer ? 3 : 2)) break;
    if (pos >= nnz || row < 1 || row > nr || col < 1 || col > nc) { pos = -1; break; }
    rows[pos] = row - 1;
    cols[pos++] = col - 1;
    offset[row]++;
  }
  if (pos == nnz) {
    for (int64_t i = 0; i < nr; i++) offset[i + 1] += offset[i];
    int64_t *fill = (int64_t *)malloc((size_t)(nr > 0 ? nr : 1) * sizeof(int64_t));
    if (fill) {
      memcpy(fill, offset, (size_t)nr * sizeof(int64_t));
      for (int64_t k = 0; k < nnz; k++) nonzero[fill[rows[k]]++] = cols[k];
      free(fill);
      rc = 0;
    }
  }
  free(rows);
  free(cols);
done:
  fclose(fp);
  return rc;
}
