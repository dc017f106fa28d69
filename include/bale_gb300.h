/*
 * bale_gb300.h -- C ABI of the GB300 (sm_103a) implementation of bale's
 * irregular-access core: histogram scatter-add (histo), index gather (ig)
 * and triangle counting on a strictly lower-triangular CSR (triangles).
 *
 * Two layers are exported from libbale_gb300.so:
 *
 *  1. Drop-ins with the reference's exact signatures.  An app that links this
 *     library instead of the reference kernels runs on one GPU unchanged.
 *     All pointers are HOST pointers (the reference's SHMEM build has
 *     SHARED == empty, libgetput/libgetput.h:151), the call is synchronous
 *     and returns the wall time in seconds of the whole call (copies
 *     included), like the reference's lgp_min_avg_max_d(...)->avg.
 *     -1.0 means failure (bad input or CUDA error), the reference's own
 *     failure return (apps/histo_src/histo_exstack.upc:58).  The message of
 *     the last failure is available from bale_last_error().
 *     Ownership follows the reference: the caller owns every array; histo
 *     ADDS into counts, ig OVERWRITES tgt, triangles write *count and *sr.
 *
 *  2. Device-resident entry points (bale_*_dev): device pointers, explicit
 *     sizes, a CUDA stream passed as void*, asynchronous.  Used for resident
 *     tables, batching and serving.
 *
 * Every index/offset is int64_t as in the reference.  Inputs are checked on
 * the device: an index outside its table, a column outside [0,row) or a
 * malformed row offset is skipped (ig writes 0 for it), counted, and reported
 * as BALE_EINPUT / -1.0 -- never an out-of-bounds access.
 */
#ifndef BALE_GB300_H
#define BALE_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define BALE_API __attribute__((visibility("default")))
#else
#define BALE_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* sparsemat_t: layout-identical to the reference (spmat/spmat.h:73-86).     */
/* With one PE, loffset/lnonzero are a plain CSR: int64[numrows+1] row       */
/* offsets and int64[nnz] column indices (pattern only, no values).          */
/* ------------------------------------------------------------------------ */
#ifndef spmat_INCLUDED
typedef struct sparsemat_t {
  int64_t local;     /* 0/1: local or distributed matrix */
  int64_t numrows;   /* total rows */
  int64_t lnumrows;  /* rows on this PE (== numrows with one PE) */
  int64_t numcols;   /* columns are in [0, numcols) */
  int64_t nnz;       /* total nonzeros */
  int64_t lnnz;      /* nonzeros on this PE */
  int64_t *offset;   /* global row offsets (== loffset with one PE) */
  int64_t *loffset;  /* row offsets, int64[lnumrows+1] */
  int64_t *nonzero;  /* global nonzeros (== lnonzero with one PE) */
  int64_t *lnonzero; /* column indices, int64[lnnz], ascending per row */
} sparsemat_t;
#endif

/* Status codes of the bale_* entry points. */
enum {
  BALE_OK = 0,
  BALE_EINVAL = 1,    /* bad argument (negative size, NULL pointer, ...) */
  BALE_EINPUT = 2,    /* input data out of range (index >= table, bad CSR) */
  BALE_ECUDA = 3,     /* a CUDA runtime call failed */
  BALE_ENOMEM = 4,    /* device or pinned allocation failed */
  BALE_ETIMEDOUT = 5, /* a bounded device-side wait gave up */
  BALE_EBUSY = 6      /* admission refused: not enough free device memory */
};

/* ======================= drop-ins: histogram ============================ */
/* apps/histo_src/histo.h:47 -- counts[index[i]] += 1 for i < len.          */
BALE_API double histo_agi(int64_t *index, int64_t len, int64_t *counts);
/* apps/histo_src/histo.h:48 -- pckindx[i] = (lindex << 16) | pe; with one  */
/* PE, lcounts[pckindx[i] >> 16] += 1.  buf_cnt (exstack buffer size) is    */
/* accepted and ignored: there is no message buffering on one GPU.          */
BALE_API double histo_exstack(int64_t *pckindx, int64_t len, int64_t *lcounts, int64_t buf_cnt);
/* apps/histo_src/histo.h:49 -- same contract as histo_exstack.             */
BALE_API double histo_exstack2(int64_t *pckindx, int64_t len, int64_t *lcounts, int64_t buf_cnt);
/* apps/histo_src/histo.h:50 -- same contract, without buf_cnt.             */
BALE_API double histo_conveyor(int64_t *pckindx, int64_t len, int64_t *lcounts);

/* ======================= drop-ins: index gather ========================= */
/* apps/ig_src/ig.h:49 -- tgt[i] = table[index[i]] for i < l_num_req.        */
BALE_API double ig_agi(int64_t *tgt, int64_t *index, int64_t l_num_req, int64_t *table);
/* apps/ig_src/ig.h:50 -- tgt[i] = ltable[pckindx[i] >> 16] (one PE).       */
BALE_API double ig_exstack(int64_t *tgt, int64_t *pckindx, int64_t l_num_req, int64_t *ltable, int64_t buf_cnt);
/* apps/ig_src/ig.h:51 -- same contract as ig_exstack.                     */
BALE_API double ig_exstack2(int64_t *tgt, int64_t *pckindx, int64_t l_num_req, int64_t *ltable, int64_t buf_cnt);
/* apps/ig_src/ig.h:52 -- same contract, without buf_cnt.                   */
BALE_API double ig_conveyor(int64_t *tgt, int64_t *pckindx, int64_t l_num_req, int64_t *ltable);

/* ======================= drop-ins: triangles ============================ */
/* apps/triangle_src/triangle.h:50 -- *count = sum over nonzeros L[i][j] of  */
/* |row_i(L) and row_j(L)| (each triangle once).  L must be strictly lower   */
/* triangular with ascending columns per row.  alg 0 and alg 1 give the same */
/* count; both are computed from L (U may be NULL).  *sr receives the number */
/* of row-j elements examined on the device (not a parity field).            */
BALE_API double triangle_agi(int64_t *count, int64_t *sr, sparsemat_t *L, sparsemat_t *U, int64_t alg);
/* apps/triangle_src/triangle.h:51 -- same contract; bufsiz ignored.        */
BALE_API double triangle_exstack_push(int64_t *count, int64_t *sr, sparsemat_t *L, sparsemat_t *U, int64_t alg, int64_t bufsiz);
/* apps/triangle_src/triangle.h:53 -- same contract; bufsiz ignored.        */
BALE_API double triangle_exstack2_push(int64_t *count, int64_t *sr, sparsemat_t *L, sparsemat_t *U, int64_t alg, int64_t bufsiz);
/* apps/triangle_src/triangle.h:54 -- same contract.                        */
BALE_API double triangle_convey_push(int64_t *count, int64_t *sr, sparsemat_t *L, sparsemat_t *U, int64_t alg);
/* apps/triangle_src/triangle.h:61 (the ALTERNATE model) -- same contract.  */
BALE_API double triangle_agi_iter(int64_t *count, int64_t *sr, sparsemat_t *L, sparsemat_t *U, int64_t alg);

/* ======================= library state ================================== */
/* Message describing the most recent failure on the calling thread ("" if */
/* none).  Replaces the reference's fprintf-and-exit error paths.          */
BALE_API const char *bale_last_error(void);
/* Facts about the current device, out[0..n): SM count, pageable host      */
/* memory access, ... via host page tables, concurrent managed access, L2   */
/* bytes, opt-in shared memory per block, host pointers usable for          */
/* registered memory, copy engines, unified addressing (-1 = unknown).      */
BALE_API int bale_device_caps(int64_t *out, int n);
/* Library version string. */
BALE_API const char *bale_version(void);
/* Release the cached device and pinned buffers the drop-ins keep between  */
/* calls (they are re-created on demand).                                  */
BALE_API void bale_release_buffers(void);

/* ======================= tuning knobs ==================================== */
/* Named launch knobs (e.g. "ig.unroll", "histo.mode", "tri.rows_per_fetch")  */
/* choose among kernel variants that compute identical results; -1 (the     */
/* default) lets the launcher pick by size class.  The autotuner sets them.  */
/* bale_tune_set returns BALE_EINVAL for an unknown name; bale_tune_get      */
/* returns -2 for one.                                                       */
BALE_API int bale_tune_set(const char *name, int64_t value);
BALE_API int64_t bale_tune_get(const char *name);
/* Apply a tuning file: one "name value" pair per line, '#' comments.        */
/* Returns the number of knobs applied, -1 if the file cannot be read.      */
BALE_API int bale_tune_load(const char *path);
BALE_API int bale_tune_count(void);
BALE_API const char *bale_tune_name(int i);

/* ======================= device-resident entry points =================== */
/* All pointers below are device pointers; stream is a cudaStream_t (NULL  */
/* = the legacy default stream).  The calls are asynchronous; a nonzero     */
/* return is an argument or launch error.  Data errors (out-of-range        */
/* indices, malformed CSR) are counted into *d_bad (one int64 in device     */
/* memory, may be NULL), which the kernels ADD to.                          */

/* counts[index[i] >> shift] += 1 for i < n (shift is 0, or 16 for packed   */
/* exstack indices).  Counters are int64, ncounts of them.                  */
BALE_API int bale_histo_dev(int64_t *d_counts, int64_t ncounts, const int64_t *d_index, int64_t n,
                   int shift, int64_t *d_bad, void *stream);
/* Measurement probe (no counterpart in the reference): n +1 reductions at  */
/* hashed positions of counts[ncounts], no index read -- the L2 reduction    */
/* rate that bounds a histogram whose table fits in L2.                     */
BALE_API int bale_l2_red_rate(int64_t *d_counts, int64_t ncounts, int64_t n, void *stream);
/* tgt[i] = table[index[i] >> shift] for i < n; out-of-range -> tgt[i] = 0. */
BALE_API int bale_ig_dev(int64_t *d_tgt, const int64_t *d_index, int64_t n, const int64_t *d_table,
                int64_t table_len, int shift, int64_t *d_bad, void *stream);
/* *d_count += triangle count of the strictly lower CSR (d_offset[n+1],     */
/* d_nonzero[nnz]); *d_work (may be NULL) += the kernels' work tally (the   */
/* default wedge kernels: elements probed, the reference's exstack pushes). */
/* With *d_bad raised the count is not meaningful.                          */
BALE_API int bale_triangle_dev(const int64_t *d_offset, const int64_t *d_nonzero, int64_t numrows,
                      int64_t nnz, int64_t *d_count, int64_t *d_work, int64_t *d_bad,
                      void *stream);
/* A graph counted repeatedly: bale_triangle_prepare validates the matrix    */
/* (malformed entries added to *d_bad) and builds its 32-bit column copy and */
/* transpose once, in device memory it owns (about 16 bytes per nonzero);   */
/* each bale_triangle_count_prepared then runs only the counting kernel.    */
/* d_offset/d_nonzero must stay valid and unchanged until release.  NULL on */
/* failure (bale_last_error).  New entry points; the reference counts once. */
typedef struct bale_tri_prepared bale_tri_prepared_t;
BALE_API bale_tri_prepared_t *bale_triangle_prepare(const int64_t *d_offset, const int64_t *d_nonzero,
                                                    int64_t numrows, int64_t nnz, int64_t *d_bad, void *stream);
BALE_API int bale_triangle_count_prepared(bale_tri_prepared_t *g, int64_t *d_count, int64_t *d_work, void *stream);
BALE_API void bale_triangle_release(bale_tri_prepared_t *g);

/* ======================= graph building on the device ================== */
/* The triangle kernels' input built in HBM: from an undirected edge list   */
/* (d_u[e], d_v[e] in [0,n); duplicates, both orientations and self loops   */
/* allowed) the strictly lower CSR of the simple graph, vertices relabelled */
/* by descending degree (ties by ascending label), columns ascending -- the */
/* reference's tidy lower matrix (spmat/spmat_utils.upc:455-473 tril,       */
/* :1055-1062 sort_nonzeros).  d_offset[n+1]; d_nonzero needs room for m    */
/* entries; *nnz receives the count.  Synchronous; BALE_EINPUT if an        */
/* endpoint is outside [0,n).  n <= 2^31, m < 2^32 - 1.  New entry points.   */
/* These, the transpose, the random permutations and the MatrixMarket       */
/* reader sort with a radix sort whose passes wait, bounded, on earlier     */
/* tiles: BALE_ETIMEDOUT if a wait gave up (the output is still exact; the  */
/* limit is the knob sort.lookback_spins).                                  */
BALE_API int bale_graph_build_dev(const int64_t *d_u, const int64_t *d_v, int64_t m, int64_t n,
                                  int64_t *d_offset, int64_t *d_nonzero, int64_t *nnz, void *stream);
/* Device scratch a build of m edges on n vertices takes (bytes). */
BALE_API int64_t bale_graph_build_workspace(int64_t m, int64_t n);
/* bale_gen_rmat's graph (include/bale_inputs.h) generated and built on the */
/* device, bit-identical: d_offset[2^scale + 1], d_nonzero room for          */
/* edgefactor * 2^scale entries.                                            */
BALE_API int bale_gen_rmat_dev(int64_t scale, int64_t edgefactor, double a, double b, double c,
                               uint64_t seed, int64_t *d_offset, int64_t *d_nonzero, int64_t *nnz,
                               void *stream);

/* spmat's transpose, permutation and random permutation on the device,    */
/* each bit-identical to the reference at one PE and synchronous:           */
/*  * bale_transpose_dev: transpose_matrix_agi (spmat/spmat_agi.upc:180-235);*/
/*    At is numcols x numrows, d_toffset[numcols+1], d_tnonzero[nnz], rows   */
/*    ascending within each row of At;                                      */
/*  * bale_permute_dev: permute_matrix_agi (spmat/spmat_agi.upc:119-173);    */
/*    row i of A goes to row rperminv[i], column j to cperminv[j], nonzeros  */
/*    keep their order; d_poffset[numrows+1], d_pnonzero[nnz];               */
/*  * bale_rand_perm_dev: rand_permp_agi(n, seed) (spmat/spmat_agi.upc:      */
/*    56-107): the permutation the reference's dart throwing yields from     */
/*    lrand48 after srand48(seed);                                          */
/*  * bale_rand_perm_exstack_dev: rand_permp_exstack(n, seed, buf_cnt)        */
/*    (spmat/spmat_exstack.upc:62-190), whose darts fly in rounds of buf_cnt; */
/*    rand_permp(n, seed) (spmat/spmat_utils.upc:63-74) is buf_cnt = 1024.    */
/*    A different permutation from rand_permp_agi's for the same seed.       */
/*  * bale_rand_perm_exstack2_dev: rand_permp_exstack2(n, seed, buf_cnt)     */
/*    (spmat/spmat_exstack2.upc:60-73), which in the reference returns       */
/*    rand_permp_exstack(n, seed, buf_cnt): the same permutation.            */
/* The random permutations take 0 <= n < 2^30.  Only the low 32 bits of     */
/* seed count (the reference's seed is an int).  As in the reference        */
/* (spmat_agi.upc:61, spmat_exstack.upc:92), a nonzero seed calls           */
/* srand48(seed) first and a zero one continues the C library's drand48     */
/* stream from wherever the caller left it; either way the call leaves that */
/* stream just past the reference's last draw, where a later lrand48() or a */
/* seed-0 call picks it up (the process's C library state, not thread-safe, */
/* like the reference's).                                                   */
/* BALE_EINPUT for malformed offsets or columns, or a rperminv/cperminv     */
/* that is not a permutation.                                               */
BALE_API int bale_transpose_dev(const int64_t *d_offset, const int64_t *d_nonzero, int64_t numrows,
                                int64_t numcols, int64_t nnz, int64_t *d_toffset, int64_t *d_tnonzero,
                                void *stream);
BALE_API int bale_permute_dev(const int64_t *d_offset, const int64_t *d_nonzero, int64_t numrows,
                              int64_t numcols, int64_t nnz, const int64_t *d_rperminv,
                              const int64_t *d_cperminv, int64_t *d_poffset, int64_t *d_pnonzero,
                              void *stream);
BALE_API int bale_rand_perm_dev(int64_t n, uint64_t seed, int64_t *d_perm, void *stream);
BALE_API int bale_rand_perm_exstack_dev(int64_t n, uint64_t seed, int64_t buf_cnt, int64_t *d_perm,
                                        void *stream);
BALE_API int bale_rand_perm_exstack2_dev(int64_t n, uint64_t seed, int64_t buf_cnt, int64_t *d_perm,
                                         void *stream);

/* MatrixMarket files of the reference's kind (spmat/spmat_utils.upc:128-149 */
/* write_matrix_mm, :217-370 read_matrix_mm_to_dist): "%%MatrixMarket matrix */
/* coordinate pattern" (or "integer", value ignored), "rows cols nnz", then  */
/* one 1-based "row col" line per nonzero.  bale_write_matrix_mm writes the   */
/* same bytes as the reference; bale_mm_header reads the banner and sizes   */
/* (comment lines after the banner are skipped); bale_read_matrix_mm_dev     */
/* parses the body on the device into d_offset[rows+1], d_nonzero[nnz],      */
/* keeping the file order of the nonzeros within each row, as the reference */
/* does.  BALE_EINPUT for an unreadable or malformed file.  Synchronous.     */
BALE_API int bale_write_matrix_mm(const sparsemat_t *A, const char *path);
BALE_API int bale_mm_header(const char *path, int64_t *numrows, int64_t *numcols, int64_t *nnz,
                            int64_t *body, int *fields);
BALE_API int bale_read_matrix_mm_dev(const char *path, int64_t *d_offset, int64_t *d_nonzero, void *stream);

/* Binary sparse matrix datasets (spmat/spmat_agi.upc:245-335               */
/* write_rowcounts / write_sparse_matrix_agi, spmat/spmat_exstack.upc:       */
/* 494-686 write_sparse_matrix_exstack, spmat/spmat_utils.upc:159-206 the    */
/* metadata file): a directory with "metadata" (numrows, numcols, nnz, the  */
/* number of writers W; one decimal per line) and per writer w "rowcnt_<w>"  */
/* and "nonzero_<w>" (raw int64 row lengths and columns of the w-th block of */
/* (numrows + W - w - 1) / W consecutive rows).  The reference at THREADS PEs */
/* writes W = THREADS.                                                      */
/*  * bale_write_sparse_matrix: the host matrix, W = 1: the same bytes as    */
/*    write_sparse_matrix_agi / _exstack at one PE;                         */
/*  * bale_write_sparse_matrix_dev: a device CSR (checked first), W writers;  */
/*    the copies overlap the file writes;                                   */
/*  * bale_sparse_matrix_header: the metadata file;                         */
/*  * bale_read_sparse_matrix_dev: any W, into d_offset[numrows+1] and       */
/*    d_nonzero[nnz] (the reference's reader is unfinished and compiled     */
/*    out); BALE_EINPUT unless the files, lengths and columns agree.         */
/*    numrows < 2^31, nnz < 2^32 - 1.                                       */
/* W <= 65536.  Synchronous.                                                */
BALE_API int bale_write_sparse_matrix(const char *dirname, const sparsemat_t *A);
BALE_API int bale_write_sparse_matrix_dev(const char *dirname, const int64_t *d_offset, const int64_t *d_nonzero,
                                          int64_t numrows, int64_t numcols, int64_t nnz, int64_t nwriters,
                                          void *stream);
BALE_API int bale_sparse_matrix_header(const char *dirname, int64_t *numrows, int64_t *numcols, int64_t *nnz,
                                       int64_t *nwriters);
BALE_API int bale_read_sparse_matrix_dev(const char *dirname, int64_t *d_offset, int64_t *d_nonzero,
                                         void *stream);

/* ======================= batched execution ============================== */
/* Many instances of uneven size in one CUDA graph: a persistent work-queue  */
/* kernel takes tiles of every instance (tile sizes per kind and size class  */
/* from the batch.* tuning knobs); ig/histo instances big enough for the     */
/* region-partitioned kernels run beside it on a second captured stream.     */
/* Create once (plans tasks, allocates the queue, captures the graph), run   */
/* any number of times, destroy.  Results equal the per-instance entry       */
/* points: histo ADDS into counts, ig OVERWRITES tgt, triangles ADD their     */
/* count into out[0].  The instances' device buffers must stay valid while   */
/* the batch exists.  New entry points; the reference has no batched form.   */
enum { BALE_KIND_HISTO = 0, BALE_KIND_IG = 1, BALE_KIND_TRIANGLES = 2 };
typedef struct bale_instance {
  int32_t kind;        /* BALE_KIND_* */
  int32_t shift;       /* 0, or 16 for the packed (index << 16) | pe form */
  int64_t n;           /* histo: updates; ig: requests; triangles: numrows */
  int64_t m;           /* histo: counters; ig: table entries; triangles: nnz */
  int64_t *out;        /* histo: counts; ig: tgt; triangles: one int64 */
  const int64_t *in;   /* histo, ig: index; triangles: row offsets[n+1] */
  const int64_t *aux;  /* ig: table; triangles: nonzeros[m]; histo: unused */
} bale_instance_t;
typedef struct bale_batch bale_batch_t;
/* NULL on failure (bale_last_error()). */
BALE_API bale_batch_t *bale_batch_create(const bale_instance_t *inst, int64_t count);
/* Launch the captured graph on stream (asynchronous). */
BALE_API int bale_batch_run(bale_batch_t *b, void *stream);
/* Out-of-range indices / malformed rows of the last run, per instance      */
/* (synchronous copy; count must equal the batch's instance count).         */
BALE_API int bale_batch_bad(bale_batch_t *b, int64_t *bad, int64_t count);
/* out[0..n): tasks, per-kind task counts (histo shared-memory, histo L2,   */
/* ig, triangle light, triangle heavy), standalone instances, instances,    */
/* side streams.                                                             */
BALE_API int bale_batch_stats(bale_batch_t *b, int64_t *out, int n);
/* side[k] = the side stream instance k runs on as its own kernels, or -1   */
/* when it goes through the work queue (count = the batch's instance count). */
BALE_API int bale_batch_plan(bale_batch_t *b, int64_t *side, int64_t count);
BALE_API void bale_batch_destroy(bale_batch_t *b);

/* ======================= serving loop =================================== */
/* Continuous batching of arriving requests against objects kept resident    */
/* in HBM (ig tables, histo counters, CSR graphs).  Registration and request */
/* admission are by free device memory.  bale_server_run replays a trace in  */
/* real time: requests are admitted as slots and arena space free up, cut    */
/* into the batched kernel's tasks, and run in "ticks" over a slice of every */
/* active request, so new requests join while long ones are running.  A    */
/* request large enough to fill the GPU alone runs as its own specialised   */
/* kernels on an express stream, beside the ticks.  Results are copied back */
/* as each request finishes.  New entry points; the                         */
/* reference has no serving form.                                           */
typedef struct bale_server bale_server_t;
typedef struct bale_request {
  int32_t kind;          /* BALE_KIND_* */
  int32_t object;        /* resident object id of the same kind */
  int32_t shift;         /* 0, or 16 for packed indices */
  int32_t reserved;
  int64_t n;             /* ig: requests; histo: updates; triangles: 0 */
  const int64_t *index;  /* host index array (ig, histo); pinned memory overlaps best */
  int64_t *out;          /* host: ig values[n]; triangles one int64; histo NULL */
  double arrival;        /* seconds after the start of bale_server_run */
} bale_request_t;
typedef struct bale_serve_stats {
  double makespan_s, p50_s, p99_s, mean_s, items_per_s;
  double gpu_busy_s;     /* sum of the ticks' and express kernels' device time */
  int64_t ticks, tasks, max_active, admission_waits, bad;
  int64_t loop_iters;    /* host scheduling iterations */
  int64_t express;       /* requests run as their own kernels on express streams */
} bale_serve_stats_t;
/* arena_bytes for per-request buffers (<= 0: a quarter of free HBM);       */
/* max_active requests in flight (<= 0: 64).  NULL on failure.               */
BALE_API bale_server_t *bale_server_create(int64_t arena_bytes, int max_active);
/* Register resident objects; return the object id (>= 0) or -status        */
/* (-BALE_EBUSY when free HBM would drop below the reserve).                */
BALE_API int bale_server_add_table(bale_server_t *s, const int64_t *host_table, int64_t n);
BALE_API int bale_server_add_counts(bale_server_t *s, int64_t ncounts);
BALE_API int bale_server_add_graph(bale_server_t *s, const int64_t *offset, const int64_t *nonzero,
                                   int64_t numrows, int64_t nnz);
BALE_API int bale_server_read_counts(bale_server_t *s, int object, int64_t *host_counts, int64_t ncounts);
/* Run the trace; latency[r] receives request r's seconds from arrival to   */
/* completion; stats may be NULL.  Histo requests add into their counters.  */
BALE_API int bale_server_run(bale_server_t *s, const bale_request_t *req, int64_t nreq, double *latency,
                             bale_serve_stats_t *stats);
BALE_API void bale_server_destroy(bale_server_t *s);

/* ======================= no-allocation gather =========================== */
/* No counterpart in the reference: an addition for callers that cannot      */
/* allocate device memory when they call (HBM already reserved by another    */
/* allocator, or a loop that cannot take cudaMalloc/cudaFree's implicit      */
/* synchronisation).  Same result as bale_ig_dev, computed by the region-    */
/* partitioned gather with its scratch in a fixed device array inside the    */
/* library (3.5 MiB = 3,670,784 bytes, held by every GPU that loads the      */
/* library until exit).  Limits: n <= 262144 requests per call (larger n ->  */
/* BALE_EINVAL with a message), table_len <= 2^32, d_index and d_tgt         */
/* 16-byte aligned.  The first call on a device looks up the array's address */
/* and caches it for the process (one context per device: do not call it    */
/* again on a device after cudaDeviceReset); make it before any stream       */
/* capture.  The stream must belong to the current device.  All calls share  */
/* the array: calls that overlap on the GPU race and must be serialised by   */
/* the caller.                                                               */
BALE_API int bale_ig_dev_noalloc(int64_t *d_tgt, const int64_t *d_index, int64_t n, const int64_t *d_table,
                                 int64_t table_len, int shift, int64_t *d_bad, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* BALE_GB300_H */
