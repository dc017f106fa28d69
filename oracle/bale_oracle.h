/*
 * bale_oracle.h -- CPU restatement of bale's histo / ig / triangles kernels.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity checker for the GPU library
 * and the source of the timed CPU baseline; nothing in the shipped library
 * links or calls it.  Every function restates one reference routine at one
 * processing element (THREADS == 1) and cites the file:line it follows.
 * The restatement is pinned against the reference itself (oracle/_ref,
 * compiled from the reference's unmodified sources) through the golden
 * vectors in tests/golden/.
 *
 * The *_mt variants split the same loops over host threads (pthreads) for
 * the multi-core CPU baseline; their results are identical to the serial
 * ones (integer sums are order-free).
 */
#ifndef BALE_ORACLE_H
#define BALE_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* histo: counts[index[i]] += 1 (apps/histo_src/histo_agi.upc:61-66). */
void orc_histo_agi(const int64_t *index, int64_t n, int64_t *counts);
/* histo, packed indices: lcounts[pckindx[i] >> 16]++ (apps/histo_src/histo_exstack.upc:64-76). */
void orc_histo_exstack(const int64_t *pckindx, int64_t n, int64_t *lcounts);
/* ig: tgt[i] = table[index[i]] (apps/ig_src/ig_agi.upc:61-64). */
void orc_ig_agi(int64_t *tgt, const int64_t *index, int64_t n, const int64_t *table);
/* ig, packed request/response: tgt[j] = ltable[pckindx[j] >> 16] (apps/ig_src/ig_exstack.upc:69-94). */
void orc_ig_exstack(int64_t *tgt, const int64_t *pckindx, int64_t n, const int64_t *ltable);

/* The exstack variants at one PE with their buffers: every package goes
 * through a buf_cnt-package send buffer, an exchange and FIFO pops
 * (exstack/exstack.upc:163-340), as in apps/histo_src/histo_exstack.upc:52-86,
 * apps/ig_src/ig_exstack.upc:54-102 and apps/triangle_src/triangle_exstack.upc:
 * 95-168.  The triangle one takes rows row0, row0 + row_step, ... only.
 * -1 when the buffers cannot be allocated or an argument is out of range. */
int orc_histo_exstack_buffered(const int64_t *pckindx, int64_t n, int64_t *lcounts, int64_t buf_cnt);
int orc_ig_exstack_buffered(int64_t *tgt, const int64_t *pckindx, int64_t n, const int64_t *ltable,
                            int64_t buf_cnt);
int64_t orc_triangle_exstack_push_buffered(const int64_t *offset, const int64_t *nonzero, int64_t numrows,
                                           int64_t bufsiz, int64_t row0, int64_t row_step, int64_t *pushed);
/* triangles alg 0, the AGI loop over rows row0, row0 + row_step, ... only. */
int64_t orc_triangle_agi_sampled(const int64_t *offset, const int64_t *nonzero, int64_t numrows, int64_t row0,
                                 int64_t row_step);

/* triangles alg 0, AGI merge scan (apps/triangle_src/triangle_agi.upc:69-99).
 * Returns the count; *pulled gets the reference's "shared refs" tally.      */
int64_t orc_triangle_agi(const int64_t *offset, const int64_t *nonzero, int64_t numrows,
                         int64_t *pulled);
/* triangles alg 0, exstack push (apps/triangle_src/triangle_exstack.upc:61-82, :108-133).
 * *pushed gets the number of wedge packages pushed.                          */
int64_t orc_triangle_exstack_push(const int64_t *offset, const int64_t *nonzero,
                                  int64_t numrows, int64_t *pushed);
/* triangles alg 1, AGI scan of U (apps/triangle_src/triangle_agi.upc:100-136):
 * sum over L's nonzeros (i,j) of |U_i and U_j|; *pulled gets the reference's
 * shared-reference tally; -1 for a NULL U. */
int64_t orc_triangle_agi_alg1(const int64_t *loff, const int64_t *lcol, int64_t n, const int64_t *uoff,
                              const int64_t *ucol, int64_t unnz, int64_t *pulled);
/* Work model printed by the reference app (apps/triangle_src/triangle.upc:325-361):
 * pulls = sum_i deg(i) * colcount(i), pushes = sum_i C(deg(i), 2).            */
void orc_triangle_work(const int64_t *offset, const int64_t *nonzero, int64_t numrows,
                       int64_t *pulls, int64_t *pushes);
/* Structural check of L (spmat/spmat_utils.upc:377-409 with unit_diagonal 0,
 * plus the tidiness the kernels rely on): 1 if strictly lower and sorted.   */
int orc_is_strict_lower_tidy(const int64_t *offset, const int64_t *nonzero, int64_t numrows);

/* Multi-threaded variants for the CPU baseline (nthreads <= 0: all cores). */
void orc_histo_agi_mt(const int64_t *index, int64_t n, int64_t *counts, int nthreads);
void orc_ig_agi_mt(int64_t *tgt, const int64_t *index, int64_t n, const int64_t *table, int nthreads);
int64_t orc_triangle_agi_mt(const int64_t *offset, const int64_t *nonzero, int64_t numrows,
                            int nthreads);
int orc_num_cpus(void);

/* Seeded inputs for the timed CPU reference arm, so that it never loads the
 * GPU library: SplitMix64 (Steele, Lea & Flood 2014) with output i =
 * mix(seed + (i+1) * 0x9E3779B97F4A7C15), the counter layout the GPU
 * library's generators use.  Uniform indices in [0, range) are the high 64
 * bits of output * range (range > 0); values are the outputs themselves.
 * Split over nthreads host threads (<= 0: all cores); same buffers for any
 * thread count.  tests/test_oracle.py pins both to the library's buffers. */
void orc_gen_uniform(int64_t *out, int64_t n, int64_t range, uint64_t seed, int nthreads);
void orc_gen_values(int64_t *out, int64_t n, uint64_t seed, int nthreads);

/* spmat_agi.upc:180-235 transpose_matrix_agi at one PE: At is numcols x
 * numrows; toffset[numcols+1], tnonzero[nnz].  Returns 0, or -1 for a column
 * outside [0, numcols). */
int orc_transpose(const int64_t *offset, const int64_t *nonzero, int64_t numrows, int64_t numcols,
                  int64_t *toffset, int64_t *tnonzero);
/* spmat_agi.upc:119-173 permute_matrix_agi at one PE: row i of A goes to row
 * rperminv[i], column j to cperminv[j]; nonzeros keep their order in the row. */
void orc_permute(const int64_t *offset, const int64_t *nonzero, int64_t numrows, const int64_t *rperminv,
                 const int64_t *cperminv, int64_t *poffset, int64_t *pnonzero);
/* spmat_agi.upc:56-107 rand_permp_agi at one PE: darts from lrand48 after
 * srand48(seed) into 2n slots, first hits kept, slots read in order. */
int orc_rand_perm(int64_t n, int64_t seed, int64_t *perm);
/* spmat_exstack.upc:62-190 rand_permp_exstack at one PE with buf_cnt-package
 * buffers (rand_permp, spmat_utils.upc:63-74, uses 1024). */
int orc_rand_perm_exstack(int64_t n, int64_t seed, int64_t buf_cnt, int64_t *perm);
/* spmat_agi.upc:286-335 write_sparse_matrix_agi at one PE: dirname/metadata,
 * rowcnt_0 and nonzero_0. */
int orc_write_dataset(const char *dirname, const int64_t *offset, const int64_t *nonzero, int64_t numrows,
                      int64_t numcols);
/* spmat_utils.upc:217-370 read_matrix_mm_to_dist at one PE: header sizes into
 * dims[3] (rows, cols, nnz) when offset is NULL; otherwise the CSR (file
 * order kept within each row).  Returns 0, or -1 for a file it rejects. */
int orc_read_mm(const char *path, int64_t *dims, int64_t *offset, int64_t *nonzero);

#ifdef __cplusplus
}
#endif
#endif
