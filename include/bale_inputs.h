/*
 * bale_inputs.h -- seeded host-side input generators of libbale_gb300.so.
 *
 * The reference draws its inputs with glibc rand() seeded per PE
 * (apps/histo_src/histo.upc:143-151, apps/ig_src/ig.upc:168-175) and builds
 * graphs with spmat's generators (spmat/spmat_utils.upc:612-691, :813-1049).
 * These generators produce the same KINDS of input from counter-based 64-bit
 * streams, so the GPU kernels and the CPU oracle receive identical buffers
 * and any size can be regenerated exactly.  The integer generators
 * (uniform, values, R-MAT, Kronecker) give the same bits on every machine;
 * the Zipf and Erdos-Renyi generators use libm log/exp and may differ in rare
 * samples across C libraries.
 *
 * Matrices are returned as one-PE sparsemat_t (offset == loffset,
 * nonzero == lnonzero) and freed with bale_free_matrix().
 */
#ifndef BALE_INPUTS_H
#define BALE_INPUTS_H

#include <stdint.h>
#include "bale_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Output i (i = 0, 1, ...) of the SplitMix64 stream started at seed. */
BALE_API uint64_t bale_splitmix64(uint64_t seed, uint64_t i);

/* out[i] = floor(splitmix64(seed, i) * range / 2^64), uniform in [0,range).
 * packed != 0 stores the reference's packed form (idx << 16) | 0
 * (apps/histo_src/histo.upc:150).  Returns BALE_OK or BALE_EINVAL. */
BALE_API int bale_gen_uniform(int64_t *out, int64_t n, int64_t range, uint64_t seed, int packed);

/* out[i] = (int64_t)splitmix64(seed, i): random 64-bit table values. */
BALE_API int bale_gen_values(int64_t *out, int64_t n, uint64_t seed);

/* The reference's ig self-check table: out[i] = -(i + 1) (apps/ig_src/ig.upc:158-161). */
BALE_API int bale_gen_negative_table(int64_t *out, int64_t n);

/* Zipf(s) over [0,range) mapped through a seeded permutation: rank r >= 0 is
 * drawn with P(r) proportional to (r+1)^-s (rejection-inversion sampling,
 * Hormann & Derflinger 1996) from stream seed_rank, then out[i] = perm(r),
 * where perm is a keyed bijection of [0,range) (a 4-round Feistel network
 * with cycle walking) keyed by seed_perm.  s > 0, s != 1. */
BALE_API int bale_gen_zipf(int64_t *out, int64_t n, int64_t range, double s, uint64_t seed_rank,
                  uint64_t seed_perm, int packed);
/* The permutation used by bale_gen_zipf: perm(r) for r in [0,range). */
BALE_API int64_t bale_keyed_perm(int64_t r, int64_t range, uint64_t key);

/* R-MAT graph (Chakrabarti, Zhan & Faloutsos 2004): 2^scale vertices,
 * edgefactor * 2^scale generated edges, quadrant probabilities (a,b,c,1-a-b-c).
 * Self-loops and duplicates are removed, the graph is symmetrised, vertices
 * are relabelled by descending degree (ties by original id; label 0 has the
 * highest degree), and the strictly lower triangle L is returned with
 * ascending columns per row. */
BALE_API sparsemat_t *bale_gen_rmat(int64_t scale, int64_t edgefactor, double a, double b, double c,
                           uint64_t seed);

/* Erdos-Renyi G(n,p), strictly lower triangle, by geometric skipping
 * (Batagelj & Brandes 2005, the method of spmat/spmat_utils.upc:612-691)
 * with uniforms from the SplitMix64 stream of seed. */
BALE_API sparsemat_t *bale_gen_erdos_renyi(int64_t n, double p, uint64_t seed);

/* Kronecker product of star graphs K_{1,m}, lower triangle, as the reference
 * builds it for `triangle -K "mode m1 m2 ..."` (apps/triangle_src/triangle.upc:
 * 252-299; spmat/spmat_utils.upc:813-1049): the specs are split in half, each
 * half becomes a local Kronecker product of stars, and the two are combined
 * into the strictly lower product.  mode 0/1/2 as in the reference. */
BALE_API sparsemat_t *bale_gen_kronecker(int mode, const int64_t *specs, int64_t nspecs);
/* The reference's closed-form triangle count for those graphs
 * (apps/triangle_src/triangle.upc:278-295); -1 for an unknown mode. */
BALE_API int64_t bale_kronecker_triangles(int mode, const int64_t *specs, int64_t nspecs);

/* Allocate an empty one-PE matrix (zeroed offsets, nnz nonzeros). */
BALE_API sparsemat_t *bale_make_matrix(int64_t numrows, int64_t numcols, int64_t nnz);
BALE_API void bale_free_matrix(sparsemat_t *m);

/* Device versions (asynchronous on stream; output in device memory), bit-  */
/* identical to bale_gen_uniform / bale_gen_values.                          */
BALE_API int bale_gen_uniform_dev(int64_t *d_out, int64_t n, int64_t range, uint64_t seed, int packed,
                                  void *stream);
BALE_API int bale_gen_values_dev(int64_t *d_out, int64_t n, uint64_t seed, void *stream);

/* Threads the generators may use (<= 0: all online CPUs).  Default: all. */
BALE_API void bale_set_host_threads(int nthreads);

#ifdef __cplusplus
}
#endif
#endif
