/*
 * Single-PE OpenSHMEM stand-in -- TEST INFRASTRUCTURE ONLY.
 *
 * Lets the reference's own SHMEM-mode C sources (libgetput, exstack,
 * exstack2, spmat, the histo/ig/triangle kernels) compile with plain gcc so
 * that they can act as the parity oracle.  With one processing element every
 * symmetric-heap access is local, so:
 *   - shmem_n_pes() == 1, shmem_my_pe() == 0;
 *   - shmem_malloc is calloc (zeroed, so runs are reproducible);
 *   - puts and gets are memmove of nelems * element size;
 *   - atomics are plain local read-modify-writes;
 *   - the *_to_all reductions copy source to target;
 *   - barriers and quiet are no-ops.
 * The semantics follow the OpenSHMEM 1.4 specification for PE_size == 1.
 * Nothing in the shipped library includes this file.
 */
#ifndef BALE_ORACLE_SHIM_SHMEM_H
#define BALE_ORACLE_SHIM_SHMEM_H

#include <stdlib.h>
#include <string.h>
#include <stddef.h>

#define _SHMEM_REDUCE_MIN_WRKDATA_SIZE 16
#define _SHMEM_REDUCE_SYNC_SIZE 16
#define _SHMEM_BCAST_SYNC_SIZE 16
#define _SHMEM_SYNC_VALUE 0L
#define SHMEM_REDUCE_MIN_WRKDATA_SIZE _SHMEM_REDUCE_MIN_WRKDATA_SIZE
#define SHMEM_REDUCE_SYNC_SIZE _SHMEM_REDUCE_SYNC_SIZE
#define SHMEM_SYNC_VALUE _SHMEM_SYNC_VALUE

static inline void shmem_init(void) {}
static inline void shmem_finalize(void) {}
static inline int shmem_n_pes(void) { return 1; }
static inline int shmem_my_pe(void) { return 0; }
static inline void shmem_barrier_all(void) {}
static inline void shmem_quiet(void) {}
static inline void shmem_fence(void) {}
static inline void shmem_global_exit(int status) { exit(status); }

static inline void *shmem_malloc(size_t size) { return calloc(size ? size : 1, 1); }
static inline void shmem_free(void *p) { free(p); }
static inline void *shmem_align(size_t alignment, size_t size) {
  void *p = NULL;
  if (posix_memalign(&p, alignment < sizeof(void *) ? sizeof(void *) : alignment, size ? size : 1))
    return NULL;
  memset(p, 0, size);
  return p;
}

#define BALE_SHIM_COPY(NAME, ELEM)                                              \
  static inline void NAME(void *dst, const void *src, size_t nelems, int pe) {  \
    (void)pe;                                                                   \
    memmove(dst, src, nelems * (ELEM));                                         \
  }
BALE_SHIM_COPY(shmem_putmem, 1)
BALE_SHIM_COPY(shmem_put32, 4)
BALE_SHIM_COPY(shmem_put64, 8)
BALE_SHIM_COPY(shmem_put128, 16)
BALE_SHIM_COPY(shmem_getmem, 1)
BALE_SHIM_COPY(shmem_get32, 4)
BALE_SHIM_COPY(shmem_get64, 8)
BALE_SHIM_COPY(shmem_get128, 16)
#undef BALE_SHIM_COPY

static inline void shmem_long_add(long *dest, long value, int pe) { (void)pe; *dest += value; }
static inline long shmem_long_fadd(long *dest, long value, int pe) {
  (void)pe; long old = *dest; *dest += value; return old;
}
static inline long shmem_long_finc(long *dest, int pe) {
  (void)pe; long old = *dest; *dest += 1; return old;
}
static inline long shmem_long_cswap(long *dest, long cond, long value, int pe) {
  (void)pe; long old = *dest; if (old == cond) *dest = value; return old;
}
static inline void shmem_longlong_p(long long *addr, long long value, int pe) { (void)pe; *addr = value; }
static inline long long shmem_longlong_g(const long long *addr, int pe) { (void)pe; return *addr; }

#define BALE_SHIM_REDUCE(NAME, T)                                               \
  static inline void NAME(T *target, const T *source, int nreduce, int PE_start, \
                          int logPE_stride, int PE_size, T *pWrk, long *pSync) { \
    (void)PE_start; (void)logPE_stride; (void)PE_size; (void)pWrk; (void)pSync;  \
    memmove(target, source, (size_t)nreduce * sizeof(T));                        \
  }
BALE_SHIM_REDUCE(shmem_long_sum_to_all, long)
BALE_SHIM_REDUCE(shmem_long_min_to_all, long)
BALE_SHIM_REDUCE(shmem_long_max_to_all, long)
BALE_SHIM_REDUCE(shmem_double_sum_to_all, double)
BALE_SHIM_REDUCE(shmem_double_min_to_all, double)
BALE_SHIM_REDUCE(shmem_double_max_to_all, double)
BALE_SHIM_REDUCE(shmem_int_or_to_all, int)
#undef BALE_SHIM_REDUCE

#endif
