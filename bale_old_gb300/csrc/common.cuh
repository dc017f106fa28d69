// common.cuh -- shared device helpers and host plumbing for libbale_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "bale_gb300.h"

namespace bale {

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// Records a printf-style message as the calling thread's last error.
void set_error(const char *fmt, ...);
// Number of SMs of the current device (cached per device).
int num_sms();
// Current device ordinal (cached per call site use).
int current_device();

// Value of a named tuning knob (tune.cu); -1 means "launcher decides".
int64_t knob(const char *name);
int64_t knob_or(const char *name, int64_t dflt);
// Automatic choice of the region-partitioned kernels (tables beyond L2 with
// enough elements to amortise the passes); thresholds are tuning knobs.
bool ig_auto_partition(int64_t n, int64_t table_len);
bool histo_auto_partition(int64_t n, int64_t ncounts);

// Device-wide scratch words owned by the library (per device): the in-kernel
// bad-input counter and the triangle work cursor.  Allocated once.
struct DeviceScratch {
  unsigned long long *words;  // kScratchWords zero-initialised u64
};
constexpr int kScratchWords = 1024;
DeviceScratch *device_scratch();
// A fresh scratch word for a launch's work cursor (ring of kScratchWords - 8
// words per device; the caller zeroes it on its stream before use).
unsigned long long *next_cursor_word();
// k (<= 4) consecutive fresh scratch words, same ring and rules.
unsigned long long *next_cursor_words(int k);
// Grow-only workspace for kernels that need scratch memory, one per (device,
// stream): launches on one stream share it in stream order, launches on
// different streams get their own.  Growing it frees the old buffer, which
// waits for the device.  Returns nullptr (error set) on allocation failure.
void *device_workspace(size_t bytes, cudaStream_t stream);
// The launchers' choices, shared with the batched and serving planners so a
// planner that supplies its own workspace takes the same path:
// launch_histo's mode (0 shared memory, 1 aggregated, 2 plain, 3 partitioned)
// and whether launch_ig uses the region partition.
int histo_mode_for(int64_t n, int64_t ncounts, const int64_t *index);
bool ig_partition_for(int64_t n, int64_t table_len, const int64_t *tgt, const int64_t *index);

#define BALE_CUDA_OK(expr)                                                        \
  do {                                                                            \
    cudaError_t _e = (expr);                                                      \
    if (_e != cudaSuccess) {                                                      \
      ::bale::set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e),   \
                        __FILE__, __LINE__);                                      \
      return BALE_ECUDA;                                                          \
    }                                                                             \
  } while (0)

// Launch entry points used by the C ABI (all asynchronous on `stream`).
int launch_ig(int64_t *tgt, const int64_t *index, int64_t n, const int64_t *table,
              int64_t table_len, int shift, unsigned long long *bad, cudaStream_t stream);
int launch_histo(int64_t *counts, int64_t ncounts, const int64_t *index, int64_t n, int shift,
                 unsigned long long *bad, cudaStream_t stream);
int launch_triangle(const int64_t *offset, const int64_t *nonzero, int64_t numrows, int64_t nnz,
                    unsigned long long *count, unsigned long long *work,
                    unsigned long long *bad, cudaStream_t stream);
// Region-partitioned gather for tables larger than L2 (ig_part.cu).
size_t ig_part_workspace_bytes(int64_t n, int64_t table_len);
bool ig_part_supported(int64_t n, int64_t table_len);
// The region partition's layout: each request becomes one u32, its offset in
// a region of 2^kIgRegionBits table entries above its position in a chunk
// of 2^kIgChunkBits requests.
constexpr int kIgChunkBits = 11;
constexpr int kIgRegionBits = 32 - kIgChunkBits;
constexpr int64_t kIgMaxRegions = int64_t(1) << (32 - kIgRegionBits);  // tables up to 2^32 entries
// direct (optional): a device word from launch_ig_skew; when it reads 1 the
// partitioned kernels return at once and the caller's direct gather runs.
int launch_ig_partitioned(int64_t *tgt, const int64_t *index, int64_t n, const int64_t *table,
                          int64_t table_len, int shift, unsigned long long *bad, void *ws,
                          unsigned long long *cursor, cudaStream_t stream, const unsigned *direct = nullptr);
// *direct = 1 when a sample of the request stream repeats its table sectors
// at least repeat_pct percent of the time (a skewed stream).
int launch_ig_skew(const int64_t *index, int64_t n, int shift, int64_t table_len, int repeat_pct, unsigned *direct,
                   cudaStream_t stream);
// Histogram over the same region partition (tables beyond L2).
size_t histo_part_workspace_bytes(int64_t n, int64_t ncounts);
int launch_histo_partitioned(int64_t *counts, int64_t ncounts, const int64_t *index, int64_t n, int shift,
                             unsigned long long *bad, void *ws, unsigned long long *cursor,
                             cudaStream_t stream);
// Bitmap/search hybrid triangle counting (tri_hybrid.cu); needs numrows < 2^32.
size_t tri_hybrid_workspace_bytes(int64_t numrows, int64_t nnz);
// run_if (optional, here and in the wedge functions below): a device word;
// the kernels return at once unless it reads 0 (hybrid) or 1 (wedge), so a
// choice made on the device picks one of the two paths.
int launch_triangle_hybrid(const int64_t *offset, const int64_t *nonzero, int64_t numrows, int64_t nnz,
                           unsigned long long *count, unsigned long long *work, unsigned long long *bad,
                           void *ws, unsigned long long *words, int rows_per_fetch, cudaStream_t stream,
                           const unsigned *run_if = nullptr);
// A public batch instance is well formed (kind, shift, sizes, pointers).
bool instance_valid(const bale_instance_t &x);
// The two halves of the hybrid: prepare (u32 column copy + heavy-row list,
// once per graph) and run (heavy and light kernels; cursors[0..1] zeroed here).
int tri_hybrid_prepare(const int64_t *offset, const int64_t *nonzero, int64_t numrows, int64_t nnz,
                       uint32_t *col32, uint32_t *heavy, unsigned long long *nheavy, cudaStream_t stream,
                       const unsigned *run_if = nullptr);
int tri_hybrid_run(const int64_t *offset, const uint32_t *col32, const uint32_t *heavy,
                   const unsigned long long *nheavy, int64_t numrows, int64_t nnz, unsigned long long *count,
                   unsigned long long *work, unsigned long long *bad, unsigned long long *cursors,
                   int rows_per_fetch, cudaStream_t stream, const unsigned *run_if = nullptr);
// Wedge-probe triangle count (tri_wedge.cu), for fewer than 2^32 - 1 rows and
// about 2^32 nonzeros.  prepare builds the u32 column copy and the transpose
// into ws (tri_wedge_workspace_bytes) and adds malformed entries to *bad (may
// be NULL); run counts from a prepared ws (cursor: two device words, zeroed
// there); launch_triangle_wedge does both.
bool tri_wedge_supported(int64_t numrows, int64_t nnz);
size_t tri_wedge_workspace_bytes(int64_t numrows, int64_t nnz);
int tri_wedge_prepare(const int64_t *offset, const int64_t *nonzero, int64_t numrows, int64_t nnz, void *ws,
                      unsigned long long *bad, cudaStream_t stream, const unsigned *run_if = nullptr);
int tri_wedge_run(const int64_t *offset, const void *ws, int64_t numrows, int64_t nnz, unsigned long long *count,
                  unsigned long long *work, unsigned long long *cursor, cudaStream_t stream,
                  const unsigned *run_if = nullptr);
int launch_triangle_wedge(const int64_t *offset, const int64_t *nonzero, int64_t numrows, int64_t nnz,
                          unsigned long long *count, unsigned long long *work, unsigned long long *bad, void *ws,
                          unsigned long long *cursor, cudaStream_t stream, const unsigned *run_if = nullptr);
// Triangle alg 1 (sum over L's nonzeros (i,j) of |U_i and U_j|, tri_alg1.cu),
// L strictly lower and U strictly upper, both n x n:
//  * check: *bad += malformed rows of L and U (run first; the others index U
//    by L's columns);
//  * transposed: *found += nonzeros (i,j) of L with i in U's row j (U is L's
//    transpose when that is nnz(L) and nnz(U) = nnz(L));
//  * count: *count += the sum, *work += the U elements looked up.
int launch_triangle_alg1_check(const int64_t *loff, const int64_t *lcol, int64_t lnnz, const int64_t *uoff,
                               const int64_t *ucol, int64_t unnz, int64_t n, unsigned long long *bad,
                               cudaStream_t stream);
int launch_triangle_alg1_transposed(const int64_t *loff, const int64_t *lcol, const int64_t *uoff,
                                    const int64_t *ucol, int64_t n, unsigned long long *found, cudaStream_t stream);
int launch_triangle_alg1_count(const int64_t *loff, const int64_t *lcol, const int64_t *uoff, const int64_t *ucol,
                               int64_t n, unsigned long long *count, unsigned long long *work, cudaStream_t stream);
// n +1 L2 reductions at hashed positions of counts (the L2 reduction-rate probe).
int launch_l2_red_rate(int64_t *counts, int64_t ncounts, int64_t n, cudaStream_t stream);
// *mapped_dst = *src by a one-thread kernel (mapped_dst: the device alias of
// mapped pinned host memory).
int launch_copy_word(const unsigned long long *src, unsigned long long *mapped_dst, cudaStream_t stream);
// max over index[i] >> shift into *out (u64, must start at 0); negatives count as huge.
int launch_index_max(const int64_t *index, int64_t n, int shift, unsigned long long *out,
                     cudaStream_t stream);

// ---------------------------------------------------------------------------
// device side
// ---------------------------------------------------------------------------
#ifdef __CUDACC__
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// Streaming 16-byte load that does not allocate in L1 and is marked
// evict-first in L2 (the index stream is read once).
__device__ __forceinline__ longlong2 ld_stream_v2(const longlong2 *p) { return __ldcs(p); }
__device__ __forceinline__ int64_t ld_stream(const int64_t *p) {
  return __ldcs(reinterpret_cast<const long long *>(p));
}
// Streaming 16-byte store (evict-first): outputs are written once.
__device__ __forceinline__ void st_stream_v2(longlong2 *p, longlong2 v) { __stcs(p, v); }
__device__ __forceinline__ void st_stream(int64_t *p, int64_t v) {
  __stcs(reinterpret_cast<long long *>(p), static_cast<long long>(v));
}
// Read-only random 8-byte load: non-coherent path, no L1 allocation (a
// random table entry is never reused by the same SM soon enough).
__device__ __forceinline__ int64_t ld_table(const int64_t *p) {
  int64_t v;
  asm("ld.global.nc.L1::no_allocate.s64 %0, [%1];" : "=l"(v) : "l"(p));
  return v;
}
// L2 cache policies (createpolicy) and loads/stores that carry them.
__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t pol;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ uint64_t policy_evict_last() {
  uint64_t pol;
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ uint4 ld_v4_u32_pol(const uint4 *p, uint64_t pol) {
  uint4 v;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.u32 {%0,%1,%2,%3}, [%4], %5;"
      : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ longlong2 ld_v2_s64_pol(const longlong2 *p, uint64_t pol) {
  longlong2 v;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.s64 {%0,%1}, [%2], %3;"
      : "=l"(v.x), "=l"(v.y) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ uint32_t ld_u32_pol(const uint32_t *p, uint64_t pol) {
  uint32_t v;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ int64_t ld_s64_pol(const int64_t *p, uint64_t pol) {
  int64_t v;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.s64 %0, [%1], %2;" : "=l"(v) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ void st_v4_u32_pol(uint4 *p, uint4 v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v4.u32 [%0], {%1,%2,%3,%4}, %5;"
               ::"l"(p), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w), "l"(pol) : "memory");
}
__device__ __forceinline__ void st_v2_s64_pol(longlong2 *p, longlong2 v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v2.s64 [%0], {%1,%2}, %3;"
               ::"l"(p), "l"(v.x), "l"(v.y), "l"(pol) : "memory");
}
__device__ __forceinline__ void st_s64_pol(int64_t *p, int64_t v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.s64 [%0], %1, %2;" ::"l"(p), "l"(v), "l"(pol) : "memory");
}
__device__ __forceinline__ void st_u32_pol(uint32_t *p, uint32_t v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.u32 [%0], %1, %2;" ::"l"(p), "r"(v), "l"(pol) : "memory");
}

// Fire-and-forget 64-bit add performed at L2 (no return value).
__device__ __forceinline__ void red_add_u64(int64_t *p, unsigned long long v) {
  asm volatile("red.global.relaxed.gpu.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
#endif

}  // namespace bale
