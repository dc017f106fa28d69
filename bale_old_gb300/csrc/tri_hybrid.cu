// tri_hybrid.cu -- triangle counting, bitmap/search hybrid over rows i (tri.mode 1;
// also the path for matrices beyond the wedge kernels' 32-bit limits).
//
// Same count as apps/triangle_src/triangle_agi.upc:69-99 (alg 0): for every
// nonzero L[i][j] after the first of row i, |row_i and row_j|.  The rows of a
// degree-ordered L are long exactly where the work is (a hub's row holds its
// higher-degree neighbours, hundreds of them), so the two sides of each
// intersection are handled by size (tri_device.cuh):
//
//  * heavy rows (label below 2^19 and at least 64 nonzeros): one CTA per row.
//    Row i becomes a bitmap over [0,i) in shared memory; each warp streams
//    whole rows j (16-byte loads from a u32 copy of the column array) and
//    tests every element against the bitmap -- one shared-memory load per
//    element instead of a binary search.  The bits are cleared by row i's own
//    columns before the next row, so the bitmap is never swept;
//  * light rows: one warp per row, row i staged in shared memory.  For each
//    neighbour j the cheaper side is searched: either row j is streamed and
//    each element is binary-searched in the part of row i before j, or each
//    element of that part of row i is binary-searched in row j.
//
// Launch sequence: convert (int64 columns -> u32), classify (heavy-row list),
// heavy kernel (rows from the list), light kernel (all other rows).
// The work tally counts row-j elements streamed plus binary-search probes.
// Validation: bad offsets, columns outside [0,i) or non-ascending rows are
// counted in *bad and the row is skipped.
#include "tri_device.cuh"

namespace bale {

namespace {

using tri::kBadCol;
using tri::kFull;
constexpr int kHeavyThreads = 512;
constexpr int kLightThreads = 256;
constexpr int kLightWarps = kLightThreads / 32;

__global__ void __launch_bounds__(256)
    tri_convert_kernel(const int64_t *__restrict__ col, int64_t nnz, uint32_t *__restrict__ col32, const unsigned *__restrict__ run_if) {
  if (tri::skipped(run_if, 0u)) return;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < nnz; k += stride) {
    const int64_t c = ld_stream(col + k);
    col32[k] = (c < 0 || c >= static_cast<int64_t>(kBadCol)) ? kBadCol : static_cast<uint32_t>(c);
  }
}

__global__ void __launch_bounds__(256)
    tri_classify_kernel(const int64_t *__restrict__ off, int64_t n, int64_t bits,
                        uint32_t *__restrict__ heavy, unsigned long long *__restrict__ nheavy, const unsigned *__restrict__ run_if) {
  if (tri::skipped(run_if, 0u)) return;
  const int64_t lim = n < bits ? n : bits;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t base = static_cast<int64_t>(blockIdx.x) * blockDim.x; base < lim; base += stride) {
    const int64_t i = base + threadIdx.x;
    const bool h = i < lim && tri::is_heavy(i, off[i], off[i + 1], bits);
    const unsigned m = __ballot_sync(kFull, h);
    unsigned long long slot = 0;
    if (lane_id() == 0 && m) slot = atomicAdd(nheavy, static_cast<unsigned long long>(__popc(m)));
    slot = __shfl_sync(kFull, slot, 0);
    if (h) heavy[slot + __popc(m & ((1u << lane_id()) - 1u))] = static_cast<uint32_t>(i);
  }
}

__device__ __forceinline__ void flush_tally(tri::Tally t, unsigned long long *count, unsigned long long *work,
                                            unsigned long long *bad) {
  t.cnt = warp_sum_u64(t.cnt);
  t.work = warp_sum_u64(t.work);
  t.bad = warp_sum_u64(t.bad);
  if (lane_id() == 0) {
    if (t.cnt) atomicAdd(count, t.cnt);
    if (t.work && work) atomicAdd(work, t.work);
    if (t.bad) atomicAdd(bad, t.bad);
  }
}

__global__ void __launch_bounds__(kHeavyThreads, 3)
    tri_heavy_kernel(const int64_t *__restrict__ off, const uint32_t *__restrict__ col, int64_t nnz,
                     const uint32_t *__restrict__ heavy, const unsigned long long *__restrict__ nheavy_p,
                     int64_t bits, unsigned long long *__restrict__ count, unsigned long long *__restrict__ work,
                     unsigned long long *__restrict__ bad, unsigned long long *__restrict__ cursor, const unsigned *__restrict__ run_if) {
  if (tri::skipped(run_if, 0u)) return;
  extern __shared__ uint32_t bm[];
  __shared__ long long sel;
  const int64_t nwords = bits >> 5;  // bits is a power of two >= 32
  const uint32_t wmask = static_cast<uint32_t>(nwords - 1);
  const unsigned long long nheavy = *nheavy_p;
  for (int64_t w = threadIdx.x; w < nwords; w += kHeavyThreads) bm[w] = 0;
  tri::Tally t;
  for (;;) {
    __syncthreads();  // sel may be rewritten
    if (threadIdx.x == 0) {
      const unsigned long long r = atomicAdd(cursor, 1ull);
      sel = r < nheavy ? static_cast<long long>(heavy[r]) : -1ll;
    }
    __syncthreads();
    const long long i = sel;
    if (i < 0) break;
    tri::heavy_row<uint32_t, kHeavyThreads>(off, col, i, nnz, bm, wmask, t);
  }
  flush_tally(t, count, work, bad);
}

__global__ void __launch_bounds__(kLightThreads)
    tri_light_kernel(const int64_t *__restrict__ off, const uint32_t *__restrict__ col, int64_t n, int64_t nnz,
                     int64_t bits, unsigned long long *__restrict__ count, unsigned long long *__restrict__ work,
                     unsigned long long *__restrict__ bad, unsigned long long *__restrict__ cursor,
                     int rows_per_fetch, const unsigned *__restrict__ run_if) {
  if (tri::skipped(run_if, 0u)) return;
  __shared__ uint32_t rowbuf[kLightWarps][tri::kLightCap];
  uint32_t *rb = rowbuf[threadIdx.x >> 5];
  tri::Tally t;
  for (;;) {
    unsigned long long r0 = 0;
    if (lane_id() == 0) r0 = atomicAdd(cursor, static_cast<unsigned long long>(rows_per_fetch));
    r0 = __shfl_sync(kFull, r0, 0);
    if (r0 >= static_cast<unsigned long long>(n)) break;
    const int64_t r1 = static_cast<int64_t>(r0) + rows_per_fetch < n ? static_cast<int64_t>(r0) + rows_per_fetch : n;
    for (int64_t i = static_cast<int64_t>(r0); i < r1; i++) tri::light_row(off, col, i, nnz, bits, rb, t);
  }
  flush_tally(t, count, work, bad);
}

bool g_heavy_attr[64];

}  // namespace

size_t tri_hybrid_workspace_bytes(int64_t numrows, int64_t nnz) {
  const int64_t lim = numrows < tri::kHeavyBits ? numrows : tri::kHeavyBits;
  return ((static_cast<size_t>(nnz > 0 ? nnz : 1) * sizeof(uint32_t) + 255) & ~size_t(255)) +
         static_cast<size_t>(lim > 0 ? lim : 1) * sizeof(uint32_t);
}

int tri_hybrid_prepare(const int64_t *offset, const int64_t *nonzero, int64_t numrows, int64_t nnz,
                       uint32_t *col32, uint32_t *heavy, unsigned long long *nheavy, cudaStream_t stream,
                       const unsigned *run_if) {
  const int sms = num_sms();
  const int64_t bits = tri::bitmap_bits(numrows);
  BALE_CUDA_OK(cudaMemsetAsync(nheavy, 0, sizeof(unsigned long long), stream));
  if (nnz > 0) {
    int64_t blocks = (nnz + 255) / 256, cap = static_cast<int64_t>(sms) * 8;
    tri_convert_kernel<<<static_cast<unsigned>(blocks < cap ? blocks : cap), 256, 0, stream>>>(nonzero, nnz, col32,
                                                                                           run_if);
    BALE_CUDA_OK(cudaGetLastError());
  }
  const int64_t lim = numrows < bits ? numrows : bits;
  int64_t blocks = (lim + 255) / 256, cap = static_cast<int64_t>(sms) * 8;
  if (blocks < 1) blocks = 1;
  tri_classify_kernel<<<static_cast<unsigned>(blocks < cap ? blocks : cap), 256, 0, stream>>>(
      offset, numrows, bits, heavy, nheavy, run_if);
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

int tri_hybrid_run(const int64_t *offset, const uint32_t *col32, const uint32_t *heavy,
                   const unsigned long long *nheavy, int64_t numrows, int64_t nnz, unsigned long long *count,
                   unsigned long long *work, unsigned long long *bad, unsigned long long *cursors,
                   int rows_per_fetch, cudaStream_t stream, const unsigned *run_if) {
  const int sms = num_sms();
  const int64_t bits = tri::bitmap_bits(numrows);
  BALE_CUDA_OK(cudaMemsetAsync(cursors, 0, 2 * sizeof(unsigned long long), stream));
  {
    const size_t smem = static_cast<size_t>(bits / 32) * sizeof(uint32_t);
    const int dev = current_device();
    if (dev >= 0 && dev < 64 && !g_heavy_attr[dev]) {
      BALE_CUDA_OK(cudaFuncSetAttribute(tri_heavy_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>((tri::kHeavyBits / 32) * sizeof(uint32_t))));
      g_heavy_attr[dev] = true;
    }
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, tri_heavy_kernel, kHeavyThreads, smem) != cudaSuccess ||
        occ < 1)
      occ = 1;
    tri_heavy_kernel<<<static_cast<unsigned>(sms * occ), kHeavyThreads, smem, stream>>>(
        offset, col32, nnz, heavy, nheavy, bits, count, work, bad, cursors, run_if);
    BALE_CUDA_OK(cudaGetLastError());
  }
  {
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, tri_light_kernel, kLightThreads, 0) != cudaSuccess ||
        occ < 1)
      occ = 1;
    int64_t blocks = static_cast<int64_t>(sms) * occ;
    const int64_t need = ((numrows + rows_per_fetch - 1) / rows_per_fetch + kLightWarps - 1) / kLightWarps;
    if (blocks > need) blocks = need > 0 ? need : 1;
    tri_light_kernel<<<static_cast<unsigned>(blocks), kLightThreads, 0, stream>>>(
        offset, col32, numrows, nnz, bits, count, work, bad, cursors + 1, rows_per_fetch, run_if);
    BALE_CUDA_OK(cudaGetLastError());
  }
  return BALE_OK;
}

int launch_triangle_hybrid(const int64_t *offset, const int64_t *nonzero, int64_t numrows, int64_t nnz,
                           unsigned long long *count, unsigned long long *work, unsigned long long *bad,
                           void *ws, unsigned long long *words, int rows_per_fetch, cudaStream_t stream,
                           const unsigned *run_if) {
  // words: [0] heavy-list length, [1] heavy cursor, [2] light cursor
  char *p = static_cast<char *>(ws);
  uint32_t *col32 = reinterpret_cast<uint32_t *>(p);
  p += (static_cast<size_t>(nnz > 0 ? nnz : 1) * sizeof(uint32_t) + 255) & ~size_t(255);
  uint32_t *heavy = reinterpret_cast<uint32_t *>(p);
  int rc = tri_hybrid_prepare(offset, nonzero, numrows, nnz, col32, heavy, words, stream, run_if);
  if (rc != BALE_OK) return rc;
  return tri_hybrid_run(offset, col32, heavy, words, numrows, nnz, count, work, bad, words + 1, rows_per_fetch,
                        stream, run_if);
}

}  // namespace bale
