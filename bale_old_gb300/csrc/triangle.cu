// triangle.cu -- exact triangle count of a strictly lower-triangular CSR L:
//   count = sum over nonzeros L[i][j] of |row_i(L) and row_j(L)|
// (apps/triangle_src/triangle_agi.upc:69-99, alg 0).  Every element w of
// row j is < j, and row i is ascending, so each triangle k < j < i is found
// exactly once: when row j's element k is matched inside row i.
//
// GPU layout of the work ("pull" form of the reference's AGI variant):
//  * a warp owns a row i at a time, fetched dynamically in small groups of
//    rows from a device cursor (row work is very uneven on skewed graphs);
//  * row i is staged in the warp's slice of shared memory (as u32 when the
//    matrix has < 2^32 rows), so each probe costs shared-memory loads only;
//  * the neighbours j of row i are taken 32 at a time; a warp prefix sum over
//    their row lengths flattens the concatenation of those rows so that
//    consecutive lanes read consecutive elements of row j (coalesced), and
//    each lane binary-searches its element in the prefix of row i that lies
//    before j;
//  * counts accumulate per lane in u64, then one atomic per warp.
// The first element of row i is skipped as in the reference (it has no
// smaller partner in row i).  Inputs are validated on the fly: a malformed
// row offset, a column outside [0,i) or a non-ascending row is counted in
// *bad and skipped, so no access ever leaves the arrays.
//
// This file also holds launch_triangle, which dispatches tri.mode 0 (this
// merge kernel), 1 (tri_hybrid.cu), 2 (tri_wedge.cu) and the default, whose
// per-graph choice between wedges and the hybrid is made on the device
// (tri_choose_kernel below).
#include "common.cuh"

namespace bale {

namespace {

constexpr int kTriThreads = 256;
constexpr int kTriWarps = kTriThreads / 32;
constexpr int kTriCap = 1024;      // row-i elements cached per warp
constexpr int kRowsPerFetchDefault = 16;  // rows claimed per cursor increment
constexpr unsigned kFull = 0xffffffffu;

// Is w in the ascending u32 run rs[0,len) (shared memory)?
__device__ __forceinline__ bool probe_smem(const uint32_t *__restrict__ rs, int64_t len, int64_t w) {
  if (w < 0 || w > 0xffffffffll) return false;
  const uint32_t ww = static_cast<uint32_t>(w);
  int64_t lo = 0, hi = len;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (rs[mid] < ww) lo = mid + 1; else hi = mid;
  }
  return lo < len && rs[lo] == ww;
}

// Is w in the ascending int64 run rg[0,len) (global memory)?
__device__ __forceinline__ bool probe_global(const int64_t *__restrict__ rg, int64_t len, int64_t w) {
  int64_t lo = 0, hi = len;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (rg[mid] < w) lo = mid + 1; else hi = mid;
  }
  return lo < len && rg[lo] == w;
}

template <bool U32>
__global__ void __launch_bounds__(kTriThreads)
    tri_rows_kernel(const int64_t *__restrict__ off, const int64_t *__restrict__ col, int64_t n,
                    int64_t nnz, unsigned long long *__restrict__ count,
                    unsigned long long *__restrict__ work, unsigned long long *__restrict__ bad,
                    unsigned long long *__restrict__ cursor, int rows_per_fetch) {
  __shared__ uint32_t rowbuf[kTriWarps][kTriCap];
  const unsigned lane = lane_id();
  uint32_t *rb = rowbuf[threadIdx.x >> 5];
  unsigned long long cnt = 0, wk = 0, nbad = 0;

  for (;;) {
    unsigned long long r0 = 0;
    if (lane == 0) r0 = atomicAdd(cursor, static_cast<unsigned long long>(rows_per_fetch));
    r0 = __shfl_sync(kFull, r0, 0);
    if (r0 >= static_cast<unsigned long long>(n)) break;
    const int64_t r1 = static_cast<int64_t>(r0) + rows_per_fetch < n ? static_cast<int64_t>(r0) + rows_per_fetch : n;

    for (int64_t i = static_cast<int64_t>(r0); i < r1; i++) {
      const int64_t b = off[i], e = off[i + 1];
      if (b < 0 || e < b || e > nnz) {
        if (lane == 0) nbad++;
        continue;
      }
      const int64_t d = e - b;
      if (d < 2) {
        if (d == 1 && lane == 0) {
          const int64_t c = col[b];
          if (c < 0 || c >= i) nbad++;
        }
        continue;
      }
      const bool cached = U32 && d <= kTriCap;
      // Stage (when it fits) and validate row i: columns in [0,i), ascending.
      bool ok = true;
      for (int64_t k = lane; k < d; k += 32) {
        const int64_t c = col[b + k];
        ok &= (c >= 0 && c < i);
        if (k > 0) ok &= c > col[b + k - 1];
        if (cached) rb[k] = static_cast<uint32_t>(c);
      }
      __syncwarp();
      if (!__all_sync(kFull, ok)) {
        if (lane == 0) nbad++;
        __syncwarp();
        continue;
      }
      const int64_t *__restrict__ rg = col + b;

      for (int64_t q0 = 1; q0 < d; q0 += 32) {
        const int64_t q = q0 + lane;
        int64_t jb = 0, jl = 0;
        if (q < d) {
          const int64_t j = cached ? static_cast<int64_t>(rb[q]) : rg[q];
          const int64_t s = off[j], t = off[j + 1];
          if (s < 0 || t < s || t > nnz) nbad++;
          else { jb = s; jl = t - s; }
        }
        int64_t inc = jl;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int64_t y = __shfl_up_sync(kFull, inc, o);
          if (static_cast<int>(lane) >= o) inc += y;
        }
        const int64_t total = __shfl_sync(kFull, inc, 31);
        if (lane == 0) wk += static_cast<unsigned long long>(total);
        for (int64_t base = 0; base < total; base += 32) {
          const int64_t kk = base + lane;
          // owner lane: the first lane whose inclusive prefix exceeds kk
          int lo = 0, hi = 31;
#pragma unroll
          for (int s = 0; s < 5; s++) {
            const int mid = (lo + hi) >> 1;
            const int64_t v = __shfl_sync(kFull, inc, mid);
            if (v > kk) hi = mid; else lo = mid + 1;
          }
          const int o = lo < 31 ? lo : 31;
          const int64_t o_inc = __shfl_sync(kFull, inc, o);
          const int64_t o_jl = __shfl_sync(kFull, jl, o);
          const int64_t o_jb = __shfl_sync(kFull, jb, o);
          if (kk < total) {
            const int64_t w = col[o_jb + (kk - (o_inc - o_jl))];
            const bool hit = cached ? probe_smem(rb, q0 + o, w) : probe_global(rg, q0 + o, w);
            cnt += hit ? 1ull : 0ull;
          }
        }
      }
      __syncwarp();  // rb is rewritten by the next row
    }
  }
  cnt = warp_sum_u64(cnt);
  wk = warp_sum_u64(wk);
  nbad = warp_sum_u64(nbad);
  if (lane == 0) {
    if (cnt) atomicAdd(count, cnt);
    if (wk && work) atomicAdd(work, wk);
    if (nbad) atomicAdd(bad, nbad);
  }
}

int g_tri_blocks_per_sm[2][64] = {{0}, {0}};

}  // namespace

// The default path per graph, chosen on the device.  The wedge path's work
// is the pushes, sum over rows of C(d,2); the hybrid's is close to the
// pulls, sum over nonzeros (i,j) of d_j.  Graphs with hubs (R-MAT: pulls
// 1.9-4x the pushes from scale 10 to 22; Kronecker products of stars, whose
// rows average hundreds of wedges per nonzero) count fastest by wedges;
// graphs without (Erdos-Renyi: pulls = pushes, 8-43 wedges per nonzero) by
// the hybrid, 10-30% faster there.  The pushes are summed exactly over the
// rows, the pulls estimated from kChooseSamples evenly spaced nonzeros; the
// last block to finish writes choice[0] = 1 (wedge) or 0 (hybrid): wedges
// when pulls >= pull_pct % of the pushes or the pushes reach push_per_nnz
// per nonzero.  Both thresholds are tuning knobs that the autotuner fits to
// measured wedge and hybrid times over R-MAT, Erdos-Renyi and Kronecker
// graphs.  The built-in values are the fit on GB300: 192 % and no push
// clause -- a product of stars with thousands of wedges per nonzero and
// pulls a third of the pushes ({3,4,5,9,16,25}) took 372 ms by wedges and
// 9.6 ms by the hybrid, R-MAT graphs (pulls 2.9-3.8x the pushes) are 2.3-3.2x
// faster by wedges, Erdos-Renyi graphs (pulls = pushes) within 25% either way.
// words: [0] pushes, [1] sampled pulls, [2] blocks done (zeroed by the caller).
constexpr int kChooseSamples = 4096;
constexpr int kChooseThreads = 256;
// Below this many nonzeros the choice (a kernel, and the skipped path's
// launches: 0.03-0.06 ms) would cost more than it can save; the wedge path
// runs directly.
constexpr int64_t kChooseMinNnz = int64_t(1) << 23;

__global__ void __launch_bounds__(kChooseThreads)
    tri_choose_kernel(const int64_t *__restrict__ off, const int64_t *__restrict__ col, int64_t n, int64_t nnz,
                      double pull_ratio, double push_per_nnz, unsigned long long *__restrict__ words,
                      unsigned *__restrict__ choice) {
  __shared__ unsigned last;
  unsigned long long pushes = 0, pulls = 0;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int64_t d = off[i + 1] - off[i];
    if (d > 1) pushes += static_cast<unsigned long long>(d) * static_cast<unsigned long long>(d - 1) / 2;
  }
  if (blockIdx.x == 0 && nnz > 0) {
    for (int s = threadIdx.x; s < kChooseSamples; s += kChooseThreads) {
      const int64_t j = col[static_cast<int64_t>((static_cast<unsigned long long>(s) * nnz) / kChooseSamples)];
      if (j >= 0 && j < n) pulls += static_cast<unsigned long long>(off[j + 1] - off[j]);  // a bad j: the paths count it
    }
  }
  pushes = warp_sum_u64(pushes);
  pulls = warp_sum_u64(pulls);
  if (lane_id() == 0) {
    if (pushes) atomicAdd(&words[0], pushes);
    if (pulls) atomicAdd(&words[1], pulls);
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&words[2], 1ull) == gridDim.x - 1 ? 1u : 0u;
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  const double push = static_cast<double>(atomicAdd(&words[0], 0ull));
  const double pull = static_cast<double>(atomicAdd(&words[1], 0ull)) * static_cast<double>(nnz) / kChooseSamples;
  const bool wedge = push == 0.0 || pull >= pull_ratio * push || push >= push_per_nnz * static_cast<double>(nnz);
  *choice = wedge ? 1u : 0u;
}

int launch_triangle(const int64_t *offset, const int64_t *nonzero, int64_t numrows, int64_t nnz,
                    unsigned long long *count, unsigned long long *work, unsigned long long *bad,
                    cudaStream_t stream) {
  if (numrows <= 0) return BALE_OK;
  // Default: per graph, wedge probes at the far vertex (tri_wedge.cu) or the
  // bitmap/search hybrid over rows i (tri_hybrid.cu), chosen on the device
  // by tri_choose_kernel; mode 2 the wedge path, mode 1 the hybrid, mode 0
  // this file's warp-per-row merge kernel for every row.
  const int64_t mode = knob("tri.mode");
  if (mode < 0 && tri_wedge_supported(numrows, nnz) && nnz >= knob_or("tri.choose_min_nnz", kChooseMinNnz)) {
    // both paths launched, the one not chosen returning at once; their
    // workspaces side by side
    const size_t wbytes = (tri_wedge_workspace_bytes(numrows, nnz) + 255) & ~size_t(255);
    char *ws = static_cast<char *>(device_workspace(wbytes + tri_hybrid_workspace_bytes(numrows, nnz), stream));
    unsigned long long *cursor = next_cursor_words(2), *hwords = next_cursor_words(3), *cw = next_cursor_words(4);
    if (!ws || !cursor || !hwords || !cw) return BALE_ENOMEM;
    unsigned *choice = reinterpret_cast<unsigned *>(cw + 3);
    BALE_CUDA_OK(cudaMemsetAsync(cw, 0, 3 * sizeof(unsigned long long), stream));
    const int64_t want = (numrows + kChooseThreads - 1) / kChooseThreads, cap = static_cast<int64_t>(num_sms()) * 4;
    const double pull_ratio = static_cast<double>(knob_or("tri.wedge_pull_pct", 192)) / 100.0;
    const int64_t ppn = knob("tri.wedge_push_per_nnz");  // -1: no push clause
    const double push_per_nnz = ppn < 0 ? 1e300 : static_cast<double>(ppn);
    tri_choose_kernel<<<static_cast<unsigned>(want < cap ? want : cap), kChooseThreads, 0, stream>>>(
        offset, nonzero, numrows, nnz, pull_ratio, push_per_nnz, cw, choice);
    BALE_CUDA_OK(cudaGetLastError());
    int rc = launch_triangle_wedge(offset, nonzero, numrows, nnz, count, work, bad, ws, cursor, stream, choice);
    if (rc != BALE_OK) return rc;
    int64_t rpf_h = knob("tri.rows_per_fetch");
    if (rpf_h < 1 || rpf_h > 4096) rpf_h = 8;
    return launch_triangle_hybrid(offset, nonzero, numrows, nnz, count, work, bad, ws + wbytes, hwords,
                                  static_cast<int>(rpf_h), stream, choice);
  }
  if ((mode < 0 || mode == 2) && tri_wedge_supported(numrows, nnz)) {
    void *ws = device_workspace(tri_wedge_workspace_bytes(numrows, nnz), stream);
    unsigned long long *cursor = next_cursor_words(2);
    if (!ws || !cursor) return BALE_ENOMEM;
    return launch_triangle_wedge(offset, nonzero, numrows, nnz, count, work, bad, ws, cursor, stream);
  }
  if (mode != 0 && numrows < 0xffffffffll) {
    int64_t rpf_h = knob("tri.rows_per_fetch");
    if (rpf_h < 1 || rpf_h > 4096) rpf_h = 8;
    void *ws = device_workspace(tri_hybrid_workspace_bytes(numrows, nnz), stream);
    unsigned long long *words = next_cursor_words(3);
    if (!ws || !words) return BALE_ENOMEM;
    return launch_triangle_hybrid(offset, nonzero, numrows, nnz, count, work, bad, ws, words,
                                  static_cast<int>(rpf_h), stream);
  }
  // Each launch takes its own cursor word from a ring so that launches on
  // different streams do not share one.
  unsigned long long *cursor = next_cursor_word();
  if (!cursor) return BALE_ECUDA;
  BALE_CUDA_OK(cudaMemsetAsync(cursor, 0, sizeof(unsigned long long), stream));

  const bool u32 = numrows <= 0xffffffffll;
  const int dev = current_device();
  int &bps = g_tri_blocks_per_sm[u32 ? 1 : 0][dev >= 0 && dev < 64 ? dev : 0];
  if (bps == 0) {
    cudaError_t e = u32 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, tri_rows_kernel<true>, kTriThreads, 0)
                        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, tri_rows_kernel<false>, kTriThreads, 0);
    if (e != cudaSuccess || bps < 1) bps = 1;
  }
  int64_t blocks = static_cast<int64_t>(num_sms()) * bps;
  int64_t rpf = knob("tri.rows_per_fetch");
  if (rpf < 1 || rpf > 4096) rpf = kRowsPerFetchDefault;
  int64_t need = (numrows + rpf - 1) / rpf;
  need = (need + kTriWarps - 1) / kTriWarps;
  if (blocks > need) blocks = need > 0 ? need : 1;
  if (u32)
    tri_rows_kernel<true><<<static_cast<int>(blocks), kTriThreads, 0, stream>>>(
        offset, nonzero, numrows, nnz, count, work, bad, cursor, static_cast<int>(rpf));
  else
    tri_rows_kernel<false><<<static_cast<int>(blocks), kTriThreads, 0, stream>>>(
        offset, nonzero, numrows, nnz, count, work, bad, cursor, static_cast<int>(rpf));
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

}  // namespace bale
