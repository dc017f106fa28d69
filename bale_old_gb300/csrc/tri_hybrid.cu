// tri_hybrid.cu -- triangle counting, bitmap/search hybrid (default mode).
//
// Same count as apps/triangle_src/triangle_agi.upc:69-99 (alg 0): for every
// nonzero L[i][j] after the first of row i, |row_i and row_j|.  The rows of a
// degree-ordered L are long exactly where the work is (a hub's row holds its
// higher-degree neighbours, hundreds of them), so the two sides of each
// intersection are handled by size:
//
//  * heavy rows (label below kHeavyBits and at least kHeavyMinDeg nonzeros):
//    one CTA per row.  Row i becomes a bitmap over [0,i) in shared memory;
//    each warp streams whole rows j (coalesced, from a u32 copy of the column
//    array) and tests every element against the bitmap -- one shared-memory
//    load per element instead of a binary search.  The bits are cleared by
//    row i's own columns before the next row, so the bitmap is never swept;
//  * light rows: one warp per row, row i staged in shared memory.  For each
//    neighbour j the cheaper side is searched: either row j is streamed and
//    each element is binary-searched in the part of row i before j, or each
//    element of that part of row i is binary-searched in row j (when
//    q * log2|row j| < |row j|).
//
// The reference's AGI scan reads every element of every row j; the work
// tally (*work) here counts row-j elements streamed plus binary-search probes.
// Validation matches the merge kernel: bad offsets, columns outside [0,i) or
// non-ascending rows are counted in *bad and the row is skipped.
#include "common.cuh"

namespace bale {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int64_t kHeavyBits = int64_t(1) << 19;  // bitmap covers labels [0, 2^19): 64 KiB
constexpr int kHeavyMinDeg = 64;
constexpr int kHeavyThreads = 512;
constexpr int kHeavyWarps = kHeavyThreads / 32;
constexpr int kLightThreads = 256;
constexpr int kLightWarps = kLightThreads / 32;
constexpr int kLightCap = 1024;
constexpr uint32_t kBadCol = 0xffffffffu;

__global__ void __launch_bounds__(256)
    tri_convert_kernel(const int64_t *__restrict__ col, int64_t nnz, uint32_t *__restrict__ col32) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < nnz; k += stride) {
    const int64_t c = ld_stream(col + k);
    col32[k] = (c < 0 || c >= static_cast<int64_t>(kBadCol)) ? kBadCol : static_cast<uint32_t>(c);
  }
}

// Rows below `bits` with at least kHeavyMinDeg nonzeros go to the heavy list.
// The light kernel applies the same test to the same raw offsets.
__device__ __forceinline__ bool is_heavy(int64_t i, int64_t b, int64_t e, int64_t bits) {
  return i < bits && e - b >= kHeavyMinDeg;
}

__global__ void __launch_bounds__(256)
    tri_classify_kernel(const int64_t *__restrict__ off, int64_t n, int64_t bits,
                        uint32_t *__restrict__ heavy, unsigned long long *__restrict__ nheavy) {
  const int64_t lim = n < bits ? n : bits;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t base = static_cast<int64_t>(blockIdx.x) * blockDim.x; base < lim; base += stride) {
    const int64_t i = base + threadIdx.x;
    const bool h = i < lim && is_heavy(i, off[i], off[i + 1], bits);
    const unsigned m = __ballot_sync(kFull, h);
    unsigned long long slot = 0;
    if (lane_id() == 0 && m) slot = atomicAdd(nheavy, static_cast<unsigned long long>(__popc(m)));
    slot = __shfl_sync(kFull, slot, 0);
    if (h) heavy[slot + __popc(m & ((1u << lane_id()) - 1u))] = static_cast<uint32_t>(i);
  }
}

__global__ void __launch_bounds__(kHeavyThreads)
    tri_heavy_kernel(const int64_t *__restrict__ off, const uint32_t *__restrict__ col, int64_t nnz,
                     const uint32_t *__restrict__ heavy, const unsigned long long *__restrict__ nheavy_p,
                     int64_t bits, unsigned long long *__restrict__ count, unsigned long long *__restrict__ work,
                     unsigned long long *__restrict__ bad, unsigned long long *__restrict__ cursor) {
  extern __shared__ uint32_t bm[];
  __shared__ long long sel;
  const unsigned lane = lane_id();
  const int warp = threadIdx.x >> 5;
  const int64_t nwords = (bits + 31) >> 5;
  const unsigned long long nheavy = *nheavy_p;
  for (int64_t w = threadIdx.x; w < nwords; w += kHeavyThreads) bm[w] = 0;
  unsigned long long cnt = 0, wk = 0, nbad = 0;
  for (;;) {
    __syncthreads();  // the previous row's bits are cleared and sel may be rewritten
    if (threadIdx.x == 0) {
      const unsigned long long r = atomicAdd(cursor, 1ull);
      sel = r < nheavy ? static_cast<long long>(heavy[r]) : -1ll;
    }
    __syncthreads();
    const long long i = sel;
    if (i < 0) break;
    const int64_t b = off[i], e = off[i + 1];
    if (b < 0 || e < b || e > nnz) {
      if (threadIdx.x == 0) nbad++;
      continue;
    }
    const int64_t d = e - b;
    bool ok = true;
    for (int64_t k = threadIdx.x; k < d; k += kHeavyThreads) {
      const uint32_t c = col[b + k];
      const bool in = static_cast<int64_t>(c) < i;
      ok &= in;
      if (k > 0) ok &= c > col[b + k - 1];
      if (in) atomicOr(&bm[c >> 5], 1u << (c & 31));
    }
    ok = __syncthreads_and(ok);
    if (ok) {
      for (int64_t q = 1 + warp; q < d; q += kHeavyWarps) {
        const uint32_t j = col[b + q];
        const int64_t s = off[j], t = off[j + 1];
        if (s < 0 || t < s || t > nnz) {
          if (lane == 0) nbad++;
          continue;
        }
        if (lane == 0) wk += static_cast<unsigned long long>(t - s);
        for (int64_t k = s + lane; k < t; k += 128) {
          uint32_t w[4];
#pragma unroll
          for (int u = 0; u < 4; u++) w[u] = (k + 32 * u < t) ? col[k + 32 * u] : kBadCol;
#pragma unroll
          for (int u = 0; u < 4; u++)
            if (static_cast<int64_t>(w[u]) < i) cnt += (bm[w[u] >> 5] >> (w[u] & 31)) & 1u;
        }
      }
    } else if (threadIdx.x == 0) {
      nbad++;
    }
    __syncthreads();
    for (int64_t k = threadIdx.x; k < d; k += kHeavyThreads) {
      const uint32_t c = col[b + k];
      if (static_cast<int64_t>(c) < i) bm[c >> 5] = 0;
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

// Is w in the ascending u32 run r[0,len)?
__device__ __forceinline__ bool search_u32(const uint32_t *__restrict__ r, int64_t len, uint32_t w) {
  int64_t lo = 0, hi = len;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (r[mid] < w) lo = mid + 1; else hi = mid;
  }
  return lo < len && r[lo] == w;
}

// Warp-wide inclusive prefix sum.
__device__ __forceinline__ int64_t warp_incl_scan(int64_t v) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(kFull, v, o);
    if (static_cast<int>(lane_id()) >= o) v += y;
  }
  return v;
}

// First lane whose inclusive prefix exceeds kk (all lanes participate).
__device__ __forceinline__ int owner_lane(int64_t inc, int64_t kk) {
  int lo = 0, hi = 31;
#pragma unroll
  for (int s = 0; s < 5; s++) {
    const int mid = (lo + hi) >> 1;
    const int64_t v = __shfl_sync(kFull, inc, mid);
    if (v > kk) hi = mid; else lo = mid + 1;
  }
  return lo < 31 ? lo : 31;
}

__global__ void __launch_bounds__(kLightThreads)
    tri_light_kernel(const int64_t *__restrict__ off, const uint32_t *__restrict__ col, int64_t n, int64_t nnz,
                     int64_t bits, unsigned long long *__restrict__ count, unsigned long long *__restrict__ work,
                     unsigned long long *__restrict__ bad, unsigned long long *__restrict__ cursor,
                     int rows_per_fetch) {
  __shared__ uint32_t rowbuf[kLightWarps][kLightCap];
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
      if (is_heavy(i, b, e, bits)) continue;  // the heavy kernel owns this row
      if (b < 0 || e < b || e > nnz) {
        if (lane == 0) nbad++;
        continue;
      }
      const int64_t d = e - b;
      if (d < 2) {
        if (d == 1 && lane == 0 && static_cast<int64_t>(col[b]) >= i) nbad++;
        continue;
      }
      const bool cached = d <= kLightCap;
      bool ok = true;
      for (int64_t k = lane; k < d; k += 32) {
        const uint32_t c = col[b + k];
        ok &= static_cast<int64_t>(c) < i;
        if (k > 0) ok &= c > col[b + k - 1];
        if (cached) rb[k] = c;
      }
      __syncwarp();
      if (!__all_sync(kFull, ok)) {
        if (lane == 0) nbad++;
        __syncwarp();
        continue;
      }
      const uint32_t *__restrict__ ri = cached ? rb : col + b;  // row i (shared or global)

      for (int64_t q0 = 1; q0 < d; q0 += 32) {
        const int64_t q = q0 + lane;
        int64_t jb = 0, jlen = 0, sl = 0, pq = 0;
        if (q < d) {
          const uint32_t j = ri[q];
          const int64_t s = off[j], t = off[j + 1];
          if (s < 0 || t < s || t > nnz) {
            nbad++;
          } else {
            jb = s;
            jlen = t - s;
            // search each of the q earlier row-i columns in row j, or stream row j
            const int64_t steps = 64 - __clzll(static_cast<unsigned long long>(jlen) + 1ull);
            if (q * steps < jlen) pq = q; else sl = jlen;
          }
        }
        // (1) streamed neighbours: every element of row j searched in ri[0,q)
        const int64_t inc = warp_incl_scan(sl);
        const int64_t tot = __shfl_sync(kFull, inc, 31);
        if (lane == 0) wk += static_cast<unsigned long long>(tot);
        for (int64_t base = 0; base < tot; base += 32) {
          const int64_t kk = base + lane;
          const int o = owner_lane(inc, kk);
          const int64_t o_inc = __shfl_sync(kFull, inc, o);
          const int64_t o_len = __shfl_sync(kFull, sl, o);
          const int64_t o_jb = __shfl_sync(kFull, jb, o);
          if (kk < tot) {
            const uint32_t w = col[o_jb + (kk - (o_inc - o_len))];
            cnt += search_u32(ri, q0 + o, w) ? 1ull : 0ull;
          }
        }
        // (2) searched neighbours: each ri[r], r < q, searched in row j
        const int64_t inc2 = warp_incl_scan(pq);
        const int64_t tot2 = __shfl_sync(kFull, inc2, 31);
        if (lane == 0) wk += static_cast<unsigned long long>(tot2);
        for (int64_t base = 0; base < tot2; base += 32) {
          const int64_t kk = base + lane;
          const int o = owner_lane(inc2, kk);
          const int64_t o_inc = __shfl_sync(kFull, inc2, o);
          const int64_t o_pq = __shfl_sync(kFull, pq, o);
          const int64_t o_jb = __shfl_sync(kFull, jb, o);
          const int64_t o_len = __shfl_sync(kFull, jlen, o);
          if (kk < tot2) {
            const uint32_t w = ri[kk - (o_inc - o_pq)];
            cnt += search_u32(col + o_jb, o_len, w) ? 1ull : 0ull;
          }
        }
      }
      __syncwarp();
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

bool g_heavy_attr[64];

}  // namespace

size_t tri_hybrid_workspace_bytes(int64_t numrows, int64_t nnz) {
  const int64_t lim = numrows < kHeavyBits ? numrows : kHeavyBits;
  return ((static_cast<size_t>(nnz > 0 ? nnz : 1) * sizeof(uint32_t) + 255) & ~size_t(255)) +
         static_cast<size_t>(lim > 0 ? lim : 1) * sizeof(uint32_t);
}

int launch_triangle_hybrid(const int64_t *offset, const int64_t *nonzero, int64_t numrows, int64_t nnz,
                           unsigned long long *count, unsigned long long *work, unsigned long long *bad,
                           void *ws, unsigned long long *words, int rows_per_fetch, cudaStream_t stream) {
  // words: [0] heavy-list length, [1] heavy cursor, [2] light cursor (zeroed here)
  const int sms = num_sms();
  char *p = static_cast<char *>(ws);
  uint32_t *col32 = reinterpret_cast<uint32_t *>(p);
  p += (static_cast<size_t>(nnz > 0 ? nnz : 1) * sizeof(uint32_t) + 255) & ~size_t(255);
  uint32_t *heavy = reinterpret_cast<uint32_t *>(p);
  const int64_t bits = numrows < kHeavyBits ? ((numrows + 31) & ~int64_t(31)) : kHeavyBits;

  BALE_CUDA_OK(cudaMemsetAsync(words, 0, 3 * sizeof(unsigned long long), stream));
  if (nnz > 0) {
    int64_t blocks = (nnz + 255) / 256, cap = static_cast<int64_t>(sms) * 8;
    tri_convert_kernel<<<static_cast<unsigned>(blocks < cap ? blocks : cap), 256, 0, stream>>>(nonzero, nnz, col32);
    BALE_CUDA_OK(cudaGetLastError());
  }
  {
    const int64_t lim = numrows < bits ? numrows : bits;
    int64_t blocks = (lim + 255) / 256, cap = static_cast<int64_t>(sms) * 8;
    if (blocks < 1) blocks = 1;
    tri_classify_kernel<<<static_cast<unsigned>(blocks < cap ? blocks : cap), 256, 0, stream>>>(
        offset, numrows, bits, heavy, words);
    BALE_CUDA_OK(cudaGetLastError());
  }
  {
    const size_t smem = static_cast<size_t>(bits / 32) * sizeof(uint32_t);
    const int dev = current_device();
    if (dev >= 0 && dev < 64 && !g_heavy_attr[dev]) {
      BALE_CUDA_OK(cudaFuncSetAttribute(tri_heavy_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>((kHeavyBits / 32) * sizeof(uint32_t))));
      g_heavy_attr[dev] = true;
    }
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, tri_heavy_kernel, kHeavyThreads, smem) != cudaSuccess ||
        occ < 1)
      occ = 1;
    tri_heavy_kernel<<<static_cast<unsigned>(sms * occ), kHeavyThreads, smem, stream>>>(
        offset, col32, nnz, heavy, words, bits, count, work, bad, words + 1);
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
        offset, col32, numrows, nnz, bits, count, work, bad, words + 2, rows_per_fetch);
    BALE_CUDA_OK(cudaGetLastError());
  }
  return BALE_OK;
}

}  // namespace bale
