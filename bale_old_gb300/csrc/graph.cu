// graph.cu -- building the triangle kernels' input on the device: the
// degree-ordered, strictly lower-triangular CSR of an undirected graph.
//
// From an edge list (or R-MAT edges generated in place, bit-identical to
// bale_gen_rmat in host/inputs.c):
//   1. keys: each edge {u,v}, u != v, becomes min << S | max (S = label
//      bits); self loops become an all-ones key that sorts last;
//   2. sort the keys (LSD radix sort below), drop the duplicates and the
//      self loops;
//   3. degrees; labels by descending degree, ties by ascending original
//      label: a second sort of (maxdeg - deg) << S | v;
//   4. each edge relabelled to row = max, col = min of the new labels, a
//      third sort, and the CSR read off the sorted keys: rows in order,
//      columns ascending within each row -- the reference's tidy lower
//      matrix (spmat/spmat_utils.upc:455-473 tril, :1055-1062 sort_nonzeros).
// The radix sort is stable, 8 bits per pass: per tile of 4096 keys a digit
// histogram, one exclusive scan over (digit, tile), then a scatter in which
// every key's rank among equal digits of its tile comes from a warp match
// and per-warp counts in shared memory.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "bale_inputs.h"
#include "common.cuh"

namespace bale {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kPer = 16;                      // keys per thread per tile
constexpr int64_t kTile = kThreads * kPer;    // 4096 keys per sort block
constexpr int kDigitBits = 8;
constexpr int kDigits = 1 << kDigitBits;      // == kThreads: one digit per thread
static_assert(kDigits == kThreads, "one digit per thread");
constexpr int kScanThreads = 1024;
constexpr int64_t kScanBlock = kScanThreads * 4;

__device__ __forceinline__ uint64_t sm64(uint64_t seed, uint64_t i) {
  uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// ---------------------------------------------------------------- scan
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *total) {
  __shared__ uint32_t warp_tot[kScanThreads / 32];
  const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
  uint32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(kFull, inc, o);
    if (static_cast<int>(lane) >= o) inc += y;
  }
  if (lane == 31) warp_tot[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    const uint32_t t = warp_tot[lane];
    uint32_t ti = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, ti, o);
      if (static_cast<int>(lane) >= o) ti += y;
    }
    warp_tot[lane] = ti - t;
    if (lane == 31) *total = ti;
  }
  __syncthreads();
  const uint32_t r = warp_tot[warp] + inc - v;
  __syncthreads();
  return r;
}

__device__ __forceinline__ void load4(const uint32_t *__restrict__ a, int64_t n, int64_t idx, uint32_t v[4]) {
#pragma unroll
  for (int q = 0; q < 4; q++) v[q] = idx + q < n ? a[idx + q] : 0u;
}

__global__ void __launch_bounds__(kScanThreads)
    scan_blocksum_kernel(const uint32_t *__restrict__ in, int64_t n, uint32_t *__restrict__ bsum) {
  __shared__ uint32_t tot;
  const int64_t idx = static_cast<int64_t>(blockIdx.x) * kScanBlock + threadIdx.x * 4;
  uint32_t v[4];
  load4(in, n, idx, v);
  block_excl_scan(v[0] + v[1] + v[2] + v[3], &tot);
  if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kScanThreads)
    scan_top_kernel(uint32_t *__restrict__ bsum, int64_t nb, uint32_t *__restrict__ total) {
  __shared__ uint32_t tot;
  uint32_t carry = 0;
  for (int64_t base = 0; base < nb; base += kScanBlock) {
    const int64_t idx = base + threadIdx.x * 4;
    uint32_t v[4];
    load4(bsum, nb, idx, v);
    uint32_t x = block_excl_scan(v[0] + v[1] + v[2] + v[3], &tot) + carry;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      if (idx + q < nb) bsum[idx + q] = x;
      x += v[q];
    }
    carry += tot;
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(kScanThreads)
    scan_apply_kernel(const uint32_t *__restrict__ in, int64_t n, const uint32_t *__restrict__ bsum,
                      uint32_t *__restrict__ out) {
  __shared__ uint32_t tot;
  const int64_t idx = static_cast<int64_t>(blockIdx.x) * kScanBlock + threadIdx.x * 4;
  uint32_t v[4];
  load4(in, n, idx, v);
  uint32_t x = block_excl_scan(v[0] + v[1] + v[2] + v[3], &tot) + bsum[blockIdx.x];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    if (idx + q < n) out[idx + q] = x;
    x += v[q];
  }
}

// ---------------------------------------------------------------- radix sort
__global__ void __launch_bounds__(kThreads)
    radix_hist_kernel(const uint64_t *__restrict__ keys, int64_t n, int shift, uint32_t *__restrict__ hist,
                      int64_t ntiles) {
  __shared__ uint32_t cnt[kDigits];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kTile;
#pragma unroll 4
  for (int r = 0; r < kPer; r++) {
    const int64_t i = base + r * kThreads + threadIdx.x;
    if (i < n) atomicAdd(&cnt[static_cast<uint32_t>(keys[i] >> shift) & (kDigits - 1)], 1u);
  }
  __syncthreads();
  hist[static_cast<int64_t>(threadIdx.x) * ntiles + blockIdx.x] = cnt[threadIdx.x];
}

// offs[d * ntiles + t]: where tile t's keys with digit d start in dst.
__global__ void __launch_bounds__(kThreads)
    radix_scatter_kernel(const uint64_t *__restrict__ src, uint64_t *__restrict__ dst, int64_t n, int shift,
                         const uint32_t *__restrict__ offs, int64_t ntiles) {
  __shared__ uint32_t base[kDigits];
  __shared__ uint32_t wcnt[kWarps][kDigits];
  const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
  base[threadIdx.x] = offs[static_cast<int64_t>(threadIdx.x) * ntiles + blockIdx.x];
#pragma unroll
  for (int w = 0; w < kWarps; w++) wcnt[w][threadIdx.x] = 0;
  __syncthreads();
  const int64_t tile = static_cast<int64_t>(blockIdx.x) * kTile;
  for (int r = 0; r < kPer; r++) {
    const int64_t i = tile + r * kThreads + threadIdx.x;
    const bool valid = i < n;
    const uint64_t key = valid ? src[i] : 0ull;
    const uint32_t d = valid ? static_cast<uint32_t>(key >> shift) & (kDigits - 1) : kDigits;  // kDigits: none
    const unsigned peers = __match_any_sync(kFull, d);
    const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
    if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    if (valid) {
      uint32_t pre = base[d] + rank;
      for (unsigned w = 0; w < warp; w++) pre += wcnt[w][d];
      dst[pre] = key;
    }
    __syncthreads();
    uint32_t t = 0;
#pragma unroll
    for (int w = 0; w < kWarps; w++) {
      t += wcnt[w][threadIdx.x];
      wcnt[w][threadIdx.x] = 0;
    }
    base[threadIdx.x] += t;
    __syncthreads();
  }
}

// ---------------------------------------------------------------- graph steps
__global__ void __launch_bounds__(256)
    rmat_keys_kernel(uint64_t *__restrict__ keys, int64_t m, int S, uint32_t ta, uint32_t tab, uint32_t tabc,
                     uint64_t seed) {
  const uint64_t draws = static_cast<uint64_t>(S + 1) / 2;  // two 32-bit levels per draw
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < m; e += stride) {
    uint64_t u = 0, v = 0, r = 0;
    for (int l = 0; l < S; l++) {
      if ((l & 1) == 0) r = sm64(seed, static_cast<uint64_t>(e) * draws + static_cast<uint64_t>(l >> 1));
      const uint32_t x = (l & 1) ? static_cast<uint32_t>(r >> 32) : static_cast<uint32_t>(r);
      const uint64_t ub = x >= tab ? 1u : 0u;
      const uint64_t vb = (x >= ta && x < tab) || x >= tabc ? 1u : 0u;
      u = (u << 1) | ub;
      v = (v << 1) | vb;
    }
    keys[e] = u == v ? ~0ull : (u < v ? (u << S) | v : (v << S) | u);
  }
}

__global__ void __launch_bounds__(256)
    edge_keys_kernel(const int64_t *__restrict__ eu, const int64_t *__restrict__ ev, int64_t m, int64_t n, int S,
                     uint64_t *__restrict__ keys, unsigned long long *__restrict__ bad) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  unsigned long long nb = 0;
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < m; e += stride) {
    const int64_t u = eu[e], v = ev[e];
    if (u < 0 || u >= n || v < 0 || v >= n) {
      nb++;
      keys[e] = ~0ull;
      continue;
    }
    const uint64_t a = static_cast<uint64_t>(u < v ? u : v), b = static_cast<uint64_t>(u < v ? v : u);
    keys[e] = a == b ? ~0ull : (a << S) | b;
  }
  nb = warp_sum_u64(nb);
  if (lane_id() == 0 && nb) atomicAdd(bad, nb);
}

// flag[e] = 1 for the first copy of each edge key (sorted input); self loops
// and rejected edges (bits at or above 2S) are dropped.
__global__ void __launch_bounds__(256)
    unique_flag_kernel(const uint64_t *__restrict__ keys, int64_t m, int S, uint32_t *__restrict__ flag) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < m; e += stride) {
    const uint64_t k = keys[e];
    flag[e] = (k >> (2 * S)) == 0 && (e == 0 || keys[e - 1] != k) ? 1u : 0u;
  }
}

// Degrees of vertices below kHubIds are counted per block in shared memory
// first: skewed graphs send most edges to a few low-labelled hubs, whose
// global counters would serialise in L2.
constexpr int kHubIds = 8192;

__global__ void __launch_bounds__(256)
    compact_degree_kernel(const uint64_t *__restrict__ keys, int64_t m, int S, int64_t n,
                          const uint32_t *__restrict__ flag, const uint32_t *__restrict__ pos,
                          uint64_t *__restrict__ out, uint32_t *__restrict__ deg) {
  __shared__ uint32_t hub[kHubIds];
  for (int h = threadIdx.x; h < kHubIds; h += 256) hub[h] = 0;
  __syncthreads();
  const uint64_t mask = (uint64_t(1) << S) - 1;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < m; e += stride) {
    if (!flag[e]) continue;
    const uint64_t k = keys[e];
    out[pos[e]] = k;
    const uint64_t a = k >> S, b = k & mask;
    if (a < kHubIds) atomicAdd(&hub[a], 1u); else atomicAdd(deg + a, 1u);
    if (b < kHubIds) atomicAdd(&hub[b], 1u); else atomicAdd(deg + b, 1u);
  }
  __syncthreads();
  for (int h = threadIdx.x; h < kHubIds && h < n; h += 256)
    if (hub[h]) atomicAdd(deg + h, hub[h]);
}

__global__ void __launch_bounds__(256)
    max_kernel(const uint32_t *__restrict__ a, int64_t n, unsigned int *__restrict__ out) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  uint32_t m = 0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    m = a[i] > m ? a[i] : m;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(kFull, m, o));
  if (lane_id() == 0 && m) atomicMax(out, m);
}

__global__ void __launch_bounds__(256)
    vertex_keys_kernel(const uint32_t *__restrict__ deg, int64_t n, int S, const unsigned int *__restrict__ maxdeg,
                       uint64_t *__restrict__ vk) {
  const uint64_t md = *maxdeg;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t v = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; v < n; v += stride)
    vk[v] = ((md - deg[v]) << S) | static_cast<uint64_t>(v);
}

__global__ void __launch_bounds__(256)
    new_label_kernel(const uint64_t *__restrict__ vk, int64_t n, int S, uint32_t *__restrict__ newid) {
  const uint64_t mask = (uint64_t(1) << S) - 1;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride)
    newid[vk[r] & mask] = static_cast<uint32_t>(r);
}

__global__ void __launch_bounds__(256)
    lower_keys_kernel(const uint64_t *__restrict__ ukeys, int64_t nu, int S, const uint32_t *__restrict__ newid,
                      uint64_t *__restrict__ lk) {
  const uint64_t mask = (uint64_t(1) << S) - 1;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < nu; e += stride) {
    const uint64_t x = newid[ukeys[e] >> S], y = newid[ukeys[e] & mask];
    lk[e] = x > y ? (x << S) | y : (y << S) | x;
  }
}

// CSR from row-major sorted keys: offset[r] = first entry of row >= r, by a
// binary search per row (rows may be empty in long runs: the isolated
// vertices all take the last labels); nonzero[e] = the column.
__global__ void __launch_bounds__(256)
    csr_offsets_kernel(const uint64_t *__restrict__ lk, int64_t nu, int64_t n, int S,
                       int64_t *__restrict__ offset) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r <= n; r += stride) {
    int64_t lo = 0, hi = nu;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (static_cast<int64_t>(lk[mid] >> S) < r) lo = mid + 1; else hi = mid;
    }
    offset[r] = lo;
  }
}

__global__ void __launch_bounds__(256)
    csr_cols_kernel(const uint64_t *__restrict__ lk, int64_t nu, int S, int64_t *__restrict__ nonzero) {
  const uint64_t mask = (uint64_t(1) << S) - 1;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < nu; e += stride)
    nonzero[e] = static_cast<int64_t>(lk[e] & mask);
}

unsigned grid_for(int64_t n) {
  const int64_t want = (n + 255) / 256, cap = static_cast<int64_t>(num_sms()) * 16;
  return static_cast<unsigned>(std::max<int64_t>(1, std::min(want, cap)));
}

int label_bits(int64_t n) {
  int S = 1;
  while ((int64_t(1) << S) < n) S++;
  return S;
}

// Workspace of one build: two key buffers (m), flags and positions (m + 1),
// the sort histogram and its scan, degrees, labels, vertex keys (n each).
struct Ws {
  uint64_t *ka, *kb, *va, *vb;
  uint32_t *flag, *pos, *hist, *hoff, *bsum, *deg, *newid;
  unsigned int *words;  // [0] scan total, [1] max degree
};

size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

size_t ws_bytes(int64_t m, int64_t n, Ws *w, char *base) {
  const int64_t mm = std::max<int64_t>(m, 1), nn = std::max<int64_t>(n, 1);
  const int64_t tiles = (std::max(mm, nn) + kTile - 1) / kTile;
  const int64_t hist_n = tiles * kDigits;
  const int64_t scan_n = std::max(mm + 1, hist_n);
  const int64_t nb = (scan_n + kScanBlock - 1) / kScanBlock + 1;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o += up256(bytes);
    return base ? base + at : nullptr;
  };
  char *p;
  p = take(8 * mm); if (w) w->ka = reinterpret_cast<uint64_t *>(p);
  p = take(8 * mm); if (w) w->kb = reinterpret_cast<uint64_t *>(p);
  p = take(8 * nn); if (w) w->va = reinterpret_cast<uint64_t *>(p);
  p = take(8 * nn); if (w) w->vb = reinterpret_cast<uint64_t *>(p);
  p = take(4 * (mm + 1)); if (w) w->flag = reinterpret_cast<uint32_t *>(p);
  p = take(4 * (mm + 1)); if (w) w->pos = reinterpret_cast<uint32_t *>(p);
  p = take(4 * hist_n); if (w) w->hist = reinterpret_cast<uint32_t *>(p);
  p = take(4 * hist_n); if (w) w->hoff = reinterpret_cast<uint32_t *>(p);
  p = take(4 * nb); if (w) w->bsum = reinterpret_cast<uint32_t *>(p);
  p = take(4 * nn); if (w) w->deg = reinterpret_cast<uint32_t *>(p);
  p = take(4 * nn); if (w) w->newid = reinterpret_cast<uint32_t *>(p);
  p = take(64); if (w) w->words = reinterpret_cast<unsigned int *>(p);
  return o;
}

// out[0,n) = exclusive prefix of in[0,n); *total = the sum.
int excl_scan(const uint32_t *in, uint32_t *out, int64_t n, uint32_t *bsum, unsigned int *total, cudaStream_t st) {
  const int64_t nb = std::max<int64_t>(1, (n + kScanBlock - 1) / kScanBlock);
  scan_blocksum_kernel<<<static_cast<unsigned>(nb), kScanThreads, 0, st>>>(in, n, bsum);
  scan_top_kernel<<<1, kScanThreads, 0, st>>>(bsum, nb, total);
  scan_apply_kernel<<<static_cast<unsigned>(nb), kScanThreads, 0, st>>>(in, n, bsum, out);
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

// Stable sort of n keys on bits [0, bits); returns the buffer holding the result.
uint64_t *radix_sort(uint64_t *a, uint64_t *b, int64_t n, int bits, Ws &w, cudaStream_t st, int *rc) {
  *rc = BALE_OK;
  if (n <= 1) return a;
  const int64_t tiles = (n + kTile - 1) / kTile;
  for (int shift = 0; shift < bits; shift += kDigitBits) {
    radix_hist_kernel<<<static_cast<unsigned>(tiles), kThreads, 0, st>>>(a, n, shift, w.hist, tiles);
    *rc = excl_scan(w.hist, w.hoff, tiles * kDigits, w.bsum, w.words, st);
    if (*rc != BALE_OK) return a;
    radix_scatter_kernel<<<static_cast<unsigned>(tiles), kThreads, 0, st>>>(a, b, n, shift, w.hoff, tiles);
    if (cudaGetLastError() != cudaSuccess) {
      *rc = BALE_ECUDA;
      return a;
    }
    std::swap(a, b);
  }
  return a;
}

// Steps 2-4 from the edge keys in w.ka (m of them).
int build_from_keys(Ws &w, int64_t m, int64_t n, int S, int64_t *d_offset, int64_t *d_nonzero, int64_t *nnz,
                    cudaStream_t st) {
  int rc = BALE_OK;
  const int kbits = std::min(64, 2 * S + 1);
  uint64_t *sorted = radix_sort(w.ka, w.kb, m, kbits, w, st, &rc);
  if (rc != BALE_OK) return rc;
  uint64_t *other = sorted == w.ka ? w.kb : w.ka;
  unique_flag_kernel<<<grid_for(m), 256, 0, st>>>(sorted, m, S, w.flag);
  rc = excl_scan(w.flag, w.pos, m, w.bsum, w.words, st);
  if (rc != BALE_OK) return rc;
  BALE_CUDA_OK(cudaMemsetAsync(w.deg, 0, static_cast<size_t>(n) * 4, st));
  compact_degree_kernel<<<grid_for(m), 256, 0, st>>>(sorted, m, S, n, w.flag, w.pos, other, w.deg);
  unsigned int nu32 = 0;
  BALE_CUDA_OK(cudaMemcpyAsync(&nu32, w.words, 4, cudaMemcpyDeviceToHost, st));
  BALE_CUDA_OK(cudaMemsetAsync(w.words + 1, 0, 4, st));
  max_kernel<<<grid_for(n), 256, 0, st>>>(w.deg, n, w.words + 1);
  unsigned int maxdeg = 0;
  BALE_CUDA_OK(cudaMemcpyAsync(&maxdeg, w.words + 1, 4, cudaMemcpyDeviceToHost, st));
  BALE_CUDA_OK(cudaStreamSynchronize(st));
  const int64_t nu = nu32;
  vertex_keys_kernel<<<grid_for(n), 256, 0, st>>>(w.deg, n, S, w.words + 1, w.va);
  int dbits = 1;
  while ((uint64_t(1) << dbits) <= maxdeg) dbits++;
  uint64_t *vs = radix_sort(w.va, w.vb, n, std::min(64, S + dbits), w, st, &rc);
  if (rc != BALE_OK) return rc;
  new_label_kernel<<<grid_for(n), 256, 0, st>>>(vs, n, S, w.newid);
  uint64_t *lk = sorted;  // the unique keys are in `other`; reuse `sorted` for the lower keys
  lower_keys_kernel<<<grid_for(nu), 256, 0, st>>>(other, nu, S, w.newid, lk);
  uint64_t *ls = radix_sort(lk, other, nu, 2 * S, w, st, &rc);
  if (rc != BALE_OK) return rc;
  csr_offsets_kernel<<<grid_for(n + 1), 256, 0, st>>>(ls, nu, n, S, d_offset);
  if (nu > 0) csr_cols_kernel<<<grid_for(nu), 256, 0, st>>>(ls, nu, S, d_nonzero);
  BALE_CUDA_OK(cudaGetLastError());
  BALE_CUDA_OK(cudaStreamSynchronize(st));
  *nnz = nu;
  return BALE_OK;
}

// ---------------------------------------------------------------- spmat ops
// CSR checks shared by transpose and permute: offsets ascending inside
// [0, nnz] with offset[numrows] == nnz, columns inside [0, numcols).
__global__ void __launch_bounds__(256)
    csr_check_kernel(const int64_t *__restrict__ off, const int64_t *__restrict__ col, int64_t numrows,
                     int64_t numcols, int64_t nnz, unsigned long long *__restrict__ bad) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  unsigned long long nb = 0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i <= numrows; i += stride) {
    const int64_t o = off[i];
    if (o < 0 || o > nnz || (i < numrows && off[i + 1] < o) || (i == numrows && o != nnz) || (i == 0 && o != 0))
      nb++;
  }
  for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < nnz; k += stride)
    if (col[k] < 0 || col[k] >= numcols) nb++;
  nb = warp_sum_u64(nb);
  if (lane_id() == 0 && nb) atomicAdd(bad, nb);
}

// keys[k] = col << rb | row, the row of nonzero k found by a binary search
// over the (checked) offsets.
__global__ void __launch_bounds__(256)
    transpose_keys_kernel(const int64_t *__restrict__ off, const int64_t *__restrict__ col, int64_t numrows,
                          int64_t nnz, int rb, uint64_t *__restrict__ keys) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < nnz; k += stride) {
    int64_t lo = 0, hi = numrows;  // the last row i with off[i] <= k
    while (hi - lo > 1) {
      const int64_t mid = (lo + hi) >> 1;
      if (off[mid] <= k) lo = mid; else hi = mid;
    }
    keys[k] = (static_cast<uint64_t>(col[k]) << rb) | static_cast<uint64_t>(lo);
  }
}

// seen[p[i]]++ for a claimed permutation p of [0, n); entries outside count as bad.
__global__ void __launch_bounds__(256)
    perm_seen_kernel(const int64_t *__restrict__ p, int64_t n, uint32_t *__restrict__ seen,
                     unsigned long long *__restrict__ bad) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  unsigned long long nb = 0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int64_t v = p[i];
    if (v < 0 || v >= n) nb++;
    else atomicAdd(seen + v, 1u);
  }
  nb = warp_sum_u64(nb);
  if (lane_id() == 0 && nb) atomicAdd(bad, nb);
}

__global__ void __launch_bounds__(256)
    perm_once_kernel(const uint32_t *__restrict__ seen, int64_t n, unsigned long long *__restrict__ bad) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  unsigned long long nb = 0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    nb += seen[i] != 1u;
  nb = warp_sum_u64(nb);
  if (lane_id() == 0 && nb) atomicAdd(bad, nb);
}

// rperm[rperminv[i]] = i; len[i] = the length of row rperm[i] of A.
__global__ void __launch_bounds__(256)
    permute_rows_kernel(const int64_t *__restrict__ off, const int64_t *__restrict__ rperminv, int64_t n,
                        uint32_t *__restrict__ rperm) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    rperm[rperminv[i]] = static_cast<uint32_t>(i);
}

__global__ void __launch_bounds__(256)
    permute_len_kernel(const int64_t *__restrict__ off, const uint32_t *__restrict__ rperm, int64_t n,
                       uint32_t *__restrict__ len) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    len[i] = static_cast<uint32_t>(off[rperm[i] + 1] - off[rperm[i]]);
}

// One warp per new row i: row rperm[i] of A, columns through cperminv.
__global__ void __launch_bounds__(256)
    permute_fill_kernel(const int64_t *__restrict__ off, const int64_t *__restrict__ col,
                        const uint32_t *__restrict__ rperm, const uint32_t *__restrict__ pstart, int64_t n,
                        int64_t nnz, const int64_t *__restrict__ cperminv, int64_t *__restrict__ poff,
                        int64_t *__restrict__ pcol) {
  const int64_t warps = static_cast<int64_t>(gridDim.x) * (blockDim.x / 32);
  const unsigned lane = lane_id();
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * (blockDim.x / 32) + (threadIdx.x >> 5); i < n; i += warps) {
    const int64_t b = off[rperm[i]], d = off[rperm[i] + 1] - b, o = pstart[i];
    if (lane == 0) poff[i] = o;
    for (int64_t t = lane; t < d; t += 32) pcol[o + t] = cperminv[col[b + t]];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) poff[n] = nnz;
}

// The drand48 generator (POSIX): X' = (0x5deece66d X + 0xb) mod 2^48,
// lrand48 = X >> 17; srand48(s) sets X = (s & 0xffffffff) << 16 | 0x330e.
// The low 48 bits of 64-bit products are exact, so u64 arithmetic suffices.
constexpr uint64_t kLcgA = 0x5deece66dull, kLcgC = 0xbull, kLcgMask = (1ull << 48) - 1;

// X after k steps from x: the affine map raised to k by squaring.
__device__ __forceinline__ uint64_t lcg_jump(uint64_t x, uint64_t k) {
  uint64_t a = kLcgA, c = kLcgC, ra = 1, rc = 0;  // result map: x -> ra x + rc
  while (k) {
    if (k & 1) {
      ra = (ra * a) & kLcgMask;
      rc = (rc * a + c) & kLcgMask;
    }
    c = (c * a + c) & kLcgMask;  // compose the map with itself
    a = (a * a) & kLcgMask;
    k >>= 1;
  }
  return (ra * x + rc) & kLcgMask;
}

// Throw t (the (t+1)-th lrand48 output) lands in slot r_t = lrand48 % m;
// keys[t] = r_t << tb | t.  Each thread takes a run of consecutive throws.
constexpr int kThrowsPerThread = 64;

__global__ void __launch_bounds__(256)
    throws_kernel(uint64_t x0, int64_t nthrows, uint64_t m, int tb, uint64_t *__restrict__ keys) {
  const int64_t first = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) * kThrowsPerThread;
  if (first >= nthrows) return;
  uint64_t x = lcg_jump(x0, static_cast<uint64_t>(first));
  const int64_t last = first + kThrowsPerThread < nthrows ? first + kThrowsPerThread : nthrows;
  for (int64_t t = first; t < last; t++) {
    x = (kLcgA * x + kLcgC) & kLcgMask;
    keys[t] = (((x >> 17) % m) << tb) | static_cast<uint64_t>(t);
  }
}

// In slot order (keys sorted by slot, then throw): the first throw at each
// slot hit it; succ[t] = 1 for those.
__global__ void __launch_bounds__(256)
    first_hit_kernel(const uint64_t *__restrict__ sk, int64_t nthrows, int tb, uint32_t *__restrict__ succ) {
  const uint64_t tmask = (uint64_t(1) << tb) - 1;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; j < nthrows; j += stride)
    succ[sk[j] & tmask] = (j == 0 || (sk[j] >> tb) != (sk[j - 1] >> tb)) ? 1u : 0u;
}

// used[j] = slot-order entry j is one of the first n hits.
__global__ void __launch_bounds__(256)
    used_kernel(const uint64_t *__restrict__ sk, int64_t nthrows, int tb, const uint32_t *__restrict__ succ,
                const uint32_t *__restrict__ rank, uint32_t n, uint32_t *__restrict__ used) {
  const uint64_t tmask = (uint64_t(1) << tb) - 1;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; j < nthrows; j += stride) {
    const uint64_t t = sk[j] & tmask;
    used[j] = succ[t] && rank[t] < n ? 1u : 0u;
  }
}

__global__ void __launch_bounds__(256)
    perm_out_kernel(const uint64_t *__restrict__ sk, int64_t nthrows, int tb, const uint32_t *__restrict__ used,
                    const uint32_t *__restrict__ upos, const uint32_t *__restrict__ rank, int64_t *__restrict__ perm) {
  const uint64_t tmask = (uint64_t(1) << tb) - 1;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; j < nthrows; j += stride)
    if (used[j]) perm[upos[j]] = rank[sk[j] & tmask];
}

// ---------------------------------------------------------------- MatrixMarket body
__device__ __forceinline__ bool is_digit(char c) { return c >= '0' && c <= '9'; }
__device__ __forceinline__ bool is_blank(char c) { return c == ' ' || c == '\t'; }

// flag[i] = 1 where an entry line starts: a digit preceded, past blanks, by
// a newline or the start of the body (comment lines start with '%').
__global__ void __launch_bounds__(256)
    mm_starts_kernel(const char *__restrict__ b, int64_t len, uint32_t *__restrict__ flag) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < len; i += stride) {
    uint32_t f = 0;
    if (is_digit(b[i])) {
      int64_t j = i - 1;
      while (j >= 0 && is_blank(b[j])) j--;
      f = (j < 0 || b[j] == '\n') ? 1u : 0u;
    }
    flag[i] = f;
  }
}

__global__ void __launch_bounds__(256)
    mm_compact_kernel(const uint32_t *__restrict__ flag, const uint32_t *__restrict__ pos, int64_t len,
                      uint32_t *__restrict__ linepos, int64_t nlines) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < len; i += stride)
    if (flag[i] && pos[i] < nlines) linepos[pos[i]] = static_cast<uint32_t>(i);
}

// An unsigned decimal at b[*p] (at least one digit, no overflow past 2^62).
__device__ __forceinline__ bool mm_uint(const char *b, int64_t len, int64_t *p, int64_t *v) {
  int64_t x = 0, q = *p;
  if (q >= len || !is_digit(b[q])) return false;
  while (q < len && is_digit(b[q])) {
    if (x > (int64_t(1) << 58)) return false;
    x = x * 10 + (b[q] - '0');
    q++;
  }
  *p = q;
  *v = x;
  return true;
}

// One thread per entry line: "row col" (or "row col value"), 1-based.
// keys[l] = (row - 1) << lb | l, cols[l] = col - 1.
__global__ void __launch_bounds__(256)
    mm_parse_kernel(const char *__restrict__ b, int64_t len, const uint32_t *__restrict__ linepos, int64_t nlines,
                    int fields, int64_t nr, int64_t nc, int lb, uint64_t *__restrict__ keys,
                    uint32_t *__restrict__ cols, unsigned long long *__restrict__ bad) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  unsigned long long nb = 0;
  for (int64_t l = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; l < nlines; l += stride) {
    int64_t p = linepos[l], r = 0, c = 0, v = 0;
    bool ok = mm_uint(b, len, &p, &r);
    while (ok && p < len && is_blank(b[p])) p++;
    ok = ok && mm_uint(b, len, &p, &c);
    if (ok && fields == 3) {
      while (p < len && is_blank(b[p])) p++;
      if (p < len && (b[p] == '-' || b[p] == '+')) p++;
      ok = mm_uint(b, len, &p, &v);
    }
    while (ok && p < len && (is_blank(b[p]) || b[p] == '\r')) p++;
    ok = ok && (p == len || b[p] == '\n') && r >= 1 && r <= nr && c >= 1 && c <= nc;
    if (!ok) {
      nb++;
      r = 1;
      c = 1;
    }
    keys[l] = (static_cast<uint64_t>(r - 1) << lb) | static_cast<uint64_t>(l);
    cols[l] = static_cast<uint32_t>(c - 1);
  }
  nb = warp_sum_u64(nb);
  if (lane_id() == 0 && nb) atomicAdd(bad, nb);
}

__global__ void __launch_bounds__(256)
    mm_cols_kernel(const uint64_t *__restrict__ sk, int64_t nlines, int lb, const uint32_t *__restrict__ cols,
                   int64_t *__restrict__ nonzero) {
  const uint64_t lmask = (uint64_t(1) << lb) - 1;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < nlines; e += stride)
    nonzero[e] = cols[sk[e] & lmask];
}

uint32_t prob_threshold(double p) {
  if (p <= 0.0) return 0;
  if (p >= 1.0) return UINT32_MAX;
  return static_cast<uint32_t>(llround(p * 4294967296.0));
}

}  // namespace
}  // namespace bale

using namespace bale;

extern "C" {

int64_t bale_graph_build_workspace(int64_t m, int64_t n) {
  if (m < 0 || n < 1) return -1;
  return static_cast<int64_t>(ws_bytes(m, n, nullptr, nullptr));
}

int bale_graph_build_dev(const int64_t *d_u, const int64_t *d_v, int64_t m, int64_t n, int64_t *d_offset,
                         int64_t *d_nonzero, int64_t *nnz, void *stream) {
  if (m < 0 || n < 1 || n > (int64_t(1) << 31) || m >= (int64_t(1) << 32) - 1 || !d_offset || !nnz ||
      (m > 0 && (!d_u || !d_v || !d_nonzero))) {
    set_error("bale_graph_build_dev: bad arguments (m=%lld, n=%lld)", static_cast<long long>(m),
              static_cast<long long>(n));
    return BALE_EINVAL;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int S = label_bits(n);
  Ws w;
  void *ws = device_workspace(ws_bytes(m, n, nullptr, nullptr), st);
  if (!ws) return BALE_ENOMEM;
  ws_bytes(m, n, &w, static_cast<char *>(ws));
  unsigned long long *bad = reinterpret_cast<unsigned long long *>(w.words + 4);
  BALE_CUDA_OK(cudaMemsetAsync(w.words, 0, 64, st));
  if (m > 0) {
    edge_keys_kernel<<<grid_for(m), 256, 0, st>>>(d_u, d_v, m, n, S, w.ka, bad);
    BALE_CUDA_OK(cudaGetLastError());
  }
  unsigned long long nbad = 0;
  BALE_CUDA_OK(cudaMemcpyAsync(&nbad, bad, 8, cudaMemcpyDeviceToHost, st));
  BALE_CUDA_OK(cudaStreamSynchronize(st));
  if (nbad) {
    set_error("bale_graph_build_dev: %llu edges with an endpoint outside [0, n)", nbad);
    return BALE_EINPUT;
  }
  return build_from_keys(w, m, n, S, d_offset, d_nonzero, nnz, st);
}

int bale_gen_rmat_dev(int64_t scale, int64_t edgefactor, double a, double b, double c, uint64_t seed,
                      int64_t *d_offset, int64_t *d_nonzero, int64_t *nnz, void *stream) {
  if (scale < 1 || scale > 31 || edgefactor < 1 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0 || !d_offset ||
      !d_nonzero || !nnz || (edgefactor << scale) >= (int64_t(1) << 32) - 1) {
    set_error("bale_gen_rmat_dev: bad arguments");
    return BALE_EINVAL;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int S = static_cast<int>(scale);
  const int64_t n = int64_t(1) << S, m = edgefactor * n;
  Ws w;
  void *ws = device_workspace(ws_bytes(m, n, nullptr, nullptr), st);
  if (!ws) return BALE_ENOMEM;
  ws_bytes(m, n, &w, static_cast<char *>(ws));
  BALE_CUDA_OK(cudaMemsetAsync(w.words, 0, 64, st));
  rmat_keys_kernel<<<grid_for(m), 256, 0, st>>>(w.ka, m, S, prob_threshold(a), prob_threshold(a + b),
                                                 prob_threshold(a + b + c), seed);
  BALE_CUDA_OK(cudaGetLastError());
  return build_from_keys(w, m, n, S, d_offset, d_nonzero, nnz, st);
}

int bale_transpose_dev(const int64_t *d_offset, const int64_t *d_nonzero, int64_t numrows, int64_t numcols,
                       int64_t nnz, int64_t *d_toffset, int64_t *d_tnonzero, void *stream) {
  if (numrows < 1 || numcols < 1 || numrows > (int64_t(1) << 31) || numcols > (int64_t(1) << 31) || nnz < 0 ||
      nnz >= (int64_t(1) << 32) - 1 || !d_offset || !d_toffset || (nnz > 0 && (!d_nonzero || !d_tnonzero))) {
    set_error("bale_transpose_dev: bad arguments");
    return BALE_EINVAL;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int rb = label_bits(numrows), cb = label_bits(numcols);
  Ws w;
  void *ws = device_workspace(ws_bytes(nnz, std::max(numrows, numcols), nullptr, nullptr), st);
  if (!ws) return BALE_ENOMEM;
  ws_bytes(nnz, std::max(numrows, numcols), &w, static_cast<char *>(ws));
  unsigned long long *bad = reinterpret_cast<unsigned long long *>(w.words + 4);
  BALE_CUDA_OK(cudaMemsetAsync(w.words, 0, 64, st));
  csr_check_kernel<<<grid_for(std::max(numrows + 1, nnz)), 256, 0, st>>>(d_offset, d_nonzero, numrows, numcols,
                                                                          nnz, bad);
  unsigned long long nbad = 0;
  BALE_CUDA_OK(cudaMemcpyAsync(&nbad, bad, 8, cudaMemcpyDeviceToHost, st));
  BALE_CUDA_OK(cudaStreamSynchronize(st));
  if (nbad) {
    set_error("bale_transpose_dev: %llu malformed offsets or columns", nbad);
    return BALE_EINPUT;
  }
  int rc = BALE_OK;
  if (nnz > 0) {
    transpose_keys_kernel<<<grid_for(nnz), 256, 0, st>>>(d_offset, d_nonzero, numrows, nnz, rb, w.ka);
    BALE_CUDA_OK(cudaGetLastError());
  }
  uint64_t *sk = radix_sort(w.ka, w.kb, nnz, rb + cb, w, st, &rc);
  if (rc != BALE_OK) return rc;
  csr_offsets_kernel<<<grid_for(numcols + 1), 256, 0, st>>>(sk, nnz, numcols, rb, d_toffset);
  if (nnz > 0) csr_cols_kernel<<<grid_for(nnz), 256, 0, st>>>(sk, nnz, rb, d_tnonzero);
  BALE_CUDA_OK(cudaGetLastError());
  BALE_CUDA_OK(cudaStreamSynchronize(st));
  return BALE_OK;
}

int bale_permute_dev(const int64_t *d_offset, const int64_t *d_nonzero, int64_t numrows, int64_t numcols,
                     int64_t nnz, const int64_t *d_rperminv, const int64_t *d_cperminv, int64_t *d_poffset,
                     int64_t *d_pnonzero, void *stream) {
  if (numrows < 1 || numcols < 1 || numrows >= (int64_t(1) << 32) - 1 || nnz < 0 ||
      nnz >= (int64_t(1) << 32) - 1 || !d_offset || !d_rperminv || !d_cperminv || !d_poffset ||
      (nnz > 0 && (!d_nonzero || !d_pnonzero))) {
    set_error("bale_permute_dev: bad arguments");
    return BALE_EINVAL;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  Ws w;
  const int64_t nmax = std::max(numrows, numcols);
  void *ws = device_workspace(ws_bytes(std::max<int64_t>(nnz, nmax), nmax, nullptr, nullptr), st);
  if (!ws) return BALE_ENOMEM;
  ws_bytes(std::max<int64_t>(nnz, nmax), nmax, &w, static_cast<char *>(ws));
  unsigned long long *bad = reinterpret_cast<unsigned long long *>(w.words + 4);
  BALE_CUDA_OK(cudaMemsetAsync(w.words, 0, 64, st));
  csr_check_kernel<<<grid_for(std::max(numrows + 1, nnz)), 256, 0, st>>>(d_offset, d_nonzero, numrows, numcols,
                                                                          nnz, bad);
  // both permutations: every label exactly once
  BALE_CUDA_OK(cudaMemsetAsync(w.deg, 0, static_cast<size_t>(numrows) * 4, st));
  perm_seen_kernel<<<grid_for(numrows), 256, 0, st>>>(d_rperminv, numrows, w.deg, bad);
  perm_once_kernel<<<grid_for(numrows), 256, 0, st>>>(w.deg, numrows, bad);
  BALE_CUDA_OK(cudaMemsetAsync(w.newid, 0, static_cast<size_t>(numcols) * 4, st));
  perm_seen_kernel<<<grid_for(numcols), 256, 0, st>>>(d_cperminv, numcols, w.newid, bad);
  perm_once_kernel<<<grid_for(numcols), 256, 0, st>>>(w.newid, numcols, bad);
  unsigned long long nbad = 0;
  BALE_CUDA_OK(cudaMemcpyAsync(&nbad, bad, 8, cudaMemcpyDeviceToHost, st));
  BALE_CUDA_OK(cudaStreamSynchronize(st));
  if (nbad) {
    set_error("bale_permute_dev: %llu malformed offsets, columns or permutation entries", nbad);
    return BALE_EINPUT;
  }
  uint32_t *rperm = w.deg, *len = w.flag, *pstart = w.pos;
  permute_rows_kernel<<<grid_for(numrows), 256, 0, st>>>(d_offset, d_rperminv, numrows, rperm);
  permute_len_kernel<<<grid_for(numrows), 256, 0, st>>>(d_offset, rperm, numrows, len);
  int rc = excl_scan(len, pstart, numrows, w.bsum, w.words, st);
  if (rc != BALE_OK) return rc;
  permute_fill_kernel<<<grid_for(numrows * 32), 256, 0, st>>>(d_offset, d_nonzero, rperm, pstart, numrows, nnz,
                                                              d_cperminv, d_poffset, d_pnonzero);
  BALE_CUDA_OK(cudaGetLastError());
  BALE_CUDA_OK(cudaStreamSynchronize(st));
  return BALE_OK;
}

int bale_rand_perm_dev(int64_t n, uint64_t seed, int64_t *d_perm, void *stream) {
  if (n < 0 || n >= (int64_t(1) << 30) || (n > 0 && !d_perm)) {
    set_error("bale_rand_perm_dev: bad arguments (n=%lld)", static_cast<long long>(n));
    return BALE_EINVAL;
  }
  if (n == 0) return BALE_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const uint64_t m = 2 * static_cast<uint64_t>(n);
  const uint64_t x0 = ((seed & 0xffffffffull) << 16) | 0x330eull;
  int mb = 1;
  while ((uint64_t(1) << mb) < m) mb++;
  // throws: about 1.39 n are needed for n distinct slots among 2n; take
  // 1.5 n + 1024 and double until the n-th first hit is among them
  for (int64_t nt = n + n / 2 + 1024;; nt *= 2) {
    int tb = 1;
    while ((int64_t(1) << tb) < nt) tb++;
    if (mb + tb > 64) {
      set_error("bale_rand_perm_dev: too many throws");
      return BALE_EINVAL;
    }
    Ws w;
    void *ws = device_workspace(ws_bytes(nt, nt, nullptr, nullptr), st);
    if (!ws) return BALE_ENOMEM;
    ws_bytes(nt, nt, &w, static_cast<char *>(ws));
    BALE_CUDA_OK(cudaMemsetAsync(w.words, 0, 64, st));
    const int64_t threads = (nt + kThrowsPerThread - 1) / kThrowsPerThread;
    throws_kernel<<<static_cast<unsigned>((threads + 255) / 256), 256, 0, st>>>(x0, nt, m, tb, w.ka);
    BALE_CUDA_OK(cudaGetLastError());
    int rc = BALE_OK;
    uint64_t *sk = radix_sort(w.ka, w.kb, nt, mb + tb, w, st, &rc);
    if (rc != BALE_OK) return rc;
    uint32_t *succ = w.flag, *rank = w.pos, *used = w.deg, *upos = w.newid;
    first_hit_kernel<<<grid_for(nt), 256, 0, st>>>(sk, nt, tb, succ);
    rc = excl_scan(succ, rank, nt, w.bsum, w.words, st);
    if (rc != BALE_OK) return rc;
    unsigned int hits = 0;
    BALE_CUDA_OK(cudaMemcpyAsync(&hits, w.words, 4, cudaMemcpyDeviceToHost, st));
    BALE_CUDA_OK(cudaStreamSynchronize(st));
    if (static_cast<int64_t>(hits) < n) continue;  // the n-th hit is further on
    used_kernel<<<grid_for(nt), 256, 0, st>>>(sk, nt, tb, succ, rank, static_cast<uint32_t>(n), used);
    rc = excl_scan(used, upos, nt, w.bsum, w.words, st);
    if (rc != BALE_OK) return rc;
    perm_out_kernel<<<grid_for(nt), 256, 0, st>>>(sk, nt, tb, used, upos, rank, d_perm);
    BALE_CUDA_OK(cudaGetLastError());
    BALE_CUDA_OK(cudaStreamSynchronize(st));
    return BALE_OK;
  }
}

int bale_read_matrix_mm_dev(const char *path, int64_t *d_offset, int64_t *d_nonzero, void *stream) {
  int64_t nr = 0, nc = 0, nnz = 0, body = 0;
  int fields = 0;
  int rc = bale_mm_header(path, &nr, &nc, &nnz, &body, &fields);
  if (rc != BALE_OK) {
    set_error("bale_read_matrix_mm_dev: %s: not a coordinate pattern/integer MatrixMarket file", path ? path : "");
    return rc;
  }
  if (!d_offset || (nnz > 0 && !d_nonzero) || nr < 1 || nr > (int64_t(1) << 31) || nnz >= (int64_t(1) << 32) - 1) {
    set_error("bale_read_matrix_mm_dev: bad arguments or sizes");
    return BALE_EINVAL;
  }
  FILE *fp = fopen(path, "rb");
  if (!fp || fseek(fp, 0, SEEK_END) != 0) {
    if (fp) fclose(fp);
    set_error("bale_read_matrix_mm_dev: cannot read %s", path);
    return BALE_EINPUT;
  }
  const int64_t len = static_cast<int64_t>(ftell(fp)) - body;
  if (len < 0 || len >= (int64_t(1) << 32) - 1) {
    fclose(fp);
    set_error("bale_read_matrix_mm_dev: %s: body of %lld bytes is outside the supported range", path,
              static_cast<long long>(len));
    return BALE_EINPUT;
  }
  std::vector<char> text(static_cast<size_t>(len > 0 ? len : 1));
  const bool read_ok = fseek(fp, static_cast<long>(body), SEEK_SET) == 0 &&
                       (len == 0 || fread(text.data(), 1, static_cast<size_t>(len), fp) == static_cast<size_t>(len));
  fclose(fp);
  if (!read_ok) {
    set_error("bale_read_matrix_mm_dev: short read of %s", path);
    return BALE_EINPUT;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int lb = 1;
  while ((int64_t(1) << lb) < std::max<int64_t>(nnz, 1)) lb++;
  // workspace: the text, start flags and their prefix (per byte), line
  // starts and columns (per entry), two key buffers, sort scratch
  const int64_t nn = std::max<int64_t>(nnz, 1), ll = std::max<int64_t>(len, 1);
  const int64_t tiles = (nn + kTile - 1) / kTile;
  const int64_t nb = (std::max(ll + 1, tiles * kDigits) + kScanBlock - 1) / kScanBlock + 1;
  const size_t need = up256(ll) + 2 * up256(4 * (ll + 1)) + 2 * up256(4 * nn) + 2 * up256(8 * nn) +
                      2 * up256(4 * tiles * kDigits) + up256(4 * nb) + 256;
  char *ws = static_cast<char *>(device_workspace(need, st));
  if (!ws) return BALE_ENOMEM;
  char *o = ws;
  auto take = [&](size_t bytes) {
    char *r = o;
    o += up256(bytes);
    return r;
  };
  char *d_text = take(ll);
  Ws w;
  w.flag = reinterpret_cast<uint32_t *>(take(4 * (ll + 1)));
  w.pos = reinterpret_cast<uint32_t *>(take(4 * (ll + 1)));
  uint32_t *linepos = reinterpret_cast<uint32_t *>(take(4 * nn));
  uint32_t *cols = reinterpret_cast<uint32_t *>(take(4 * nn));
  w.ka = reinterpret_cast<uint64_t *>(take(8 * nn));
  w.kb = reinterpret_cast<uint64_t *>(take(8 * nn));
  w.hist = reinterpret_cast<uint32_t *>(take(4 * tiles * kDigits));
  w.hoff = reinterpret_cast<uint32_t *>(take(4 * tiles * kDigits));
  w.bsum = reinterpret_cast<uint32_t *>(take(4 * nb));
  w.words = reinterpret_cast<unsigned int *>(take(64));
  w.va = w.vb = nullptr;
  w.deg = w.newid = nullptr;
  unsigned long long *bad = reinterpret_cast<unsigned long long *>(w.words + 4);
  BALE_CUDA_OK(cudaMemsetAsync(w.words, 0, 64, st));
  if (len > 0) BALE_CUDA_OK(cudaMemcpyAsync(d_text, text.data(), static_cast<size_t>(len), cudaMemcpyHostToDevice, st));
  mm_starts_kernel<<<grid_for(ll), 256, 0, st>>>(d_text, len, w.flag);
  rc = excl_scan(w.flag, w.pos, len, w.bsum, w.words, st);
  if (rc != BALE_OK) return rc;
  unsigned int lines = 0;
  BALE_CUDA_OK(cudaMemcpyAsync(&lines, w.words, 4, cudaMemcpyDeviceToHost, st));
  BALE_CUDA_OK(cudaStreamSynchronize(st));
  if (static_cast<int64_t>(lines) != nnz) {
    set_error("bale_read_matrix_mm_dev: %s: %lld nonzeros in the header, %u entry lines", path,
              static_cast<long long>(nnz), lines);
    return BALE_EINPUT;
  }
  if (nnz > 0) {
    mm_compact_kernel<<<grid_for(ll), 256, 0, st>>>(w.flag, w.pos, len, linepos, nnz);
    mm_parse_kernel<<<grid_for(nnz), 256, 0, st>>>(d_text, len, linepos, nnz, fields, nr, nc, lb, w.ka, cols, bad);
    BALE_CUDA_OK(cudaGetLastError());
  }
  unsigned long long nbad = 0;
  BALE_CUDA_OK(cudaMemcpyAsync(&nbad, bad, 8, cudaMemcpyDeviceToHost, st));
  BALE_CUDA_OK(cudaStreamSynchronize(st));
  if (nbad) {
    set_error("bale_read_matrix_mm_dev: %s: %llu malformed or out-of-range entries", path, nbad);
    return BALE_EINPUT;
  }
  int rb = 1;
  while ((int64_t(1) << rb) < nr) rb++;
  uint64_t *sk = radix_sort(w.ka, w.kb, nnz, rb + lb, w, st, &rc);
  if (rc != BALE_OK) return rc;
  csr_offsets_kernel<<<grid_for(nr + 1), 256, 0, st>>>(sk, nnz, nr, lb, d_offset);
  if (nnz > 0) mm_cols_kernel<<<grid_for(nnz), 256, 0, st>>>(sk, nnz, lb, cols, d_nonzero);
  BALE_CUDA_OK(cudaGetLastError());
  BALE_CUDA_OK(cudaStreamSynchronize(st));
  return BALE_OK;
}

}  // extern "C"
