// tri_device.cuh -- per-row procedures of the bitmap/search triangle count,
// shared by the standalone kernels (tri_hybrid.cu) and the batched work-queue
// kernel (batch.cu).  C is the column element type: uint32_t (a compacted
// copy, kBadCol marking a column that does not fit) or int64_t (the
// reference's own sparsemat_t array).
//
// The count is the reference's alg 0 (apps/triangle_src/triangle_agi.upc:69-99):
// for every nonzero L[i][j] after the first of row i, |row_i and row_j|.
#pragma once

#include "common.cuh"

namespace bale {
namespace tri {

constexpr unsigned kFull = 0xffffffffu;
constexpr int64_t kHeavyBits = int64_t(1) << 19;  // heavy rows: labels below 2^19 (64 KiB bitmap)
constexpr int kHeavyMinDeg = 64;                  // ... with at least 64 nonzeros
constexpr int kLightCap = 1024;                   // row-i elements a warp keeps in shared memory
constexpr uint32_t kBadCol = 0xffffffffu;

__device__ __forceinline__ int64_t colv(const uint32_t *c, int64_t k) { return static_cast<int64_t>(c[k]); }
__device__ __forceinline__ int64_t colv(const int64_t *c, int64_t k) { return c[k]; }

// Rows below `bits` with at least kHeavyMinDeg nonzeros are heavy.  Both the
// heavy and the light procedures apply this test to the same raw offsets, so
// every row is handled (and validated) by exactly one of them.
__device__ __forceinline__ bool is_heavy(int64_t i, int64_t b, int64_t e, int64_t bits) {
  return i < bits && e - b >= kHeavyMinDeg;
}

// A path's kernels return at once when a device-made choice picked the
// other one (run_if: null, or a word that must read `want`).
__device__ __forceinline__ bool skipped(const unsigned *run_if, unsigned want) {
  return run_if && *run_if != want;
}

// Bit w of the row-i bitmap.  The word index is masked to the power-of-two
// bitmap size, so a malformed row j never indexes outside it; such a row is
// itself flagged when it is processed as row i, which fails the whole count.
__device__ __forceinline__ uint32_t bit_of(const uint32_t *__restrict__ bm, uint32_t wmask, uint32_t w) {
  return __funnelshift_r(bm[(w >> 5) & wmask], 0u, w) & 1u;
}

// Number of elements of the run r[0,len) whose bit is set (whole warp).
__device__ __forceinline__ uint32_t count_in_bitmap(const uint32_t *__restrict__ bm, uint32_t wmask,
                                                    const uint32_t *__restrict__ r, int64_t len) {
  const unsigned lane = lane_id();
  uint32_t c = 0;
  int64_t head = static_cast<int64_t>(((16u - (reinterpret_cast<uintptr_t>(r) & 15u)) & 15u) >> 2);
  if (head > len) head = len;
  if (static_cast<int64_t>(lane) < head) c += bit_of(bm, wmask, r[lane]);
  const uint4 *__restrict__ r4 = reinterpret_cast<const uint4 *>(r + head);
  const int64_t n4 = (len - head) >> 2;
  int64_t v = lane;
  for (; v + 32 < n4; v += 64) {
    const uint4 x = r4[v], y = r4[v + 32];
    c += bit_of(bm, wmask, x.x) + bit_of(bm, wmask, x.y) + bit_of(bm, wmask, x.z) + bit_of(bm, wmask, x.w);
    c += bit_of(bm, wmask, y.x) + bit_of(bm, wmask, y.y) + bit_of(bm, wmask, y.z) + bit_of(bm, wmask, y.w);
  }
  if (v < n4) {
    const uint4 x = r4[v];
    c += bit_of(bm, wmask, x.x) + bit_of(bm, wmask, x.y) + bit_of(bm, wmask, x.z) + bit_of(bm, wmask, x.w);
  }
  const int64_t tail = head + 4 * n4;
  if (tail + static_cast<int64_t>(lane) < len) c += bit_of(bm, wmask, r[tail + lane]);
  return c;
}

__device__ __forceinline__ uint32_t count_in_bitmap(const uint32_t *__restrict__ bm, uint32_t wmask,
                                                    const int64_t *__restrict__ r, int64_t len) {
  const unsigned lane = lane_id();
  uint32_t c = 0;
  const int64_t head = (reinterpret_cast<uintptr_t>(r) & 15u) ? 1 : 0;
  if (lane == 0 && head && len > 0) c += bit_of(bm, wmask, static_cast<uint32_t>(r[0]));
  const longlong2 *__restrict__ r2 = reinterpret_cast<const longlong2 *>(r + head);
  const int64_t n2 = len > head ? (len - head) >> 1 : 0;
  for (int64_t v = lane; v < n2; v += 32) {
    const longlong2 x = r2[v];
    c += bit_of(bm, wmask, static_cast<uint32_t>(x.x)) + bit_of(bm, wmask, static_cast<uint32_t>(x.y));
  }
  const int64_t tail = head + 2 * n2;
  if (lane == 0 && tail < len) c += bit_of(bm, wmask, static_cast<uint32_t>(r[tail]));
  return c;
}

// Is w in the ascending run r[0,len)?
template <typename R>
__device__ __forceinline__ bool search_run(const R *__restrict__ r, int64_t len, int64_t w) {
  int64_t lo = 0, hi = len;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (colv(r, mid) < w) lo = mid + 1; else hi = mid;
  }
  return lo < len && colv(r, lo) == w;
}

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

struct Tally {
  unsigned long long cnt = 0, work = 0, bad = 0;
};

// One light row, processed by a whole warp; rb is the warp's kLightCap-entry
// shared-memory slot.  Heavy rows are skipped (their owner validates them).
// For each neighbour j at position q the cheaper side is searched: stream
// row j and binary-search each element in ri[0,q), or binary-search each of
// ri[0,q) in row j (when q * log2|row j| < |row j|).
template <typename C>
__device__ void light_row(const int64_t *__restrict__ off, const C *__restrict__ col, int64_t i, int64_t nnz,
                          int64_t bits, uint32_t *__restrict__ rb, Tally &t) {
  const unsigned lane = lane_id();
  const int64_t b = off[i], e = off[i + 1];
  if (is_heavy(i, b, e, bits)) return;
  if (b < 0 || e < b || e > nnz) {
    if (lane == 0) t.bad++;
    return;
  }
  const int64_t d = e - b;
  if (d < 2) {
    if (d == 1 && lane == 0) {
      const int64_t c = colv(col, b);
      if (c < 0 || c >= i) t.bad++;
    }
    return;
  }
  const bool cached = d <= kLightCap && i <= 0xffffffffll;  // cached columns are < i
  bool ok = true;
  for (int64_t k = lane; k < d; k += 32) {
    const int64_t c = colv(col, b + k);
    ok &= c >= 0 && c < i;
    if (k > 0) ok &= c > colv(col, b + k - 1);
    if (cached) rb[k] = static_cast<uint32_t>(c);
  }
  __syncwarp();
  if (!__all_sync(kFull, ok)) {
    if (lane == 0) t.bad++;
    __syncwarp();
    return;
  }
  const C *__restrict__ rg = col + b;
  for (int64_t q0 = 1; q0 < d; q0 += 32) {
    const int64_t q = q0 + lane;
    int64_t jb = 0, jlen = 0, sl = 0, pq = 0;
    if (q < d) {
      const int64_t j = cached ? static_cast<int64_t>(rb[q]) : colv(rg, q);
      const int64_t s = off[j], u = off[j + 1];
      if (s < 0 || u < s || u > nnz) {
        t.bad++;
      } else {
        jb = s;
        jlen = u - s;
        const int64_t steps = 64 - __clzll(static_cast<unsigned long long>(jlen) + 1ull);
        if (q * steps < jlen) pq = q; else sl = jlen;
      }
    }
    // (1) streamed neighbours: every element of row j searched in ri[0,q)
    const int64_t inc = warp_incl_scan(sl);
    const int64_t tot = __shfl_sync(kFull, inc, 31);
    if (lane == 0) t.work += static_cast<unsigned long long>(tot);
    for (int64_t base = 0; base < tot; base += 32) {
      const int64_t kk = base + lane;
      const int o = owner_lane(inc, kk);
      const int64_t o_inc = __shfl_sync(kFull, inc, o);
      const int64_t o_len = __shfl_sync(kFull, sl, o);
      const int64_t o_jb = __shfl_sync(kFull, jb, o);
      if (kk < tot) {
        const int64_t w = colv(col, o_jb + (kk - (o_inc - o_len)));
        const bool hit = cached ? search_run(rb, q0 + o, w) : search_run(rg, q0 + o, w);
        t.cnt += hit ? 1ull : 0ull;
      }
    }
    // (2) searched neighbours: each ri[r], r < q, searched in row j
    const int64_t inc2 = warp_incl_scan(pq);
    const int64_t tot2 = __shfl_sync(kFull, inc2, 31);
    if (lane == 0) t.work += static_cast<unsigned long long>(tot2);
    for (int64_t base = 0; base < tot2; base += 32) {
      const int64_t kk = base + lane;
      const int o = owner_lane(inc2, kk);
      const int64_t o_inc = __shfl_sync(kFull, inc2, o);
      const int64_t o_pq = __shfl_sync(kFull, pq, o);
      const int64_t o_jb = __shfl_sync(kFull, jb, o);
      const int64_t o_len = __shfl_sync(kFull, jlen, o);
      if (kk < tot2) {
        const int64_t r = kk - (o_inc - o_pq);
        const int64_t w = cached ? static_cast<int64_t>(rb[r]) : colv(rg, r);
        t.cnt += search_run(col + o_jb, o_len, w) ? 1ull : 0ull;
      }
    }
  }
  __syncwarp();
}

// One heavy row, processed by the whole block (THREADS threads); bm is a
// zeroed bitmap of (wmask+1) words in shared memory and is zero again on
// return.  Every thread must call this with the same i.
template <typename C, int THREADS>
__device__ void heavy_row(const int64_t *__restrict__ off, const C *__restrict__ col, int64_t i, int64_t nnz,
                          uint32_t *__restrict__ bm, uint32_t wmask, Tally &t) {
  const unsigned lane = lane_id();
  const int warp = threadIdx.x >> 5;
  const int64_t b = off[i], e = off[i + 1];
  if (b < 0 || e < b || e > nnz) {
    if (threadIdx.x == 0) t.bad++;
    return;
  }
  const int64_t d = e - b;
  bool ok = true;
  for (int64_t k = threadIdx.x; k < d; k += THREADS) {
    const int64_t c = colv(col, b + k);
    const bool in = c >= 0 && c < i;
    ok &= in;
    if (k > 0) ok &= c > colv(col, b + k - 1);
    if (in) atomicOr(&bm[static_cast<uint32_t>(c) >> 5], 1u << (static_cast<uint32_t>(c) & 31));
  }
  ok = __syncthreads_and(ok);
  if (ok) {
    for (int64_t q = 1 + warp; q < d; q += THREADS / 32) {
      const int64_t j = colv(col, b + q);
      const int64_t s = off[j], u = off[j + 1];
      if (s < 0 || u < s || u > nnz) {
        if (lane == 0) t.bad++;
        continue;
      }
      if (lane == 0) t.work += static_cast<unsigned long long>(u - s);
      t.cnt += count_in_bitmap(bm, wmask, col + s, u - s);
    }
  } else if (threadIdx.x == 0) {
    t.bad++;
  }
  __syncthreads();
  for (int64_t k = threadIdx.x; k < d; k += THREADS) {
    const int64_t c = colv(col, b + k);
    if (c >= 0 && c < i) bm[static_cast<uint32_t>(c) >> 5] = 0;
  }
  __syncthreads();
}

// Smallest power of two >= 32 covering min(numrows, kHeavyBits) labels.
__host__ __device__ inline int64_t bitmap_bits(int64_t numrows) {
  int64_t bits = 32;
  while (bits < numrows && bits < kHeavyBits) bits <<= 1;
  return bits;
}

}  // namespace tri
}  // namespace bale
