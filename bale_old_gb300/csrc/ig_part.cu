// ig_part.cu -- index gather for tables larger than L2, by region partitioning.
//
// A random 8-byte read of a table that does not fit in L2 costs far more
// DRAM traffic than its 8 bytes: the line it lands in is fetched whole and
// is almost never reused before eviction.  bale's exstack/conveyor variants
// (apps/ig_src/ig_exstack.upc:69-94) solve the same problem across PEs by
// sending each request to the PE that owns the table slice and shipping the
// reply back.  Here the "PEs" are L2-sized regions of the table and the
// exchange happens through HBM in three coalesced passes:
//
//  1. partition: each 2048-request chunk is counting-sorted in shared memory
//     by region (region = 2^21 entries = 16 MiB), whole chunks by a kernel
//     without per-element bounds checks.  Each request becomes one
//     u32 (offset in its region << 11 | position in its chunk), written back
//     grouped by region, plus the chunk's region boundaries (u16);
//  2. gather: (region, chunk) segments are processed region-major, so at any
//     time the whole GPU reads one region, which stays resident in L2; the
//     table values are written next to their requests;
//  3. unpermute: each chunk scatters its values to their positions in a
//     shared-memory tile, which is stored to tgt with 16-byte stores.
//
// Per request that is ~46 bytes of streaming traffic (8 index + 4+4+4 entry
// + 8+8 value + 8 output) and the table is read about once, instead of one
// mostly wasted DRAM line per request.  Table reads may allocate in L1: a
// skewed request stream keeps its hot entries there instead of queueing on
// their L2 slices.
//
// A strongly skewed stream (Zipf-like, most requests on few entries) is
// better served by the direct gather, whose L1 and L2 keep the hot entries
// for every request.  ig_skew_kernel samples the index stream and writes the
// choice to a device word; the three kernels here return at once when it
// chose the direct gather, and the direct gather returns when it did not.
#include "common.cuh"

namespace bale {

namespace {

constexpr int kThreads = 256;
constexpr int kCBits = kIgChunkBits;
constexpr int kChunk = 1 << kCBits;       // requests per chunk: 2048
constexpr int kRBits = kIgRegionBits;     // log2(entries per region) = 21: 16 MiB of table
constexpr int kMaxRegions = static_cast<int>(kIgMaxRegions);
constexpr int kPer = kChunk / kThreads;   // requests per thread in the partition and unpermute
static_assert(kPer % 4 == 0, "whole 16-byte vectors per thread");
constexpr int kDescPerClaim = 8;          // (region, chunk) segments a warp claims at once

// Exclusive scan of a[0,m) in shared memory, in place; a[m] = total.
// m <= kThreads * 8.  Called by all threads of the block.
__device__ void block_exclusive_scan(uint32_t *a, int m) {
  __shared__ uint32_t warp_tot[kThreads / 32];
  const int per = (m + kThreads - 1) / kThreads;
  const int lo = threadIdx.x * per;
  uint32_t sum = 0;
  for (int i = 0; i < per; i++)
    if (lo + i < m) sum += a[lo + i];
  // inclusive warp scan of per-thread sums
  uint32_t inc = sum;
  const unsigned lane = lane_id();
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
    if (static_cast<int>(lane) >= o) inc += y;
  }
  if (lane == 31) warp_tot[threadIdx.x >> 5] = inc;
  __syncthreads();
  uint32_t wbase = 0;
  for (int w = 0; w < static_cast<int>(threadIdx.x >> 5); w++) wbase += warp_tot[w];
  uint32_t run = wbase + inc - sum;  // exclusive prefix of this thread's slice
  for (int i = 0; i < per; i++) {
    if (lo + i < m) {
      uint32_t v = a[lo + i];
      a[lo + i] = run;
      run += v;
    }
  }
  if (threadIdx.x == kThreads - 1) a[m] = wbase + inc;
  __syncthreads();
}

// Partition of one chunk of any length (the last, partial chunk of a call):
// chunk c = chunk0 + blockIdx.x.
__global__ void __launch_bounds__(kThreads)
    igp_partition_kernel(const int64_t *__restrict__ index, int64_t n, uint64_t tlen, int shift, int nreg,
                         uint32_t *__restrict__ entries, uint16_t *__restrict__ starts, int64_t chunk0,
                         const unsigned *__restrict__ direct) {
  __shared__ uint32_t hist[kMaxRegions + 2];
  __shared__ __align__(16) uint32_t stage[kChunk];
  if (direct && *direct) return;
  const int64_t c = chunk0 + blockIdx.x;
  const int64_t base = c * kChunk;
  const int len = static_cast<int>(n - base < kChunk ? n - base : kChunk);
  for (int i = threadIdx.x; i < nreg + 2; i += kThreads) hist[i] = 0;
  __syncthreads();
  uint32_t key[kPer], reg[kPer], rank[kPer];
#pragma unroll
  for (int s = 0; s < kPer; s++) {
    const int e = s * kThreads + threadIdx.x;
    if (e < len) {
      const uint64_t k = static_cast<uint64_t>(index[base + e] >> shift);
      const bool ok = k < tlen;
      reg[s] = ok ? static_cast<uint32_t>(k >> kRBits) : static_cast<uint32_t>(nreg);
      key[s] = ok ? ((static_cast<uint32_t>(k) << kCBits) | static_cast<uint32_t>(e)) : static_cast<uint32_t>(e);
      rank[s] = atomicAdd(&hist[reg[s]], 1u);
    }
  }
  __syncthreads();
  block_exclusive_scan(hist, nreg + 1);  // hist[b] = start of region b; hist[nreg+1] = len
  uint16_t *st = starts + c * (nreg + 2);
  for (int i = threadIdx.x; i < nreg + 2; i += kThreads) st[i] = static_cast<uint16_t>(hist[i]);
#pragma unroll
  for (int s = 0; s < kPer; s++)
    if (s * kThreads + static_cast<int>(threadIdx.x) < len) stage[hist[reg[s]] + rank[s]] = key[s];
  __syncthreads();
  for (int i = threadIdx.x; i < len; i += kThreads) entries[base + i] = stage[i];
}

// Partition of whole chunks (every chunk but a partial last one), with no
// per-element bounds checks: branches and their bookkeeping were most of the
// instructions of the general kernel, which made it instruction-bound; this
// one moves its 12 bytes per request at close to the HBM rate.  The region
// ranks come from shared-memory atomics on one counter per region; for up to
// 62 regions (tables up to 62 * 2^21 entries) one warp scans the counters.
template <int SHIFT>
__global__ void __launch_bounds__(kThreads)
    igp_partition_full_kernel(const int64_t *__restrict__ index, uint64_t tlen, int nreg,
                              uint32_t *__restrict__ entries, uint16_t *__restrict__ starts,
                              const unsigned *__restrict__ direct) {
  __shared__ uint32_t hist[kMaxRegions + 2];
  __shared__ __align__(16) uint32_t stage[kChunk];  // read back as uint4
  if (direct && *direct) return;
  const int t = threadIdx.x;
  const int64_t c = blockIdx.x;
  const uint64_t pol = policy_evict_first();
  const longlong2 *src = reinterpret_cast<const longlong2 *>(index + c * kChunk);
  longlong2 v[kPer / 2];
#pragma unroll
  for (int h = 0; h < kPer / 2; h++) v[h] = ld_v2_s64_pol(src + h * kThreads + t, pol);
  for (int i = t; i < nreg + 2; i += kThreads) hist[i] = 0;
  __syncthreads();
  uint32_t key[kPer], reg[kPer], rank[kPer];
#pragma unroll
  for (int h = 0; h < kPer / 2; h++) {
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const int s = 2 * h + j;
      const uint64_t k = static_cast<uint64_t>((j ? v[h].y : v[h].x) >> SHIFT);
      const uint32_t e = static_cast<uint32_t>(2 * (h * kThreads + t) + j);  // position in the chunk
      const bool ok = k < tlen;
      reg[s] = ok ? static_cast<uint32_t>(k >> kRBits) : static_cast<uint32_t>(nreg);
      key[s] = ok ? ((static_cast<uint32_t>(k) << kCBits) | e) : e;  // the shift drops the region bits
      rank[s] = atomicAdd(&hist[reg[s]], 1u);
    }
  }
  __syncthreads();
  uint16_t *st = starts + c * (nreg + 2);
  if (nreg + 2 <= 64) {
    if (t < 32) {  // counters 2t and 2t+1 per lane: nreg + 1 regions and the total
      const int r0 = 2 * t, r1 = 2 * t + 1;
      const uint32_t a0 = r0 <= nreg ? hist[r0] : 0u, a1 = r1 <= nreg ? hist[r1] : 0u;
      uint32_t inc = a0 + a1;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (t >= o) inc += y;
      }
      const uint32_t ex = inc - a0 - a1;
      if (r0 <= nreg + 1) {
        hist[r0] = ex;
        st[r0] = static_cast<uint16_t>(ex);
      }
      if (r1 <= nreg + 1) {
        hist[r1] = ex + a0;
        st[r1] = static_cast<uint16_t>(ex + a0);
      }
    }
  } else {
    block_exclusive_scan(hist, nreg + 1);
    for (int i = t; i < nreg + 2; i += kThreads) st[i] = static_cast<uint16_t>(hist[i]);
  }
  __syncthreads();
#pragma unroll
  for (int s = 0; s < kPer; s++) stage[hist[reg[s]] + rank[s]] = key[s];
  __syncthreads();
  uint4 *dst = reinterpret_cast<uint4 *>(entries + c * kChunk);
#pragma unroll
  for (int q = 0; q < kPer / 4; q++)
    st_v4_u32_pol(dst + q * kThreads + t, reinterpret_cast<const uint4 *>(stage)[q * kThreads + t], pol);
}

// Both partition kernels over the n requests: whole chunks, then the partial
// last one.
int launch_partition(const int64_t *index, int64_t n, uint64_t tlen, int shift, int nreg, uint32_t *entries,
                     uint16_t *starts, const unsigned *direct, cudaStream_t stream) {
  const int64_t nfull = n / kChunk;
  if (nfull > 0) {
    if (shift == 16)
      igp_partition_full_kernel<16><<<static_cast<unsigned>(nfull), kThreads, 0, stream>>>(index, tlen, nreg, entries,
                                                                                        starts, direct);
    else
      igp_partition_full_kernel<0><<<static_cast<unsigned>(nfull), kThreads, 0, stream>>>(index, tlen, nreg, entries,
                                                                                       starts, direct);
    BALE_CUDA_OK(cudaGetLastError());
  }
  if (n % kChunk) {
    igp_partition_kernel<<<1, kThreads, 0, stream>>>(index, n, tlen, shift, nreg, entries, starts, nfull, direct);
    BALE_CUDA_OK(cudaGetLastError());
  }
  return BALE_OK;
}

// Segment (region b, chunk c): entries[c*kChunk + s .. c*kChunk + e).
__global__ void __launch_bounds__(kThreads)
    igp_gather_kernel(const uint32_t *__restrict__ entries, const uint16_t *__restrict__ starts,
                      int64_t nchunks, int nreg, const int64_t *__restrict__ table,
                      int64_t *__restrict__ val, unsigned long long *__restrict__ cursor,
                      unsigned long long *__restrict__ bad, const unsigned *__restrict__ direct) {
  if (direct && *direct) return;
  const unsigned lane = lane_id();
  const uint64_t ef = policy_evict_first();
  const int64_t total = static_cast<int64_t>(nreg + 1) * nchunks;
  unsigned long long nbad = 0;
  for (;;) {
    unsigned long long d0 = 0;
    if (lane == 0) d0 = atomicAdd(cursor, static_cast<unsigned long long>(kDescPerClaim));
    d0 = __shfl_sync(0xffffffffu, d0, 0);
    if (static_cast<int64_t>(d0) >= total) break;
    for (int g = 0; g < kDescPerClaim; g++) {
      const int64_t d = static_cast<int64_t>(d0) + g;
      if (d >= total) break;
      const int b = static_cast<int>(d / nchunks);
      const int64_t c = d - static_cast<int64_t>(b) * nchunks;
      const uint16_t *st = starts + c * (nreg + 2) + b;
      const int s = st[0], e = st[1];
      const uint32_t *ent = entries + c * kChunk;
      int64_t *vo = val + c * kChunk;
      if (b < nreg) {
        const int64_t *reg = table + (static_cast<int64_t>(b) << kRBits);
        for (int k = s + static_cast<int>(lane); k < e; k += 128) {
          uint32_t kk[4];
          int64_t v[4];
#pragma unroll
          for (int u = 0; u < 4; u++)
            kk[u] = (k + 32 * u < e) ? ld_u32_pol(ent + k + 32 * u, ef) : 0u;
#pragma unroll
          for (int u = 0; u < 4; u++)
            v[u] = (k + 32 * u < e) ? __ldg(reg + (kk[u] >> kCBits)) : 0;  // may allocate in L1
#pragma unroll
          for (int u = 0; u < 4; u++)
            if (k + 32 * u < e) st_s64_pol(vo + k + 32 * u, v[u], ef);
        }
      } else {
        for (int k = s + static_cast<int>(lane); k < e; k += 32) {
          st_s64_pol(vo + k, 0, ef);  // out-of-range request: value 0, counted
          nbad++;
        }
      }
    }
  }
  nbad = warp_sum_u64(nbad);
  if (lane == 0 && nbad) atomicAdd(bad, nbad);
}

// Histogram over the same partition: region-major L2 reductions, so the
// counters of one region stay in L2 while every chunk's updates to it land.
__global__ void __launch_bounds__(kThreads)
    igp_histo_kernel(const uint32_t *__restrict__ entries, const uint16_t *__restrict__ starts,
                     int64_t nchunks, int nreg, int64_t *__restrict__ counts,
                     unsigned long long *__restrict__ cursor, unsigned long long *__restrict__ bad) {
  const unsigned lane = lane_id();
  const uint64_t ef = policy_evict_first();
  const int64_t total = static_cast<int64_t>(nreg + 1) * nchunks;
  unsigned long long nbad = 0;
  for (;;) {
    unsigned long long d0 = 0;
    if (lane == 0) d0 = atomicAdd(cursor, static_cast<unsigned long long>(kDescPerClaim));
    d0 = __shfl_sync(0xffffffffu, d0, 0);
    if (static_cast<int64_t>(d0) >= total) break;
    for (int g = 0; g < kDescPerClaim; g++) {
      const int64_t d = static_cast<int64_t>(d0) + g;
      if (d >= total) break;
      const int b = static_cast<int>(d / nchunks);
      const int64_t c = d - static_cast<int64_t>(b) * nchunks;
      const uint16_t *st = starts + c * (nreg + 2) + b;
      const int s = st[0], e = st[1];
      if (b == nreg) {  // out-of-range updates: counted, not applied
        if (lane == 0) nbad += static_cast<unsigned long long>(e - s);
        continue;
      }
      const uint32_t *ent = entries + c * kChunk;
      int64_t *reg = counts + (static_cast<int64_t>(b) << kRBits);
      for (int k = s + static_cast<int>(lane); k < e; k += 32)
        red_add_u64(reg + (ld_u32_pol(ent + k, ef) >> kCBits), 1ull);
    }
  }
  if (lane == 0 && nbad) atomicAdd(bad, nbad);
}

__global__ void __launch_bounds__(kThreads)
    igp_unpermute_kernel(const uint32_t *__restrict__ entries, const int64_t *__restrict__ val,
                         int64_t *__restrict__ tgt, int64_t n, const unsigned *__restrict__ direct) {
  __shared__ __align__(16) int64_t tile[kChunk];
  if (direct && *direct) return;
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kChunk;
  const int len = static_cast<int>(n - base < kChunk ? n - base : kChunk);
  const uint64_t ef = policy_evict_first();
  if (len == kChunk) {
#pragma unroll
    for (int q = 0; q < kPer / 4; q++) {
      const int at = q * kThreads + threadIdx.x;  // entries 4 at..4 at+3
      const uint4 e = ld_v4_u32_pol(reinterpret_cast<const uint4 *>(entries + base) + at, ef);
      const longlong2 *vp = reinterpret_cast<const longlong2 *>(val + base) + 2 * at;
      const longlong2 v0 = ld_v2_s64_pol(vp, ef), v1 = ld_v2_s64_pol(vp + 1, ef);
      tile[e.x & (kChunk - 1)] = v0.x;
      tile[e.y & (kChunk - 1)] = v0.y;
      tile[e.z & (kChunk - 1)] = v1.x;
      tile[e.w & (kChunk - 1)] = v1.y;
    }
  } else {
    for (int i = threadIdx.x; i < len; i += kThreads)
      tile[entries[base + i] & (kChunk - 1)] = val[base + i];
  }
  __syncthreads();
  longlong2 *out = reinterpret_cast<longlong2 *>(tgt + base);
  for (int p = threadIdx.x; 2 * p < len; p += kThreads) {
    if (2 * p + 1 < len) st_stream_v2(out + p, make_longlong2(tile[2 * p], tile[2 * p + 1]));
    else st_stream(tgt + base + 2 * p, tile[2 * p]);
  }
}

// Is the request stream skewed enough for the direct gather?  One block
// samples kSkewSamples requests (runs spread evenly over the stream),
// inserts their 32-byte table sectors into a shared-memory hash set and
// counts the samples whose sector was already there.  *direct = 1 when at least repeat_pct
// percent of them were: Zipf(s) requests over 2^26 entries repeat 0.04%
// (uniform), 36% (s = 1.01), 55% (s = 1.1) and 83% (s = 1.3) of an
// 8192-sample, and the direct gather overtakes the partitioned one between
// 36% and 55%.
constexpr int kSkewSamples = 8192;
constexpr int kSkewSlots = 2 * kSkewSamples;  // the set is never more than half full
constexpr int kSkewThreads = 1024;
constexpr int kSkewRun = 128;                       // consecutive requests per run (1 KiB)
constexpr int kSkewRuns = kSkewSamples / kSkewRun;  // 64
static_assert(kSkewSamples % kSkewThreads == 0 && kSkewSamples % kSkewRun == 0, "whole samples");

__global__ void __launch_bounds__(kSkewThreads)
    ig_skew_kernel(const int64_t *__restrict__ index, int64_t n, int shift, uint64_t tlen, int repeat_pct,
                   unsigned *__restrict__ direct) {
  extern __shared__ uint32_t set[];  // kSkewSlots words (dynamic: above the static limit)
  __shared__ unsigned repeats;
  for (int i = threadIdx.x; i < kSkewSlots; i += kSkewThreads) set[i] = 0;
  if (threadIdx.x == 0) repeats = 0;
  __syncthreads();
  // kSkewRuns runs of kSkewRun consecutive requests, evenly spaced: whole
  // lines, so the one block needs few memory transactions
  const int64_t step = n / kSkewRuns;  // >= kSkewRun: callers sample streams of at least kSkewSamples
  constexpr int kPer = kSkewSamples / kSkewThreads;
  int64_t raw[kPer];
#pragma unroll
  for (int r = 0; r < kPer; r++) {
    const int t = threadIdx.x + r * kSkewThreads;
    raw[r] = index[static_cast<int64_t>(t / kSkewRun) * step + t % kSkewRun];
  }
  unsigned mine = 0;
#pragma unroll
  for (int r = 0; r < kPer; r++) {
    const uint64_t k = static_cast<uint64_t>(raw[r] >> shift);
    const uint32_t key = k < tlen ? static_cast<uint32_t>(k >> 2) + 1u : 0xffffffffu;  // 0 marks a free slot
    uint32_t h = (key * 0x9e3779b1u) >> (32 - 14);  // kSkewSlots = 2^14
    for (int probe = 0; probe < kSkewSlots; probe++) {
      const uint32_t old = atomicCAS(&set[h], 0u, key);
      if (old == 0u) break;
      if (old == key) {
        mine++;
        break;
      }
      h = (h + 1u) & (kSkewSlots - 1u);
    }
  }
  if (mine) atomicAdd(&repeats, mine);
  __syncthreads();
  if (threadIdx.x == 0) *direct = repeats * 100u >= static_cast<unsigned>(repeat_pct) * kSkewSamples ? 1u : 0u;
}
static_assert(kSkewSlots == 1 << 14, "the hash takes the top 14 bits");

}  // namespace

size_t ig_part_workspace_bytes(int64_t n, int64_t table_len) {
  const int64_t nchunks = (n + kChunk - 1) / kChunk;
  const int64_t nreg = (table_len + (int64_t(1) << kRBits) - 1) >> kRBits;
  size_t b = 0;
  b += static_cast<size_t>(nchunks) * kChunk * sizeof(uint32_t);  // entries
  b += static_cast<size_t>(nchunks) * kChunk * sizeof(int64_t);   // values
  b += ((static_cast<size_t>(nchunks) * (nreg + 2) * sizeof(uint16_t)) + 255) & ~size_t(255);
  return b;
}

// Entries and region starts only (no values): the histogram's workspace.
size_t histo_part_workspace_bytes(int64_t n, int64_t ncounts) {
  const int64_t nchunks = (n + kChunk - 1) / kChunk;
  const int64_t nreg = (ncounts + (int64_t(1) << kRBits) - 1) >> kRBits;
  return static_cast<size_t>(nchunks) * kChunk * sizeof(uint32_t) +
         (((static_cast<size_t>(nchunks) * (nreg + 2) * sizeof(uint16_t)) + 255) & ~size_t(255));
}

int launch_histo_partitioned(int64_t *counts, int64_t ncounts, const int64_t *index, int64_t n, int shift,
                             unsigned long long *bad, void *ws, unsigned long long *cursor,
                             cudaStream_t stream) {
  const int64_t nchunks = (n + kChunk - 1) / kChunk;
  const int nreg = static_cast<int>((ncounts + (int64_t(1) << kRBits) - 1) >> kRBits);
  uint32_t *entries = static_cast<uint32_t *>(ws);
  uint16_t *starts = reinterpret_cast<uint16_t *>(static_cast<char *>(ws) +
                                                  static_cast<size_t>(nchunks) * kChunk * sizeof(uint32_t));
  BALE_CUDA_OK(cudaMemsetAsync(cursor, 0, sizeof(unsigned long long), stream));
  int rc = launch_partition(index, n, static_cast<uint64_t>(ncounts), shift, nreg, entries, starts, nullptr, stream);
  if (rc != BALE_OK) return rc;
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, igp_histo_kernel, kThreads, 0) != cudaSuccess || occ < 1)
    occ = 1;
  int64_t blocks = static_cast<int64_t>(num_sms()) * occ;
  const int64_t warps_needed = ((nreg + 1) * nchunks + kDescPerClaim - 1) / kDescPerClaim;
  if (blocks * (kThreads / 32) > warps_needed) blocks = (warps_needed + (kThreads / 32) - 1) / (kThreads / 32);
  if (blocks < 1) blocks = 1;
  igp_histo_kernel<<<static_cast<unsigned>(blocks), kThreads, 0, stream>>>(entries, starts, nchunks, nreg,
                                                                         counts, cursor, bad);
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

bool ig_part_supported(int64_t n, int64_t table_len) {
  return n > 0 && table_len > 0 && table_len <= (int64_t(kMaxRegions) << kRBits);
}

int launch_ig_skew(const int64_t *index, int64_t n, int shift, int64_t table_len, int repeat_pct, unsigned *direct,
                   cudaStream_t stream) {
  if (n < kSkewSamples) {
    BALE_CUDA_OK(cudaMemsetAsync(direct, 0, sizeof(unsigned), stream));
    return BALE_OK;
  }
  const int smem = kSkewSlots * static_cast<int>(sizeof(uint32_t));
  BALE_CUDA_OK(cudaFuncSetAttribute(ig_skew_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  ig_skew_kernel<<<1, kSkewThreads, smem, stream>>>(index, n, shift, static_cast<uint64_t>(table_len), repeat_pct,
                                                    direct);
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

int launch_ig_partitioned(int64_t *tgt, const int64_t *index, int64_t n, const int64_t *table,
                          int64_t table_len, int shift, unsigned long long *bad, void *ws,
                          unsigned long long *cursor, cudaStream_t stream, const unsigned *direct) {
  const int64_t nchunks = (n + kChunk - 1) / kChunk;
  const int nreg = static_cast<int>((table_len + (int64_t(1) << kRBits) - 1) >> kRBits);
  char *p = static_cast<char *>(ws);
  uint32_t *entries = reinterpret_cast<uint32_t *>(p);
  p += static_cast<size_t>(nchunks) * kChunk * sizeof(uint32_t);
  int64_t *val = reinterpret_cast<int64_t *>(p);
  p += static_cast<size_t>(nchunks) * kChunk * sizeof(int64_t);
  uint16_t *starts = reinterpret_cast<uint16_t *>(p);

  BALE_CUDA_OK(cudaMemsetAsync(cursor, 0, sizeof(unsigned long long), stream));
  int rc = launch_partition(index, n, static_cast<uint64_t>(table_len), shift, nreg, entries, starts, direct, stream);
  if (rc != BALE_OK) return rc;
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, igp_gather_kernel, kThreads, 0) != cudaSuccess || occ < 1)
    occ = 1;
  int64_t blocks = static_cast<int64_t>(num_sms()) * occ;
  const int64_t warps_needed = ((nreg + 1) * nchunks + kDescPerClaim - 1) / kDescPerClaim;
  if (blocks * (kThreads / 32) > warps_needed) blocks = (warps_needed + (kThreads / 32) - 1) / (kThreads / 32);
  if (blocks < 1) blocks = 1;
  igp_gather_kernel<<<static_cast<unsigned>(blocks), kThreads, 0, stream>>>(entries, starts, nchunks, nreg,
                                                                          table, val, cursor, bad, direct);
  BALE_CUDA_OK(cudaGetLastError());
  igp_unpermute_kernel<<<static_cast<unsigned>(nchunks), kThreads, 0, stream>>>(entries, val, tgt, n, direct);
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

}  // namespace bale
