// histo.cu -- histogram scatter-add: counts[index[i] >> shift] += 1.
//
// Replaces the remote atomic of apps/histo_src/histo_agi.upc:61-66 and the
// push/exchange/pull of apps/histo_src/histo_exstack.upc:64-76.  bale's
// aggregation layer (exstack/conveyors: bin updates by destination, then move
// them in bulk) becomes on-chip work:
//
//  * small tables (fit in shared memory): every block keeps a private u32
//    copy of the whole table in shared memory, counts its slice of updates
//    with shared-memory atomics, then flushes the non-zero counters to HBM
//    with one L2 reduction each;
//  * larger tables: one fire-and-forget L2 reduction per update
//    (red.global.add.u64).  For tables that live in L2 this is bound by the
//    L2 reduction rate, otherwise by one DRAM sector read and write-back per
//    update;
//  * tables well beyond L2: the updates are first partitioned by 16 MiB
//    region (ig_part.cu's partition), so the reductions of one region at a
//    time stay in L2;
//  * skewed updates (mode 1, chosen by the tuner or the caller): the lanes
//    that hit the same counter are grouped with __match_any_sync and the
//    leader adds the group size with one reduction.
//
// The drop-ins ADD into the caller's counts (apps/histo_src/histo.upc:210-213
// relies on accumulation across models).
#include "common.cuh"

namespace bale {

namespace {

constexpr int kHistoThreads = 256;
constexpr int kSmemThreads = 512;
// Largest table kept privately in shared memory (u32 counters, 192 KiB).
constexpr int64_t kSmemMaxCounters = 48 * 1024;

template <bool AGG>
__device__ __forceinline__ void histo_add(int64_t *__restrict__ counts, uint64_t ncounts,
                                          int64_t raw, int shift, unsigned &nbad) {
  uint64_t k = static_cast<uint64_t>(raw >> shift);
  const bool ok = k < ncounts;
  if (AGG) {
    // All 32 lanes call this together (warp-uniform loop), so the full mask
    // is valid.  Invalid lanes get a key no valid lane can share.
    unsigned long long key = ok ? k : ~0ull;
    unsigned peers = __match_any_sync(0xffffffffu, key);
    if (ok && (__ffs(peers) - 1) == static_cast<int>(lane_id()))
      red_add_u64(counts + k, static_cast<unsigned long long>(__popc(peers)));
  } else if (ok) {
    red_add_u64(counts + k, 1ull);
  }
  if (!ok) nbad++;
}

template <int UNROLL, bool AGG>
__global__ void __launch_bounds__(kHistoThreads)
    histo_global_kernel(int64_t *__restrict__ counts, uint64_t ncounts,
                        const int64_t *__restrict__ index, int64_t n, int shift,
                        unsigned long long *__restrict__ bad) {
  const longlong2 *__restrict__ idx2 = reinterpret_cast<const longlong2 *>(index);
  const int64_t npairs = n >> 1;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  int64_t warp0 = static_cast<int64_t>(blockIdx.x) * blockDim.x + (threadIdx.x & ~31u);
  int64_t p = warp0 + lane_id();
  unsigned nbad = 0;
  // Warp-uniform trip condition so that __match_any_sync sees all lanes.
  for (; warp0 + 31 + (UNROLL - 1) * stride < npairs; warp0 += UNROLL * stride, p += UNROLL * stride) {
    longlong2 ix[UNROLL];
#pragma unroll
    for (int u = 0; u < UNROLL; u++) ix[u] = ld_stream_v2(idx2 + p + u * stride);
#pragma unroll
    for (int u = 0; u < UNROLL; u++) {
      histo_add<AGG>(counts, ncounts, ix[u].x, shift, nbad);
      histo_add<AGG>(counts, ncounts, ix[u].y, shift, nbad);
    }
  }
  for (; p < npairs; p += stride) {
    longlong2 ix = ld_stream_v2(idx2 + p);
    histo_add<false>(counts, ncounts, ix.x, shift, nbad);
    histo_add<false>(counts, ncounts, ix.y, shift, nbad);
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0)
    histo_add<false>(counts, ncounts, index[n - 1], shift, nbad);
  unsigned long long b = warp_sum_u64(nbad);
  if (b && lane_id() == 0) atomicAdd(bad, b);
}

__global__ void __launch_bounds__(kHistoThreads)
    histo_scalar_kernel(int64_t *__restrict__ counts, uint64_t ncounts,
                        const int64_t *__restrict__ index, int64_t n, int shift,
                        unsigned long long *__restrict__ bad) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  unsigned nbad = 0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    histo_add<false>(counts, ncounts, ld_stream(index + i), shift, nbad);
  unsigned long long b = warp_sum_u64(nbad);
  if (b && lane_id() == 0) atomicAdd(bad, b);
}

// Block-private shared-memory histogram, then one flush per non-zero counter.
// Each block handles a contiguous slice of at most 2^31 updates, so a u32
// counter cannot overflow.
__global__ void __launch_bounds__(kSmemThreads)
    histo_smem_kernel(int64_t *__restrict__ counts, uint32_t ncounts,
                      const int64_t *__restrict__ index, int64_t n, int64_t per_block, int shift,
                      unsigned long long *__restrict__ bad) {
  extern __shared__ uint32_t sc[];
  for (uint32_t c = threadIdx.x; c < ncounts; c += blockDim.x) sc[c] = 0;
  __syncthreads();
  const int64_t lo = static_cast<int64_t>(blockIdx.x) * per_block;
  const int64_t hi = lo + per_block < n ? lo + per_block : n;
  unsigned nbad = 0;
  // 16-byte loads over the aligned interior of [lo,hi), scalar at the ends.
  int64_t a = (lo + 1) & ~static_cast<int64_t>(1);
  if (a > hi) a = hi;
  int64_t e = a + ((hi - a) & ~static_cast<int64_t>(1));
  for (int64_t i = lo + threadIdx.x; i < a; i += blockDim.x) {
    uint64_t k = static_cast<uint64_t>(ld_stream(index + i) >> shift);
    if (k < ncounts) atomicAdd(&sc[k], 1u); else nbad++;
  }
  const longlong2 *__restrict__ idx2 = reinterpret_cast<const longlong2 *>(index + a);
  const int64_t np = (e - a) >> 1;
  for (int64_t p = threadIdx.x; p < np; p += blockDim.x) {
    longlong2 ix = ld_stream_v2(idx2 + p);
    uint64_t k0 = static_cast<uint64_t>(ix.x >> shift), k1 = static_cast<uint64_t>(ix.y >> shift);
    if (k0 < ncounts) atomicAdd(&sc[k0], 1u); else nbad++;
    if (k1 < ncounts) atomicAdd(&sc[k1], 1u); else nbad++;
  }
  for (int64_t i = e + threadIdx.x; i < hi; i += blockDim.x) {
    uint64_t k = static_cast<uint64_t>(ld_stream(index + i) >> shift);
    if (k < ncounts) atomicAdd(&sc[k], 1u); else nbad++;
  }
  __syncthreads();
  for (uint32_t c = threadIdx.x; c < ncounts; c += blockDim.x) {
    uint32_t v = sc[c];
    if (v) red_add_u64(counts + c, v);
  }
  unsigned long long b = warp_sum_u64(nbad);
  if (b && lane_id() == 0) atomicAdd(bad, b);
}

bool g_smem_attr_set[64] = {false};

// The L2 reduction rate the histogram is bound by when its table lives in
// L2: n +1 reductions at hashed positions of counts, with no index stream
// to read -- the histogram's update minus its input.
__global__ void __launch_bounds__(256) l2_red_rate_kernel(int64_t *__restrict__ counts, uint64_t m, int64_t n) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    uint64_t x = static_cast<uint64_t>(i) * 0x9E3779B97F4A7C15ull;
    x ^= x >> 29;
    red_add_u64(counts + __umul64hi(x, m), 1ull);
  }
}

}  // namespace

int launch_l2_red_rate(int64_t *counts, int64_t ncounts, int64_t n, cudaStream_t stream) {
  if (n <= 0 || ncounts <= 0) return BALE_OK;
  const int64_t want = (n + 255) / 256, full = static_cast<int64_t>(num_sms()) * 8;
  l2_red_rate_kernel<<<static_cast<unsigned>(want < full ? want : full), 256, 0, stream>>>(
      counts, static_cast<uint64_t>(ncounts), n);
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

// Mode: 0 shared-memory private table, 1 warp-aggregated L2 reductions,
// 2 plain L2 reductions, 3 region-partitioned L2 reductions.  Automatic:
// shared memory when the table fits; plain L2 reductions while the table
// lives in L2 (uniform updates rarely collide inside a warp, so the
// aggregation's __match_any_sync costs more than it saves -- it pays only
// for skewed updates, which the tuner or the caller can select); the
// region partition once the table is well beyond L2.
int histo_mode_for(int64_t n, int64_t ncounts, const int64_t *index) {
  const bool aligned = (reinterpret_cast<uintptr_t>(index) & 15) == 0;
  int64_t mode = knob("histo.mode");
  if (mode < 0 || mode > 3) {
    if (ncounts <= kSmemMaxCounters) mode = 0;
    else if (histo_auto_partition(n, ncounts)) mode = 3;
    else mode = 2;
  }
  if (mode == 0 && ncounts > kSmemMaxCounters) mode = 2;
  if (!aligned && (mode == 0 || mode == 3)) mode = 2;
  if (mode == 3 && ncounts > (kIgMaxRegions << kIgRegionBits)) mode = 2;
  return static_cast<int>(mode);
}

int launch_histo(int64_t *counts, int64_t ncounts, const int64_t *index, int64_t n, int shift,
                 unsigned long long *bad, cudaStream_t stream) {
  if (n <= 0) return BALE_OK;
  const int sms = num_sms();
  const bool aligned = (reinterpret_cast<uintptr_t>(index) & 15) == 0;
  const int64_t mode = histo_mode_for(n, ncounts, index);
  if (mode == 3) {
    void *ws = device_workspace(histo_part_workspace_bytes(n, ncounts), stream);
    unsigned long long *cursor = next_cursor_word();
    if (!ws || !cursor) return BALE_ENOMEM;
    return launch_histo_partitioned(counts, ncounts, index, n, shift, bad, ws, cursor, stream);
  }

  if (mode == 0) {
    const size_t smem = static_cast<size_t>(ncounts) * sizeof(uint32_t);
    const int dev = current_device();
    if (dev >= 0 && dev < 64 && !g_smem_attr_set[dev]) {
      BALE_CUDA_OK(cudaFuncSetAttribute(histo_smem_kernel,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(kSmemMaxCounters * sizeof(uint32_t))));
      g_smem_attr_set[dev] = true;
    }
    // Blocks resident per SM given the shared-memory footprint.
    int per_sm = smem <= 48 * 1024 ? 4 : (smem <= 96 * 1024 ? 2 : 1);
    // Each block should see several updates per counter so that the flush
    // (ncounts reductions per block) stays a small share of the work.
    int64_t upc = knob("histo.smem_updates_per_counter");
    if (upc <= 0) upc = 4;
    int64_t blocks = n / (upc * (ncounts > 0 ? ncounts : 1));
    int64_t cap = static_cast<int64_t>(sms) * per_sm;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    int64_t per_block = (n + blocks - 1) / blocks;
    while (per_block > (int64_t(1) << 31)) {  // u32 shared counters
      blocks *= 2;
      per_block = (n + blocks - 1) / blocks;
    }
    per_block = (per_block + 1) & ~static_cast<int64_t>(1);
    blocks = (n + per_block - 1) / per_block;
    histo_smem_kernel<<<static_cast<int>(blocks), kSmemThreads, smem, stream>>>(
        counts, static_cast<uint32_t>(ncounts), index, n, per_block, shift, bad);
    BALE_CUDA_OK(cudaGetLastError());
    return BALE_OK;
  }

  int64_t want = (n / 2 + kHistoThreads - 1) / kHistoThreads;
  int64_t bps = knob("histo.blocks_per_sm");
  if (bps <= 0) bps = 8;
  int64_t full = static_cast<int64_t>(sms) * bps;
  int blocks = static_cast<int>(want < full ? (want > 0 ? want : 1) : full);
  int64_t unroll = knob("histo.unroll");
  if (unroll != 1 && unroll != 2 && unroll != 4 && unroll != 8) unroll = 4;
  using HistoKernel = void (*)(int64_t *, uint64_t, const int64_t *, int64_t, int, unsigned long long *);
  HistoKernel k;
  if (!aligned) {
    k = histo_scalar_kernel;
  } else if (mode == 1) {
    k = unroll == 1 ? histo_global_kernel<1, true> : unroll == 2 ? histo_global_kernel<2, true>
      : unroll == 8 ? histo_global_kernel<8, true> : histo_global_kernel<4, true>;
  } else {
    k = unroll == 1 ? histo_global_kernel<1, false> : unroll == 2 ? histo_global_kernel<2, false>
      : unroll == 8 ? histo_global_kernel<8, false> : histo_global_kernel<4, false>;
  }
  k<<<blocks, kHistoThreads, 0, stream>>>(counts, static_cast<uint64_t>(ncounts), index, n, shift, bad);
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

}  // namespace bale
