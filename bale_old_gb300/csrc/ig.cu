// ig.cu -- index gather: tgt[i] = table[index[i] >> shift].
//
// Replaces the per-request remote get of apps/ig_src/ig_agi.upc:61-64 and the
// request/response exchange of apps/ig_src/ig_exstack.upc:69-94: on one GPU
// the table is in HBM and each request is one random 8-byte load.  The cost
// is one 32-byte DRAM sector per request plus the two 8-byte streams, so the
// kernel is built to keep enough independent sector reads in flight: every
// thread issues 2*UNROLL table loads before it consumes any of them, index and
// output move as 16-byte streaming accesses (evict-first), and the grid is a
// whole number of resident waves over the SMs.  The table loads can carry an
// L2 evict-last policy so that the part of the table that fits in L2 stays
// there while the streams pass through.
//
// launch_ig dispatches: this direct gather for tables that fit L2 and for
// short request streams; for large tables with many requests (the
// ig.part_min_* knobs) the region-partitioned gather of ig_part.cu, preceded
// by its device-side skew test, which hands strongly skewed streams back to
// the direct gather here.
#include "common.cuh"

namespace bale {

namespace {

// Table-load flavours (knob "ig.table_policy").
enum TablePolicy { kNoAlloc = 0, kEvictLast = 1, kEvictFirst = 2, kCached = 3 };

template <int TPOL>
__device__ __forceinline__ int64_t ld_table_pol(const int64_t *p, uint64_t pol) {
  int64_t v;
  if (TPOL == kNoAlloc) {
    asm("ld.global.nc.L1::no_allocate.s64 %0, [%1];" : "=l"(v) : "l"(p));
  } else if (TPOL == kCached) {
    asm("ld.global.nc.s64 %0, [%1];" : "=l"(v) : "l"(p));
  } else {
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.s64 %0, [%1], %2;" : "=l"(v) : "l"(p), "l"(pol));
  }
  return v;
}

template <int TPOL>
__device__ __forceinline__ uint64_t make_policy() {
  uint64_t pol = 0;
  if (TPOL == kEvictLast) asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  if (TPOL == kEvictFirst) asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

// Loads table[k] for a checked index k; out-of-range indices (including
// negative ones, which are huge as unsigned) produce 0 and are counted.
template <int TPOL>
__device__ __forceinline__ int64_t gather_one(const int64_t *__restrict__ table, uint64_t tlen,
                                              int64_t raw, int shift, uint64_t pol, unsigned &nbad) {
  uint64_t k = static_cast<uint64_t>(raw >> shift);
  if (k < tlen) return ld_table_pol<TPOL>(table + k, pol);
  nbad++;
  return 0;
}

// only_if (optional): run only when *only_if is 1 (the skew test chose
// this gather over the partitioned one).
template <int UNROLL, int TPOL>
__global__ void __launch_bounds__(512)
    ig_gather_kernel(int64_t *__restrict__ tgt, const int64_t *__restrict__ index, int64_t n,
                     const int64_t *__restrict__ table, uint64_t tlen, int shift,
                     unsigned long long *__restrict__ bad, const unsigned *__restrict__ only_if) {
  if (only_if && !*only_if) return;
  const longlong2 *__restrict__ idx2 = reinterpret_cast<const longlong2 *>(index);
  longlong2 *__restrict__ out2 = reinterpret_cast<longlong2 *>(tgt);
  const uint64_t pol = make_policy<TPOL>();
  const int64_t npairs = n >> 1;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  unsigned nbad = 0;

  // Main body: UNROLL pairs per thread per trip, all loads issued first.
  for (; p + (UNROLL - 1) * stride < npairs; p += UNROLL * stride) {
    longlong2 ix[UNROLL];
#pragma unroll
    for (int u = 0; u < UNROLL; u++) ix[u] = ld_stream_v2(idx2 + p + u * stride);
    longlong2 v[UNROLL];
#pragma unroll
    for (int u = 0; u < UNROLL; u++) {
      v[u].x = gather_one<TPOL>(table, tlen, ix[u].x, shift, pol, nbad);
      v[u].y = gather_one<TPOL>(table, tlen, ix[u].y, shift, pol, nbad);
    }
#pragma unroll
    for (int u = 0; u < UNROLL; u++) st_stream_v2(out2 + p + u * stride, v[u]);
  }
  // Remaining pairs.
  for (; p < npairs; p += stride) {
    longlong2 ix = ld_stream_v2(idx2 + p);
    longlong2 v;
    v.x = gather_one<TPOL>(table, tlen, ix.x, shift, pol, nbad);
    v.y = gather_one<TPOL>(table, tlen, ix.y, shift, pol, nbad);
    st_stream_v2(out2 + p, v);
  }
  // Odd last element.
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    tgt[n - 1] = gather_one<TPOL>(table, tlen, index[n - 1], shift, pol, nbad);
  }
  unsigned long long b = warp_sum_u64(nbad);
  if (b && lane_id() == 0) atomicAdd(bad, b);
}

// Scalar variant for index/tgt arrays that are not 16-byte aligned.
__global__ void __launch_bounds__(256)
    ig_gather_scalar_kernel(int64_t *__restrict__ tgt, const int64_t *__restrict__ index,
                            int64_t n, const int64_t *__restrict__ table, uint64_t tlen,
                            int shift, unsigned long long *__restrict__ bad) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  unsigned nbad = 0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += stride)
    st_stream(tgt + i, gather_one<kNoAlloc>(table, tlen, ld_stream(index + i), shift, 0, nbad));
  unsigned long long b = warp_sum_u64(nbad);
  if (b && lane_id() == 0) atomicAdd(bad, b);
}

// max(index[i] >> shift) as unsigned (a negative index compares as huge).
__global__ void __launch_bounds__(256)
    index_max_kernel(const int64_t *__restrict__ index, int64_t n, int shift,
                     unsigned long long *__restrict__ out) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  unsigned long long m = 0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += stride) {
    unsigned long long k = static_cast<unsigned long long>(ld_stream(index + i) >> shift);
    m = k > m ? k : m;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long t = __shfl_xor_sync(0xffffffffu, m, o);
    m = t > m ? t : m;
  }
  if (lane_id() == 0 && m) atomicMax(out, m);
}

using IgKernel = void (*)(int64_t *, const int64_t *, int64_t, const int64_t *, uint64_t, int,
                          unsigned long long *, const unsigned *);

template <int U>
IgKernel pick_policy(int pol) {
  switch (pol) {
    case kEvictLast: return ig_gather_kernel<U, kEvictLast>;
    case kEvictFirst: return ig_gather_kernel<U, kEvictFirst>;
    case kCached: return ig_gather_kernel<U, kCached>;
    default: return ig_gather_kernel<U, kNoAlloc>;
  }
}

IgKernel pick_kernel(int unroll, int pol) {
  switch (unroll) {
    case 1: return pick_policy<1>(pol);
    case 2: return pick_policy<2>(pol);
    case 8: return pick_policy<8>(pol);
    default: return pick_policy<4>(pol);
  }
}

int g_l2_fetch_set[64];

}  // namespace

// Tables well beyond what L2 can hold go through the region-partitioned
// gather (ig_part.cu) when there are enough requests to amortise its passes.
namespace {

// The skew test's threshold (knob ig.skew_repeat_pct; 0 turns the test off):
// the share of sampled requests whose table sector repeats within the sample.
constexpr int64_t kSkewRepeatPct = 45;

// The direct gather k over n requests, as many blocks as are resident (knob
// ig.blocks_per_sm overrides) and no more than the work needs.
int launch_direct(IgKernel k, int threads, int unroll, int64_t *tgt, const int64_t *index, int64_t n,
                  const int64_t *table, int64_t table_len, int shift, unsigned long long *bad,
                  const unsigned *only_if, cudaStream_t stream) {
  int64_t bps = knob("ig.blocks_per_sm");
  if (bps <= 0) {
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, threads, 0) != cudaSuccess || occ < 1) occ = 1;
    bps = occ;
  }
  const int64_t want = (n / 2 + static_cast<int64_t>(threads) * unroll - 1) / (static_cast<int64_t>(threads) * unroll);
  const int64_t full = static_cast<int64_t>(num_sms()) * bps;
  const int blocks = static_cast<int>(want < full ? (want > 0 ? want : 1) : full);
  k<<<blocks, threads, 0, stream>>>(tgt, index, n, table, static_cast<uint64_t>(table_len), shift, bad, only_if);
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

}  // namespace

bool ig_partition_for(int64_t n, int64_t table_len, const int64_t *tgt, const int64_t *index) {
  const bool aligned = ((reinterpret_cast<uintptr_t>(tgt) | reinterpret_cast<uintptr_t>(index)) & 15) == 0;
  const int64_t mode = knob("ig.mode");
  return aligned && ig_part_supported(n, table_len) && (mode == 1 || (mode < 0 && ig_auto_partition(n, table_len)));
}

int launch_ig(int64_t *tgt, const int64_t *index, int64_t n, const int64_t *table,
              int64_t table_len, int shift, unsigned long long *bad, cudaStream_t stream) {
  if (n <= 0) return BALE_OK;
  const int sms = num_sms();
  const bool aligned = ((reinterpret_cast<uintptr_t>(tgt) | reinterpret_cast<uintptr_t>(index)) & 15) == 0;

  const int64_t fetch = knob("ig.l2_fetch");
  if (fetch >= 0) {
    const int dev = current_device();
    if (dev >= 0 && dev < 64 && g_l2_fetch_set[dev] != fetch + 1) {
      BALE_CUDA_OK(cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, static_cast<size_t>(fetch)));
      g_l2_fetch_set[dev] = static_cast<int>(fetch + 1);
    }
  }
  if (ig_partition_for(n, table_len, tgt, index)) {
    void *ws = device_workspace(ig_part_workspace_bytes(n, table_len), stream);
    unsigned long long *cursor = next_cursor_word();  // a slot of 4 words: [0] cursor, [1] the skew choice
    if (!ws || !cursor) return BALE_ENOMEM;
    // Left to the size rule (ig.mode -1), a skewed stream goes to the direct
    // gather with L1-allocating table loads instead, chosen on the device.
    int64_t pct = knob("ig.skew_repeat_pct");
    if (pct < 0) pct = kSkewRepeatPct;
    if (knob("ig.mode") >= 0 || pct == 0 || pct > 100)
      return launch_ig_partitioned(tgt, index, n, table, table_len, shift, bad, ws, cursor, stream);
    unsigned *direct = reinterpret_cast<unsigned *>(cursor + 1);
    int rc = launch_ig_skew(index, n, shift, table_len, static_cast<int>(pct), direct, stream);
    if (rc == BALE_OK) rc = launch_ig_partitioned(tgt, index, n, table, table_len, shift, bad, ws, cursor, stream, direct);
    if (rc != BALE_OK) return rc;
    return launch_direct(ig_gather_kernel<4, kCached>, 256, 4, tgt, index, n, table, table_len, shift, bad, direct,
                         stream);
  }
  if (!aligned) {
    int64_t want = (n + 255) / 256, full = static_cast<int64_t>(sms) * 8;
    int blocks = static_cast<int>(want < full ? want : full);
    ig_gather_scalar_kernel<<<blocks, 256, 0, stream>>>(tgt, index, n, table,
                                                        static_cast<uint64_t>(table_len), shift, bad);
    BALE_CUDA_OK(cudaGetLastError());
    return BALE_OK;
  }
  int64_t unroll = knob("ig.unroll");
  if (unroll != 1 && unroll != 2 && unroll != 4 && unroll != 8) unroll = 4;
  int64_t pol = knob("ig.table_policy");
  if (pol < 0 || pol > 3) pol = kEvictLast;
  int64_t threads = knob("ig.threads");
  if (threads != 128 && threads != 256 && threads != 512) threads = 256;
  return launch_direct(pick_kernel(static_cast<int>(unroll), static_cast<int>(pol)), static_cast<int>(threads),
                       static_cast<int>(unroll), tgt, index, n, table, table_len, shift, bad, nullptr, stream);
}

// One word from device memory to a mapped host word, written by the kernel:
// no copy engine is involved, so it never queues behind large copies.
__global__ void copy_word_kernel(const unsigned long long *__restrict__ src, volatile unsigned long long *dst) {
  *dst = *src;
}

int launch_copy_word(const unsigned long long *src, unsigned long long *mapped_dst, cudaStream_t stream) {
  copy_word_kernel<<<1, 1, 0, stream>>>(src, mapped_dst);
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

int launch_index_max(const int64_t *index, int64_t n, int shift, unsigned long long *out,
                     cudaStream_t stream) {
  if (n <= 0) return BALE_OK;
  int64_t want = (n + 255) / 256;
  int64_t full = static_cast<int64_t>(num_sms()) * 8;
  int blocks = static_cast<int>(want < full ? want : full);
  index_max_kernel<<<blocks, 256, 0, stream>>>(index, n, shift, out);
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

}  // namespace bale
