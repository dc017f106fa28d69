// sort.cu -- the stable LSD radix sort of 64-bit keys and the u32 exclusive
// scan the graph build and spmat's operations share.
//
// The radix sort takes 8 bits per pass over tiles of 4096 keys.  In a pass,
// every key's rank among equal digits of its tile comes from a warp match and
// per-warp counts in shared memory; the tile is laid out in shared memory in
// sorted order and leaves run by run.  Where a tile's runs start in the
// output comes, below 2^30 keys, from a single sweep (the published Onesweep
// scheme of Adinets and Merrill, 2022): one histogram kernel counts the
// digits of every pass in one read of the keys, and within a pass each tile
// takes the next tile number from a counter, publishes its digit counts and
// adds up its predecessors' by looking back over their published words, so a
// pass is one kernel that reads and writes each key once.  Larger sorts, or
// the knob sort.onesweep = 0, take the three-step pass: a per-tile digit
// histogram kernel, an exclusive scan over (digit, tile), then the scatter.
#include <algorithm>

#include "sort.cuh"

namespace bale {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kThreads = kSortThreads;
constexpr int kWarps = kThreads / 32;
constexpr int kPer = kSortPer;
static_assert(kDigits == kThreads, "one digit per thread");

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

// offs[d * ntiles + t]: where tile t's keys with digit d start in dst.  Each
// warp ranks a contiguous eighth of the tile in index order with warp-private
// digit counts (no block barrier per round); the warps' counts are scanned
// per digit, the tile is laid out in shared memory in sorted order, and the
// threads then write consecutive sorted positions, so each digit's run leaves
// the block as whole lines.  Stable: within a digit, tile index order.
constexpr int kWarpSlice = static_cast<int>(kTile) / kWarps;  // 512 keys per warp
static_assert(kWarpSlice == 32 * kPer, "a warp's slice is kPer rounds of 32");

// A single-sweep pass's tile words: flag in the top two bits, a count below.
constexpr uint32_t kStAggregate = 1u << 30;  // the tile's own digit count
constexpr uint32_t kStPrefix = 2u << 30;     // the count of the digit in this and every earlier tile
constexpr uint32_t kStValue = kStAggregate - 1;

struct Lookback {
  const uint32_t *start;   // the pass's digit starts in the output
  unsigned int *counter;   // tiles claimed so far in the pass
  uint32_t *status;        // the pass's tile words, zero before it
  uint32_t *next;          // the next pass's tile words, zeroed here
  int64_t spins;           // polls without progress before a wait gives up
  unsigned int *err;       // set when a wait gave up
  int withhold;            // tile 0 publishes nothing (the bounded-wait test: its successors' waits run out)
};

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_relaxed(uint32_t *p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Digit d in tiles [0, t), from their published words: WIDTH earlier tiles
// are read at once, nearest first, adding counts up to the first inclusive
// prefix; a word not yet published is read again, and after lb.spins reads
// that make no progress the wait gives up (*gave_up, with an undercount that
// the caller replaces).  Eight at once measured best (R-MAT scale-22 build:
// 4 -> 9.83 ms, 8 -> 9.61, 16 -> 9.72, 32 -> 10.06).
constexpr int kLookWidth = 8;

template <int WIDTH>
__device__ __forceinline__ uint32_t look_back(const Lookback &lb, int64_t t, unsigned d, bool *gave_up) {
  uint32_t sum = 0;
  int64_t j = t - 1, polls = 0;  // the nearest tile not yet added
  for (;;) {
    uint32_t v[WIDTH];
#pragma unroll
    for (int q = 0; q < WIDTH; q++) v[q] = j - q >= 0 ? ld_relaxed(lb.status + (j - q) * kDigits + d) : kStPrefix;
    int used = 0;
    bool reached = false, blocked = false;
#pragma unroll
    for (int q = 0; q < WIDTH; q++) {
      if (reached || blocked) continue;
      if (v[q] == 0) {
        blocked = true;
      } else {
        sum += v[q] & kStValue;
        used++;
        reached = (v[q] & kStPrefix) != 0;
      }
    }
    if (reached) return sum;
    j -= used;
    if (used == 0 && ++polls > lb.spins) {
      *gave_up = true;
      return sum;
    }
  }
}

// Four blocks per SM (64 registers, 36 bytes of spills) hide the shared-memory
// latency better than three at 80 registers: R-MAT scale-22 build 10.57 ->
// 10.02 ms, transpose 4.21 -> 4.10 ms.
//
// LOOKBACK: the tile is the next unclaimed one, so every tile it waits on
// belongs to a block already running; it publishes its digit counts before
// its own look-back and its inclusive prefix right after.  A poll loop gives
// up after lb.spins reads of one unpublished word; the block then counts the
// earlier tiles' digits from their keys and sets *lb.err, so the output is
// still the sorted keys and the caller reports the wait.
template <bool LOOKBACK>
__global__ void __launch_bounds__(kThreads, 4)
    radix_scatter_kernel(const uint64_t *__restrict__ src, uint64_t *__restrict__ dst, int64_t n, int shift,
                         const uint32_t *__restrict__ offs, int64_t ntiles, Lookback lb) {
  __shared__ uint64_t sorted[kTile];
  __shared__ uint32_t wcnt[kWarps][kDigits];  // counts per warp, then their exclusive prefix over warps
  __shared__ uint32_t gbase[kDigits];         // where each digit's run starts in dst
  __shared__ uint32_t wsum[kWarps];
  __shared__ uint32_t claimed;
  const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
#pragma unroll
  for (int w = 0; w < kWarps; w++) wcnt[w][threadIdx.x] = 0;
  if constexpr (LOOKBACK) {
    if (threadIdx.x == 0) claimed = atomicAdd(lb.counter, 1u);
    lb.next[static_cast<int64_t>(blockIdx.x) * kDigits + threadIdx.x] = 0;
  } else {
    gbase[threadIdx.x] = offs[static_cast<int64_t>(threadIdx.x) * ntiles + blockIdx.x];
  }
  __syncthreads();
  const int64_t t = LOOKBACK ? static_cast<int64_t>(claimed) : static_cast<int64_t>(blockIdx.x);
  const int64_t tile = t * kTile;
  const int64_t first = tile + static_cast<int64_t>(warp) * kWarpSlice + lane;
  uint64_t key[kPer];
  uint32_t dr[kPer];  // digit << 16 | rank among the warp's keys of that digit (kDigits: no key)
#pragma unroll
  for (int r = 0; r < kPer; r++) {
    const int64_t i = first + r * 32;
    const bool valid = i < n;
    key[r] = valid ? src[i] : 0ull;
    const uint32_t d = valid ? static_cast<uint32_t>(key[r] >> shift) & (kDigits - 1) : kDigits;
    // the lowest lane of each digit adds the digit's keys to the warp's count
    // and hands the count before them to the others
    const unsigned peers = __match_any_sync(kFull, d);
    const uint32_t below = __popc(peers & ((1u << lane) - 1u));
    uint32_t prior = 0;
    if (valid && below == 0) prior = atomicAdd(&wcnt[warp][d], __popc(peers));
    prior = __shfl_sync(kFull, prior, __ffs(peers) - 1);
    dr[r] = d << 16 | (prior + below);
  }
  __syncthreads();
  // thread d: digit d's warp prefixes and its count in the tile, then the
  // exclusive scan of the counts over digits
  uint32_t cnt = 0;
#pragma unroll
  for (int w = 0; w < kWarps; w++) {
    const uint32_t c = wcnt[w][threadIdx.x];
    wcnt[w][threadIdx.x] = cnt;
    cnt += c;
  }
  uint32_t *mine = nullptr;
  if constexpr (LOOKBACK) {
    mine = lb.status + t * kDigits + threadIdx.x;
    if (t > 0 || !lb.withhold) st_relaxed(mine, (t == 0 ? kStPrefix : kStAggregate) | cnt);
  }
  uint32_t inc = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(kFull, inc, o);
    if (static_cast<int>(lane) >= o) inc += y;
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  uint32_t before = 0;
  for (unsigned w = 0; w < warp; w++) before += wsum[w];
  const uint32_t start = before + inc - cnt;  // digit d = threadIdx.x starts here in the sorted tile
  // one table per use: each warp's place for digit d in the sorted tile, and
  // the shift from a sorted position to its place in dst
#pragma unroll
  for (int w = 0; w < kWarps; w++) wcnt[w][threadIdx.x] += start;
  if constexpr (!LOOKBACK) gbase[threadIdx.x] -= start;
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kPer; r++) {
    const uint32_t d = dr[r] >> 16;
    if (d < kDigits) sorted[wcnt[warp][d] + (dr[r] & 0xffffu)] = key[r];
  }
  if constexpr (LOOKBACK) {
    // the tile is laid out before its look-back: the earlier tiles have had
    // that long to publish
    bool gave_up = false;
    uint32_t before_tiles = t > 0 ? look_back<kLookWidth>(lb, t, threadIdx.x, &gave_up) : 0u;  // digit d in tiles [0, t)
    if (__syncthreads_or(gave_up)) {
      // a wait gave up: count the digits of tiles [0, t) from their keys
      // (exact, so the pass still writes a permutation), and report it
      uint32_t *recount = wcnt[0];  // free: the layout above is done
      recount[threadIdx.x] = 0;
      __syncthreads();
      for (int64_t i = threadIdx.x; i < tile; i += kThreads)
        atomicAdd(&recount[static_cast<uint32_t>(src[i] >> shift) & (kDigits - 1)], 1u);
      __syncthreads();
      before_tiles = recount[threadIdx.x];
      if (threadIdx.x == 0) atomicOr(lb.err, 1u);
    }
    if (t > 0) st_relaxed(mine, kStPrefix | (before_tiles + cnt));
    gbase[threadIdx.x] = lb.start[threadIdx.x] + before_tiles - start;
  }
  __syncthreads();
  const int tile_n = static_cast<int>(n - tile < kTile ? n - tile : kTile);
  for (int j = threadIdx.x; j < tile_n; j += kThreads) {
    const uint64_t k = sorted[j];
    const uint32_t d = static_cast<uint32_t>(k >> shift) & (kDigits - 1);
    const uint32_t at = gbase[d] + j;  // gbase[d] - start[d] + j, modulo 2^32
    if (LOOKBACK ? at < n : true) dst[at] = k;
  }
}

// Digit counts of every pass in one read of the keys: osw[p * kDigits + d]
// += the keys whose digit p (the 8 bits from shift0 + 8p) is d.  The two
// halves of the block count apart, halving the collisions of skewed digits.
__global__ void __launch_bounds__(kThreads)
    onesweep_hist_kernel(const uint64_t *__restrict__ keys, int64_t n, int shift0, int passes,
                         uint32_t *__restrict__ osw) {
  __shared__ uint32_t h[2][kOsPasses][kDigits];
#pragma unroll
  for (int p = 0; p < kOsPasses; p++) h[0][p][threadIdx.x] = h[1][p][threadIdx.x] = 0;
  __syncthreads();
  uint32_t(*mine)[kDigits] = h[threadIdx.x >> 7];
  const int64_t stride = static_cast<int64_t>(gridDim.x) * kThreads;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * kThreads + threadIdx.x; i < n; i += stride) {
    const uint64_t k = keys[i] >> shift0;
#pragma unroll
    for (int p = 0; p < kOsPasses; p++)
      if (p < passes) atomicAdd(&mine[p][static_cast<uint32_t>(k >> (8 * p)) & (kDigits - 1)], 1u);
  }
  __syncthreads();
  for (int p = 0; p < passes; p++) {
    const uint32_t v = h[0][p][threadIdx.x] + h[1][p][threadIdx.x];
    if (v) atomicAdd(&osw[p * kDigits + threadIdx.x], v);
  }
}

// Block p: pass p's digit counts into their exclusive prefix, in place.
__global__ void __launch_bounds__(kThreads) onesweep_starts_kernel(uint32_t *__restrict__ osw) {
  __shared__ uint32_t wtot[kWarps];
  const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
  uint32_t *h = osw + blockIdx.x * kDigits;
  const uint32_t v = h[threadIdx.x];
  uint32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(kFull, inc, o);
    if (static_cast<int>(lane) >= o) inc += y;
  }
  if (lane == 31) wtot[warp] = inc;
  __syncthreads();
  uint32_t before = 0;
  for (unsigned w = 0; w < warp; w++) before += wtot[w];
  h[threadIdx.x] = before + inc - v;
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

// CSR checks shared by transpose, permute and the dataset writer and reader: offsets ascending inside
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

}  // namespace

unsigned grid_for(int64_t n) {
  const int64_t want = (n + 255) / 256, cap = static_cast<int64_t>(num_sms()) * 16;
  return static_cast<unsigned>(std::max<int64_t>(1, std::min(want, cap)));
}

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
  p = take(4 * kOsWords); if (w) w->osw = reinterpret_cast<uint32_t *>(p);
  p = take(64); if (w) w->words = reinterpret_cast<unsigned int *>(p);
  return o;
}

int excl_scan(const uint32_t *in, uint32_t *out, int64_t n, uint32_t *bsum, unsigned int *total, cudaStream_t st) {
  const int64_t nb = std::max<int64_t>(1, (n + kScanBlock - 1) / kScanBlock);
  scan_blocksum_kernel<<<static_cast<unsigned>(nb), kScanThreads, 0, st>>>(in, n, bsum);
  scan_top_kernel<<<1, kScanThreads, 0, st>>>(bsum, nb, total);
  scan_apply_kernel<<<static_cast<unsigned>(nb), kScanThreads, 0, st>>>(in, n, bsum, out);
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

namespace {

// The three-step pass: per-tile histograms, their scan, the scatter.
int radix_pass_scanned(const uint64_t *a, uint64_t *b, int64_t n, int shift, Ws &w, cudaStream_t st) {
  const int64_t tiles = (n + kTile - 1) / kTile;
  radix_hist_kernel<<<static_cast<unsigned>(tiles), kThreads, 0, st>>>(a, n, shift, w.hist, tiles);
  const int rc = excl_scan(w.hist, w.hoff, tiles * kDigits, w.bsum, w.words, st);
  if (rc != BALE_OK) return rc;
  radix_scatter_kernel<false><<<static_cast<unsigned>(tiles), kThreads, 0, st>>>(a, b, n, shift, w.hoff, tiles,
                                                                                 Lookback{});
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

bool single_sweep(int64_t n) { return n < (int64_t(1) << 30) && knob_or("sort.onesweep", 1) != 0; }

// `passes` single-sweep passes over the digits from shift0, ping-ponging
// between *a and *b (on return *a holds the result).  The tile words of the
// even passes live in w.hist, the odd ones' in w.hoff: each pass zeroes the
// other array for the next.
int single_sweep_sort(uint64_t **a, uint64_t **b, int64_t n, int shift0, int passes, Ws &w, cudaStream_t st) {
  if (passes <= 0) return BALE_OK;
  const int64_t tiles = (n + kTile - 1) / kTile;
  BALE_CUDA_OK(cudaMemsetAsync(w.osw, 0, 4 * kOsWords, st));
  BALE_CUDA_OK(cudaMemsetAsync(w.hist, 0, 4 * static_cast<size_t>(tiles) * kDigits, st));
  const unsigned hblocks = static_cast<unsigned>(std::min<int64_t>(tiles, static_cast<int64_t>(num_sms()) * 4));
  onesweep_hist_kernel<<<hblocks, kThreads, 0, st>>>(*a, n, shift0, passes, w.osw);
  onesweep_starts_kernel<<<passes, kThreads, 0, st>>>(w.osw);
  const int64_t spins = knob_or("sort.lookback_spins", int64_t(1) << 22);
  const int withhold = knob_or("sort.test_withhold", 0) != 0;
  for (int p = 0; p < passes; p++) {
    Lookback lb{w.osw + p * kDigits, w.osw + kOsPasses * kDigits + p, p % 2 ? w.hoff : w.hist,
                p % 2 ? w.hist : w.hoff, spins, w.words + kSortErrWord, withhold};
    radix_scatter_kernel<true><<<static_cast<unsigned>(tiles), kThreads, 0, st>>>(*a, *b, n, shift0 + 8 * p,
                                                                                nullptr, tiles, lb);
    BALE_CUDA_OK(cudaGetLastError());
    std::swap(*a, *b);
  }
  return BALE_OK;
}

}  // namespace

int radix_pass(const uint64_t *a, uint64_t *b, int64_t n, int shift, Ws &w, cudaStream_t st) {
  if (n < 1) return BALE_OK;
  if (!single_sweep(n)) return radix_pass_scanned(a, b, n, shift, w, st);
  uint64_t *x = const_cast<uint64_t *>(a), *y = b;  // one pass reads x only
  return single_sweep_sort(&x, &y, n, shift, 1, w, st);
}

int sort_status(const unsigned int *words, cudaStream_t st, const char *who) {
  unsigned int e = 0;
  BALE_CUDA_OK(cudaMemcpyAsync(&e, words + kSortErrWord, 4, cudaMemcpyDeviceToHost, st));
  BALE_CUDA_OK(cudaStreamSynchronize(st));
  if (e) {
    set_error("%s: a radix sort pass gave up waiting for an earlier tile (knob sort.lookback_spins)", who);
    return BALE_ETIMEDOUT;
  }
  return BALE_OK;
}

int label_bits(int64_t n) {
  int S = 1;
  while ((int64_t(1) << S) < n) S++;
  return S;
}

int csr_from_keys(const uint64_t *sk, int64_t nk, int64_t nrows, int S, int64_t *offset, int64_t *nonzero,
                  cudaStream_t st) {
  csr_offsets_kernel<<<grid_for(nrows + 1), 256, 0, st>>>(sk, nk, nrows, S, offset);
  if (nonzero && nk > 0) csr_cols_kernel<<<grid_for(nk), 256, 0, st>>>(sk, nk, S, nonzero);
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

void launch_csr_check(const int64_t *off, const int64_t *col, int64_t numrows, int64_t numcols, int64_t nnz,
                      unsigned long long *bad, cudaStream_t st) {
  csr_check_kernel<<<grid_for(std::max(numrows + 1, nnz)), 256, 0, st>>>(off, col, numrows, numcols, nnz, bad);
}

uint64_t *radix_sort(uint64_t *a, uint64_t *b, int64_t n, int bits, Ws &w, cudaStream_t st, int *rc) {
  *rc = BALE_OK;
  if (n <= 1) return a;
  if (single_sweep(n)) {
    *rc = single_sweep_sort(&a, &b, n, 0, (bits + kDigitBits - 1) / kDigitBits, w, st);
    return a;
  }
  for (int shift = 0; shift < bits; shift += kDigitBits) {
    *rc = radix_pass_scanned(a, b, n, shift, w, st);
    if (*rc != BALE_OK) return a;
    std::swap(a, b);
  }
  return a;
}

}  // namespace bale
