// tri_wedge.cu -- triangle counting by wedge probes at the far vertex, for
// matrices below 2^32 rows and nonzeros.  The default mode runs it for every
// such matrix below 2^23 nonzeros, and above that when the device-side
// choice in triangle.cu finds the graph has hubs (pulls well above pushes).
//
// The count is the reference's alg 0 (apps/triangle_src/triangle_agi.upc:69-99):
// the sum over nonzeros L[i][j] of |row_i and row_j|.  Rows ascend and row j
// lies in [0,j), so row_i and row_j = row_i[0,p) and row_j, where p is the
// position of j in row i.  That is the exstack "push" form
// (apps/triangle_src/triangle_exstack.upc:108-133): for each (i,j), every w
// of row i below j goes to j's owner, which looks it up in row j.  Its work
// is sum_i C(d_i,2) probes instead of the sum of deg(j) row-j elements the
// AGI loop scans; on the degree-ordered R-MAT graph of scale 22 that is
// 7.2 G probes against 28.9 G.
//
// Here "j's owner" is a CTA or a warp, and the incoming wedges of each j are
// grouped through the transpose of L, built on the device:
//   1. scan: validate every row (offsets inside [0,nnz], columns ascending in
//      [0,i)), write the u32 column copy, count each j's incoming (i, p > 0);
//   2. exclusive scan of the counts -> in_off;
//   3. fill: in_rec[in_off[j] + t] = {k - p, p}, the start and length of the
//      prefix row_i[0,p) (k is the nonzero's index);
//   4. count: one warp per j.  Row j's columns below 2^16 become a bitmap in
//      the warp's own 8 KiB of shared memory (so no block-wide barrier is
//      ever needed) and its few columns above 2^16 a short sorted list beside
//      it; the warp tests every element of the incoming prefixes -- one
//      shared-memory load per element for the bitmap part -- then clears the
//      bits it set.  On a degree-ordered matrix the labels below 2^16 are the
//      hubs, where nearly all probes land (94% at R-MAT scale 22).
//   5. dense pairs: a pair (i,j) whose prefix is longer than the ceil(j/32)
//      words of a bitmap of [0,j) (plus a margin), for j below 2^14, gets no
//      record in steps 1-3; step 1 also builds the column bitmaps of the rows
//      below 2^14, and one warp per row i ANDs row i's bits with row j's and
//      counts them (54% of the scale-22 probes become 1.28 G word ANDs).
// Steps 1-3 and the bitmaps depend only on the matrix (a resident graph does
// them once).  A malformed row raises *bad in step 1 and the later steps then
// return at once; every index stays inside its array either way.  The work
// tally is the number of probes, sum_i C(d_i,2) -- the reference's exstack
// push count -- with each dense pair counted as the p probes it replaces.
#include <algorithm>

#include "tri_device.cuh"

namespace bale {

namespace {

using tri::kBadCol;
using tri::kFull;

constexpr int kScanThreads = 256;
constexpr int kScanWarps = kScanThreads / 32;
constexpr int kPsumThreads = 1024;
constexpr int kPsumPer = 4;
constexpr int64_t kPsumBlock = static_cast<int64_t>(kPsumThreads) * kPsumPer;  // counts per scan block
constexpr int kWarpThreads = 256;
constexpr int kWarpWarps = kWarpThreads / 32;
constexpr int kWarpBitsMax = 16;  // bitmap of 2^16 labels (8 KiB) per warp
constexpr int kOvf = 256;         // columns at or above 2^16 a warp keeps in shared memory
constexpr int kUnroll = 4;        // rounds of 32 nonzeros in flight per warp (scan, fill)
constexpr int kHub = 8192;        // labels whose incoming counts and slots live in shared memory
constexpr int kScanBlocksPerSm = 6;
constexpr int kFillUnroll = 4;     // the fill's rounds in flight
constexpr int kProbeInFlight = 5;  // 16-byte prefix vectors per lane in flight when probing
constexpr int kStagedInFlight = 2; // the same for prefixes probed against staged short rows
constexpr int kDenseHubs = 16384;  // rows j below this keep a bitmap of their columns for dense pairs
constexpr int kDenseThreads = 256;

// Workspace words: [0] nonzero when the scan met a dense pair, [1] malformed
// entries seen by the scan, [2] the dense-pair margin (negative: no dense
// pairs), [3] the bitmap rows (a multiple of 128).
enum { kWDenseAny = 0, kWBad = 1, kWDenseOv = 2, kWDenseHubs = 3, kWords = 4 };

// A nonzero (i, j) at position p of row i is a dense pair when j has a
// column bitmap (j < hubs) and its prefix row_i[0,p) is longer than the
// bitmap's ceil(j/32) words plus the margin ov: then one AND and popcount
// per word of [0,j) costs less than p probes.  Dense pairs get no record;
// wedge_dense_kernel counts them.
__device__ __forceinline__ bool dense_pair(uint32_t j, uint32_t p, int64_t ov, uint32_t hubs) {
  return ov >= 0 && j < hubs && static_cast<int64_t>(p) > static_cast<int64_t>((j + 31u) >> 5) + ov;
}

struct Layout {
  size_t col32, in_cnt, in_off, bsum, in_rec, hubs, bits, words, total;
  uint32_t dense_hubs;  // rows with a column bitmap: min(kDenseHubs, numrows rounded up to 128)
};

size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

Layout layout(int64_t n, int64_t nnz) {
  Layout l;
  const size_t nz = static_cast<size_t>(nnz > 0 ? nnz : 1);
  const size_t nb = static_cast<size_t>((n + kPsumBlock - 1) / kPsumBlock) + 1;
  size_t o = 0;
  l.col32 = o;  o += up256(nz * 4);
  l.in_cnt = o; o += up256(static_cast<size_t>(n) * 4 + 4);
  l.in_off = o; o += up256(static_cast<size_t>(n + 1) * 4);
  l.bsum = o;   o += up256(nb * 4);
  l.in_rec = o; o += up256(nz * 8);
  l.hubs = o;   o += up256(static_cast<size_t>(num_sms()) * kScanBlocksPerSm * kHub * 4);
  // a multiple of 128, so each row's bitmap starts on a 16-byte boundary
  l.dense_hubs = static_cast<uint32_t>(std::min<int64_t>(kDenseHubs, (n + 127) / 128 * 128));
  l.bits = o;   o += up256(static_cast<size_t>(l.dense_hubs) * (l.dense_hubs / 32) * 4);
  l.words = o;  o += up256(kWords * 8);
  l.total = o;
  return l;
}

__device__ __forceinline__ uint32_t incl_scan_u32(uint32_t v) {
  const unsigned lane = lane_id();
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(kFull, v, o);
    if (static_cast<int>(lane) >= o) v += y;
  }
  return v;
}

// Is w in the ascending run r[0,len)?
__device__ __forceinline__ bool search_u32(const uint32_t *__restrict__ r, uint32_t len, uint32_t w) {
  uint32_t lo = 0, hi = len;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (r[mid] < w) lo = mid + 1; else hi = mid;
  }
  return lo < len && r[lo] == w;
}

// The lane owning position bb + lane of a sequence flattened over the warp,
// where lane r covers [inc_r - len_r, inc_r) and the inclusive prefixes
// inc_r strictly increase over the lanes that cover anything (len >= 1)
// and stay at the total beyond them.  Without a search: the owner is the
// number of lanes ending at or before bb (a ballot) plus the number ending
// inside (bb, bb + lane] (bits of one OR-reduction; the ends are distinct).
__device__ __forceinline__ int flat_owner(uint32_t inc, uint32_t bb) {
  const unsigned lane = lane_id();
  const uint32_t a = __popc(__ballot_sync(kFull, inc <= bb));
  const uint32_t x = inc - bb;
  const uint32_t ends = __reduce_or_sync(kFull, (inc > bb && x < 32u) ? (1u << x) : 0u);
  const uint32_t o = a + __popc(ends & ((2u << lane) - 1u));
  return o < 32u ? static_cast<int>(o) : 31;
}

// The nonzeros of 32 consecutive rows, flattened over the warp.  The rows'
// offsets are loaded one per lane; rows whose offsets are not inside
// [0,nnz] count as bad.  The non-empty rows are compacted to the low lanes
// through the warp's 32-entry staging slot so that their prefixes strictly
// increase (flat_owner's condition).
struct RowGroup {
  uint32_t b = 0, d = 0, row = 0, inc = 0, tot = 0;
  unsigned nbad = 0;
  __device__ __forceinline__ void load(const int64_t *__restrict__ off, int64_t n, int64_t nnz, int64_t r0,
                                       uint4 *slot) {
    const unsigned lane = lane_id();
    const int64_t i = r0 + lane;
    uint32_t mb = 0, md = 0;
    if (i < n) {
      const int64_t bb = off[i], e = off[i + 1];
      if (bb < 0 || e < bb || e > nnz) {
        nbad = 1;
      } else {
        mb = static_cast<uint32_t>(bb);
        md = static_cast<uint32_t>(e - bb);
      }
    }
    const unsigned m = __ballot_sync(kFull, md > 0);
    if (md > 0) slot[__popc(m & ((1u << lane) - 1u))] = make_uint4(mb, md, lane, 0u);
    __syncwarp();
    if (lane < static_cast<unsigned>(__popc(m))) {
      const uint4 t = slot[lane];
      b = t.x;
      d = t.y;
      row = t.z;
    }
    __syncwarp();
    inc = incl_scan_u32(d);
    tot = __shfl_sync(kFull, inc, 31);
  }
  // Nonzero index k, its position p in its row and the row (relative to the
  // group) of flattened position bb + lane (all lanes call; valid for < tot).
  __device__ __forceinline__ void at(uint32_t bb, uint32_t &k, uint32_t &p, uint32_t &r) const {
    const int o = flat_owner(inc, bb);
    const uint32_t ob = __shfl_sync(kFull, b, o);
    const uint32_t ox = __shfl_sync(kFull, inc - d, o);
    r = __shfl_sync(kFull, row, o);
    p = bb + lane_id() - ox;
    k = ob + p;
  }
};

// Incoming counts of hub labels (below kHub) are accumulated per block in
// shared memory: on a degree-ordered matrix nearly every row starts with
// the same few hubs, and their global counters would serialise in L2.  Each
// block's hub counts go to hubs[block][label] (for the fill's slot bases)
// and into in_cnt once.
__global__ void __launch_bounds__(kScanThreads)
    wedge_scan_kernel(const int64_t *__restrict__ off, const int64_t *__restrict__ col, int64_t n, int64_t nnz,
                      uint32_t *__restrict__ col32, uint32_t *__restrict__ in_cnt, uint32_t *__restrict__ hubs,
                      unsigned long long *__restrict__ words, unsigned long long *__restrict__ bad, int64_t ov,
                      uint32_t dhubs, const unsigned *__restrict__ run_if) {
  if (tri::skipped(run_if, 1u)) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    words[kWDenseOv] = static_cast<unsigned long long>(ov);
    words[kWDenseHubs] = dhubs;
  }
  __shared__ uint4 stage[kScanWarps][32];
  __shared__ uint32_t hub[kHub];
  for (int h = threadIdx.x; h < kHub; h += kScanThreads) hub[h] = 0;
  __syncthreads();
  const int64_t groups = (n + 31) / 32;
  const int64_t warps = static_cast<int64_t>(gridDim.x) * kScanWarps;
  const unsigned lane = lane_id();
  unsigned long long nbad = 0;
  bool any_dense = false;
  for (int64_t g = static_cast<int64_t>(blockIdx.x) * kScanWarps + (threadIdx.x >> 5); g < groups; g += warps) {
    RowGroup rg;
    rg.load(off, n, nnz, g * 32, stage[threadIdx.x >> 5]);
    nbad += rg.nbad;
    uint32_t carry = 0;  // the element before this batch (lane 31 of the last round)
    for (uint32_t base = 0; base < rg.tot; base += 32 * kUnroll) {
      uint32_t k[kUnroll], p[kUnroll], r[kUnroll], cu[kUnroll];
      int64_t c[kUnroll];
#pragma unroll
      for (int u = 0; u < kUnroll; u++) {
        rg.at(base + 32 * u, k[u], p[u], r[u]);
        c[u] = base + 32 * u + lane < rg.tot ? ld_stream(col + k[u]) : 0;
        cu[u] = (c[u] >= 0 && c[u] < static_cast<int64_t>(kBadCol)) ? static_cast<uint32_t>(c[u]) : kBadCol;
      }
#pragma unroll
      for (int u = 0; u < kUnroll; u++) {
        // the previous element of the same row: lane - 1 of this round, or
        // lane 31 of the previous one (flattened positions are consecutive)
        uint32_t prv = __shfl_up_sync(kFull, cu[u], 1);
        const uint32_t last = __shfl_sync(kFull, u == 0 ? carry : cu[u > 0 ? u - 1 : 0], 31);
        if (lane == 0) prv = last;
        if (base + 32 * u + lane < rg.tot) {
          const int64_t i = g * 32 + r[u];
          const bool ok = c[u] >= 0 && c[u] < i && (p[u] == 0 || cu[u] > prv);
          col32[k[u]] = ok ? cu[u] : kBadCol;
          if (!ok) nbad++;
          else if (p[u] > 0 && dense_pair(cu[u], p[u], ov, dhubs)) {
            any_dense = true;
          } else if (p[u] > 0) {
            if (cu[u] < static_cast<uint32_t>(kHub)) atomicAdd(&hub[cu[u]], 1u);
            else atomicAdd(in_cnt + cu[u], 1u);
          }
        }
      }
      carry = cu[kUnroll - 1];
    }
  }
  nbad = warp_sum_u64(nbad);
  if (lane == 0 && nbad) {
    atomicAdd(words + kWBad, nbad);
    if (bad) atomicAdd(bad, nbad);
  }
  if (__syncthreads_or(any_dense) && threadIdx.x == 0) words[kWDenseAny] = 1;
  uint32_t *mine = hubs + static_cast<size_t>(blockIdx.x) * kHub;
  for (int h = threadIdx.x; h < kHub; h += kScanThreads) {
    const uint32_t v = hub[h];
    mine[h] = v;
    if (v) atomicAdd(in_cnt + h, v);
  }
}

// hubs[b][h] becomes the exclusive prefix over blocks b of the hub counts.
__global__ void __launch_bounds__(256) wedge_hubscan_kernel(uint32_t *__restrict__ hubs, int nblocks, const unsigned *__restrict__ run_if) {
  if (tri::skipped(run_if, 1u)) return;
  const int h = blockIdx.x * 256 + threadIdx.x;
  if (h >= kHub) return;
  uint32_t run = 0;
  for (int b = 0; b < nblocks; b++) {
    uint32_t *x = hubs + static_cast<size_t>(b) * kHub + h;
    const uint32_t v = *x;
    *x = run;
    run += v;
  }
}

// Sum of 4 counts per thread, returned as the thread's exclusive prefix
// within the block; *total receives the block's sum (all threads).
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *total) {
  __shared__ uint32_t warp_tot[kPsumThreads / 32];
  const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
  const uint32_t inc = incl_scan_u32(v);
  if (lane == 31) warp_tot[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    const uint32_t t = warp_tot[lane];
    const uint32_t ti = incl_scan_u32(t);
    warp_tot[lane] = ti - t;  // exclusive warp offsets
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

__global__ void __launch_bounds__(kPsumThreads)
    wedge_blocksum_kernel(const uint32_t *__restrict__ in_cnt, int64_t n, uint32_t *__restrict__ bsum, const unsigned *__restrict__ run_if) {
  if (tri::skipped(run_if, 1u)) return;
  __shared__ uint32_t tot;
  const int64_t idx = static_cast<int64_t>(blockIdx.x) * kPsumBlock + static_cast<int64_t>(threadIdx.x) * kPsumPer;
  uint32_t v[4];
  load4(in_cnt, n, idx, v);
  block_excl_scan(v[0] + v[1] + v[2] + v[3], &tot);
  if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

// One block: exclusive scan of the nb block sums in place; in_off[n] = total.
__global__ void __launch_bounds__(kPsumThreads)
    wedge_topscan_kernel(uint32_t *__restrict__ bsum, int64_t nb, uint32_t *__restrict__ in_off, int64_t n, const unsigned *__restrict__ run_if) {
  if (tri::skipped(run_if, 1u)) return;
  __shared__ uint32_t tot;
  uint32_t carry = 0;
  for (int64_t base = 0; base < nb; base += kPsumBlock) {
    const int64_t idx = base + static_cast<int64_t>(threadIdx.x) * kPsumPer;
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
  if (threadIdx.x == 0) in_off[n] = carry;
}

// in_off[j] = exclusive prefix of the counts; the counts are zeroed for the fill.
__global__ void __launch_bounds__(kPsumThreads)
    wedge_offsets_kernel(uint32_t *__restrict__ in_cnt, int64_t n, const uint32_t *__restrict__ bsum,
                         uint32_t *__restrict__ in_off, const unsigned *__restrict__ run_if) {
  if (tri::skipped(run_if, 1u)) return;
  __shared__ uint32_t tot;
  const int64_t idx = static_cast<int64_t>(blockIdx.x) * kPsumBlock + static_cast<int64_t>(threadIdx.x) * kPsumPer;
  uint32_t v[4];
  load4(in_cnt, n, idx, v);
  uint32_t x = block_excl_scan(v[0] + v[1] + v[2] + v[3], &tot) + bsum[blockIdx.x];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    if (idx + q < n) {
      in_off[idx + q] = x;
      in_cnt[idx + q] = 0;
    }
    x += v[q];
  }
}

// Same grid and the same rows per block as the scan, so a block's hub
// records take the slots in_off[h] + hubs[block][h] onwards, handed out by
// shared-memory counters; other labels take global ones.
__global__ void __launch_bounds__(kScanThreads)
    wedge_fill_kernel(const int64_t *__restrict__ off, const uint32_t *__restrict__ col32, int64_t n, int64_t nnz,
                      const uint32_t *__restrict__ in_off, uint32_t *__restrict__ in_cnt,
                      const uint32_t *__restrict__ hubs, uint2 *__restrict__ in_rec,
                      const unsigned long long *__restrict__ words, const unsigned *__restrict__ run_if) {
  if (tri::skipped(run_if, 1u)) return;
  __shared__ uint4 stage[kScanWarps][32];
  __shared__ uint32_t hubslot[kHub];
  if (words[kWBad]) return;
  const int64_t ov = static_cast<int64_t>(words[kWDenseOv]);
  const uint32_t dhubs = static_cast<uint32_t>(words[kWDenseHubs]);
  {
    const uint32_t *mine = hubs + static_cast<size_t>(blockIdx.x) * kHub;
    for (int h = threadIdx.x; h < kHub; h += kScanThreads) hubslot[h] = h < n ? in_off[h] + mine[h] : 0u;
    __syncthreads();
  }
  const int64_t groups = (n + 31) / 32;
  const int64_t warps = static_cast<int64_t>(gridDim.x) * kScanWarps;
  const unsigned lane = lane_id();
  for (int64_t g = static_cast<int64_t>(blockIdx.x) * kScanWarps + (threadIdx.x >> 5); g < groups; g += warps) {
    RowGroup rg;
    rg.load(off, n, nnz, g * 32, stage[threadIdx.x >> 5]);
    for (uint32_t base = 0; base < rg.tot; base += 32 * kFillUnroll) {
      uint32_t k[kFillUnroll], p[kFillUnroll], c[kFillUnroll], slot[kFillUnroll];
#pragma unroll
      for (int u = 0; u < kFillUnroll; u++) {
        uint32_t r;
        rg.at(base + 32 * u, k[u], p[u], r);
        c[u] = base + 32 * u + lane < rg.tot ? col32[k[u]] : kBadCol;
        // the first nonzero of a row closes no wedge; dense pairs are counted apart
        if (p[u] == 0 || (c[u] != kBadCol && dense_pair(c[u], p[u], ov, dhubs))) c[u] = kBadCol;
      }
#pragma unroll
      for (int u = 0; u < kFillUnroll; u++)
        slot[u] = c[u] == kBadCol               ? 0u
                  : c[u] < static_cast<uint32_t>(kHub) ? atomicAdd(&hubslot[c[u]], 1u)
                                                : in_off[c[u]] + atomicAdd(in_cnt + c[u], 1u);
#pragma unroll
      for (int u = 0; u < kFillUnroll; u++)
        if (c[u] != kBadCol) in_rec[slot[u]] = make_uint2(k[u] - p[u], p[u]);
    }
  }
}

// Is element w of an incoming prefix in row j?  Labels below `lim` are
// tested in the bitmap; with OVF the others are searched in row j's sorted
// tail [lim, j) -- kept in shared memory when it has at most kOvf entries.
template <bool OVF>
struct RowJ {
  const uint32_t *bm;
  uint32_t wmask, lim;
  const uint32_t *tail;  // shared-memory copy, or the tail in col32
  uint32_t ntail;
  __device__ __forceinline__ uint32_t has(uint32_t w) const {
    if (!OVF || w < lim) return tri::bit_of(bm, wmask, w);
    return search_u32(tail, ntail, w) ? 1u : 0u;
  }
  // elements of x (element indices base..base+3) inside [s, s + len)
  __device__ __forceinline__ uint32_t test4(uint4 x, uint32_t base, uint32_t s, uint32_t len) const {
    const uint32_t o = base - s;  // wraps for elements before s
    uint32_t c = 0;
    if (o < len) c += has(x.x);
    if (o + 1u < len) c += has(x.y);
    if (o + 2u < len) c += has(x.z);
    if (o + 3u < len) c += has(x.w);
    return c;
  }
};

// Probes of up to 32 prefixes (lane l holds record l; {0,0} for none; real
// records have p >= 1) against row j: every element of each prefix
// row_i[s, s+p) is tested.  The prefixes' 16-byte vectors are flattened over
// the warp so every lane has a vector whatever the prefix lengths,
// kProbeInFlight vectors per lane in flight.
template <bool OVF>
__device__ __forceinline__ void probe_records(const RowJ<OVF> rj, const uint4 *__restrict__ col4, uint32_t nvec_all,
                                              uint2 rec, unsigned long long &cnt, unsigned long long &wk) {
  const unsigned lane = lane_id();
  const uint32_t s = rec.x, p = rec.y;
  const uint32_t v0 = s >> 2;
  const uint32_t nv = p ? ((s + p + 3u) >> 2) - v0 : 0u;
  const uint32_t inc = incl_scan_u32(nv);
  const uint32_t tot = __shfl_sync(kFull, inc, 31);
  const uint32_t q = v0 - (inc - nv);  // vector index = q + flattened position
  wk += p;
  for (uint32_t base = 0; base < tot; base += 32 * kProbeInFlight) {
    uint4 xv[kProbeInFlight];
    uint32_t vi[kProbeInFlight], ps[kProbeInFlight], pl[kProbeInFlight];
    bool act[kProbeInFlight];
#pragma unroll
    for (int h = 0; h < kProbeInFlight; h++) {
      const uint32_t bb = base + 32u * h;
      const int o = flat_owner(inc, bb);
      vi[h] = __shfl_sync(kFull, q, o) + bb + lane;
      ps[h] = __shfl_sync(kFull, s, o);
      pl[h] = __shfl_sync(kFull, p, o);
      act[h] = bb + lane < tot && vi[h] < nvec_all;
      xv[h] = act[h] ? col4[vi[h]] : make_uint4(0u, 0u, 0u, 0u);
    }
#pragma unroll
    for (int h = 0; h < kProbeInFlight; h++)
      if (act[h]) cnt += rj.test4(xv[h], vi[h] << 2, ps[h], pl[h]);
  }
}

// Probes of up to 32 prefixes of different rows j (lane l holds record l
// and the place of its row j in the warp's staging buffer, stg[ro, ro + rl)),
// each element binary-searched in its staged row; flattened as above, with
// kStagedInFlight vectors per lane in flight.
__device__ __forceinline__ void probe_records_staged(const uint32_t *__restrict__ stg, uint32_t ro, uint32_t rl,
                                                     const uint4 *__restrict__ col4, uint32_t nvec_all, uint2 rec,
                                                     unsigned long long &cnt, unsigned long long &wk) {
  const unsigned lane = lane_id();
  const uint32_t s = rec.x, p = rec.y;
  const uint32_t v0 = s >> 2;
  const uint32_t nv = p ? ((s + p + 3u) >> 2) - v0 : 0u;
  const uint32_t inc = incl_scan_u32(nv);
  const uint32_t tot = __shfl_sync(kFull, inc, 31);
  const uint32_t q = v0 - (inc - nv);
  wk += p;
  for (uint32_t base = 0; base < tot; base += 32 * kStagedInFlight) {
    uint4 xv[kStagedInFlight];
    uint32_t vi[kStagedInFlight], ps[kStagedInFlight], pl[kStagedInFlight], oro[kStagedInFlight],
        orl[kStagedInFlight];
    bool act[kStagedInFlight];
#pragma unroll
    for (int h = 0; h < kStagedInFlight; h++) {
      const uint32_t bb = base + 32u * h;
      const int o = flat_owner(inc, bb);
      vi[h] = __shfl_sync(kFull, q, o) + bb + lane;
      ps[h] = __shfl_sync(kFull, s, o);
      pl[h] = __shfl_sync(kFull, p, o);
      oro[h] = __shfl_sync(kFull, ro, o);
      orl[h] = __shfl_sync(kFull, rl, o);
      act[h] = bb + lane < tot && vi[h] < nvec_all;
      xv[h] = act[h] ? col4[vi[h]] : make_uint4(0u, 0u, 0u, 0u);
    }
#pragma unroll
    for (int h = 0; h < kStagedInFlight; h++) {
      if (!act[h]) continue;
      const uint32_t e = (vi[h] << 2) - ps[h];  // wraps for elements before the prefix
      const uint32_t *r = stg + oro[h];
      if (e < pl[h] && search_u32(r, orl[h], xv[h].x)) cnt++;
      if (e + 1u < pl[h] && search_u32(r, orl[h], xv[h].y)) cnt++;
      if (e + 2u < pl[h] && search_u32(r, orl[h], xv[h].z)) cnt++;
      if (e + 3u < pl[h] && search_u32(r, orl[h], xv[h].w)) cnt++;
    }
  }
}

__device__ __forceinline__ void flush(unsigned long long cnt, unsigned long long wk, unsigned long long *count,
                                      unsigned long long *work) {
  cnt = warp_sum_u64(cnt);
  wk = warp_sum_u64(wk);
  if (lane_id() == 0) {
    if (cnt) atomicAdd(count, cnt);
    if (wk && work) atomicAdd(work, wk);
  }
}

// One warp per row j, each warp with its own bitmap of 2^wbits labels and a
// kOvf-entry tail list in shared memory.  Rows below wlim = min(n, 2^wbits)
// (all columns inside the bitmap) are claimed one at a time in label order,
// which on a degree-ordered matrix starts with the rows that close the most
// wedges; the rest 32 at a time, one lane checking each for incoming
// prefixes so that empty ones cost no serial loads.
__global__ void __launch_bounds__(kWarpThreads, 3)
    wedge_count_kernel(const int64_t *__restrict__ off, const uint32_t *__restrict__ col32,
                       const uint32_t *__restrict__ in_off, const uint2 *__restrict__ in_rec, int64_t n, int64_t wlim,
                       int wbits, uint32_t nvec_all, uint32_t stage_max, const unsigned long long *__restrict__ words,
                       unsigned long long *__restrict__ count, unsigned long long *__restrict__ work,
                       unsigned long long *__restrict__ cursor, const unsigned *__restrict__ run_if) {
  if (tri::skipped(run_if, 1u)) return;
  extern __shared__ uint32_t wsm[];
  if (words[kWBad]) return;
  const unsigned lane = lane_id();
  const uint32_t nw = 1u << (wbits - 5);
  uint32_t *bm = wsm + static_cast<size_t>(threadIdx.x >> 5) * (nw + kOvf);
  uint32_t *ovf = bm + nw;
  const uint32_t lim = 1u << wbits;
  const uint4 *__restrict__ col4 = reinterpret_cast<const uint4 *>(col32);  // col32 is 256-byte aligned
  for (uint32_t w = lane; w < nw; w += 32) bm[w] = 0;
  __syncwarp();
  unsigned long long cnt = 0, wk = 0;
  const unsigned long long nbig = static_cast<unsigned long long>(wlim);
  // Two queues: rows below wlim one at a time (cursor[0], issue-bound work)
  // and claims of 32 rows above it (cursor[1], latency-bound); each warp
  // alternates between them so that the two kinds overlap on every SM.
  bool big_done = false, small_done = false;
  for (unsigned it = 0;; it++) {
    if (big_done && small_done) break;
    const bool take_big = !big_done && (small_done || (it & 1u) == 0);
    unsigned long long t = 0;
    if (lane == 0) t = atomicAdd(cursor + (take_big ? 0 : 1), 1ull);
    t = __shfl_sync(kFull, t, 0);
    int64_t j0, j1;
    if (take_big) {
      if (t >= nbig) {
        big_done = true;
        continue;
      }
      j0 = static_cast<int64_t>(t);
      j1 = j0 + 1;
    } else {
      j0 = wlim + static_cast<int64_t>(t) * 32;
      if (j0 >= n) {
        small_done = true;
        continue;
      }
      j1 = j0 + 32 < n ? j0 + 32 : n;
    }
    // rows of this claim with incoming prefixes and a non-empty row j
    const int64_t jl = j0 + lane;
    bool live = false;
    uint32_t lb = 0, ld = 0, lr0 = 0, lnr = 0;
    if (jl < j1) {
      lr0 = in_off[jl];
      lnr = in_off[jl + 1] - lr0;
      const int64_t bb = off[jl], dd = off[jl + 1] - bb;
      live = lnr > 0 && dd > 0;
      lb = static_cast<uint32_t>(bb);
      ld = static_cast<uint32_t>(dd);
    }
    if (!take_big) {
      // Rows above wlim: the short ones (at most stage_max columns, where a
      // binary search beats setting and clearing a bitmap) are staged in the
      // warp's buffer -- as many at a time as fit -- and all their prefixes
      // probed flattened, so they cost a few memory round trips per claim
      // instead of a few per row.  The bitmap area is the buffer, zeroed
      // again after each batch.
      uint4 *slot = reinterpret_cast<uint4 *>(ovf + kOvf) - 32;
      uint32_t *stg = bm;
      const uint32_t cap = nw + kOvf - 128;
      const bool fits = live && ld <= stage_max;
      const unsigned lm = __ballot_sync(kFull, fits);
      if (fits) slot[__popc(lm & ((1u << lane) - 1u))] = make_uint4(lb, ld, lr0, lnr);
      __syncwarp();
      const unsigned m = __popc(lm);
      uint32_t cb = 0, cd = 0, cr0 = 0, cnr = 0;
      if (lane < m) {
        const uint4 v = slot[lane];
        cb = v.x;
        cd = v.y;
        cr0 = v.z;
        cnr = v.w;
      }
      __syncwarp();
      const uint32_t incd = incl_scan_u32(cd);  // strictly increasing over lanes < m (cd >= 1)
      for (unsigned t0 = 0; t0 < m;) {
        const uint32_t base_s = __shfl_sync(kFull, incd - cd, t0);
        const unsigned fm = __ballot_sync(kFull, lane >= t0 && lane < m && incd - base_s <= cap);
        const unsigned t1 = 32u - __clz(fm);  // lanes [t0, t1) fit (lane t0 always does)
        const uint32_t end_s = __shfl_sync(kFull, incd, t1 - 1);
        for (uint32_t g = base_s; g < end_s; g += 32) {
          const int o = flat_owner(incd, g);
          const uint32_t ob = __shfl_sync(kFull, cb, o), ox = __shfl_sync(kFull, incd - cd, o);
          if (g + lane < end_s) stg[g + lane - base_s] = col32[ob + (g + lane - ox)];
        }
        __syncwarp();
        const uint32_t cn = lane >= t0 && lane < t1 ? cnr : 0u;
        const uint32_t incr = incl_scan_u32(cn);
        const uint32_t totr = __shfl_sync(kFull, incr, 31);
        for (uint32_t base = 0; base < totr; base += 32) {
          const int o = flat_owner(incr, base);
          const uint32_t o0 = __shfl_sync(kFull, cr0, o), ox = __shfl_sync(kFull, incr - cn, o);
          const uint32_t ro = __shfl_sync(kFull, incd - cd, o) - base_s, rl = __shfl_sync(kFull, cd, o);
          const uint2 rec = base + lane < totr ? in_rec[o0 + (base + lane - ox)] : make_uint2(0u, 0u);
          probe_records_staged(stg, ro, rl, col4, nvec_all, rec, cnt, wk);
        }
        __syncwarp();
        for (uint32_t g = lane; g < end_s - base_s; g += 32) stg[g] = 0;
        __syncwarp();
        t0 = t1;
      }
      // longer rows: one at a time below, on the (zero) bitmap
      live = live && !fits;
      if (!__any_sync(kFull, live)) continue;
    }
    unsigned todo = __ballot_sync(kFull, live);
    while (todo) {
      const int64_t j = j0 + __ffs(todo) - 1;
      todo &= todo - 1;
      const uint32_t r0 = in_off[j], nrec = in_off[j + 1] - r0;
      const int64_t b = off[j], d = off[j + 1] - b;
      if (j < wlim) {
        for (int64_t k = lane; k < d; k += 32) {
          const uint32_t c = col32[b + k];
          atomicOr(&bm[(c >> 5) & (nw - 1u)], 1u << (c & 31));
        }
        __syncwarp();
        const RowJ<false> rj{bm, nw - 1u, lim, nullptr, 0u};
        for (uint32_t r = 0; r < nrec; r += 32) {
          const uint2 rec = r + lane < nrec ? in_rec[r0 + r + lane] : make_uint2(0u, 0u);
          probe_records(rj, col4, nvec_all, rec, cnt, wk);
        }
      } else {
        // columns below lim go to the bitmap, the ascending tail [lim, j) to the list
        uint32_t below = 0;
        for (int64_t k = lane; k < d; k += 32) {
          const uint32_t c = col32[b + k];
          if (c < lim) {
            atomicOr(&bm[c >> 5], 1u << (c & 31));
            below++;
          }
        }
        below = __reduce_add_sync(kFull, below);
        const uint32_t ntail = static_cast<uint32_t>(d) - below;
        const bool cached = ntail <= static_cast<uint32_t>(kOvf);
        if (cached)
          for (uint32_t k = lane; k < ntail; k += 32) ovf[k] = col32[b + below + k];
        __syncwarp();
        const RowJ<true> rj{bm, nw - 1u, lim, cached ? ovf : col32 + b + below, ntail};
        for (uint32_t r = 0; r < nrec; r += 32) {
          const uint2 rec = r + lane < nrec ? in_rec[r0 + r + lane] : make_uint2(0u, 0u);
          probe_records(rj, col4, nvec_all, rec, cnt, wk);
        }
      }
      __syncwarp();
      for (int64_t k = lane; k < d; k += 32) {
        const uint32_t c = col32[b + k];
        if (c < lim) bm[(c >> 5) & (nw - 1u)] = 0;
      }
      __syncwarp();
    }
  }
  flush(cnt, wk, count, work);
}

// Column bitmaps of the rows j below dhubs (their columns all lie in
// [0, j)), built when the scan met a dense pair: row j's at bits + j *
// (dhubs / 32), its words zeroed up to a multiple of 4 past ceil(j/32) (the
// dense kernel reads 16-byte vectors) before its bits are set.
__global__ void __launch_bounds__(256)
    wedge_hubbits_kernel(const int64_t *__restrict__ off, const uint32_t *__restrict__ col32, int64_t n,
                         uint32_t *__restrict__ bits, const unsigned long long *__restrict__ words,
                         const unsigned *__restrict__ run_if) {
  if (tri::skipped(run_if, 1u)) return;
  if (words[kWBad] || !words[kWDenseAny] || static_cast<int64_t>(words[kWDenseOv]) < 0) return;
  const uint32_t dhubs = static_cast<uint32_t>(words[kWDenseHubs]);
  const uint32_t stride = dhubs / 32;
  const unsigned lane = lane_id();
  const int64_t rows = static_cast<int64_t>(dhubs) < n ? static_cast<int64_t>(dhubs) : n;
  const int64_t warps = static_cast<int64_t>(gridDim.x) * 8;
  for (int64_t j = static_cast<int64_t>(blockIdx.x) * 8 + (threadIdx.x >> 5); j < rows; j += warps) {
    uint32_t *row = bits + static_cast<size_t>(j) * stride;
    const uint32_t nz = ((((static_cast<uint32_t>(j) + 31u) >> 5) + 3u) >> 2) << 2;
    for (uint32_t w = lane; w < nz; w += 32) row[w] = 0;
    __syncwarp();
    for (int64_t k = off[j] + lane; k < off[j + 1]; k += 32) {
      const uint32_t c = col32[k];
      if (c < static_cast<uint32_t>(j)) atomicOr(&row[c >> 5], 1u << (c & 31));  // the scan checked c < j
    }
  }
}

// The dense pairs: one warp per row i that has any, with row i's columns
// below its largest dense j as bits in the warp's shared memory.  Each pair
// (i, j) adds popc(row_i & row_j) over the ceil(j/32) words of [0, j) --
// row j's bits all lie below j.  The 16-byte vectors of up to 32 pairs are
// flattened over the lanes, kDenseInFlight of them per lane in flight, so a
// pair costs no round trip of its own.  As the probe kernel would have, each
// pair adds p to the work tally when row j has columns.
constexpr int kDenseInFlight = 4;

__global__ void __launch_bounds__(kDenseThreads)
    wedge_dense_kernel(const int64_t *__restrict__ off, const uint32_t *__restrict__ col32, int64_t n,
                       const uint32_t *__restrict__ bits, const unsigned long long *__restrict__ words,
                       unsigned long long *__restrict__ count, unsigned long long *__restrict__ work,
                       const unsigned *__restrict__ run_if) {
  if (tri::skipped(run_if, 1u)) return;
  if (words[kWBad] || !words[kWDenseAny]) return;
  const int64_t ov = static_cast<int64_t>(words[kWDenseOv]);
  const uint32_t dhubs = static_cast<uint32_t>(words[kWDenseHubs]);
  if (ov < 0 || dhubs == 0) return;
  __shared__ __align__(16) uint32_t bmall[kDenseThreads / 32][kDenseHubs / 32];
  __shared__ uint32_t stage[kDenseThreads / 32][32];
  const unsigned lane = lane_id();
  uint32_t *bm = bmall[threadIdx.x >> 5];
  uint32_t *stg = stage[threadIdx.x >> 5];
  for (int w = lane; w < kDenseHubs / 32; w += 32) bm[w] = 0;
  __syncwarp();
  const uint32_t stride = dhubs / 32;
  unsigned long long cnt = 0, wk = 0;
  const int64_t warps = static_cast<int64_t>(gridDim.x) * (kDenseThreads / 32);
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * (kDenseThreads / 32) + (threadIdx.x >> 5); i < n; i += warps) {
    const int64_t b = off[i], d = off[i + 1] - b;
    if (d < ov + 2) continue;  // p <= d - 1 must exceed ov + 1
    uint32_t jmax = 0;
    for (int64_t k = lane; k < d; k += 32) {
      const uint32_t c = col32[b + k];
      if (dense_pair(c, static_cast<uint32_t>(k), ov, dhubs)) jmax = c > jmax ? c : jmax;
    }
    jmax = __reduce_max_sync(kFull, jmax);
    if (jmax == 0) continue;  // a dense j is at least ov + 2
    for (int64_t k = lane; k < d; k += 32) {
      const uint32_t c = col32[b + k];
      if (c < jmax) atomicOr(&bm[c >> 5], 1u << (c & 31));
    }
    __syncwarp();
    for (int64_t k0 = 0; k0 < d; k0 += 32) {
      const int64_t k = k0 + lane;
      const uint32_t c = k < d ? col32[b + k] : kBadCol;
      const bool dn = k < d && dense_pair(c, static_cast<uint32_t>(k), ov, dhubs);
      if (dn && off[c + 1] > off[c]) wk += static_cast<unsigned long long>(k);
      const unsigned m = __ballot_sync(kFull, dn);
      if (!m) continue;
      // the dense columns to the low lanes, so their vector counts strictly increase
      if (dn) stg[__popc(m & ((1u << lane) - 1u))] = c;
      __syncwarp();
      const unsigned nd = __popc(m);
      const uint32_t cj = lane < nd ? stg[lane] : 0u;
      __syncwarp();
      // 16-byte vectors of [0, j): the last may reach past ceil(j/32) words,
      // where row j's bitmap is zero (its stride is a multiple of 4 words)
      const uint32_t nv = lane < nd ? (((cj + 31u) >> 5) + 3u) >> 2 : 0u;
      const uint32_t inc = incl_scan_u32(nv);
      const uint32_t tot = __shfl_sync(kFull, inc, 31);
      const uint4 *bm4 = reinterpret_cast<const uint4 *>(bm);
      const uint4 *bits4 = reinterpret_cast<const uint4 *>(bits);
      const uint32_t stride4 = stride >> 2;
      uint32_t sum = 0;  // at most 32 pairs of at most 2^14 common columns each
      for (uint32_t base = 0; base < tot; base += 32u * kDenseInFlight) {
        uint4 x[kDenseInFlight], y[kDenseInFlight];
        bool act[kDenseInFlight];
#pragma unroll
        for (int h = 0; h < kDenseInFlight; h++) {
          const uint32_t bb = base + 32u * h;
          const int o = flat_owner(inc, bb);
          const uint32_t j = __shfl_sync(kFull, cj, o);
          const uint32_t v = bb + lane - __shfl_sync(kFull, inc - nv, o);
          act[h] = bb + lane < tot;
          // an idle lane reads vector 0 of row j, and its sum is dropped
          const uint32_t va = act[h] ? v : 0u;
          x[h] = bits4[static_cast<size_t>(j) * stride4 + va];
          y[h] = bm4[va];
        }
#pragma unroll
        for (int h = 0; h < kDenseInFlight; h++) {
          const uint32_t t = __popc(x[h].x & y[h].x) + __popc(x[h].y & y[h].y) + __popc(x[h].z & y[h].z) +
                             __popc(x[h].w & y[h].w);
          sum += act[h] ? t : 0u;
        }
      }
      cnt += sum;
    }
    __syncwarp();
    for (int64_t k = lane; k < d; k += 32) {
      const uint32_t c = col32[b + k];
      if (c < jmax) bm[c >> 5] = 0;
    }
    __syncwarp();
  }
  flush(cnt, wk, count, work);
}

bool g_count_attr[64];

// log2 of the per-warp bitmap: min(16, labels rounded up to a power of two >= 32).
int warp_bits(int64_t numrows) {
  int wb = 5;
  while (wb < kWarpBitsMax && (int64_t(1) << wb) < numrows) wb++;
  return wb;
}

size_t count_smem(int wb) { return ((size_t(1) << (wb - 5)) + kOvf) * sizeof(uint32_t) * kWarpWarps; }

}  // namespace

bool tri_wedge_supported(int64_t numrows, int64_t nnz) {
  // u32 labels, edge indices and vector element indices (up to nnz + 3)
  return numrows > 0 && numrows < 0xffffffffll && nnz >= 0 && nnz < 0xffffff00ll;
}

size_t tri_wedge_workspace_bytes(int64_t numrows, int64_t nnz) { return layout(numrows, nnz).total; }

int tri_wedge_prepare(const int64_t *offset, const int64_t *nonzero, int64_t numrows, int64_t nnz, void *ws,
                      unsigned long long *bad, cudaStream_t stream, const unsigned *run_if) {
  if (!tri_wedge_supported(numrows, nnz)) return BALE_EINVAL;
  const Layout l = layout(numrows, nnz);
  char *p = static_cast<char *>(ws);
  uint32_t *col32 = reinterpret_cast<uint32_t *>(p + l.col32);
  uint32_t *in_cnt = reinterpret_cast<uint32_t *>(p + l.in_cnt);
  uint32_t *in_off = reinterpret_cast<uint32_t *>(p + l.in_off);
  uint32_t *bsum = reinterpret_cast<uint32_t *>(p + l.bsum);
  uint2 *in_rec = reinterpret_cast<uint2 *>(p + l.in_rec);
  uint32_t *hubs = reinterpret_cast<uint32_t *>(p + l.hubs);
  uint32_t *bits = reinterpret_cast<uint32_t *>(p + l.bits);
  unsigned long long *words = reinterpret_cast<unsigned long long *>(p + l.words);
  const int sms = num_sms();
  // dense pairs (tri.dense 0: none) and their margin over the bitmap's words
  const int64_t ov = knob_or("tri.dense", 1) == 0 ? -1 : knob_or("tri.dense_ov", 32);
  BALE_CUDA_OK(cudaMemsetAsync(in_cnt, 0, static_cast<size_t>(numrows) * 4, stream));
  BALE_CUDA_OK(cudaMemsetAsync(words, 0, kWords * sizeof(unsigned long long), stream));
  const int64_t groups = (numrows + 31) / 32;
  int64_t sblocks = (groups + kScanWarps - 1) / kScanWarps;
  const int64_t scap = static_cast<int64_t>(sms) * kScanBlocksPerSm;  // the hubs array holds this many blocks
  if (sblocks > scap) sblocks = scap;
  wedge_scan_kernel<<<static_cast<unsigned>(sblocks), kScanThreads, 0, stream>>>(
      offset, nonzero, numrows, nnz, col32, in_cnt, hubs, words, bad, ov, l.dense_hubs, run_if);
  BALE_CUDA_OK(cudaGetLastError());
  if (ov >= 0 && l.dense_hubs > 0) {
    wedge_hubbits_kernel<<<static_cast<unsigned>((l.dense_hubs + 7) / 8), 256, 0, stream>>>(offset, col32, numrows,
                                                                                            bits, words, run_if);
    BALE_CUDA_OK(cudaGetLastError());
  }
  wedge_hubscan_kernel<<<kHub / 256, 256, 0, stream>>>(hubs, static_cast<int>(sblocks), run_if);
  BALE_CUDA_OK(cudaGetLastError());
  const int64_t nb = (numrows + kPsumBlock - 1) / kPsumBlock;
  wedge_blocksum_kernel<<<static_cast<unsigned>(nb), kPsumThreads, 0, stream>>>(in_cnt, numrows, bsum, run_if);
  BALE_CUDA_OK(cudaGetLastError());
  wedge_topscan_kernel<<<1, kPsumThreads, 0, stream>>>(bsum, nb, in_off, numrows, run_if);
  BALE_CUDA_OK(cudaGetLastError());
  wedge_offsets_kernel<<<static_cast<unsigned>(nb), kPsumThreads, 0, stream>>>(in_cnt, numrows, bsum, in_off,
                                                                               run_if);
  BALE_CUDA_OK(cudaGetLastError());
  wedge_fill_kernel<<<static_cast<unsigned>(sblocks), kScanThreads, 0, stream>>>(offset, col32, numrows, nnz, in_off,
                                                                                 in_cnt, hubs, in_rec, words, run_if);
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

int tri_wedge_run(const int64_t *offset, const void *ws, int64_t numrows, int64_t nnz, unsigned long long *count,
                  unsigned long long *work, unsigned long long *cursor, cudaStream_t stream, const unsigned *run_if) {
  if (!tri_wedge_supported(numrows, nnz)) return BALE_EINVAL;
  const Layout l = layout(numrows, nnz);
  const char *p = static_cast<const char *>(ws);
  const uint32_t *col32 = reinterpret_cast<const uint32_t *>(p + l.col32);
  const uint32_t *in_off = reinterpret_cast<const uint32_t *>(p + l.in_off);
  const uint2 *in_rec = reinterpret_cast<const uint2 *>(p + l.in_rec);
  const uint32_t *bits = reinterpret_cast<const uint32_t *>(p + l.bits);
  const unsigned long long *words = reinterpret_cast<const unsigned long long *>(p + l.words);
  const int sms = num_sms();
  const int wb = warp_bits(numrows);
  const int64_t wlim = numrows < (int64_t(1) << wb) ? numrows : (int64_t(1) << wb);
  const uint32_t nvec_all = static_cast<uint32_t>((nnz + 3) / 4);
  const uint32_t stage_max = static_cast<uint32_t>(knob_or("tri.wedge_stage_max", 64));
  const size_t smem = count_smem(wb);
  const int dev = current_device();
  BALE_CUDA_OK(cudaMemsetAsync(cursor, 0, 2 * sizeof(unsigned long long), stream));
  if (dev >= 0 && dev < 64 && !g_count_attr[dev]) {
    BALE_CUDA_OK(cudaFuncSetAttribute(wedge_count_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(count_smem(kWarpBitsMax))));
    g_count_attr[dev] = true;
  }
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, wedge_count_kernel, kWarpThreads, smem) != cudaSuccess ||
      occ < 1)
    occ = 1;
  int64_t blocks = static_cast<int64_t>(sms) * occ;
  const int64_t claims = wlim + (numrows - wlim + 31) / 32;  // both queues
  const int64_t need = (claims + kWarpWarps - 1) / kWarpWarps;
  if (blocks > need) blocks = need > 0 ? need : 1;
  wedge_count_kernel<<<static_cast<unsigned>(blocks), kWarpThreads, smem, stream>>>(
      offset, col32, in_off, in_rec, numrows, wlim, wb, nvec_all, stage_max, words, count, work, cursor, run_if);
  BALE_CUDA_OK(cudaGetLastError());
  // the dense pairs the prepare step left out of the records (none when its
  // margin was negative: the kernel returns at once)
  const int64_t dgroups = (numrows + kDenseThreads / 32 - 1) / (kDenseThreads / 32);
  wedge_dense_kernel<<<static_cast<unsigned>(std::min<int64_t>(dgroups, static_cast<int64_t>(sms) * 8)), kDenseThreads,
                       0, stream>>>(offset, col32, numrows, bits, words, count, work, run_if);
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

int launch_triangle_wedge(const int64_t *offset, const int64_t *nonzero, int64_t numrows, int64_t nnz,
                          unsigned long long *count, unsigned long long *work, unsigned long long *bad, void *ws,
                          unsigned long long *cursor, cudaStream_t stream, const unsigned *run_if) {
  const int rc = tri_wedge_prepare(offset, nonzero, numrows, nnz, ws, bad, stream, run_if);
  if (rc != BALE_OK) return rc;
  return tri_wedge_run(offset, ws, numrows, nnz, count, work, cursor, stream, run_if);
}

}  // namespace bale
