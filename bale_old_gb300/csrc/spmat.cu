// spmat.cu -- spmat's operations at one PE on the device, each bit-identical
// to the reference:
//   * transpose_matrix_agi and permute_matrix_agi (spmat/spmat_agi.upc:
//     119-235): a key pass and a sort; a warp per permuted row;
//   * rand_permp_agi and rand_permp_exstack (spmat/spmat_agi.upc:56-107,
//     spmat/spmat_exstack.upc:62-190): dart throwing decided in parallel,
//     the throws grouped by slot region so that their claims stay in L2;
//   * read_matrix_mm_to_dist (spmat/spmat_utils.upc:217-370): the body
//     parsed on the device, a stable sort keeping each row's file order;
//   * binary datasets (spmat/spmat_agi.upc:245-335): row lengths and
//     columns streamed between device memory and the files through two
//     pinned chunks.
// The sorts are sort.cu's stable radix sort.
#include <sys/stat.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "sort.cuh"

namespace bale {
namespace {

constexpr unsigned kFull = 0xffffffffu;

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

// The lane owning flattened position bb + lane, where lane r covers
// [inc_r - len_r, inc_r), the inclusive prefixes inc_r strictly increase over
// the lanes that cover anything and stay at the total beyond them: the lanes
// ending at or before bb (a ballot) plus those ending inside (bb, bb + lane]
// (bits of one OR-reduction; the ends are distinct).
__device__ __forceinline__ int flat_owner64(int64_t inc, int64_t bb) {
  const unsigned lane = lane_id();
  const uint32_t a = __popc(__ballot_sync(kFull, inc <= bb));
  const int64_t x = inc - bb;
  const uint32_t ends = __reduce_or_sync(kFull, (x > 0 && x < 32) ? (1u << static_cast<uint32_t>(x)) : 0u);
  const uint32_t o = a + __popc(ends & ((2u << lane) - 1u));
  return o < 32u ? static_cast<int>(o) : 31;
}

// keys[k] = col << rb | row for every nonzero of a checked CSR.  A warp
// takes 32 rows and flattens their nonzeros over its lanes (empty rows
// dropped, so the prefixes strictly increase): each lane knows its
// nonzero's row without a search, and the reads and writes coalesce.
__global__ void __launch_bounds__(256)
    transpose_keys_kernel(const int64_t *__restrict__ off, const int64_t *__restrict__ col, int64_t numrows,
                          int rb, uint64_t *__restrict__ keys) {
  __shared__ longlong2 stage[8][32];
  const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
  const int64_t groups = (numrows + 31) / 32;
  const int64_t warps = static_cast<int64_t>(gridDim.x) * 8;
  for (int64_t g = static_cast<int64_t>(blockIdx.x) * 8 + warp; g < groups; g += warps) {
    const int64_t i = g * 32 + lane;
    int64_t b = 0, d = 0;
    if (i < numrows) {
      b = off[i];
      d = off[i + 1] - b;
    }
    const unsigned live = __ballot_sync(kFull, d > 0);
    if (d > 0) stage[warp][__popc(live & ((1u << lane) - 1u))] = make_longlong2(b, (d << 5) | lane);
    __syncwarp();
    int64_t mb = 0, md = 0, mrow = 0;
    if (lane < static_cast<unsigned>(__popc(live))) {
      const longlong2 t = stage[warp][lane];
      mb = t.x;
      md = t.y >> 5;
      mrow = g * 32 + (t.y & 31);
    }
    __syncwarp();
    int64_t inc = md;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(kFull, inc, o);
      if (static_cast<int>(lane) >= o) inc += y;
    }
    const int64_t tot = __shfl_sync(kFull, inc, 31);
    for (int64_t bb = 0; bb < tot; bb += 32) {
      const int o = flat_owner64(inc, bb);
      const int64_t ob = __shfl_sync(kFull, mb, o), ox = __shfl_sync(kFull, inc - md, o);
      const int64_t orow = __shfl_sync(kFull, mrow, o);
      if (bb + lane < tot) {
        const int64_t k = ob + (bb + lane - ox);
        keys[k] = (static_cast<uint64_t>(col[k]) << rb) | static_cast<uint64_t>(orow);
      }
    }
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

__device__ __forceinline__ uint64_t lcg_step(uint64_t x) { return (kLcgA * x + kLcgC) & kLcgMask; }

// The LCG's affine map applied 32 times, x -> kLcgA32 x + kLcgC32 (mod 2^48).
struct LcgMap {
  uint64_t a, c;
};
constexpr LcgMap lcg_power(int k) {
  LcgMap m{1, 0};
  for (int i = 0; i < k; i++) m = {(m.a * kLcgA) & kLcgMask, (m.c * kLcgA + kLcgC) & kLcgMask};
  return m;
}
constexpr LcgMap kLcg32 = lcg_power(32);

// Dart throwing (rand_permp_agi, spmat/spmat_agi.upc:56-107; rand_permp_exstack,
// spmat/spmat_exstack.upc:62-190).  Throw t lands in slot r_t = lrand48() % m
// for the lrand48 output number idx(t) = t + lost(t): the exstack form loses
// one draw each time a round of per_round throws finds its buffer full, which
// happens in every round before round cap and in none after it, so lost(t) =
// min(t / per_round, cap) (per_round = 0: nothing is lost).  A throw takes its
// slot exactly when no earlier throw hit it (a slot, once taken, stays
// taken), so owner[r] = min{t : r_t = r} decides every throw at once.
//
// The owner and target arrays hold 2n words (512 MB at n = 2^26), far beyond
// L2, and the throws land at random.  So the throws become keys slot << tb |
// t, one stable radix pass groups them by slot region (2^kDartRegionBits
// slots, 64 MiB of owner), and the passes that touch owner and target sweep
// the keys in that order: at any time the GPU works on one or two regions,
// whose slices stay in L2.  The hits are bits of a bitmap (12.5 MB at
// 2^26, L2-resident); S(t), the hits before throw t, is a prefix count of it.
constexpr int kThrowsPerThread = 64;
constexpr int kDartRoundsMax = 4096;
constexpr int kDartRegionBits = 22;

__device__ __forceinline__ int64_t dart_lost(int64_t t, int64_t per_round, int64_t cap) {
  if (!per_round) return 0;
  const int64_t k = t / per_round;
  return k < cap ? k : cap;
}

// The slot of throw t, alone (one jump ahead).
__device__ __forceinline__ uint32_t dart_slot(uint64_t x0, int64_t t, int64_t per_round, int64_t cap, uint32_t m) {
  const uint64_t x = lcg_jump(x0, static_cast<uint64_t>(t + dart_lost(t, per_round, cap)));
  return static_cast<uint32_t>(lcg_step(x) >> 17) % m;
}

// keys[t - t_begin] = r_t << tb | t for throws [t_begin, t_end).  A warp
// takes kThrowsPerThread runs of 32 consecutive throws, lane l throw l of
// each run: one jump ahead, then the 32-step map (plus a single step per
// draw lost in between), so the key stores coalesce.
__global__ void __launch_bounds__(256)
    dart_keys_kernel(uint64_t x0, int64_t t_begin, int64_t t_end, int64_t per_round, int64_t cap, uint32_t m, int tb,
                     uint64_t *__restrict__ keys) {
  const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  int64_t t = t_begin + warp * (32 * kThrowsPerThread) + lane_id();
  if (t >= t_end) return;
  int64_t lost = dart_lost(t, per_round, cap);
  uint64_t x = lcg_jump(x0, static_cast<uint64_t>(t + lost));
  for (int r = 0; r < kThrowsPerThread && t < t_end; r++) {
    const uint64_t y = lcg_step(x);  // output idx(t)
    keys[t - t_begin] = (static_cast<uint64_t>(static_cast<uint32_t>(y >> 17) % m) << tb) | static_cast<uint64_t>(t);
    t += 32;
    const int64_t lost2 = dart_lost(t, per_round, cap);
    x = (kLcg32.a * x + kLcg32.c) & kLcgMask;
    for (int64_t e = lost; e < lost2; e++) x = lcg_step(x);
    lost = lost2;
  }
}

// The passes over the region-grouped keys: each block takes kDartKeysPerBlock
// consecutive keys and blocks start in order, so the GPU's working set moves
// through the regions one at a time; the keys themselves stream past L2
// (evict-first) instead of pushing the region's slices out.
constexpr int kDartKeysPerThread = 16;
constexpr int64_t kDartKeysPerBlock = 256 * kDartKeysPerThread;

__device__ __forceinline__ uint64_t dart_key(const uint64_t *__restrict__ keys, int64_t i, uint64_t pol) {
  return static_cast<uint64_t>(ld_s64_pol(reinterpret_cast<const int64_t *>(keys) + i, pol));
}

__global__ void __launch_bounds__(256)
    dart_claim_kernel(const uint64_t *__restrict__ keys, int64_t nkeys, int tb, uint32_t *__restrict__ owner) {
  const uint64_t tmask = (uint64_t(1) << tb) - 1, pol = policy_evict_first();
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kDartKeysPerBlock + threadIdx.x;
#pragma unroll 4
  for (int r = 0; r < kDartKeysPerThread; r++) {
    const int64_t i = base + r * 256;
    if (i >= nkeys) break;
    const uint64_t k = dart_key(keys, i, pol);
    atomicMin(&owner[k >> tb], static_cast<uint32_t>(k & tmask));
  }
}

__global__ void __launch_bounds__(256)
    dart_hitbits_kernel(const uint64_t *__restrict__ keys, int64_t nkeys, int tb, const uint32_t *__restrict__ owner,
                        uint32_t *__restrict__ bits) {
  const uint64_t tmask = (uint64_t(1) << tb) - 1, pol = policy_evict_first();
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kDartKeysPerBlock + threadIdx.x;
#pragma unroll 4
  for (int r = 0; r < kDartKeysPerThread; r++) {
    const int64_t i = base + r * 256;
    if (i >= nkeys) break;
    const uint64_t k = dart_key(keys, i, pol);
    const uint32_t t = static_cast<uint32_t>(k & tmask);
    if (owner[k >> tb] == t) atomicOr(&bits[t >> 5], 1u << (t & 31));
  }
}

__global__ void __launch_bounds__(256)
    dart_popc_kernel(const uint32_t *__restrict__ bits, int64_t nwords, uint32_t *__restrict__ pc) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t w = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; w < nwords; w += stride)
    pc[w] = __popc(bits[w]);
}

__device__ __forceinline__ bool dart_hit(const uint32_t *__restrict__ bits, int64_t t) {
  return (bits[t >> 5] >> (t & 31)) & 1u;
}

// S(t): the hits among throws [0, t).
__device__ __forceinline__ int64_t dart_S(const uint32_t *__restrict__ bits, const uint32_t *__restrict__ wpre,
                                          int64_t t) {
  return static_cast<int64_t>(wpre[t >> 5]) + __popc(bits[t >> 5] & ((1u << (t & 31)) - 1u));
}

// rand_permp_agi: dart i is thrown until it hits, so the hit of throw t
// carries dart S(t); only the first n hits are thrown.
__global__ void __launch_bounds__(256)
    dart_place_agi_kernel(const uint64_t *__restrict__ keys, int64_t nkeys, int tb, const uint32_t *__restrict__ bits,
                          const uint32_t *__restrict__ wpre, int64_t n, uint32_t *__restrict__ target) {
  const uint64_t tmask = (uint64_t(1) << tb) - 1, pol = policy_evict_first();
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kDartKeysPerBlock + threadIdx.x;
#pragma unroll 4
  for (int r = 0; r < kDartKeysPerThread; r++) {
    const int64_t i = base + r * 256;
    if (i >= nkeys) break;
    const uint64_t k = dart_key(keys, i, pol);
    const int64_t t = static_cast<int64_t>(k & tmask);
    if (!dart_hit(bits, t)) continue;
    const int64_t d = dart_S(bits, wpre, t);
    if (d < n) target[k >> tb] = static_cast<uint32_t>(d);
  }
}

// rand_permp_exstack throws rounds of per_round darts while more than
// per_round are pending; the first round k* that finds at most per_round
// pending starts at throw k* per_round: the first k with S(k per_round) >=
// n - per_round.  words[1] = k*, or ~0u when the throws so far fall short.
__global__ void dart_kstar_kernel(const uint32_t *__restrict__ bits, const uint32_t *__restrict__ wpre,
                                  int64_t nthrows, int64_t per_round, int64_t n, unsigned int *__restrict__ words) {
  if (threadIdx.x | blockIdx.x) return;
  const int64_t need = n - per_round;
  int64_t lo = 0, hi = nthrows / per_round;  // S(hi per_round) reaches need; find the first k that does
  if (dart_S(bits, wpre, hi * per_round) < need) {
    words[1] = ~0u;
    return;
  }
  while (lo < hi) {
    const int64_t mid = lo + (hi - lo) / 2;
    if (dart_S(bits, wpre, mid * per_round) >= need) hi = mid;
    else lo = mid + 1;
  }
  words[1] = static_cast<unsigned int>(lo);
}

// Throws from t0 on are drawn again for the rounds from k* on (no draw is
// lost there): forget their claims and hits.
__global__ void __launch_bounds__(256)
    dart_forget_kernel(uint32_t *__restrict__ owner, int64_t m, uint32_t t0, uint32_t *__restrict__ bits,
                       int64_t nwords) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  const int64_t w0 = t0 >> 5;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < m || i < nwords; i += stride) {
    if (i < m && owner[i] != ~0u && owner[i] >= t0) owner[i] = ~0u;
    if (i >= w0 && i < nwords) bits[i] &= i == w0 ? (1u << (t0 & 31)) - 1u : 0u;
  }
}

// The rounds from k* on throw every pending dart: round q starts at
// rstart[q] with as many throws as darts were pending.  words[2] = the end
// of the last round, words[3] = the round count, words[4] = 0 (done), 1
// (more throws needed) or 2 (more than kDartRoundsMax rounds).
__global__ void dart_rounds_kernel(const uint32_t *__restrict__ bits, const uint32_t *__restrict__ wpre,
                                   int64_t nthrows, int64_t t0, int64_t n, uint32_t *__restrict__ rstart,
                                   unsigned int *__restrict__ words) {
  if (threadIdx.x | blockIdx.x) return;
  int64_t start = t0, size = n - dart_S(bits, wpre, t0);
  int q = 0;
  while (size > 0) {
    if (start + size > nthrows) {
      words[4] = 1;
      return;
    }
    if (q >= kDartRoundsMax) {
      words[4] = 2;
      return;
    }
    rstart[q++] = static_cast<uint32_t>(start);
    const int64_t hits = dart_S(bits, wpre, start + size) - dart_S(bits, wpre, start);
    start += size;
    size -= hits;
  }
  rstart[q] = static_cast<uint32_t>(start);
  words[2] = static_cast<unsigned int>(start);
  words[3] = static_cast<unsigned int>(q);
  words[4] = 0;
}

// The darts of rand_permp_exstack.  A round pops its buffer in throw order
// and sends the missed darts back in that order; they are written backwards
// in front of the unthrown darts, so the missed dart of rank r (of ms) is
// thrown next at position ms - 1 - r of the following round, and the rest
// of that round throws new darts in order.  Rounds before k* are per_round
// throws from k per_round; with Rj(k) = k per_round - S(k per_round) darts
// sent back before round k, round k opens with Rj(k) - Rj(k-1) returned
// darts and continues with new darts from k per_round - Rj(k-1) on.  From
// k* on the rounds are rstart[0..nrounds].  Each thread that throws a new
// dart follows it to its hit and records it in the slot (found again from
// the generator).  words[5] counts chains that ran past the last round
// (none, for consistent inputs).
__global__ void __launch_bounds__(256)
    dart_chase_kernel(uint64_t x0, uint32_t m, const uint32_t *__restrict__ bits, const uint32_t *__restrict__ wpre,
                      int64_t per_round, int64_t kstar, const uint32_t *__restrict__ rstart, int nrounds,
                      uint32_t *__restrict__ target, unsigned int *__restrict__ words) {
  const int64_t t0 = kstar * per_round, tend = rstart[nrounds], t1 = rstart[1];
  auto sent_back = [&](int64_t k) -> int64_t {  // Rj(k)
    return k <= 0 ? 0 : k * per_round - dart_S(bits, wpre, k * per_round);
  };
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < tend; t += stride) {
    int64_t k, j;
    if (t < t0) {
      k = t / per_round;
      j = t - k * per_round;
    } else if (t < t1) {
      k = kstar;
      j = t - t0;
    } else {
      continue;  // the rounds after k* throw returned darts only
    }
    const int64_t before = sent_back(k - 1), back = sent_back(k) - before;
    if (j < back) continue;
    const uint32_t dart = static_cast<uint32_t>(k * per_round - before + j - back);
    int64_t cur = t;
    while (!dart_hit(bits, cur)) {
      int64_t s, s2;
      if (cur < t0) {
        s = cur / per_round * per_round;
        s2 = s + per_round;
      } else {
        int lo = 0, hi = nrounds - 1;  // the last round starting at or before cur
        while (lo < hi) {
          const int mid = (lo + hi + 1) / 2;
          if (rstart[mid] <= cur) lo = mid;
          else hi = mid - 1;
        }
        s = rstart[lo];
        s2 = rstart[lo + 1];
      }
      const int64_t ss = dart_S(bits, wpre, s), missed = (s2 - s) - (dart_S(bits, wpre, s2) - ss);
      const int64_t rank = (cur - dart_S(bits, wpre, cur)) - (s - ss);
      const int64_t nc = s2 + missed - 1 - rank;  // in [s2, s2 + missed) when consistent
      cur = nc < s2 ? tend : nc;
      if (cur >= tend) break;
    }
    if (cur >= tend) {
      atomicAdd(&words[5], 1u);
      continue;
    }
    target[dart_slot(x0, cur, per_round, kstar, m)] = dart;
  }
}

__global__ void __launch_bounds__(256)
    dart_taken_kernel(const uint32_t *__restrict__ target, int64_t m, uint32_t *__restrict__ taken) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t s = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; s < m; s += stride)
    taken[s] = target[s] != ~0u ? 1u : 0u;
}

// The permutation is the darts in slot order.
__global__ void __launch_bounds__(256)
    dart_perm_kernel(const uint32_t *__restrict__ target, const uint32_t *__restrict__ pos, int64_t m, int64_t n,
                     int64_t *__restrict__ perm) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t s = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; s < m; s += stride)
    if (target[s] != ~0u && pos[s] < n) perm[pos[s]] = target[s];
}

// ---------------------------------------------------------------- random permutations (host)
struct DartWs {
  uint64_t *ka, *kb;                        // keys, and the region pass's output
  uint32_t *owner, *target, *pos;           // per slot
  uint32_t *bits, *pc, *wpre;               // hit bits per throw, popcounts and their prefix per word
  uint32_t *hist, *hoff, *bsum, *rstart;    // radix pass, scans, rounds
  unsigned int *words;  // [0] scan total, [1] k*, [2] last throw, [3] rounds, [4] rounds status, [5] lost chains
};

size_t dart_ws(int64_t m, int64_t nkeys, int64_t nbits, DartWs *w, char *base) {
  const int64_t tiles = (nkeys + kTile - 1) / kTile;
  const int64_t nwords = (nbits >> 5) + 2;
  const int64_t scan_n = std::max(std::max(m, nwords), tiles * kDigits) + 1;
  const int64_t nb = (scan_n + kScanBlock - 1) / kScanBlock + 1;
  size_t o = 0;
  auto take = [&](size_t bytes) -> char * {
    const size_t at = o;
    o += up256(bytes);
    return base ? base + at : nullptr;
  };
  char *p;
  p = take(8 * nkeys); if (w) w->ka = reinterpret_cast<uint64_t *>(p);
  p = take(8 * nkeys); if (w) w->kb = reinterpret_cast<uint64_t *>(p);
  p = take(4 * m); if (w) w->owner = reinterpret_cast<uint32_t *>(p);
  p = take(4 * m); if (w) w->target = reinterpret_cast<uint32_t *>(p);
  p = take(4 * m); if (w) w->pos = reinterpret_cast<uint32_t *>(p);
  p = take(4 * nwords); if (w) w->bits = reinterpret_cast<uint32_t *>(p);
  p = take(4 * (nwords + 1)); if (w) w->pc = reinterpret_cast<uint32_t *>(p);
  p = take(4 * (nwords + 1)); if (w) w->wpre = reinterpret_cast<uint32_t *>(p);
  p = take(4 * tiles * kDigits); if (w) w->hist = reinterpret_cast<uint32_t *>(p);
  p = take(4 * tiles * kDigits); if (w) w->hoff = reinterpret_cast<uint32_t *>(p);
  p = take(4 * nb); if (w) w->bsum = reinterpret_cast<uint32_t *>(p);
  p = take(4 * (kDartRoundsMax + 1)); if (w) w->rstart = reinterpret_cast<uint32_t *>(p);
  p = take(64); if (w) w->words = reinterpret_cast<unsigned int *>(p);
  return o;
}

int read_words(const unsigned int *d_words, unsigned int *h, int count, cudaStream_t st) {
  BALE_CUDA_OK(cudaMemcpyAsync(h, d_words, 4 * count, cudaMemcpyDeviceToHost, st));
  BALE_CUDA_OK(cudaStreamSynchronize(st));
  return BALE_OK;
}

// Keys of throws [t_begin, t_end) grouped by slot region (stable); returns
// the buffer holding them (w.ka or w.kb).
uint64_t *dart_region_keys(uint64_t x0, int64_t t_begin, int64_t t_end, int64_t per_round, int64_t cap, int64_t m,
                           int tb, DartWs &w, cudaStream_t st, int *rc) {
  *rc = BALE_OK;
  const int64_t nk = t_end - t_begin;
  const int64_t warps = (nk + 32 * kThrowsPerThread - 1) / (32 * kThrowsPerThread);
  dart_keys_kernel<<<static_cast<unsigned>((warps + 7) / 8), 256, 0, st>>>(x0, t_begin, t_end, per_round, cap,
                                                                           static_cast<uint32_t>(m), tb, w.ka);
  if (m <= (int64_t(1) << kDartRegionBits) || nk <= 1) return w.ka;  // one region: its slices fit in L2 as they are
  Ws rw;
  rw.hist = w.hist;
  rw.hoff = w.hoff;
  rw.bsum = w.bsum;
  rw.words = w.words;
  *rc = radix_pass(w.ka, w.kb, nk, tb + kDartRegionBits, rw, st);  // the region is the 8 bits from there
  return *rc == BALE_OK ? w.kb : w.ka;
}

// The hit bits of the keys' throws set in w.bits, then S: wpre[w] = hits in
// words [0, w) (wpre[nwords] = all of them, also in words[0]).
int dart_claims(const uint64_t *keys, int64_t nk, int tb, int64_t nwords, DartWs &w, cudaStream_t st) {
  const unsigned blocks = static_cast<unsigned>((nk + kDartKeysPerBlock - 1) / kDartKeysPerBlock);
  dart_claim_kernel<<<blocks, 256, 0, st>>>(keys, nk, tb, w.owner);
  dart_hitbits_kernel<<<blocks, 256, 0, st>>>(keys, nk, tb, w.owner, w.bits);
  dart_popc_kernel<<<grid_for(nwords), 256, 0, st>>>(w.bits, nwords, w.pc);
  BALE_CUDA_OK(cudaMemsetAsync(w.pc + nwords, 0, 4, st));
  return excl_scan(w.pc, w.wpre, nwords + 1, w.bsum, w.words, st);
}

// rand_permp_agi (per_round = 0) or rand_permp_exstack with buffers of
// per_round darts (1 <= per_round <= n), for 1 <= n < 2^30.  The throws
// needed are not known in advance: about 1.39 n hit n distinct slots of 2n.
// Take 1.5 n + 1024 (and for the exstack rounds from k* on, which throw at
// most per_round pending darts, 2 per_round + 1024) and double while short.
int rand_perm_darts(int64_t n, uint64_t seed, int64_t per_round, int64_t *d_perm, cudaStream_t st,
                    const char *who) {
  const int64_t m = 2 * n;
  const uint64_t x0 = ((seed & 0xffffffffull) << 16) | 0x330eull;
  for (int grow = 0; grow < 6; grow++) {
    int64_t nt = (n + n / 2 + 1024) << grow, tail = 0;
    if (per_round) {
      nt = (nt + per_round - 1) / per_round * per_round;
      tail = (2 * per_round + 1024) << grow;
    }
    const int64_t cap = nt + tail;  // throws numbered below cap
    if (cap >= int64_t(0xffffffff)) break;
    int tb = 1;
    while ((int64_t(1) << tb) < cap + 1) tb++;
    const int64_t nwords = (cap >> 5) + 2;
    DartWs w;
    void *ws = device_workspace(dart_ws(m, std::max(nt, tail), cap, nullptr, nullptr), st);
    if (!ws) return BALE_ENOMEM;
    dart_ws(m, std::max(nt, tail), cap, &w, static_cast<char *>(ws));
    BALE_CUDA_OK(cudaMemsetAsync(w.owner, 0xff, 4 * m, st));
    BALE_CUDA_OK(cudaMemsetAsync(w.target, 0xff, 4 * m, st));
    BALE_CUDA_OK(cudaMemsetAsync(w.bits, 0, 4 * nwords, st));
    BALE_CUDA_OK(cudaMemsetAsync(w.words, 0, 64, st));
    int rc = BALE_OK;
    const uint64_t *keys = dart_region_keys(x0, 0, nt, per_round, INT64_MAX, m, tb, w, st, &rc);
    if (rc != BALE_OK || (rc = dart_claims(keys, nt, tb, nwords, w, st)) != BALE_OK) return rc;
    unsigned int h[6] = {0, 0, 0, 0, 0, 0};
    if (!per_round) {
      if ((rc = read_words(w.words, h, 1, st)) != BALE_OK) return rc;
      if (static_cast<int64_t>(h[0]) < n) continue;
      dart_place_agi_kernel<<<static_cast<unsigned>((nt + kDartKeysPerBlock - 1) / kDartKeysPerBlock), 256, 0, st>>>(
          keys, nt, tb, w.bits, w.wpre, n, w.target);
    } else {
      dart_kstar_kernel<<<1, 32, 0, st>>>(w.bits, w.wpre, nt, per_round, n, w.words);
      if ((rc = read_words(w.words, h, 2, st)) != BALE_OK) return rc;
      if (h[1] == ~0u) continue;
      const int64_t kstar = h[1], t0 = kstar * per_round, t2 = t0 + tail;
      dart_forget_kernel<<<grid_for(std::max(m, nwords)), 256, 0, st>>>(w.owner, m, static_cast<uint32_t>(t0), w.bits,
                                                                         nwords);
      const uint64_t *tk = dart_region_keys(x0, t0, t2, per_round, kstar, m, tb, w, st, &rc);
      if (rc != BALE_OK || (rc = dart_claims(tk, tail, tb, nwords, w, st)) != BALE_OK) return rc;
      dart_rounds_kernel<<<1, 32, 0, st>>>(w.bits, w.wpre, t2, t0, n, w.rstart, w.words);
      if ((rc = read_words(w.words, h, 5, st)) != BALE_OK) return rc;
      if (h[4] == 1) continue;
      if (h[4] != 0) {
        set_error("%s: more than %d rounds of returned darts", who, kDartRoundsMax);
        return BALE_EINVAL;
      }
      dart_chase_kernel<<<grid_for(h[2]), 256, 0, st>>>(x0, static_cast<uint32_t>(m), w.bits, w.wpre, per_round,
                                                        kstar, w.rstart, static_cast<int>(h[3]), w.target, w.words);
    }
    dart_taken_kernel<<<grid_for(m), 256, 0, st>>>(w.target, m, w.owner);
    if ((rc = excl_scan(w.owner, w.pos, m, w.bsum, w.words, st)) != BALE_OK) return rc;
    dart_perm_kernel<<<grid_for(m), 256, 0, st>>>(w.target, w.pos, m, n, d_perm);
    BALE_CUDA_OK(cudaGetLastError());
    if ((rc = read_words(w.words, h, 6, st)) != BALE_OK) return rc;
    if (static_cast<int64_t>(h[0]) != n || h[5] != 0) {
      set_error("%s: %u darts placed of %lld (%u lost)", who, h[0], static_cast<long long>(n), h[5]);
      return BALE_EINVAL;
    }
    return BALE_OK;
  }
  set_error("%s: too many throws for n = %lld", who, static_cast<long long>(n));
  return BALE_EINVAL;
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

// ---------------------------------------------------------------- binary datasets
// cnt[i] = offset[i+1] - offset[i] of a checked CSR.
__global__ void __launch_bounds__(256)
    ds_lengths_kernel(const int64_t *__restrict__ off, int64_t n, int64_t *__restrict__ cnt) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    cnt[i] = off[i + 1] - off[i];
}

// out[j] = v[idx[j]] for j < k (the offsets at the writers' first rows).
__global__ void ds_gather_kernel(const int64_t *__restrict__ v, const int64_t *__restrict__ idx, int64_t k,
                                 int64_t *__restrict__ out) {
  for (int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; j < k;
       j += static_cast<int64_t>(gridDim.x) * blockDim.x)
    out[j] = v[idx[j]];
}

// Row lengths read from the files (in off[0..n)) become 32-bit lengths;
// bad counts lengths outside [0, nnz], *sum adds them all (64-bit, so a
// sum past 2^32 is seen).
__global__ void __launch_bounds__(256)
    ds_counts_kernel(const int64_t *__restrict__ cnt, int64_t n, int64_t nnz, uint32_t *__restrict__ len,
                     unsigned long long *__restrict__ sum, unsigned long long *__restrict__ bad) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  unsigned long long s = 0, nb = 0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int64_t c = cnt[i];
    const bool ok = c >= 0 && c <= nnz;
    nb += ok ? 0 : 1;
    s += ok ? static_cast<unsigned long long>(c) : 0;
    len[i] = ok ? static_cast<uint32_t>(c) : 0u;
  }
  s = warp_sum_u64(s);
  nb = warp_sum_u64(nb);
  if (lane_id() == 0) {
    if (s) atomicAdd(sum, s);
    if (nb) atomicAdd(bad, nb);
  }
}

__global__ void __launch_bounds__(256)
    ds_offsets_kernel(const uint32_t *__restrict__ pos, int64_t n, int64_t total, int64_t *__restrict__ off) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i <= n; i += stride)
    off[i] = i < n ? static_cast<int64_t>(pos[i]) : total;
}

// File transfers go through two pinned chunks kept for the process: the
// copy of one chunk overlaps the fwrite (or fread) of the other.  One
// transfer at a time holds them.
constexpr size_t kIoChunk = size_t(8) << 20;

struct IoStaging {
  std::mutex mu;
  char *buf[2] = {nullptr, nullptr};
};

IoStaging &io_staging() {
  static IoStaging s;
  return s;
}

// With the staging lock held: the two chunks, allocated on first use.
int io_buffers(IoStaging &io) {
  for (char *&b : io.buf)
    if (!b && cudaHostAlloc(reinterpret_cast<void **>(&b), kIoChunk, cudaHostAllocPortable) != cudaSuccess) {
      b = nullptr;
      cudaGetLastError();
      return BALE_ENOMEM;
    }
  return BALE_OK;
}

struct IoEvents {
  cudaEvent_t ev[2] = {nullptr, nullptr};
  ~IoEvents() {
    for (cudaEvent_t e : ev)
      if (e) {
        cudaEventSynchronize(e);
        cudaEventDestroy(e);
      }
  }
  int make() {
    for (cudaEvent_t &e : ev)
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
        e = nullptr;
        return BALE_ECUDA;
      }
    return BALE_OK;
  }
};

// bytes of device memory at src appended to fp.
int dev_to_file(IoStaging &io, FILE *fp, const char *src, size_t bytes, cudaStream_t st) {
  IoEvents e;
  if (e.make() != BALE_OK) return BALE_ECUDA;
  const size_t chunks = (bytes + kIoChunk - 1) / kIoChunk;
  auto len = [&](size_t k) { return std::min(kIoChunk, bytes - k * kIoChunk); };
  for (size_t k = 0; k < chunks && k < 2; k++) {
    BALE_CUDA_OK(cudaMemcpyAsync(io.buf[k], src + k * kIoChunk, len(k), cudaMemcpyDeviceToHost, st));
    BALE_CUDA_OK(cudaEventRecord(e.ev[k], st));
  }
  for (size_t k = 0; k < chunks; k++) {
    const int b = static_cast<int>(k & 1);
    BALE_CUDA_OK(cudaEventSynchronize(e.ev[b]));
    if (fwrite(io.buf[b], 1, len(k), fp) != len(k)) return BALE_EINPUT;
    if (k + 2 < chunks) {
      BALE_CUDA_OK(cudaMemcpyAsync(io.buf[b], src + (k + 2) * kIoChunk, len(k + 2), cudaMemcpyDeviceToHost, st));
      BALE_CUDA_OK(cudaEventRecord(e.ev[b], st));
    }
  }
  return BALE_OK;
}

// bytes read from fp into device memory at dst.  Returns with the copies
// finished (the events are waited for on every path).
int file_to_dev(IoStaging &io, FILE *fp, char *dst, size_t bytes, cudaStream_t st) {
  IoEvents e;
  if (e.make() != BALE_OK) return BALE_ECUDA;
  bool used[2] = {false, false};
  for (size_t k = 0, at = 0; at < bytes; k++, at += kIoChunk) {
    const int b = static_cast<int>(k & 1);
    const size_t n = std::min(kIoChunk, bytes - at);
    if (used[b]) BALE_CUDA_OK(cudaEventSynchronize(e.ev[b]));
    if (fread(io.buf[b], 1, n, fp) != n) return BALE_EINPUT;
    BALE_CUDA_OK(cudaMemcpyAsync(dst + at, io.buf[b], n, cudaMemcpyHostToDevice, st));
    BALE_CUDA_OK(cudaEventRecord(e.ev[b], st));
    used[b] = true;
  }
  return BALE_OK;
}

// The first row of each of the W writers' blocks, and numrows at the end.
std::vector<int64_t> writer_rows(int64_t numrows, int64_t writers) {
  std::vector<int64_t> first(static_cast<size_t>(writers) + 1, 0);
  for (int64_t w = 0; w < writers; w++) first[w + 1] = first[w] + (numrows + writers - w - 1) / writers;
  return first;
}

// Closes a FILE on every return path.
struct FileGuard {
  FILE *f;
  ~FileGuard() {
    if (f) fclose(f);
  }
};

int64_t file_bytes(const char *path) {
  struct stat sb;
  if (stat(path, &sb) != 0 || !S_ISREG(sb.st_mode)) return -1;
  return static_cast<int64_t>(sb.st_size);
}

constexpr int64_t kMaxWriters = int64_t(1) << 16;

}  // namespace
}  // namespace bale

using namespace bale;

extern "C" {

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
    transpose_keys_kernel<<<grid_for(numrows * 32), 256, 0, st>>>(d_offset, d_nonzero, numrows, rb, w.ka);
    BALE_CUDA_OK(cudaGetLastError());
  }
  uint64_t *sk = radix_sort(w.ka, w.kb, nnz, rb + cb, w, st, &rc);
  if (rc != BALE_OK) return rc;
  rc = csr_from_keys(sk, nnz, numcols, rb, d_toffset, d_tnonzero, st);
  if (rc != BALE_OK) return rc;
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
  return rand_perm_darts(n, seed, 0, d_perm, static_cast<cudaStream_t>(stream), "bale_rand_perm_dev");
}

int bale_rand_perm_exstack_dev(int64_t n, uint64_t seed, int64_t buf_cnt, int64_t *d_perm, void *stream) {
  if (n < 0 || n >= (int64_t(1) << 30) || buf_cnt < 1 || (n > 0 && !d_perm)) {
    set_error("bale_rand_perm_exstack_dev: bad arguments (n=%lld, buf_cnt=%lld)", static_cast<long long>(n),
              static_cast<long long>(buf_cnt));
    return BALE_EINVAL;
  }
  if (n == 0) return BALE_OK;
  // a buffer that holds every dart never fills: the same as one of n
  return rand_perm_darts(n, seed, std::min(buf_cnt, n), d_perm, static_cast<cudaStream_t>(stream),
                         "bale_rand_perm_exstack_dev");
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
  FileGuard guard{fp};
  const int64_t len = static_cast<int64_t>(ftell(fp)) - body;
  if (len < 0 || len >= (int64_t(1) << 32) - 1) {
    set_error("bale_read_matrix_mm_dev: %s: body of %lld bytes is outside the supported range", path,
              static_cast<long long>(len));
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
  if (len > 0) {  // the body, through the pinned chunks (reads overlap the copies)
    IoStaging &io = io_staging();
    std::lock_guard<std::mutex> lock(io.mu);
    if (io_buffers(io) != BALE_OK) return BALE_ENOMEM;
    rc = fseek(fp, static_cast<long>(body), SEEK_SET) == 0 ? file_to_dev(io, fp, d_text, static_cast<size_t>(len), st)
                                                           : BALE_EINPUT;
  }
  if (rc != BALE_OK) {
    set_error("bale_read_matrix_mm_dev: short read of %s", path);
    return rc;
  }
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
  if ((rc = csr_from_keys(sk, nnz, nr, lb, d_offset, nullptr, st)) != BALE_OK) return rc;
  if (nnz > 0) mm_cols_kernel<<<grid_for(nnz), 256, 0, st>>>(sk, nnz, lb, cols, d_nonzero);
  BALE_CUDA_OK(cudaGetLastError());
  BALE_CUDA_OK(cudaStreamSynchronize(st));
  return BALE_OK;
}

int bale_write_sparse_matrix_dev(const char *dirname, const int64_t *d_offset, const int64_t *d_nonzero,
                                 int64_t numrows, int64_t numcols, int64_t nnz, int64_t nwriters, void *stream) {
  if (!dirname || !d_offset || (nnz > 0 && !d_nonzero) || numrows < 0 || numcols < 0 || nnz < 0 || nwriters < 1 ||
      nwriters > kMaxWriters) {
    set_error("bale_write_sparse_matrix_dev: bad arguments");
    return BALE_EINVAL;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const std::vector<int64_t> first = writer_rows(numrows, nwriters);
  const size_t nw = static_cast<size_t>(nwriters) + 1;
  const size_t need = up256(8 * std::max<int64_t>(numrows, 1)) + 2 * up256(8 * nw) + 256;
  char *ws = static_cast<char *>(device_workspace(need, st));
  if (!ws) return BALE_ENOMEM;
  int64_t *cnt = reinterpret_cast<int64_t *>(ws);
  int64_t *d_first = reinterpret_cast<int64_t *>(ws + up256(8 * std::max<int64_t>(numrows, 1)));
  int64_t *d_bound = d_first + up256(8 * nw) / 8;
  unsigned long long *bad = reinterpret_cast<unsigned long long *>(d_bound + up256(8 * nw) / 8);
  BALE_CUDA_OK(cudaMemsetAsync(bad, 0, 8, st));
  csr_check_kernel<<<grid_for(std::max(numrows + 1, nnz)), 256, 0, st>>>(d_offset, d_nonzero, numrows, numcols,
                                                                          nnz, bad);
  if (numrows > 0) ds_lengths_kernel<<<grid_for(numrows), 256, 0, st>>>(d_offset, numrows, cnt);
  BALE_CUDA_OK(cudaMemcpyAsync(d_first, first.data(), 8 * nw, cudaMemcpyHostToDevice, st));
  ds_gather_kernel<<<1, 256, 0, st>>>(d_offset, d_first, static_cast<int64_t>(nw), d_bound);
  BALE_CUDA_OK(cudaGetLastError());
  std::vector<int64_t> bound(nw);
  unsigned long long nbad = 0;
  BALE_CUDA_OK(cudaMemcpyAsync(bound.data(), d_bound, 8 * nw, cudaMemcpyDeviceToHost, st));
  BALE_CUDA_OK(cudaMemcpyAsync(&nbad, bad, 8, cudaMemcpyDeviceToHost, st));
  BALE_CUDA_OK(cudaStreamSynchronize(st));
  if (nbad) {
    set_error("bale_write_sparse_matrix_dev: %llu malformed offsets or columns", nbad);
    return BALE_EINPUT;
  }
  IoStaging &io = io_staging();
  std::lock_guard<std::mutex> lock(io.mu);
  if (io_buffers(io) != BALE_OK) return BALE_ENOMEM;
  mkdir(dirname, 0770);  // may exist already, as in the reference
  std::vector<char> name(strlen(dirname) + 32);
  snprintf(name.data(), name.size(), "%s/metadata", dirname);
  FILE *fp = fopen(name.data(), "w");
  bool ok = fp && fprintf(fp, "%lld\n%lld\n%lld\n%lld\n", static_cast<long long>(numrows),
                          static_cast<long long>(numcols), static_cast<long long>(nnz),
                          static_cast<long long>(nwriters)) > 0;
  if (fp && fclose(fp) != 0) ok = false;
  int rc = ok ? BALE_OK : BALE_EINPUT;
  for (int64_t w = 0; rc == BALE_OK && w < nwriters; w++) {
    for (int part = 0; rc == BALE_OK && part < 2; part++) {
      snprintf(name.data(), name.size(), part ? "%s/nonzero_%lld" : "%s/rowcnt_%lld", dirname,
               static_cast<long long>(w));
      fp = fopen(name.data(), "wb");
      if (!fp) {
        rc = BALE_EINPUT;
        break;
      }
      const char *src = part ? reinterpret_cast<const char *>(d_nonzero + bound[w])
                             : reinterpret_cast<const char *>(cnt + first[w]);
      const size_t bytes = 8 * static_cast<size_t>(part ? bound[w + 1] - bound[w] : first[w + 1] - first[w]);
      rc = bytes ? dev_to_file(io, fp, src, bytes, st) : BALE_OK;
      if (fclose(fp) != 0 && rc == BALE_OK) rc = BALE_EINPUT;
    }
  }
  if (rc != BALE_OK) set_error("bale_write_sparse_matrix_dev: cannot write the dataset %s", dirname);
  return rc;
}

int bale_read_sparse_matrix_dev(const char *dirname, int64_t *d_offset, int64_t *d_nonzero, void *stream) {
  int64_t nr = 0, nc = 0, nnz = 0, writers = 0;
  int rc = bale_sparse_matrix_header(dirname, &nr, &nc, &nnz, &writers);
  if (rc != BALE_OK) {
    set_error("bale_read_sparse_matrix_dev: %s: no readable metadata file", dirname ? dirname : "");
    return rc;
  }
  if (!d_offset || (nnz > 0 && !d_nonzero) || nr >= (int64_t(1) << 31) || nnz >= (int64_t(1) << 32) - 1 ||
      writers > kMaxWriters) {
    set_error("bale_read_sparse_matrix_dev: bad arguments or sizes");
    return BALE_EINVAL;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const std::vector<int64_t> first = writer_rows(nr, writers);
  const size_t nw = static_cast<size_t>(writers) + 1;
  // each writer's files: rowcnt_<w> holds its rows' lengths, nonzero_<w>
  // whole int64 columns; the columns of all writers add up to nnz
  std::vector<int64_t> nzstart(nw, 0);
  std::vector<char> name(strlen(dirname) + 32);
  for (int64_t w = 0; w < writers; w++) {
    snprintf(name.data(), name.size(), "%s/rowcnt_%lld", dirname, static_cast<long long>(w));
    const int64_t rb = file_bytes(name.data());
    snprintf(name.data(), name.size(), "%s/nonzero_%lld", dirname, static_cast<long long>(w));
    const int64_t nb = file_bytes(name.data());
    if (rb != 8 * (first[w + 1] - first[w]) || nb < 0 || nb % 8 || nzstart[w] + nb / 8 > nnz) {
      set_error("bale_read_sparse_matrix_dev: %s: files of writer %lld do not match the metadata", dirname,
                static_cast<long long>(w));
      return BALE_EINPUT;
    }
    nzstart[w + 1] = nzstart[w] + nb / 8;
  }
  if (nzstart[writers] != nnz) {
    set_error("bale_read_sparse_matrix_dev: %s: %lld nonzeros in the files, %lld in the metadata", dirname,
              static_cast<long long>(nzstart[writers]), static_cast<long long>(nnz));
    return BALE_EINPUT;
  }
  const int64_t n1 = nr + 1;
  const int64_t nb = (n1 + kScanBlock - 1) / kScanBlock + 1;
  const size_t need = 2 * up256(4 * n1) + up256(4 * nb) + 2 * up256(8 * nw) + 256;
  char *ws = static_cast<char *>(device_workspace(need, st));
  if (!ws) return BALE_ENOMEM;
  char *o = ws;
  auto take = [&](size_t bytes) {
    char *r = o;
    o += up256(bytes);
    return r;
  };
  uint32_t *len = reinterpret_cast<uint32_t *>(take(4 * n1));
  uint32_t *pos = reinterpret_cast<uint32_t *>(take(4 * n1));
  uint32_t *bsum = reinterpret_cast<uint32_t *>(take(4 * nb));
  int64_t *d_first = reinterpret_cast<int64_t *>(take(8 * nw));
  int64_t *d_bound = reinterpret_cast<int64_t *>(take(8 * nw));
  unsigned int *words = reinterpret_cast<unsigned int *>(take(64));
  unsigned long long *sum = reinterpret_cast<unsigned long long *>(words + 4), *bad = sum + 1, *bad_csr = sum + 2;
  BALE_CUDA_OK(cudaMemsetAsync(words, 0, 64, st));
  {
    IoStaging &io = io_staging();
    std::lock_guard<std::mutex> lock(io.mu);
    if (io_buffers(io) != BALE_OK) return BALE_ENOMEM;
    for (int64_t w = 0; w < writers; w++) {
      for (int part = 0; part < 2; part++) {
        snprintf(name.data(), name.size(), part ? "%s/nonzero_%lld" : "%s/rowcnt_%lld", dirname,
                 static_cast<long long>(w));
        const size_t bytes = 8 * static_cast<size_t>(part ? nzstart[w + 1] - nzstart[w] : first[w + 1] - first[w]);
        if (!bytes) continue;
        char *dst = part ? reinterpret_cast<char *>(d_nonzero + nzstart[w]) : reinterpret_cast<char *>(d_offset + first[w]);
        FILE *fp = fopen(name.data(), "rb");
        rc = fp ? file_to_dev(io, fp, dst, bytes, st) : BALE_EINPUT;
        if (fp) fclose(fp);
        if (rc != BALE_OK) {
          set_error("bale_read_sparse_matrix_dev: cannot read %s", name.data());
          return rc;
        }
      }
    }
  }
  if (nr > 0) {
    ds_counts_kernel<<<grid_for(nr), 256, 0, st>>>(d_offset, nr, nnz, len, sum, bad);
    if ((rc = excl_scan(len, pos, nr, bsum, words, st)) != BALE_OK) return rc;
  }
  ds_offsets_kernel<<<grid_for(n1), 256, 0, st>>>(pos, nr, nnz, d_offset);
  csr_check_kernel<<<grid_for(std::max(n1, nnz)), 256, 0, st>>>(d_offset, d_nonzero, nr, nc, nnz, bad_csr);
  BALE_CUDA_OK(cudaMemcpyAsync(d_first, first.data(), 8 * nw, cudaMemcpyHostToDevice, st));
  ds_gather_kernel<<<1, 256, 0, st>>>(d_offset, d_first, static_cast<int64_t>(nw), d_bound);
  BALE_CUDA_OK(cudaGetLastError());
  std::vector<int64_t> bound(nw);
  unsigned long long h[3] = {0, 0, 0};
  BALE_CUDA_OK(cudaMemcpyAsync(bound.data(), d_bound, 8 * nw, cudaMemcpyDeviceToHost, st));
  BALE_CUDA_OK(cudaMemcpyAsync(h, sum, 24, cudaMemcpyDeviceToHost, st));
  BALE_CUDA_OK(cudaStreamSynchronize(st));
  if (h[1] || h[0] != static_cast<unsigned long long>(nnz) || h[2] || bound != nzstart) {
    set_error("bale_read_sparse_matrix_dev: %s: row lengths, columns or writer blocks are inconsistent "
              "(%llu bad lengths, lengths sum to %llu of %lld, %llu bad offsets or columns)",
              dirname, h[1], h[0], static_cast<long long>(nnz), h[2]);
    return BALE_EINPUT;
  }
  return BALE_OK;
}

}  // extern "C"
