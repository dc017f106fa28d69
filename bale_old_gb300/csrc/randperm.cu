// randperm.cu -- spmat's random permutations at one PE on the device, each
// bit-identical to the reference: rand_permp_agi (spmat/spmat_agi.upc:
// 56-107) and rand_permp_exstack (spmat/spmat_exstack.upc:62-190; rand_permp,
// spmat/spmat_utils.upc:63-74, is the latter with buffers of 1024).  Dart
// throwing decided in parallel, the throws grouped by slot region so that
// their claims stay in L2.
#include <algorithm>
#include <climits>
#include <cstdlib>

#include "sort.cuh"

namespace bale {
namespace {

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

// rand_permp_agi stops drawing at the throw that places its n-th dart:
// words[6] = the smallest t with S(t + 1) >= n (the caller has checked that
// the throws so far hold n hits).
__global__ void dart_nth_hit_kernel(const uint32_t *__restrict__ bits, const uint32_t *__restrict__ wpre,
                                    int64_t nthrows, int64_t n, unsigned int *__restrict__ words) {
  if (threadIdx.x | blockIdx.x) return;
  int64_t lo = 0, hi = nthrows - 1;
  while (lo < hi) {
    const int64_t mid = lo + (hi - lo) / 2;
    if (dart_S(bits, wpre, mid + 1) >= n) hi = mid;
    else lo = mid + 1;
  }
  words[6] = static_cast<unsigned int>(lo);
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
  uint32_t *osw;                            // radix pass: digit starts and tile counter
  unsigned int *words;  // [0] scan total, [1] k*, [2] last throw, [3] rounds, [4] rounds status, [5] lost chains,
                        // [6] the throw of rand_permp_agi's n-th hit, [kSortErrWord] a radix wait gave up
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
  p = take(4 * kOsWords); if (w) w->osw = reinterpret_cast<uint32_t *>(p);
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
  rw.osw = w.osw;
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
//
// x0 is the generator's state before the first draw; *draws receives the
// number of lrand48 draws the reference makes (rand_permp_agi: up to the
// throw of the n-th hit; rand_permp_exstack: up to the end of the last
// round, plus the draw lost by each of the k* rounds that found the buffer
// full).
int rand_perm_darts(int64_t n, uint64_t x0, int64_t per_round, int64_t *d_perm, cudaStream_t st, const char *who,
                    int64_t *draws) {
  const int64_t m = 2 * n;
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
    unsigned int h[7] = {0, 0, 0, 0, 0, 0, 0};
    int64_t kstar_used = 0;
    if (!per_round) {
      if ((rc = read_words(w.words, h, 1, st)) != BALE_OK) return rc;
      if (static_cast<int64_t>(h[0]) < n) continue;
      dart_place_agi_kernel<<<static_cast<unsigned>((nt + kDartKeysPerBlock - 1) / kDartKeysPerBlock), 256, 0, st>>>(
          keys, nt, tb, w.bits, w.wpre, n, w.target);
      dart_nth_hit_kernel<<<1, 32, 0, st>>>(w.bits, w.wpre, nt, n, w.words);
    } else {
      dart_kstar_kernel<<<1, 32, 0, st>>>(w.bits, w.wpre, nt, per_round, n, w.words);
      if ((rc = read_words(w.words, h, 2, st)) != BALE_OK) return rc;
      if (h[1] == ~0u) continue;
      const int64_t kstar = h[1], t0 = kstar * per_round, t2 = t0 + tail;
      kstar_used = kstar;
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
    if ((rc = read_words(w.words, h, 7, st)) != BALE_OK || (rc = sort_status(w.words, st, who)) != BALE_OK)
      return rc;
    if (static_cast<int64_t>(h[0]) != n || h[5] != 0) {
      set_error("%s: %u darts placed of %lld (%u lost)", who, h[0], static_cast<long long>(n), h[5]);
      return BALE_EINVAL;
    }
    *draws = per_round ? static_cast<int64_t>(h[2]) + kstar_used : static_cast<int64_t>(h[6]) + 1;
    return BALE_OK;
  }
  set_error("%s: too many throws for n = %lld", who, static_cast<long long>(n));
  return BALE_EINVAL;
}

// The reference reseeds only when its int seed is nonzero (spmat_agi.upc:61,
// spmat_exstack.upc:92: `if (seed != 0) srand48(seed)`); with 0 it continues
// the C library's drand48 stream from wherever the caller left it, and with
// any seed it leaves that stream just past its last draw, where a later
// lrand48() or seed-0 call picks it up.  The entry points do the same with
// the process's C library state: seed48 installs a state and returns the
// previous one, so reading it is two calls.  (Like the reference, this is
// not safe against other threads drawing from the same stream meanwhile.)
uint64_t libc_drand48_state() {
  unsigned short probe[3] = {0, 0, 0};
  const unsigned short *prev = seed48(probe);
  unsigned short keep[3] = {prev[0], prev[1], prev[2]};
  seed48(keep);
  return static_cast<uint64_t>(keep[0]) | static_cast<uint64_t>(keep[1]) << 16 | static_cast<uint64_t>(keep[2]) << 32;
}

void set_libc_drand48_state(uint64_t x) {
  unsigned short s[3] = {static_cast<unsigned short>(x & 0xffff), static_cast<unsigned short>(x >> 16 & 0xffff),
                         static_cast<unsigned short>(x >> 32 & 0xffff)};
  seed48(s);
}

uint64_t host_lcg_jump(uint64_t x, uint64_t k) {
  uint64_t a = kLcgA, c = kLcgC, ra = 1, rc = 0;
  while (k) {
    if (k & 1) {
      ra = (ra * a) & kLcgMask;
      rc = (rc * a + c) & kLcgMask;
    }
    c = (c * a + c) & kLcgMask;
    a = (a * a) & kLcgMask;
    k >>= 1;
  }
  return (ra * x + rc) & kLcgMask;
}

// The generator's state before the first draw: srand48(seed) for a seed
// whose low 32 bits (the reference's int) are nonzero, else the C library's.
uint64_t start_state(uint64_t seed) {
  if ((seed & 0xffffffffull) == 0) return libc_drand48_state();
  const uint64_t x0 = ((seed & 0xffffffffull) << 16) | 0x330eull;
  set_libc_drand48_state(x0);  // srand48(seed), as the reference does before it draws
  return x0;
}

// The darts, then the C library's stream left past the reference's last draw.
int rand_perm_entry(int64_t n, uint64_t seed, int64_t per_round, int64_t *d_perm, cudaStream_t st, const char *who) {
  const uint64_t x0 = start_state(seed);
  if (n == 0) return BALE_OK;  // the reference draws nothing either
  int64_t draws = 0;
  const int rc = rand_perm_darts(n, x0, per_round, d_perm, st, who, &draws);
  if (rc == BALE_OK) set_libc_drand48_state(host_lcg_jump(x0, static_cast<uint64_t>(draws)));
  return rc;
}

}  // namespace
}  // namespace bale

using namespace bale;

extern "C" {

int bale_rand_perm_dev(int64_t n, uint64_t seed, int64_t *d_perm, void *stream) {
  if (n < 0 || n >= (int64_t(1) << 30) || (n > 0 && !d_perm)) {
    set_error("bale_rand_perm_dev: bad arguments (n=%lld)", static_cast<long long>(n));
    return BALE_EINVAL;
  }
  return rand_perm_entry(n, seed, 0, d_perm, static_cast<cudaStream_t>(stream), "bale_rand_perm_dev");
}

int bale_rand_perm_exstack_dev(int64_t n, uint64_t seed, int64_t buf_cnt, int64_t *d_perm, void *stream) {
  if (n < 0 || n >= (int64_t(1) << 30) || buf_cnt < 1 || (n > 0 && !d_perm)) {
    set_error("bale_rand_perm_exstack_dev: bad arguments (n=%lld, buf_cnt=%lld)", static_cast<long long>(n),
              static_cast<long long>(buf_cnt));
    return BALE_EINVAL;
  }
  // a buffer that holds every dart never fills: the same as one of n
  return rand_perm_entry(n, seed, std::min(buf_cnt, std::max<int64_t>(n, 1)), d_perm,
                         static_cast<cudaStream_t>(stream), "bale_rand_perm_exstack_dev");
}

// The reference's rand_permp_exstack2 returns rand_permp_exstack(N, seed,
// buf_cnt) (spmat/spmat_exstack2.upc:60-73; its own exstack2 form is
// compiled out), so this is that permutation too.
int bale_rand_perm_exstack2_dev(int64_t n, uint64_t seed, int64_t buf_cnt, int64_t *d_perm, void *stream) {
  if (n < 0 || n >= (int64_t(1) << 30) || buf_cnt < 1 || (n > 0 && !d_perm)) {
    set_error("bale_rand_perm_exstack2_dev: bad arguments (n=%lld, buf_cnt=%lld)", static_cast<long long>(n),
              static_cast<long long>(buf_cnt));
    return BALE_EINVAL;
  }
  return rand_perm_entry(n, seed, std::min(buf_cnt, std::max<int64_t>(n, 1)), d_perm,
                         static_cast<cudaStream_t>(stream), "bale_rand_perm_exstack2_dev");
}

}  // extern "C"
