// graph.cu -- building the triangle kernels' input on the device: the
// degree-ordered, strictly lower-triangular CSR of an undirected graph.
//
// From an edge list (or R-MAT edges generated in place, bit-identical to
// bale_gen_rmat in host/inputs.c):
//   1. keys: each edge {u,v}, u != v, becomes min << S | max (S = label
//      bits); self loops become an all-ones key that sorts last;
//   2. sort the keys (LSD radix sort), drop the duplicates and the
//      self loops;
//   3. degrees; labels by descending degree, ties by ascending original
//      label: a second sort of (maxdeg - deg) << S | v;
//   4. each edge relabelled to row = max, col = min of the new labels, a
//      third sort, and the CSR read off the sorted keys: rows in order,
//      columns ascending within each row -- the reference's tidy lower
//      matrix (spmat/spmat_utils.upc:455-473 tril, :1055-1062 sort_nonzeros).
// The sorts are sort.cu's stable radix sort.
#include <algorithm>
#include <cmath>
#include <vector>

#include "bale_inputs.h"
#include "sort.cuh"

namespace bale {
namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ uint64_t sm64(uint64_t seed, uint64_t i) {
  uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
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
  const unsigned lane = lane_id();
  const int64_t warps = static_cast<int64_t>(gridDim.x) * (blockDim.x >> 5);
  // warp-contiguous runs of 32 sorted keys: the smaller endpoint a repeats
  // along the run, so its lanes add once per distinct a
  for (int64_t e0 = (static_cast<int64_t>(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; e0 < m;
       e0 += warps * 32) {
    const int64_t e = e0 + lane;
    const bool keep = e < m && flag[e];
    const uint64_t k = keep ? keys[e] : ~0ull;
    if (keep) out[pos[e]] = k;
    const uint64_t a = k >> S;
    const unsigned peers = __match_any_sync(kFull, a);
    if (keep && (peers & ((1u << lane) - 1u)) == 0) {
      const uint32_t c = __popc(peers);
      if (a < kHubIds) atomicAdd(&hub[a], c); else atomicAdd(deg + a, c);
    }
    if (keep) {
      const uint64_t b = k & mask;
      if (b < kHubIds) atomicAdd(&hub[b], 1u); else atomicAdd(deg + b, 1u);
    }
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

// R-MAT quadrant probability as a 32-bit threshold on a uniform draw.
uint32_t prob_threshold(double p) {
  if (p <= 0.0) return 0;
  if (p >= 1.0) return UINT32_MAX;
  return static_cast<uint32_t>(llround(p * 4294967296.0));
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
  // few blocks: each flushes its kHubIds shared counters at the end
  compact_degree_kernel<<<std::min<unsigned>(grid_for(m), num_sms() * 4), 256, 0, st>>>(sorted, m, S, n, w.flag,
                                                                                    w.pos, other, w.deg);
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
  rc = csr_from_keys(ls, nu, n, S, d_offset, d_nonzero, st);
  if (rc != BALE_OK) return rc;
  BALE_CUDA_OK(cudaGetLastError());
  if ((rc = sort_status(w.words, st, "graph build")) != BALE_OK) return rc;
  *nnz = nu;
  return BALE_OK;
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

}  // extern "C"
