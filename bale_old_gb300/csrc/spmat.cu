// spmat.cu -- spmat's transpose and permutation at one PE on the device,
// each bit-identical to the reference: transpose_matrix_agi and
// permute_matrix_agi (spmat/spmat_agi.upc:119-235).  The transpose is a key
// pass and sort.cu's stable radix sort; the permutation a warp per permuted
// row.  The random permutations are in randperm.cu, the MatrixMarket and
// dataset files in spmat_io.cu.
#include <algorithm>

#include "sort.cuh"

namespace bale {
namespace {

constexpr unsigned kFull = 0xffffffffu;

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
  launch_csr_check(d_offset, d_nonzero, numrows, numcols, nnz, bad, st);
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
  return sort_status(w.words, st, "bale_transpose_dev");
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
  launch_csr_check(d_offset, d_nonzero, numrows, numcols, nnz, bad, st);
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

}  // extern "C"
