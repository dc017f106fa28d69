// ig.cu -- index gather: tgt[i] = table[index[i] >> shift].
//
// Replaces the per-request remote get of apps/ig_src/ig_agi.upc:61-64 and the
// request/response exchange of apps/ig_src/ig_exstack.upc:69-94: on one GPU
// the table is in HBM and each request is one random 8-byte load.  The cost
// is one 32-byte DRAM sector per request plus the two streams, so the kernel
// is built to keep enough independent sector reads in flight: every thread
// issues 2*UNROLL table loads before it consumes any of them, index and
// output move as 16-byte streaming accesses, and the grid is a whole number
// of waves over the SMs.
#include "common.cuh"

namespace bale {

namespace {

constexpr int kIgThreads = 256;

// Loads table[k] for a checked index k; out-of-range indices (including
// negative ones, which are huge as unsigned) produce 0 and are counted.
__device__ __forceinline__ int64_t gather_one(const int64_t *__restrict__ table, uint64_t tlen,
                                              int64_t raw, int shift, unsigned &nbad) {
  uint64_t k = static_cast<uint64_t>(raw >> shift);
  if (k < tlen) return ld_table(table + k);
  nbad++;
  return 0;
}

template <int UNROLL>
__global__ void __launch_bounds__(kIgThreads)
    ig_gather_kernel(int64_t *__restrict__ tgt, const int64_t *__restrict__ index, int64_t n,
                     const int64_t *__restrict__ table, uint64_t tlen, int shift,
                     unsigned long long *__restrict__ bad) {
  const longlong2 *__restrict__ idx2 = reinterpret_cast<const longlong2 *>(index);
  longlong2 *__restrict__ out2 = reinterpret_cast<longlong2 *>(tgt);
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
      v[u].x = gather_one(table, tlen, ix[u].x, shift, nbad);
      v[u].y = gather_one(table, tlen, ix[u].y, shift, nbad);
    }
#pragma unroll
    for (int u = 0; u < UNROLL; u++) st_stream_v2(out2 + p + u * stride, v[u]);
  }
  // Remaining pairs.
  for (; p < npairs; p += stride) {
    longlong2 ix = ld_stream_v2(idx2 + p);
    longlong2 v;
    v.x = gather_one(table, tlen, ix.x, shift, nbad);
    v.y = gather_one(table, tlen, ix.y, shift, nbad);
    st_stream_v2(out2 + p, v);
  }
  // Odd last element.
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    tgt[n - 1] = gather_one(table, tlen, index[n - 1], shift, nbad);
  }
  unsigned long long b = warp_sum_u64(nbad);
  if (b && lane_id() == 0) atomicAdd(bad, b);
}

// Scalar variant for index/tgt arrays that are not 16-byte aligned.
__global__ void __launch_bounds__(kIgThreads)
    ig_gather_scalar_kernel(int64_t *__restrict__ tgt, const int64_t *__restrict__ index,
                            int64_t n, const int64_t *__restrict__ table, uint64_t tlen,
                            int shift, unsigned long long *__restrict__ bad) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  unsigned nbad = 0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += stride)
    st_stream(tgt + i, gather_one(table, tlen, ld_stream(index + i), shift, nbad));
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

}  // namespace

int launch_ig(int64_t *tgt, const int64_t *index, int64_t n, const int64_t *table,
              int64_t table_len, int shift, unsigned long long *bad, cudaStream_t stream) {
  if (n <= 0) return BALE_OK;
  const int sms = num_sms();
  const bool aligned = ((reinterpret_cast<uintptr_t>(tgt) | reinterpret_cast<uintptr_t>(index)) & 15) == 0;
  // 8 resident blocks of 256 threads per SM; fewer blocks for small inputs.
  int64_t want = (n / 2 + kIgThreads - 1) / kIgThreads;
  int64_t full = static_cast<int64_t>(sms) * 8;
  int blocks = static_cast<int>(want < full ? (want > 0 ? want : 1) : full);
  if (aligned) {
    ig_gather_kernel<4><<<blocks, kIgThreads, 0, stream>>>(tgt, index, n, table,
                                                          static_cast<uint64_t>(table_len), shift, bad);
  } else {
    ig_gather_scalar_kernel<<<blocks, kIgThreads, 0, stream>>>(
        tgt, index, n, table, static_cast<uint64_t>(table_len), shift, bad);
  }
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
