// tri_alg1.cu -- triangle counting with the reference's alg 1: the sum over
// the nonzeros L[i][j] of |U_i and U_j|, where U is the upper-triangular
// matrix the caller passes (apps/triangle_src/triangle_agi.upc:100-136, and
// the exstack variants' alg 1, apps/triangle_src/triangle_exstack.upc:
// 134-158, which push U's row i to row j's owner).
//
// The apps pass U = transpose(L) (apps/triangle_src/triangle.upc:306-307).
// Then the sum counts every triangle once -- a triangle a < b < c is counted
// at L's nonzero (b, a), whose U rows share c -- exactly as alg 0 does, so
// the count is the alg-0 count of L and the fast kernels compute it.  This
// file decides on the device whether U is L's transpose: it is when U is a
// tidy strictly upper matrix with as many nonzeros as L and every nonzero
// (i, j) of L has i in U's row j.  For any other tidy upper U the sum is
// computed as written: a warp per row i of L streams, for each j of the row,
// U's row j from the first column not below U_i's smallest and looks each
// element up in U_i (binary search), which is the reference's backward merge
// with its early stop, in parallel.
#include "common.cuh"

namespace bale {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ bool find_i64(const int64_t *__restrict__ r, int64_t len, int64_t w) {
  int64_t lo = 0, hi = len;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (r[mid] < w) lo = mid + 1;
    else hi = mid;
  }
  return lo < len && r[lo] == w;
}

__device__ __forceinline__ int64_t lower_bound_i64(const int64_t *__restrict__ r, int64_t len, int64_t w) {
  int64_t lo = 0, hi = len;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (r[mid] < w) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// A tidy triangular CSR, a warp per row: offsets inside [0, nnz] and not
// decreasing, columns strictly ascending, each in (row, n) for an upper
// matrix or [0, row) for a lower one.  Malformed rows are counted in *bad.
template <bool UPPER>
__global__ void __launch_bounds__(kThreads)
    alg1_check_kernel(const int64_t *__restrict__ off, const int64_t *__restrict__ col, int64_t n, int64_t nnz,
                      unsigned long long *__restrict__ bad) {
  const unsigned lane = lane_id();
  const int64_t warps = static_cast<int64_t>(gridDim.x) * (kThreads / 32);
  unsigned long long nbad = 0;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * (kThreads / 32) + (threadIdx.x >> 5); r < n; r += warps) {
    const int64_t b = off[r], e = off[r + 1];
    if (b < 0 || e < b || e > nnz) {
      nbad += lane == 0;
      continue;
    }
    bool ok = true;
    for (int64_t t = b + lane; t < e; t += 32) {
      const int64_t c = col[t];
      ok &= UPPER ? (c > r && c < n) : (c >= 0 && c < r);
      if (t > b) ok &= col[t - 1] < c;
    }
    nbad += __any_sync(0xffffffffu, !ok) && lane == 0;
  }
  if (lane == 0 && nbad) atomicAdd(bad, nbad);
}

// found += the nonzeros (i, j) of L with i in U's row j.
__global__ void __launch_bounds__(kThreads)
    alg1_transpose_kernel(const int64_t *__restrict__ loff, const int64_t *__restrict__ lcol,
                          const int64_t *__restrict__ uoff, const int64_t *__restrict__ ucol, int64_t n,
                          unsigned long long *__restrict__ found) {
  const unsigned lane = lane_id();
  const int64_t warps = static_cast<int64_t>(gridDim.x) * (kThreads / 32);
  unsigned long long f = 0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * (kThreads / 32) + (threadIdx.x >> 5); i < n; i += warps) {
    for (int64_t k = loff[i] + lane; k < loff[i + 1]; k += 32) {
      const int64_t j = lcol[k];
      f += find_i64(ucol + uoff[j], uoff[j + 1] - uoff[j], i) ? 1u : 0u;
    }
  }
  f = warp_sum_u64(f);
  if (lane == 0 && f) atomicAdd(found, f);
}

// count += sum over L's nonzeros (i, j) of |U_i and U_j|; work += the U_j
// elements looked up.
__global__ void __launch_bounds__(kThreads)
    alg1_count_kernel(const int64_t *__restrict__ loff, const int64_t *__restrict__ lcol,
                      const int64_t *__restrict__ uoff, const int64_t *__restrict__ ucol, int64_t n,
                      unsigned long long *__restrict__ count, unsigned long long *__restrict__ work) {
  const unsigned lane = lane_id();
  const int64_t warps = static_cast<int64_t>(gridDim.x) * (kThreads / 32);
  unsigned long long cnt = 0, wk = 0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * (kThreads / 32) + (threadIdx.x >> 5); i < n; i += warps) {
    const int64_t ub = uoff[i], ulen = uoff[i + 1] - ub;
    if (ulen == 0) continue;  // no third vertex above i
    const int64_t *ui = ucol + ub;
    const int64_t umin = ui[0];
    for (int64_t k = loff[i]; k < loff[i + 1]; k++) {
      const int64_t j = lcol[k];
      const int64_t jb = uoff[j], jlen = uoff[j + 1] - jb;
      const int64_t s = lower_bound_i64(ucol + jb, jlen, umin);
      for (int64_t t = s + lane; t < jlen; t += 32) {
        cnt += find_i64(ui, ulen, ucol[jb + t]) ? 1u : 0u;
        wk++;
      }
    }
  }
  cnt = warp_sum_u64(cnt);
  wk = warp_sum_u64(wk);
  if (lane == 0) {
    if (cnt) atomicAdd(count, cnt);
    if (wk && work) atomicAdd(work, wk);
  }
}

int grid_for_rows(int64_t n) {
  const int64_t want = (n + (kThreads / 32) - 1) / (kThreads / 32);
  const int64_t full = static_cast<int64_t>(num_sms()) * 8;
  return static_cast<int>(want < full ? (want > 0 ? want : 1) : full);
}

}  // namespace

int launch_triangle_alg1_check(const int64_t *loff, const int64_t *lcol, int64_t lnnz, const int64_t *uoff,
                               const int64_t *ucol, int64_t unnz, int64_t n, unsigned long long *bad,
                               cudaStream_t stream) {
  if (n <= 0) return BALE_OK;
  const int g = grid_for_rows(n);
  alg1_check_kernel<false><<<g, kThreads, 0, stream>>>(loff, lcol, n, lnnz, bad);
  BALE_CUDA_OK(cudaGetLastError());
  alg1_check_kernel<true><<<g, kThreads, 0, stream>>>(uoff, ucol, n, unnz, bad);
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

int launch_triangle_alg1_transposed(const int64_t *loff, const int64_t *lcol, const int64_t *uoff,
                                    const int64_t *ucol, int64_t n, unsigned long long *found, cudaStream_t stream) {
  if (n <= 0) return BALE_OK;
  alg1_transpose_kernel<<<grid_for_rows(n), kThreads, 0, stream>>>(loff, lcol, uoff, ucol, n, found);
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

int launch_triangle_alg1_count(const int64_t *loff, const int64_t *lcol, const int64_t *uoff, const int64_t *ucol,
                               int64_t n, unsigned long long *count, unsigned long long *work, cudaStream_t stream) {
  if (n <= 0) return BALE_OK;
  alg1_count_kernel<<<grid_for_rows(n), kThreads, 0, stream>>>(loff, lcol, uoff, ucol, n, count, work);
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

}  // namespace bale
