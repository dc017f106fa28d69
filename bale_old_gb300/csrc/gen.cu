// gen.cu -- device-side input generators, bit-identical to the host ones in
// host/inputs.c (integer-only SplitMix64 streams), so large inputs can be
// made directly in HBM and checked against host-generated ones.
#include "bale_inputs.h"
#include "common.cuh"

namespace bale {
namespace {

__device__ __forceinline__ uint64_t sm64(uint64_t seed, uint64_t i) {
  uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

__global__ void __launch_bounds__(256)
    gen_uniform_kernel(int64_t *__restrict__ out, int64_t n, uint64_t range, uint64_t seed, int packed) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint64_t r = sm64(seed, static_cast<uint64_t>(i));
    const uint64_t v = range ? __umul64hi(r, range) : r;
    out[i] = packed ? static_cast<int64_t>(v << 16) : static_cast<int64_t>(v);
  }
}

}  // namespace
}  // namespace bale

using namespace bale;

extern "C" {

int bale_gen_uniform_dev(int64_t *d_out, int64_t n, int64_t range, uint64_t seed, int packed, void *stream) {
  if (n < 0 || range <= 0 || (n > 0 && !d_out) || (packed && range > (int64_t(1) << 47))) {
    set_error("bale_gen_uniform_dev: bad arguments");
    return BALE_EINVAL;
  }
  if (n == 0) return BALE_OK;
  int64_t blocks = (n + 255) / 256, cap = static_cast<int64_t>(num_sms()) * 16;
  gen_uniform_kernel<<<static_cast<unsigned>(blocks < cap ? blocks : cap), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      d_out, n, static_cast<uint64_t>(range), seed, packed);
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

int bale_gen_values_dev(int64_t *d_out, int64_t n, uint64_t seed, void *stream) {
  if (n < 0 || (n > 0 && !d_out)) {
    set_error("bale_gen_values_dev: bad arguments");
    return BALE_EINVAL;
  }
  if (n == 0) return BALE_OK;
  int64_t blocks = (n + 255) / 256, cap = static_cast<int64_t>(num_sms()) * 16;
  gen_uniform_kernel<<<static_cast<unsigned>(blocks < cap ? blocks : cap), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      d_out, n, 0, seed, 0);
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

}  // extern "C"
