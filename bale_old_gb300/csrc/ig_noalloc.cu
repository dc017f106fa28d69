// ig_noalloc.cu -- bale_ig_dev_noalloc: the region-partitioned index gather
// with all of its scratch in one fixed device array inside this library.
//
// Why it exists: some callers of an index gather cannot allocate device
// memory at the moment they call.  A serving process whose HBM has been
// reserved up front by another allocator (a framework's caching allocator, or
// a memory pool sized to the whole device) gets cudaMalloc failures even
// though its own buffers are ready, and a latency-critical loop cannot accept
// the device-wide synchronisation that cudaMalloc/cudaFree may imply.  The
// regular entry point (bale_ig_dev) grows a workspace with cudaMalloc on
// demand; this one never allocates: the partition scratch for up to
// kNoAllocMaxRequests requests lives in g_ig_noalloc_scratch, a file-scope
// __device__ array that every GPU which loads the library holds until the
// process exits (3.5 MiB: 3,670,784 bytes).
//
// Set-up: the first call on each device, with that device current, looks up
// the array's device address with cudaGetSymbolAddress and caches it; make
// that first call before any stream capture.  The cache assumes one CUDA
// context per device for the life of the process: after cudaDeviceReset the
// cached address is stale, so a process that resets a device must not call
// this entry point on it again.  The stream must belong to the current
// device, whose array the call uses.  Host code never passes the
// array's name to a kernel: in host code the name is only a host-side
// stand-in, not a device address.
//
// Sharing: every call uses the same array, which keeps the previous call's
// contents.  The work cursor is cleared on the stream at the start of each
// call and every other scratch word is written before it is read, so stale
// contents never leak into a result -- but calls that overlap on the GPU
// (different streams, or different host threads) race on the array and must
// be serialised by the caller.
#include <mutex>

#include "common.cuh"

namespace bale {

namespace {

constexpr int64_t kNoAllocMaxRequests = int64_t(1) << 18;       // per call
constexpr int64_t kNoAllocMaxTable = kIgMaxRegions << kIgRegionBits;  // 2^32 entries
constexpr int64_t kChunk = int64_t(1) << kIgChunkBits;            // requests per partition chunk
constexpr int64_t kMaxChunks = kNoAllocMaxRequests / kChunk;      // 128
constexpr size_t kEntriesBytes = kNoAllocMaxRequests * sizeof(uint32_t);
constexpr size_t kValuesBytes = kNoAllocMaxRequests * sizeof(int64_t);
constexpr size_t kStartsBytes = ((kMaxChunks * (kIgMaxRegions + 2) * sizeof(uint16_t)) + 255) & ~size_t(255);
constexpr size_t kWordsOffset = kEntriesBytes + kValuesBytes + kStartsBytes;
constexpr size_t kScratchBytes = kWordsOffset + 256;  // [0] work cursor, [1] discarded bad count
static_assert(kScratchBytes == 3670784, "the documented size of the fixed scratch array");

static __device__ __align__(256) unsigned char g_ig_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
void *g_base[64] = {nullptr};

// Device address of g_ig_noalloc_scratch on the current device (looked up
// once per device; no allocation).
int scratch_base(void **out) {
  int dev = 0;
  BALE_CUDA_OK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("bale_ig_dev_noalloc: device ordinal %d out of range", dev);
    return BALE_EINVAL;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_base[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_ig_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      set_error("bale_ig_dev_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return BALE_ECUDA;
    }
    g_base[dev] = p;
  }
  *out = g_base[dev];
  return BALE_OK;
}

}  // namespace

}  // namespace bale

extern "C" int bale_ig_dev_noalloc(int64_t *d_tgt, const int64_t *d_index, int64_t n, const int64_t *d_table,
                                   int64_t table_len, int shift, int64_t *d_bad, void *stream) {
  using namespace bale;
  if (n < 0 || table_len < 0 || (shift != 0 && shift != 16) ||
      (n > 0 && (!d_tgt || !d_index || (table_len > 0 && !d_table)))) {
    set_error("bale_ig_dev_noalloc: bad arguments");
    return BALE_EINVAL;
  }
  if (n > kNoAllocMaxRequests) {
    set_error("bale_ig_dev_noalloc: %lld requests exceed the fixed scratch limit of %lld requests per call",
              static_cast<long long>(n), static_cast<long long>(kNoAllocMaxRequests));
    return BALE_EINVAL;
  }
  if (table_len > kNoAllocMaxTable) {
    set_error("bale_ig_dev_noalloc: table of %lld entries exceeds the limit of %lld entries",
              static_cast<long long>(table_len), static_cast<long long>(kNoAllocMaxTable));
    return BALE_EINVAL;
  }
  if (((reinterpret_cast<uintptr_t>(d_tgt) | reinterpret_cast<uintptr_t>(d_index)) & 15) != 0) {
    set_error("bale_ig_dev_noalloc: d_index and d_tgt must be 16-byte aligned");
    return BALE_EINVAL;
  }
  if (n == 0) return BALE_OK;
  void *base = nullptr;
  int rc = scratch_base(&base);
  if (rc != BALE_OK) return rc;
  unsigned char *p = static_cast<unsigned char *>(base);
  unsigned long long *words = reinterpret_cast<unsigned long long *>(p + kWordsOffset);
  unsigned long long *bad = d_bad ? reinterpret_cast<unsigned long long *>(d_bad) : words + 1;
  // The partitioned launcher lays out entries, values and region starts for
  // this call's n from the start of the array; for n <= kNoAllocMaxRequests
  // they end before kWordsOffset.  It zeroes the cursor on the stream first.
  return launch_ig_partitioned(d_tgt, d_index, n, d_table, table_len, shift, bad, p, words,
                               static_cast<cudaStream_t>(stream));
}
