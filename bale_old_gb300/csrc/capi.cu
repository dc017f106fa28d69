// capi.cu -- the C ABI of libbale_gb300.so (declared in include/bale_gb300.h).
//
// Drop-ins keep the reference signatures (apps/histo_src/histo.h:47-50,
// apps/ig_src/ig.h:49-52, apps/triangle_src/triangle.h:50-61): host arrays
// in, host arrays out, synchronous, wall seconds returned, -1.0 on failure.
// The reference's signatures carry no table length (the SHARED arrays'
// extents are implied by the app), so the drop-ins derive the extent the
// call can touch from the data: the largest index, computed on the device
// after the index array is uploaded.  Exactly counts[0..max] / table[0..max]
// are moved, which the reference would also have been allowed to access.
#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <mutex>
#include <vector>

#include "common.cuh"

namespace bale {

// ---------------------------------------------------------------------------
// errors, device facts, scratch
// ---------------------------------------------------------------------------
static thread_local char t_err[512] = "";

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(t_err, sizeof(t_err), fmt, ap);
  va_end(ap);
}

int current_device() {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess) return 0;
  return d;
}

int num_sms() {
  static int cache[64] = {0};
  int d = current_device();
  if (d < 0 || d >= 64) d = 0;
  if (cache[d] == 0) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, d) != cudaSuccess || v <= 0) v = 1;
    cache[d] = v;
  }
  return cache[d];
}

static std::mutex g_scratch_mu;
static DeviceScratch g_scratch[64];

DeviceScratch *device_scratch() {
  int d = current_device();
  if (d < 0 || d >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  DeviceScratch &s = g_scratch[d];
  if (!s.words) {
    void *p = nullptr;
    if (cudaMalloc(&p, kScratchWords * sizeof(unsigned long long)) != cudaSuccess) {
      set_error("cudaMalloc of %d scratch words failed", kScratchWords);
      return nullptr;
    }
    if (cudaMemset(p, 0, kScratchWords * sizeof(unsigned long long)) != cudaSuccess) {
      cudaFree(p);
      set_error("cudaMemset of scratch words failed");
      return nullptr;
    }
    s.words = static_cast<unsigned long long *>(p);
  }
  return &s;
}

static unsigned long long g_ring = 0;

unsigned long long *next_cursor_word() { return next_cursor_words(1); }

unsigned long long *next_cursor_words(int k) {
  if (k < 1 || k > 4) return nullptr;
  DeviceScratch *ds = device_scratch();
  if (!ds) return nullptr;
  // slots of 4 words starting at word 8
  const int nslots = (kScratchWords - 8) / 4;
  const int slot = static_cast<int>(__atomic_fetch_add(&g_ring, 1ull, __ATOMIC_RELAXED) % nslots);
  return ds->words + 8 + 4 * slot;
}

// Scratch word layout used by the synchronous drop-ins (serialised by
// g_dropin_mu): [0] bad-input count, [1] index max, [2] triangle count,
// [3] triangle work.  [7] absorbs bad counts the caller does not want.
enum { kWordBad = 0, kWordMax = 1, kWordCount = 2, kWordWork = 3, kWordFound = 4, kWordDiscard = 7 };

// ---------------------------------------------------------------------------
// drop-in state: a stream and grow-only device buffers per device
// ---------------------------------------------------------------------------
struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  int ensure(size_t bytes) {
    if (bytes <= cap && p) return BALE_OK;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = bytes < 256 ? 256 : bytes;
    if (cudaMalloc(&p, want) != cudaSuccess) {
      cudaGetLastError();
      set_error("cudaMalloc(%zu bytes) failed", want);
      return BALE_ENOMEM;
    }
    cap = want;
    return BALE_OK;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

struct DropinState {
  cudaStream_t stream = nullptr;
  cudaStream_t s_comp = nullptr, s_down = nullptr;  // the pipelined gather's compute and download streams
  DevBuf buf[4];
  unsigned long long *h_max = nullptr;  // mapped pinned per-chunk maxima (host address)
  unsigned long long *h_max_dev = nullptr;  // ... and their device alias
  size_t h_max_cap = 0;
};

static std::mutex g_dropin_mu;
static DropinState g_state[64];

// One grow-only workspace per (device, stream): work on one stream runs in
// order, so launches on the same stream may share it, while launches on
// different streams (the batched graph's side streams, the serving loop's
// express streams, callers' own streams) never see each other's data.
static std::mutex g_ws_mu;
static std::map<std::pair<int, cudaStream_t>, DevBuf> g_ws;

void *device_workspace(size_t bytes, cudaStream_t stream) {
  int d = current_device();
  if (d < 0) return nullptr;
  std::lock_guard<std::mutex> lk(g_ws_mu);
  DevBuf &b = g_ws[{d, stream}];
  if (b.ensure(bytes) != BALE_OK) return nullptr;
  return b.p;
}

static DropinState *dropin_state() {
  int d = current_device();
  if (d < 0 || d >= 64) return nullptr;
  DropinState &s = g_state[d];
  if (!s.stream) {
    if (cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s.s_comp, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s.s_down, cudaStreamNonBlocking) != cudaSuccess) {
      set_error("cudaStreamCreate failed");
      s.stream = s.s_comp = s.s_down = nullptr;
      return nullptr;
    }
  }
  return &s;
}

static double now_seconds() {
  using namespace std::chrono;
  return duration_cast<duration<double>>(steady_clock::now().time_since_epoch()).count();
}

#define DROPIN_TRY(expr)             \
  do {                               \
    int _rc = (expr);                \
    if (_rc != BALE_OK) return -1.0; \
  } while (0)

#define DROPIN_CUDA(expr)                                                          \
  do {                                                                             \
    cudaError_t _e = (expr);                                                       \
    if (_e != cudaSuccess) {                                                       \
      set_error("%s failed: %s", #expr, cudaGetErrorString(_e));                   \
      return -1.0;                                                                 \
    }                                                                              \
  } while (0)

// Upload index[0,n) into buf[0] and find the largest (shifted) index; the
// result is the number of table entries the call touches (max + 1).
static double extent_of(DropinState *st, DeviceScratch *ds, const int64_t *index, int64_t n,
                        int shift, int64_t *extent) {
  const size_t bytes = static_cast<size_t>(n) * sizeof(int64_t);
  DROPIN_TRY(st->buf[0].ensure(bytes));
  DROPIN_CUDA(cudaMemsetAsync(ds->words, 0, 8 * sizeof(unsigned long long), st->stream));
  DROPIN_CUDA(cudaMemcpyAsync(st->buf[0].p, index, bytes, cudaMemcpyHostToDevice, st->stream));
  DROPIN_TRY(launch_index_max(static_cast<const int64_t *>(st->buf[0].p), n, shift,
                              ds->words + kWordMax, st->stream));
  unsigned long long mx = 0;
  DROPIN_CUDA(cudaMemcpyAsync(&mx, ds->words + kWordMax, sizeof(mx), cudaMemcpyDeviceToHost, st->stream));
  DROPIN_CUDA(cudaStreamSynchronize(st->stream));
  if (mx >= (1ull << 60)) {
    set_error("index out of range (negative or >= 2^60): max index %llu", mx);
    return -1.0;
  }
  *extent = static_cast<int64_t>(mx) + 1;
  return 0.0;
}

static double histo_dropin(const int64_t *index, int64_t n, int64_t *counts, int shift) {
  const double t0 = now_seconds();
  if (n < 0 || (n > 0 && (!index || !counts))) {
    set_error("histo: bad arguments (len=%lld)", static_cast<long long>(n));
    return -1.0;
  }
  if (n == 0) return now_seconds() - t0;
  std::lock_guard<std::mutex> lk(g_dropin_mu);
  DropinState *st = dropin_state();
  DeviceScratch *ds = device_scratch();
  if (!st || !ds) return -1.0;
  int64_t extent = 0;
  if (extent_of(st, ds, index, n, shift, &extent) < 0) return -1.0;
  const size_t cbytes = static_cast<size_t>(extent) * sizeof(int64_t);
  DROPIN_TRY(st->buf[1].ensure(cbytes));
  int64_t *d_counts = static_cast<int64_t *>(st->buf[1].p);
  DROPIN_CUDA(cudaMemcpyAsync(d_counts, counts, cbytes, cudaMemcpyHostToDevice, st->stream));
  DROPIN_TRY(launch_histo(d_counts, extent, static_cast<const int64_t *>(st->buf[0].p), n, shift,
                          ds->words + kWordBad, st->stream));
  DROPIN_CUDA(cudaMemcpyAsync(counts, d_counts, cbytes, cudaMemcpyDeviceToHost, st->stream));
  unsigned long long bad = 0;
  DROPIN_CUDA(cudaMemcpyAsync(&bad, ds->words + kWordBad, sizeof(bad), cudaMemcpyDeviceToHost, st->stream));
  DROPIN_CUDA(cudaStreamSynchronize(st->stream));
  if (bad) {
    set_error("histo: %llu out-of-range indices", bad);
    return -1.0;
  }
  return now_seconds() - t0;
}

// Events of one pipelined call, destroyed on every return path.
struct EventSet {
  std::vector<cudaEvent_t> ev;
  ~EventSet() {
    for (auto e : ev)
      if (e) cudaEventDestroy(e);
  }
  cudaEvent_t make() {
    cudaEvent_t e = nullptr;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
    ev.push_back(e);
    return e;
  }
};

// Large gathers are pipelined in chunks of requests so that the copies in
// both directions and the gathers overlap.  The table's extent is not known
// before the requests are (the reference passes no table length), so:
//   1. chunk 0 is uploaded and its largest index found; the table is then
//      uploaded up to it (plus a margin for later chunks' larger indices);
//   2. the other chunks are uploaded behind it, each with its maximum, and
//      each is gathered as soon as it and the table are on the device and
//      copied back on a third stream while later chunks still upload;
//   3. a chunk whose indices reach beyond the uploaded part first extends
//      the device table on the gather stream (into a larger buffer, after
//      the uploads, only when the margin is used up).
// Results are identical to the single-pass path; the call stays synchronous.
static double ig_dropin_pipelined(int64_t *tgt, const int64_t *index, int64_t n, const int64_t *table, int shift,
                                  int64_t chunk, DropinState *st, DeviceScratch *ds, double t0) {
  const int64_t nch = (n + chunk - 1) / chunk;
  const size_t ibytes = static_cast<size_t>(n) * sizeof(int64_t);
  DROPIN_TRY(st->buf[0].ensure(ibytes));  // index
  DROPIN_TRY(st->buf[2].ensure(ibytes));  // output
  DROPIN_TRY(st->buf[3].ensure(static_cast<size_t>(nch) * sizeof(unsigned long long)));  // chunk maxima
  if (st->h_max_cap < static_cast<size_t>(nch)) {
    if (st->h_max) cudaFreeHost(st->h_max);
    st->h_max = st->h_max_dev = nullptr;
    st->h_max_cap = 0;
    void *hp = nullptr, *dp = nullptr;
    DROPIN_CUDA(cudaHostAlloc(&hp, static_cast<size_t>(nch) * sizeof(unsigned long long), cudaHostAllocMapped));
    st->h_max = static_cast<unsigned long long *>(hp);
    DROPIN_CUDA(cudaHostGetDevicePointer(&dp, hp, 0));
    st->h_max_dev = static_cast<unsigned long long *>(dp);
    st->h_max_cap = static_cast<size_t>(nch);
  }
  int64_t *d_idx = static_cast<int64_t *>(st->buf[0].p);
  int64_t *d_out = static_cast<int64_t *>(st->buf[2].p);
  unsigned long long *d_max = static_cast<unsigned long long *>(st->buf[3].p);
  unsigned long long *h_max = st->h_max, *h_max_dev = st->h_max_dev;
  EventSet es;
  DevBuf grown;  // a larger table buffer, if a chunk needs one
  // Every failure drains the streams first: copies into the caller's host
  // buffers may still be in flight.
  auto fail = [&]() -> double {
    cudaStreamSynchronize(st->stream);
    cudaStreamSynchronize(st->s_comp);
    cudaStreamSynchronize(st->s_down);
    cudaGetLastError();
    grown.release();
    return -1.0;
  };
#define PIPE_TRY(expr)                  \
  do {                                  \
    if ((expr) != BALE_OK) return fail(); \
  } while (0)
#define PIPE_CUDA(expr)                                                          \
  do {                                                                           \
    cudaError_t _e = (expr);                                                     \
    if (_e != cudaSuccess) {                                                     \
      set_error("%s failed: %s", #expr, cudaGetErrorString(_e));                 \
      return fail();                                                             \
    }                                                                            \
  } while (0)
  std::vector<cudaEvent_t> ev_max(static_cast<size_t>(nch)), ev_up(static_cast<size_t>(nch)),
      ev_gat(static_cast<size_t>(nch));
  for (int64_t k = 0; k < nch; k++) {
    ev_max[k] = es.make();
    ev_up[k] = es.make();
    ev_gat[k] = es.make();
    if (!ev_max[k] || !ev_up[k] || !ev_gat[k]) {
      set_error("ig: cudaEventCreate failed");
      return fail();
    }
  }
  cudaEvent_t ev_tab = es.make();
  if (!ev_tab) {
    set_error("ig: cudaEventCreate failed");
    return fail();
  }
  PIPE_CUDA(cudaMemsetAsync(ds->words, 0, 8 * sizeof(unsigned long long), st->stream));
  PIPE_CUDA(cudaMemsetAsync(d_max, 0, static_cast<size_t>(nch) * sizeof(unsigned long long), st->stream));
  auto upload = [&](int64_t k) -> int {
    const int64_t lo = k * chunk, len = std::min(chunk, n - lo);
    if (cudaMemcpyAsync(d_idx + lo, index + lo, static_cast<size_t>(len) * 8, cudaMemcpyHostToDevice,
                        st->stream) != cudaSuccess ||
        cudaEventRecord(ev_up[k], st->stream) != cudaSuccess)
      return BALE_ECUDA;
    // the maximum goes to the host by a kernel's write, not a copy: a
    // device-to-host copy here would queue behind the result downloads
    int rc = launch_index_max(d_idx + lo, len, shift, d_max + k, st->stream);
    if (rc == BALE_OK) rc = launch_copy_word(d_max + k, h_max_dev + k, st->stream);
    if (rc != BALE_OK) return rc;
    if (cudaEventRecord(ev_max[k], st->stream) != cudaSuccess) return BALE_ECUDA;
    return BALE_OK;
  };
  auto too_big = [&](unsigned long long m) {
    if (m < (1ull << 60)) return false;
    set_error("index out of range (negative or >= 2^60): max index %llu", m);
    return true;
  };
  if (upload(0) != BALE_OK) {
    set_error("ig: upload failed");
    return fail();
  }
  PIPE_CUDA(cudaEventSynchronize(ev_max[0]));
  if (too_big(h_max[0])) {
    return fail();
  }
  int64_t ext = static_cast<int64_t>(h_max[0]) + 1;  // table entries on the device
  size_t cap = static_cast<size_t>(ext) + static_cast<size_t>(ext) / 4 + 1024;
  PIPE_TRY(st->buf[1].ensure(cap * sizeof(int64_t)));
  int64_t *d_tab = static_cast<int64_t *>(st->buf[1].p);
  PIPE_CUDA(cudaMemcpyAsync(d_tab, table, static_cast<size_t>(ext) * 8, cudaMemcpyHostToDevice, st->stream));
  PIPE_CUDA(cudaEventRecord(ev_tab, st->stream));
  for (int64_t k = 1; k < nch; k++)
    if (upload(k) != BALE_OK) {
      set_error("ig: upload failed");
      return fail();
    }
  PIPE_CUDA(cudaStreamWaitEvent(st->s_comp, ev_tab, 0));
  for (int64_t k = 0; k < nch; k++) {
    PIPE_CUDA(cudaEventSynchronize(ev_max[k]));
    if (too_big(h_max[k])) {
      return fail();
    }
    const int64_t need = static_cast<int64_t>(h_max[k]) + 1;
    if (need > ext) {
      // Extend the device table to this chunk's largest index, on the gather
      // stream (usually a few entries: independent chunks of random requests
      // have nearly the same maximum).  Only when the buffer's margin is used
      // up is a larger buffer taken -- sized from every chunk's maximum, so
      // this waits for the uploads -- after the gathers reading the old one.
      int64_t top = need;
      if (static_cast<size_t>(need) > cap) {
        PIPE_CUDA(cudaStreamSynchronize(st->stream));
        for (int64_t r = k; r < nch; r++) {
          if (too_big(h_max[r])) return fail();
          top = std::max<int64_t>(top, static_cast<int64_t>(h_max[r]) + 1);
        }
        PIPE_CUDA(cudaStreamSynchronize(st->s_comp));
        PIPE_TRY(grown.ensure(static_cast<size_t>(top) * sizeof(int64_t)));
        PIPE_CUDA(cudaMemcpyAsync(grown.p, d_tab, static_cast<size_t>(ext) * 8, cudaMemcpyDeviceToDevice,
                                  st->s_comp));
        d_tab = static_cast<int64_t *>(grown.p);
        cap = static_cast<size_t>(top);
      }
      PIPE_CUDA(cudaMemcpyAsync(d_tab + ext, table + ext, static_cast<size_t>(top - ext) * 8,
                                cudaMemcpyHostToDevice, st->s_comp));
      ext = top;
    }
    const int64_t lo = k * chunk, len = std::min(chunk, n - lo);
    PIPE_CUDA(cudaStreamWaitEvent(st->s_comp, ev_up[k], 0));
    PIPE_TRY(launch_ig(d_out + lo, d_idx + lo, len, d_tab, ext, shift, ds->words + kWordBad, st->s_comp));
    PIPE_CUDA(cudaEventRecord(ev_gat[k], st->s_comp));
    PIPE_CUDA(cudaStreamWaitEvent(st->s_down, ev_gat[k], 0));
    PIPE_CUDA(cudaMemcpyAsync(tgt + lo, d_out + lo, static_cast<size_t>(len) * 8, cudaMemcpyDeviceToHost,
                                st->s_down));
  }
  unsigned long long bad = 0;
  PIPE_CUDA(cudaStreamSynchronize(st->s_comp));
  PIPE_CUDA(cudaMemcpyAsync(&bad, ds->words + kWordBad, sizeof(bad), cudaMemcpyDeviceToHost, st->s_down));
  PIPE_CUDA(cudaStreamSynchronize(st->s_down));
  PIPE_CUDA(cudaStreamSynchronize(st->stream));
  grown.release();
#undef PIPE_TRY
#undef PIPE_CUDA
  if (bad) {
    set_error("ig: %llu out-of-range indices", bad);
    return -1.0;
  }
  return now_seconds() - t0;
}

static double ig_dropin(int64_t *tgt, const int64_t *index, int64_t n, const int64_t *table,
                        int shift) {
  const double t0 = now_seconds();
  if (n < 0 || (n > 0 && (!index || !tgt || !table))) {
    set_error("ig: bad arguments (l_num_req=%lld)", static_cast<long long>(n));
    return -1.0;
  }
  if (n == 0) return now_seconds() - t0;
  std::lock_guard<std::mutex> lk(g_dropin_mu);
  DropinState *st = dropin_state();
  DeviceScratch *ds = device_scratch();
  if (!st || !ds) return -1.0;
  const int64_t chunk = knob_or("dropin.ig_chunk", int64_t(1) << 24);
  if (chunk > 0 && n > 2 * chunk) return ig_dropin_pipelined(tgt, index, n, table, shift, chunk, st, ds, t0);
  int64_t extent = 0;
  if (extent_of(st, ds, index, n, shift, &extent) < 0) return -1.0;
  const size_t tbytes = static_cast<size_t>(extent) * sizeof(int64_t);
  const size_t obytes = static_cast<size_t>(n) * sizeof(int64_t);
  DROPIN_TRY(st->buf[1].ensure(tbytes));
  DROPIN_TRY(st->buf[2].ensure(obytes));
  DROPIN_CUDA(cudaMemcpyAsync(st->buf[1].p, table, tbytes, cudaMemcpyHostToDevice, st->stream));
  DROPIN_TRY(launch_ig(static_cast<int64_t *>(st->buf[2].p), static_cast<const int64_t *>(st->buf[0].p), n,
                       static_cast<const int64_t *>(st->buf[1].p), extent, shift, ds->words + kWordBad,
                       st->stream));
  DROPIN_CUDA(cudaMemcpyAsync(tgt, st->buf[2].p, obytes, cudaMemcpyDeviceToHost, st->stream));
  unsigned long long bad = 0;
  DROPIN_CUDA(cudaMemcpyAsync(&bad, ds->words + kWordBad, sizeof(bad), cudaMemcpyDeviceToHost, st->stream));
  DROPIN_CUDA(cudaStreamSynchronize(st->stream));
  if (bad) {
    set_error("ig: %llu out-of-range indices", bad);
    return -1.0;
  }
  return now_seconds() - t0;
}

// The triangle drop-ins.  alg 0 counts from L alone; any other alg is the
// reference's alg 1 (apps/triangle_src/triangle_agi.upc:100-136), the sum
// over L's nonzeros (i,j) of |U_i and U_j| with the caller's U, which must be
// given (the reference returns -1 for a NULL U).  When U is L's transpose,
// as the apps pass it, that sum is alg 0's count and the alg-0 kernels run;
// for any other tidy upper U it is computed as written (tri_alg1.cu).
static double triangle_dropin(int64_t *count, int64_t *sr, sparsemat_t *L, sparsemat_t *U, int64_t alg) {
  const double t0 = now_seconds();
  if (!count || !sr || !L) {
    set_error("triangle: NULL count, sr or L");
    return -1.0;
  }
  const int64_t n = L->lnumrows;
  if (n < 0 || (n > 0 && !L->loffset)) {
    set_error("triangle: bad matrix (lnumrows=%lld)", static_cast<long long>(n));
    return -1.0;
  }
  const int64_t nnz = n > 0 ? L->loffset[n] : 0;
  if (nnz < 0 || (nnz > 0 && !L->lnonzero)) {
    set_error("triangle: bad matrix (nnz=%lld)", static_cast<long long>(nnz));
    return -1.0;
  }
  const bool alg1 = alg != 0;
  int64_t unnz = 0;
  if (alg1) {
    if (!U) {
      set_error("triangle: alg %lld needs U (NULL given)", static_cast<long long>(alg));
      return -1.0;
    }
    if (U->lnumrows != n || (n > 0 && !U->loffset)) {
      set_error("triangle: U must have L's %lld rows", static_cast<long long>(n));
      return -1.0;
    }
    unnz = n > 0 ? U->loffset[n] : 0;
    if (unnz < 0 || (unnz > 0 && !U->lnonzero)) {
      set_error("triangle: bad U (nnz=%lld)", static_cast<long long>(unnz));
      return -1.0;
    }
  }
  std::lock_guard<std::mutex> lk(g_dropin_mu);
  DropinState *st = dropin_state();
  DeviceScratch *ds = device_scratch();
  if (!st || !ds) return -1.0;
  const size_t obytes = static_cast<size_t>(n + 1) * sizeof(int64_t);
  const size_t cbytes = static_cast<size_t>(nnz > 0 ? nnz : 1) * sizeof(int64_t);
  DROPIN_TRY(st->buf[0].ensure(obytes));
  DROPIN_TRY(st->buf[1].ensure(cbytes));
  DROPIN_CUDA(cudaMemsetAsync(ds->words, 0, 8 * sizeof(unsigned long long), st->stream));
  DROPIN_CUDA(cudaMemcpyAsync(st->buf[0].p, L->loffset, obytes, cudaMemcpyHostToDevice, st->stream));
  if (nnz > 0)
    DROPIN_CUDA(cudaMemcpyAsync(st->buf[1].p, L->lnonzero, static_cast<size_t>(nnz) * sizeof(int64_t),
                                cudaMemcpyHostToDevice, st->stream));
  const int64_t *d_loff = static_cast<const int64_t *>(st->buf[0].p);
  const int64_t *d_lcol = static_cast<const int64_t *>(st->buf[1].p);
  bool general_alg1 = false;
  if (alg1 && n > 0) {
    DROPIN_TRY(st->buf[2].ensure(obytes));
    DROPIN_TRY(st->buf[3].ensure(static_cast<size_t>(unnz > 0 ? unnz : 1) * sizeof(int64_t)));
    DROPIN_CUDA(cudaMemcpyAsync(st->buf[2].p, U->loffset, obytes, cudaMemcpyHostToDevice, st->stream));
    if (unnz > 0)
      DROPIN_CUDA(cudaMemcpyAsync(st->buf[3].p, U->lnonzero, static_cast<size_t>(unnz) * sizeof(int64_t),
                                  cudaMemcpyHostToDevice, st->stream));
    const int64_t *d_uoff = static_cast<const int64_t *>(st->buf[2].p);
    const int64_t *d_ucol = static_cast<const int64_t *>(st->buf[3].p);
    DROPIN_TRY(launch_triangle_alg1_check(d_loff, d_lcol, nnz, d_uoff, d_ucol, unnz, n, ds->words + kWordBad,
                                          st->stream));
    unsigned long long bad = 0;
    DROPIN_CUDA(cudaMemcpyAsync(&bad, ds->words + kWordBad, sizeof(bad), cudaMemcpyDeviceToHost, st->stream));
    DROPIN_CUDA(cudaStreamSynchronize(st->stream));
    if (bad) {
      set_error("triangle: L is not strictly lower or U not strictly upper tidy CSR (%llu bad rows)", bad);
      return -1.0;
    }
    DROPIN_TRY(launch_triangle_alg1_transposed(d_loff, d_lcol, d_uoff, d_ucol, n, ds->words + kWordFound,
                                               st->stream));
    unsigned long long found = 0;
    DROPIN_CUDA(cudaMemcpyAsync(&found, ds->words + kWordFound, sizeof(found), cudaMemcpyDeviceToHost, st->stream));
    DROPIN_CUDA(cudaStreamSynchronize(st->stream));
    general_alg1 = !(unnz == nnz && found == static_cast<unsigned long long>(nnz));
    if (general_alg1)
      DROPIN_TRY(launch_triangle_alg1_count(d_loff, d_lcol, d_uoff, d_ucol, n, ds->words + kWordCount,
                                            ds->words + kWordWork, st->stream));
  }
  if (!general_alg1)
    DROPIN_TRY(launch_triangle(d_loff, d_lcol, n, nnz, ds->words + kWordCount, ds->words + kWordWork,
                               ds->words + kWordBad, st->stream));
  unsigned long long w[4] = {0, 0, 0, 0};
  DROPIN_CUDA(cudaMemcpyAsync(w, ds->words, sizeof(w), cudaMemcpyDeviceToHost, st->stream));
  DROPIN_CUDA(cudaStreamSynchronize(st->stream));
  if (w[kWordBad]) {
    set_error("triangle: L is not a strictly lower-triangular tidy CSR (%llu bad rows/offsets)",
              w[kWordBad]);
    return -1.0;
  }
  *count = static_cast<int64_t>(w[kWordCount]);
  *sr = static_cast<int64_t>(w[kWordWork]);
  return now_seconds() - t0;
}

}  // namespace bale

using namespace bale;

extern "C" {

double histo_agi(int64_t *index, int64_t len, int64_t *counts) {
  return histo_dropin(index, len, counts, 0);
}
double histo_exstack(int64_t *pckindx, int64_t len, int64_t *lcounts, int64_t buf_cnt) {
  (void)buf_cnt;
  return histo_dropin(pckindx, len, lcounts, 16);
}
double histo_exstack2(int64_t *pckindx, int64_t len, int64_t *lcounts, int64_t buf_cnt) {
  (void)buf_cnt;
  return histo_dropin(pckindx, len, lcounts, 16);
}
double histo_conveyor(int64_t *pckindx, int64_t len, int64_t *lcounts) {
  return histo_dropin(pckindx, len, lcounts, 16);
}

double ig_agi(int64_t *tgt, int64_t *index, int64_t l_num_req, int64_t *table) {
  return ig_dropin(tgt, index, l_num_req, table, 0);
}
double ig_exstack(int64_t *tgt, int64_t *pckindx, int64_t l_num_req, int64_t *ltable, int64_t buf_cnt) {
  (void)buf_cnt;
  return ig_dropin(tgt, pckindx, l_num_req, ltable, 16);
}
double ig_exstack2(int64_t *tgt, int64_t *pckindx, int64_t l_num_req, int64_t *ltable, int64_t buf_cnt) {
  (void)buf_cnt;
  return ig_dropin(tgt, pckindx, l_num_req, ltable, 16);
}
double ig_conveyor(int64_t *tgt, int64_t *pckindx, int64_t l_num_req, int64_t *ltable) {
  return ig_dropin(tgt, pckindx, l_num_req, ltable, 16);
}

double triangle_agi(int64_t *count, int64_t *sr, sparsemat_t *L, sparsemat_t *U, int64_t alg) {
  return triangle_dropin(count, sr, L, U, alg);
}
double triangle_exstack_push(int64_t *count, int64_t *sr, sparsemat_t *L, sparsemat_t *U, int64_t alg,
                             int64_t bufsiz) {
  (void)bufsiz;
  return triangle_dropin(count, sr, L, U, alg);
}
double triangle_exstack2_push(int64_t *count, int64_t *sr, sparsemat_t *L, sparsemat_t *U, int64_t alg,
                              int64_t bufsiz) {
  (void)bufsiz;
  return triangle_dropin(count, sr, L, U, alg);
}
double triangle_convey_push(int64_t *count, int64_t *sr, sparsemat_t *L, sparsemat_t *U, int64_t alg) {
  return triangle_dropin(count, sr, L, U, alg);
}
double triangle_agi_iter(int64_t *count, int64_t *sr, sparsemat_t *L, sparsemat_t *U, int64_t alg) {
  return triangle_dropin(count, sr, L, U, alg);
}

int bale_device_caps(int64_t *out, int n) {
  if (!out || n <= 0) return BALE_EINVAL;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return BALE_ECUDA;
  const cudaDeviceAttr attrs[] = {cudaDevAttrMultiProcessorCount,
                                  cudaDevAttrPageableMemoryAccess,
                                  cudaDevAttrPageableMemoryAccessUsesHostPageTables,
                                  cudaDevAttrConcurrentManagedAccess,
                                  cudaDevAttrL2CacheSize,
                                  cudaDevAttrMaxSharedMemoryPerBlockOptin,
                                  cudaDevAttrCanUseHostPointerForRegisteredMem,
                                  cudaDevAttrAsyncEngineCount,
                                  cudaDevAttrUnifiedAddressing};
  const int na = static_cast<int>(sizeof(attrs) / sizeof(attrs[0]));
  for (int i = 0; i < n; i++) {
    int v = -1;
    if (i < na && cudaDeviceGetAttribute(&v, attrs[i], dev) != cudaSuccess) v = -1;
    out[i] = v;
  }
  return BALE_OK;
}

const char *bale_last_error(void) { return t_err; }
const char *bale_version(void) { return "bale_gb300 0.1 (sm_103a)"; }

void bale_release_buffers(void) {
  std::lock_guard<std::mutex> lk(g_dropin_mu);
  for (int d = 0; d < 64; d++)
    for (auto &b : g_state[d].buf) b.release();
  std::lock_guard<std::mutex> lk2(g_ws_mu);
  for (auto &kv : g_ws) kv.second.release();
  g_ws.clear();
}

int bale_histo_dev(int64_t *d_counts, int64_t ncounts, const int64_t *d_index, int64_t n, int shift,
                   int64_t *d_bad, void *stream) {
  if (n < 0 || ncounts < 0 || (shift != 0 && shift != 16) || (n > 0 && (!d_counts || !d_index))) {
    set_error("bale_histo_dev: bad arguments");
    return BALE_EINVAL;
  }
  if (n == 0) return BALE_OK;
  DeviceScratch *ds = device_scratch();
  if (!ds) return BALE_ECUDA;
  unsigned long long *bad = d_bad ? reinterpret_cast<unsigned long long *>(d_bad) : ds->words + kWordDiscard;
  return launch_histo(d_counts, ncounts, d_index, n, shift, bad, static_cast<cudaStream_t>(stream));
}

int bale_l2_red_rate(int64_t *d_counts, int64_t ncounts, int64_t n, void *stream) {
  if (n < 0 || ncounts < 0 || (n > 0 && (!d_counts || ncounts == 0))) {
    set_error("bale_l2_red_rate: bad arguments");
    return BALE_EINVAL;
  }
  return launch_l2_red_rate(d_counts, ncounts, n, static_cast<cudaStream_t>(stream));
}

int bale_ig_dev(int64_t *d_tgt, const int64_t *d_index, int64_t n, const int64_t *d_table, int64_t table_len,
                int shift, int64_t *d_bad, void *stream) {
  if (n < 0 || table_len < 0 || (shift != 0 && shift != 16) ||
      (n > 0 && (!d_tgt || !d_index || (table_len > 0 && !d_table)))) {
    set_error("bale_ig_dev: bad arguments");
    return BALE_EINVAL;
  }
  if (n == 0) return BALE_OK;
  DeviceScratch *ds = device_scratch();
  if (!ds) return BALE_ECUDA;
  unsigned long long *bad = d_bad ? reinterpret_cast<unsigned long long *>(d_bad) : ds->words + kWordDiscard;
  return launch_ig(d_tgt, d_index, n, d_table, table_len, shift, bad, static_cast<cudaStream_t>(stream));
}

int bale_triangle_dev(const int64_t *d_offset, const int64_t *d_nonzero, int64_t numrows, int64_t nnz,
                      int64_t *d_count, int64_t *d_work, int64_t *d_bad, void *stream) {
  if (numrows < 0 || nnz < 0 || !d_count || (numrows > 0 && !d_offset) || (nnz > 0 && !d_nonzero)) {
    set_error("bale_triangle_dev: bad arguments");
    return BALE_EINVAL;
  }
  if (numrows == 0) return BALE_OK;
  DeviceScratch *ds = device_scratch();
  if (!ds) return BALE_ECUDA;
  unsigned long long *bad = d_bad ? reinterpret_cast<unsigned long long *>(d_bad) : ds->words + kWordDiscard;
  return launch_triangle(d_offset, d_nonzero, numrows, nnz, reinterpret_cast<unsigned long long *>(d_count),
                         reinterpret_cast<unsigned long long *>(d_work), bad,
                         static_cast<cudaStream_t>(stream));
}

struct bale_tri_prepared {
  const int64_t *offset = nullptr, *nonzero = nullptr;
  int64_t numrows = 0, nnz = 0;
  bool wedge = false;        // else each count runs the general path
  void *ws = nullptr;        // the wedge kernels' prepared form
  unsigned long long *cursor = nullptr;
};

bale_tri_prepared_t *bale_triangle_prepare(const int64_t *d_offset, const int64_t *d_nonzero, int64_t numrows,
                                           int64_t nnz, int64_t *d_bad, void *stream) {
  if (numrows < 0 || nnz < 0 || (numrows > 0 && !d_offset) || (nnz > 0 && !d_nonzero)) {
    set_error("bale_triangle_prepare: bad arguments");
    return nullptr;
  }
  bale_tri_prepared *g = new (std::nothrow) bale_tri_prepared();
  if (!g) {
    set_error("bale_triangle_prepare: out of host memory");
    return nullptr;
  }
  g->offset = d_offset;
  g->nonzero = d_nonzero;
  g->numrows = numrows;
  g->nnz = nnz;
  const int64_t mode = knob("tri.mode");
  g->wedge = (mode < 0 || mode == 2) && tri_wedge_supported(numrows, nnz);
  if (g->wedge) {
    DeviceScratch *ds = device_scratch();
    const size_t bytes = tri_wedge_workspace_bytes(numrows, nnz);
    if (!ds || cudaMalloc(&g->ws, bytes) != cudaSuccess || cudaMalloc(&g->cursor, 16) != cudaSuccess) {
      cudaGetLastError();
      set_error("bale_triangle_prepare: cudaMalloc of %zu bytes failed", bytes);
      bale_triangle_release(g);
      return nullptr;
    }
    unsigned long long *bad = d_bad ? reinterpret_cast<unsigned long long *>(d_bad) : ds->words + kWordDiscard;
    if (tri_wedge_prepare(d_offset, d_nonzero, numrows, nnz, g->ws, bad, static_cast<cudaStream_t>(stream)) !=
        BALE_OK) {
      bale_triangle_release(g);
      return nullptr;
    }
  }
  return g;
}

int bale_triangle_count_prepared(bale_tri_prepared_t *g, int64_t *d_count, int64_t *d_work, void *stream) {
  if (!g || !d_count) {
    set_error("bale_triangle_count_prepared: bad arguments");
    return BALE_EINVAL;
  }
  if (g->numrows == 0) return BALE_OK;
  if (!g->wedge)
    return bale_triangle_dev(g->offset, g->nonzero, g->numrows, g->nnz, d_count, d_work, nullptr, stream);
  return tri_wedge_run(g->offset, g->ws, g->numrows, g->nnz, reinterpret_cast<unsigned long long *>(d_count),
                       reinterpret_cast<unsigned long long *>(d_work), g->cursor, static_cast<cudaStream_t>(stream));
}

void bale_triangle_release(bale_tri_prepared_t *g) {
  if (!g) return;
  if (g->ws || g->cursor) cudaDeviceSynchronize();  // no count in flight may still read them
  cudaFree(g->ws);
  cudaFree(g->cursor);
  delete g;
}

}  // extern "C"
