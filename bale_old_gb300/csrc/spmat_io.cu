// spmat_io.cu -- spmat's files on the device side: read_matrix_mm_to_dist
// (spmat/spmat_utils.upc:217-370), the body parsed on the device with a
// stable sort keeping each row's file order, and the binary datasets
// (spmat/spmat_agi.upc:245-335), row lengths and columns streamed between
// device memory and the files through two pinned chunks.  The host-only
// writers and header readers are in host/mmio.c.
#include <sys/stat.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "sort.cuh"

namespace bale {
namespace {

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
                      2 * up256(4 * tiles * kDigits) + up256(4 * nb) + up256(4 * kOsWords) + 256;
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
  w.osw = reinterpret_cast<uint32_t *>(take(4 * kOsWords));
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
  return sort_status(w.words, st, "bale_read_matrix_mm_dev");
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
  launch_csr_check(d_offset, d_nonzero, numrows, numcols, nnz, bad, st);
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
  launch_csr_check(d_offset, d_nonzero, nr, nc, nnz, bad_csr, st);
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
