// sort.cuh -- the stable LSD radix sort of 64-bit keys, the u32 exclusive
// scan and the CSR helpers shared by the graph build (graph.cu) and spmat's
// operations (spmat.cu, randperm.cu, spmat_io.cu).
#pragma once

#include "common.cuh"

namespace bale {

constexpr int kSortThreads = 256;                   // threads per sort block: one digit each
constexpr int kSortPer = 16;                        // keys per thread per tile
constexpr int64_t kTile = kSortThreads * kSortPer;  // 4096 keys per sort block
constexpr int kDigitBits = 8;
constexpr int kDigits = 1 << kDigitBits;
constexpr int kScanThreads = 1024;
constexpr int64_t kScanBlock = kScanThreads * 4;    // elements per scan block

constexpr int kOsPasses = 8;                                // digit passes of a 64-bit key
constexpr int kOsWords = kOsPasses * kDigits + kOsPasses;  // per pass: digit starts; then its tile counter
// words[kSortErrWord] is set when a sort pass's bounded wait gave up.  Every
// caller zeroes words before its first sort and reads it with sort_status.
constexpr int kSortErrWord = 15;

// Workspace of one graph build: two key buffers (m), flags and positions
// (m + 1), the sort's per-tile words and their scan, degrees, labels, vertex
// keys (n each).  The sort and the scan use hist, hoff, bsum, osw and words only.
struct Ws {
  uint64_t *ka, *kb, *va, *vb;
  uint32_t *flag, *pos, *hist, *hoff, *bsum, *deg, *newid;
  uint32_t *osw;        // kOsWords: the single-sweep sort's digit starts and tile counters
  unsigned int *words;  // [0] scan total, [1] max degree, [kSortErrWord] a sort wait gave up
};

size_t up256(size_t x);
// Blocks for a grid-stride loop over n items (at most 16 per SM).
unsigned grid_for(int64_t n);
// Bytes of a Ws for m edge keys and n vertices; with base, also lays it out in w.
size_t ws_bytes(int64_t m, int64_t n, Ws *w, char *base);
// out[0,n) = exclusive prefix of in[0,n); *total = the sum.
int excl_scan(const uint32_t *in, uint32_t *out, int64_t n, uint32_t *bsum, unsigned int *total, cudaStream_t st);
// One stable pass over the 8 bits from `shift`: a into b.
int radix_pass(const uint64_t *a, uint64_t *b, int64_t n, int shift, Ws &w, cudaStream_t st);
// BALE_ETIMEDOUT (with the error text naming `who`) when a sort since words
// was zeroed gave up a wait, else BALE_OK; synchronises st.
int sort_status(const unsigned int *words, cudaStream_t st, const char *who);
// Bits for labels [0, n): the least S with 2^S >= n (at least 1).
int label_bits(int64_t n);
// A CSR read off keys sorted by row: key = row << S | column (low S bits).
// offset[r] = the first key of row >= r (r in [0, nrows]); nonzero[e] = the
// column of key e (skipped when nonzero is null).
int csr_from_keys(const uint64_t *sk, int64_t nk, int64_t nrows, int S, int64_t *offset, int64_t *nonzero,
                  cudaStream_t st);
// Adds to *bad the malformed entries of a CSR: offsets not ascending inside
// [0, nnz] with offset[0] = 0 and offset[numrows] = nnz, columns outside
// [0, numcols).  Asynchronous.
void launch_csr_check(const int64_t *off, const int64_t *col, int64_t numrows, int64_t numcols, int64_t nnz,
                      unsigned long long *bad, cudaStream_t st);
// Stable sort of n keys on bits [0, bits); returns the buffer holding the result.
uint64_t *radix_sort(uint64_t *a, uint64_t *b, int64_t n, int bits, Ws &w, cudaStream_t st, int *rc);

}  // namespace bale
