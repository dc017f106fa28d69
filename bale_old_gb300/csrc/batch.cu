// batch.cu -- hundreds of uneven histo / ig / triangle instances in one
// persistent, CUDA-graph-captured work-queue launch.
//
// A plain run launches every instance's kernels separately: small instances
// leave most of the GPU idle and every launch pays its fixed cost.  Here a
// host planner cuts every instance into tiles (tasks) sized per kind and size
// class (the batch.* tuning knobs, set by the autotuner), orders them
// longest-first, and one persistent kernel -- two 512-thread blocks per SM,
// 96 KiB of shared memory and 64 registers a thread -- pulls tasks from a
// device queue until it is empty:
//
//   histo, table <= 24 Ki counters : the task's updates are counted in a
//                                    shared-memory copy of the table, then
//                                    flushed with one L2 reduction per counter;
//   histo, larger table            : plain red.global.add.u64 per update;
//   ig                             : direct gather, 8 loads in flight/thread;
//   triangles, light rows          : warps take rows of the task's range
//                                    (tri_device.cuh light_row);
//   triangles, heavy rows          : the whole block per heavy row, row i as
//                                    a shared-memory bitmap (heavy_row).
//
// Instances large enough to fill the GPU by themselves (the standalone rule:
// the partition thresholds, batch.standalone_min elements, or
// batch.standalone_min_edges nonzeros for a graph) run their specialised
// kernels instead -- region-partitioned ig / histo, the wedge triangle
// kernels -- on up to batch.streams captured side streams, longest first to
// the least loaded, in parallel with the queue.  The whole run -- queue
// reset, the persistent kernel and those launches -- is one CUDA graph,
// replayed by bale_batch_run.
//
// Results match the per-instance entry points bit for bit: histo ADDS into
// its counts, ig OVERWRITES tgt, triangles ADD their count into out[0].
// Out-of-range indices and malformed rows are counted per instance.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "batch.cuh"

namespace bale {
namespace q {

namespace {


__device__ __forceinline__ void add_bad(unsigned long long *bad, unsigned long long v) {
  v = warp_sum_u64(v);
  if (lane_id() == 0 && v) atomicAdd(bad, v);
}

__device__ void cta_histo_smem(const Inst &in, int64_t lo, int64_t hi, uint32_t *sm, unsigned long long *bad) {
  const uint64_t m = static_cast<uint64_t>(in.m);
  for (uint64_t c = threadIdx.x; c < m; c += kThreads) sm[c] = 0;
  __syncthreads();
  unsigned long long nb = 0;
  for (int64_t i = lo + threadIdx.x; i < hi; i += kThreads) {
    const uint64_t k = static_cast<uint64_t>(ld_stream(in.in + i) >> in.shift);
    if (k < m) atomicAdd(&sm[k], 1u); else nb++;
  }
  __syncthreads();
  for (uint64_t c = threadIdx.x; c < m; c += kThreads) {
    const uint32_t v = sm[c];
    if (v) red_add_u64(in.out + c, v);
  }
  add_bad(bad, nb);
}

__device__ void cta_histo_l2(const Inst &in, int64_t lo, int64_t hi, unsigned long long *bad) {
  const uint64_t m = static_cast<uint64_t>(in.m);
  unsigned long long nb = 0;
  for (int64_t i = lo + threadIdx.x; i < hi; i += 4 * kThreads) {
    int64_t r[4];
#pragma unroll
    for (int u = 0; u < 4; u++) r[u] = (i + u * kThreads < hi) ? ld_stream(in.in + i + u * kThreads) : -1;
#pragma unroll
    for (int u = 0; u < 4; u++) {
      if (i + u * kThreads < hi) {
        const uint64_t k = static_cast<uint64_t>(r[u] >> in.shift);
        if (k < m) red_add_u64(in.out + k, 1ull); else nb++;
      }
    }
  }
  add_bad(bad, nb);
}

__device__ void cta_ig(const Inst &in, int64_t lo, int64_t hi, unsigned long long *bad) {
  const uint64_t m = static_cast<uint64_t>(in.m);
  unsigned long long nb = 0;
  constexpr int U = 8;
  for (int64_t i = lo + threadIdx.x; i < hi; i += U * kThreads) {
    int64_t r[U], v[U];
#pragma unroll
    for (int u = 0; u < U; u++) r[u] = (i + u * kThreads < hi) ? ld_stream(in.in + i + u * kThreads) : 0;
#pragma unroll
    for (int u = 0; u < U; u++) {
      const uint64_t k = static_cast<uint64_t>(r[u] >> in.shift);
      const bool live = i + u * kThreads < hi;
      v[u] = 0;
      if (live && k < m) v[u] = ld_table(in.aux + k);
      else if (live) nb++;
    }
#pragma unroll
    for (int u = 0; u < U; u++)
      if (i + u * kThreads < hi) st_stream(in.out + i + u * kThreads, v[u]);
  }
  add_bad(bad, nb);
}

__device__ void flush_tri(const tri::Tally &t0, const Inst &in, unsigned long long *bad, unsigned long long *work) {
  tri::Tally t = t0;
  t.cnt = warp_sum_u64(t.cnt);
  t.work = warp_sum_u64(t.work);
  t.bad = warp_sum_u64(t.bad);
  if (lane_id() == 0) {
    if (t.cnt) atomicAdd(reinterpret_cast<unsigned long long *>(in.out), t.cnt);
    if (t.work) atomicAdd(work, t.work);
    if (t.bad) atomicAdd(bad, t.bad);
  }
}

__device__ void cta_tri_light(const Inst &in, int64_t lo, int64_t hi, uint32_t *sm, unsigned long long *cursor,
                              unsigned long long *bad, unsigned long long *work) {
  if (threadIdx.x == 0) *cursor = static_cast<unsigned long long>(lo);
  __syncthreads();
  uint32_t *rb = sm + (threadIdx.x >> 5) * tri::kLightCap;
  tri::Tally t;
  for (;;) {
    unsigned long long r = 0;
    if (lane_id() == 0) r = atomicAdd(cursor, 1ull);
    r = __shfl_sync(0xffffffffu, r, 0);
    if (static_cast<int64_t>(r) >= hi) break;
    tri::light_row(in.in, in.aux, static_cast<int64_t>(r), in.m, in.bits, rb, t);
  }
  flush_tri(t, in, bad, work);
}

__device__ void cta_tri_heavy(const Inst &in, int64_t lo, int64_t hi, uint32_t *sm, unsigned long long *bad,
                              unsigned long long *work) {
  const int64_t nwords = in.bits >> 5;
  for (int64_t w = threadIdx.x; w < nwords; w += kThreads) sm[w] = 0;
  __syncthreads();
  tri::Tally t;
  for (int64_t r = lo; r < hi; r++) {
    const int64_t b = in.in[r], e = in.in[r + 1];  // the same value in every thread
    if (!tri::is_heavy(r, b, e, in.bits)) continue;
    tri::heavy_row<int64_t, kThreads>(in.in, in.aux, r, in.m, sm, static_cast<uint32_t>(nwords - 1), t);
  }
  flush_tri(t, in, bad, work);
}

__global__ void __launch_bounds__(kThreads, 2)
    batch_kernel(const Task *__restrict__ tasks, int64_t ntasks, const Inst *__restrict__ insts,
                 unsigned long long *__restrict__ head, unsigned long long *__restrict__ bad,
                 unsigned long long *__restrict__ work) {
  extern __shared__ __align__(16) uint32_t sm[];
  __shared__ long long sel;
  __shared__ unsigned long long row_cursor;
  for (;;) {
    __syncthreads();  // the previous task is finished with shared memory
    if (threadIdx.x == 0) {
      const unsigned long long t = atomicAdd(head, 1ull);
      sel = t < static_cast<unsigned long long>(ntasks) ? static_cast<long long>(t) : -1ll;
    }
    __syncthreads();
    const long long ti = sel;
    if (ti < 0) break;
    const Task tk = tasks[ti];
    const Inst in = insts[tk.inst];
    unsigned long long *ib = bad + tk.inst;
    switch (tk.kind) {
      case kHistoSmem: cta_histo_smem(in, tk.lo, tk.hi, sm, ib); break;
      case kHistoL2: cta_histo_l2(in, tk.lo, tk.hi, ib); break;
      case kIgDirect: cta_ig(in, tk.lo, tk.hi, ib); break;
      case kTriLight: cta_tri_light(in, tk.lo, tk.hi, sm, &row_cursor, ib, work); break;
      case kTriHeavy: cta_tri_heavy(in, tk.lo, tk.hi, sm, ib, work); break;
      default: break;
    }
  }
}

bool g_batch_attr[64];

// size class of an instance: 0 small (< 2^18 elements), 1 medium (< 2^23), 2 large
int size_class(int64_t n) { return n < (int64_t(1) << 18) ? 0 : (n < (int64_t(1) << 23) ? 1 : 2); }

int64_t tuned(const char *base, int cls, int64_t dflt) {
  static const char *suffix[3] = {".small", ".medium", ".large"};
  char name[64];
  snprintf(name, sizeof(name), "%s%s", base, suffix[cls]);
  const int64_t v = knob(name);
  return v > 0 ? v : dflt;
}

}  // namespace

Inst make_inst(const bale_instance_t &x) {
  Inst d;
  d.kind = x.kind;
  d.shift = x.shift;
  d.n = x.n;
  d.m = x.m;
  d.out = x.out;
  d.in = x.in;
  d.aux = x.aux;
  d.bits = x.kind == BALE_KIND_TRIANGLES ? tri::bitmap_bits(x.n) : 0;
  return d;
}

void plan_tasks(const bale_instance_t &x, int32_t k, const int64_t *host_off, std::vector<Planned> &plan) {
  if (x.n == 0) return;
  const int cls = size_class(x.kind == BALE_KIND_TRIANGLES ? x.m : x.n);
  if (x.kind == BALE_KIND_HISTO) {
    if (x.m <= kSmemCounters) {
      // each task sees several updates per counter so the flush stays cheap
      int64_t tile = tuned("batch.histo_tile", cls, int64_t(1) << 17);
      tile = std::max<int64_t>(tile, 4 * x.m);
      for (int64_t lo = 0; lo < x.n; lo += tile)
        plan.push_back({{kHistoSmem, k, lo, std::min(x.n, lo + tile)},
                        static_cast<double>(std::min(tile, x.n - lo)) * 0.5 + static_cast<double>(x.m)});
    } else {
      const int64_t tile = tuned("batch.histo_l2_tile", cls, int64_t(1) << 17);
      for (int64_t lo = 0; lo < x.n; lo += tile)
        plan.push_back({{kHistoL2, k, lo, std::min(x.n, lo + tile)}, static_cast<double>(std::min(tile, x.n - lo))});
    }
  } else if (x.kind == BALE_KIND_IG) {
    const int64_t tile = tuned("batch.ig_tile", cls, int64_t(1) << 17);
    for (int64_t lo = 0; lo < x.n; lo += tile)
      plan.push_back({{kIgDirect, k, lo, std::min(x.n, lo + tile)},
                      static_cast<double>(std::min(tile, x.n - lo)) * (x.m * 8 > (int64_t(96) << 20) ? 2.0 : 1.0)});
  } else {
    // Row degrees are known exactly and cheaply: every heavy row gets its own
    // task (or a few per task); light rows are cut into tasks of about the
    // same number of nonzeros.
    const int64_t bits = tri::bitmap_bits(x.n);
    const int64_t lim = std::min<int64_t>(x.n, bits);
    const double avg = static_cast<double>(x.m) / static_cast<double>(x.n);
    const int64_t hrows = tuned("batch.tri_heavy_rows", cls, 1);
    for (int64_t i = 0; i < lim;) {
      if (host_off[i + 1] - host_off[i] >= tri::kHeavyMinDeg) {
        int64_t j = i, nh = 0;
        double c = 0;
        while (j < lim && nh < hrows) {
          const int64_t dj = host_off[j + 1] - host_off[j];
          if (dj >= tri::kHeavyMinDeg) {
            c += static_cast<double>(dj) * 4.0 * avg;
            nh++;
          }
          j++;
        }
        plan.push_back({{kTriHeavy, k, i, j}, c});
        i = j;
      } else {
        i++;
      }
    }
    const int64_t lnnz = tuned("batch.tri_light_rows", cls, 1 << 15);  // nonzeros per light task
    int64_t lo = 0;
    while (lo < x.n) {
      int64_t hi = lo, acc = 0;
      while (hi < x.n && (hi == lo || acc < lnnz)) {
        acc += host_off[hi + 1] - host_off[hi];
        hi++;
      }
      plan.push_back({{kTriLight, k, lo, hi}, static_cast<double>(acc) * 2.0 * avg + 64.0});
      lo = hi;
    }
  }
}

int64_t queue_blocks() {
  const int dev = current_device();
  if (dev >= 0 && dev < 64 && !g_batch_attr[dev]) {
    if (cudaFuncSetAttribute(batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(kSmemBytes)) != cudaSuccess)
      return 0;
    g_batch_attr[dev] = true;
  }
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_kernel, kThreads, kSmemBytes) != cudaSuccess || occ < 1)
    occ = 1;
  return static_cast<int64_t>(num_sms()) * occ;
}

int launch_queue(const Task *d_tasks, int64_t ntasks, const Inst *d_inst, unsigned long long *words,
                 unsigned long long *bad, int64_t blocks, cudaStream_t stream) {
  if (ntasks <= 0) return BALE_OK;
  if (blocks > ntasks) blocks = ntasks;
  if (blocks < 1) blocks = 1;
  batch_kernel<<<static_cast<unsigned>(blocks), kThreads, kSmemBytes, stream>>>(d_tasks, ntasks, d_inst, words, bad,
                                                                                  words + 1);
  BALE_CUDA_OK(cudaGetLastError());
  return BALE_OK;
}

}  // namespace q
}  // namespace bale

struct bale_batch {
  int device = 0;
  int64_t count = 0;
  bale::q::Inst *d_inst = nullptr;
  bale::q::Task *d_tasks = nullptr;
  int64_t ntasks = 0;
  int64_t ntasks_kind[5] = {0, 0, 0, 0, 0};
  unsigned long long *d_words = nullptr;  // [0] queue head, [1] work, then 4 words per standalone instance
  unsigned long long *d_bad = nullptr;    // per instance
  void *d_ws = nullptr;                   // workspaces of the standalone instances, one region each
  std::vector<int64_t> standalone;
  std::vector<int> side_of;  // per instance: its side stream, or -1 (work queue)
  cudaStream_t s_main = nullptr;
  std::vector<cudaStream_t> s_side;
  cudaEvent_t ev_fork = nullptr;
  std::vector<cudaEvent_t> ev_join;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace bale {
namespace {

void destroy(bale_batch *b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  for (auto e : b->ev_join) cudaEventDestroy(e);
  if (b->s_main) cudaStreamDestroy(b->s_main);
  for (auto st : b->s_side) cudaStreamDestroy(st);
  cudaFree(b->d_inst);
  cudaFree(b->d_tasks);
  cudaFree(b->d_words);
  cudaFree(b->d_bad);
  cudaFree(b->d_ws);
  delete b;
}


}  // namespace
namespace q {

// Would this instance use the region-partitioned kernels on its own?
bool partition_worthy(const bale_instance_t &x) {
  if (x.kind == BALE_KIND_IG) return ig_partition_for(x.n, x.m, x.out, x.in);
  if (x.kind == BALE_KIND_HISTO) return histo_mode_for(x.n, x.m, x.in) == 3;
  return false;
}

// Instances large enough to fill the GPU by themselves run as their own
// kernels (the same ones the per-instance entry points use) on side streams
// of the graph; the work queue takes the rest.
bool goes_standalone(const bale_instance_t &x) {
  if (knob("batch.standalone") == 0 || x.n == 0) return false;
  if (partition_worthy(x)) return true;
  if (x.kind == BALE_KIND_TRIANGLES) return x.m >= knob_or("batch.standalone_min_edges", int64_t(1) << 21);
  return x.n >= knob_or("batch.standalone_min", int64_t(1) << 23);
}

size_t standalone_ws(const bale_instance_t &x) {
  size_t need = 0;
  if (x.kind == BALE_KIND_IG && partition_worthy(x)) need = ig_part_workspace_bytes(x.n, x.m);
  else if (x.kind == BALE_KIND_HISTO && partition_worthy(x)) need = histo_part_workspace_bytes(x.n, x.m);
  else if (x.kind == BALE_KIND_TRIANGLES)
    need = tri_wedge_supported(x.n, x.m) ? tri_wedge_workspace_bytes(x.n, x.m) : tri_hybrid_workspace_bytes(x.n, x.m);
  return (need + 255) & ~size_t(255);
}

double standalone_cost(const bale_instance_t &x) {
  if (x.kind == BALE_KIND_TRIANGLES) return 15.0 * static_cast<double>(x.m);
  return static_cast<double>(x.n) * (x.kind == BALE_KIND_IG ? 1.5 : 1.0);
}

int launch_standalone(const bale_instance_t &x, unsigned long long *bad, void *ws, unsigned long long *words,
                      cudaStream_t st) {
  if (x.kind == BALE_KIND_IG) {
    if (partition_worthy(x)) return launch_ig_partitioned(x.out, x.in, x.n, x.aux, x.m, x.shift, bad, ws, words, st);
    return launch_ig(x.out, x.in, x.n, x.aux, x.m, x.shift, bad, st);
  }
  if (x.kind == BALE_KIND_HISTO) {
    if (partition_worthy(x)) return launch_histo_partitioned(x.out, x.m, x.in, x.n, x.shift, bad, ws, words, st);
    return launch_histo(x.out, x.m, x.in, x.n, x.shift, bad, st);
  }
  if (tri_wedge_supported(x.n, x.m))
    return launch_triangle_wedge(x.in, x.aux, x.n, x.m, reinterpret_cast<unsigned long long *>(x.out), nullptr, bad,
                                 ws, words, st);
  return launch_triangle_hybrid(x.in, x.aux, x.n, x.m, reinterpret_cast<unsigned long long *>(x.out), nullptr, bad,
                                ws, words, 8, st);
}

}  // namespace q

bool instance_valid(const bale_instance_t &x) {
  const bool ok_kind = x.kind == BALE_KIND_HISTO || x.kind == BALE_KIND_IG || x.kind == BALE_KIND_TRIANGLES;
  const bool ok_shift = x.shift == 0 || x.shift == 16;
  const bool ok_ptr = x.kind == BALE_KIND_TRIANGLES
                          ? (x.out && (x.n == 0 || x.in) && (x.m == 0 || x.aux))
                          : (x.n == 0 || (x.in && x.out && (x.kind != BALE_KIND_IG || x.m == 0 || x.aux)));
  return ok_kind && ok_shift && x.n >= 0 && x.m >= 0 && ok_ptr &&
         !(x.kind == BALE_KIND_TRIANGLES && x.n >= 0xffffffffll);
}

}  // namespace bale

using namespace bale;
using namespace bale::q;

extern "C" {

bale_batch_t *bale_batch_create(const bale_instance_t *inst, int64_t count) {
  if (count < 0 || (count > 0 && !inst)) {
    set_error("bale_batch_create: bad arguments");
    return nullptr;
  }
  bale_batch *b = new (std::nothrow) bale_batch();
  if (!b) {
    set_error("bale_batch_create: out of host memory");
    return nullptr;
  }
  b->count = count;
  if (cudaGetDevice(&b->device) != cudaSuccess) b->device = 0;
#define BATCH_CUDA(expr)                                                                  \
  do {                                                                                    \
    cudaError_t _e = (expr);                                                              \
    if (_e != cudaSuccess) {                                                              \
      set_error("bale_batch_create: %s failed: %s", #expr, cudaGetErrorString(_e));       \
      cudaGetLastError();                                                                 \
      destroy(b);                                                                         \
      return nullptr;                                                                     \
    }                                                                                     \
  } while (0)

  std::vector<Inst> di(static_cast<size_t>(count));
  for (int64_t k = 0; k < count; k++) {
    if (!instance_valid(inst[k])) {
      set_error("bale_batch_create: instance %lld is invalid", static_cast<long long>(k));
      destroy(b);
      return nullptr;
    }
    di[static_cast<size_t>(k)] = make_inst(inst[k]);
  }

  // ---- plan: standalone instances, then the work queue ----
  std::vector<Planned> plan;
  std::vector<size_t> ws_off;
  size_t ws_total = 256;
  std::vector<int64_t> host_off;
  for (int64_t k = 0; k < count; k++) {
    const bale_instance_t &x = inst[k];
    if (x.n == 0) continue;
    if (goes_standalone(x)) {
      b->standalone.push_back(k);
      ws_off.push_back(ws_total);
      ws_total += standalone_ws(x);
      continue;
    }
    if (x.kind == BALE_KIND_TRIANGLES) {
      host_off.resize(static_cast<size_t>(x.n + 1));
      BATCH_CUDA(cudaMemcpy(host_off.data(), x.in, sizeof(int64_t) * static_cast<size_t>(x.n + 1),
                            cudaMemcpyDeviceToHost));
    }
    plan_tasks(x, static_cast<int32_t>(k), host_off.data(), plan);
  }
  // longest first
  std::stable_sort(plan.begin(), plan.end(), [](const Planned &a, const Planned &c) { return a.cost > c.cost; });
  std::vector<Task> tasks;
  tasks.reserve(plan.size());
  for (auto &p : plan) {
    tasks.push_back(p.t);
    b->ntasks_kind[p.t.kind]++;
  }
  b->ntasks = static_cast<int64_t>(tasks.size());

  // ---- device state ----
  const size_t nw = 2 + 4 * b->standalone.size();
  BATCH_CUDA(cudaMalloc(&b->d_inst, sizeof(Inst) * std::max<size_t>(1, di.size())));
  BATCH_CUDA(cudaMalloc(&b->d_tasks, sizeof(Task) * std::max<size_t>(1, tasks.size())));
  BATCH_CUDA(cudaMalloc(&b->d_words, sizeof(unsigned long long) * nw));
  BATCH_CUDA(cudaMalloc(&b->d_bad, sizeof(unsigned long long) * std::max<int64_t>(1, count)));
  if (!b->standalone.empty()) BATCH_CUDA(cudaMalloc(&b->d_ws, ws_total));
  if (!di.empty()) BATCH_CUDA(cudaMemcpy(b->d_inst, di.data(), sizeof(Inst) * di.size(), cudaMemcpyHostToDevice));
  if (!tasks.empty())
    BATCH_CUDA(cudaMemcpy(b->d_tasks, tasks.data(), sizeof(Task) * tasks.size(), cudaMemcpyHostToDevice));
  BATCH_CUDA(cudaMemset(b->d_words, 0, sizeof(unsigned long long) * nw));
  BATCH_CUDA(cudaMemset(b->d_bad, 0, sizeof(unsigned long long) * std::max<int64_t>(1, count)));
  int64_t blocks = queue_blocks();
  if (blocks < 1) {
    set_error("bale_batch_create: the queue kernel cannot be configured");
    destroy(b);
    return nullptr;
  }
  const int64_t qb = knob("batch.queue_blocks");
  if (qb > 0 && qb < blocks) blocks = qb;

  // side streams for the standalone instances, longest first to the least loaded
  int64_t nside = knob_or("batch.streams", 4);
  if (nside < 1) nside = 1;
  nside = std::min<int64_t>(nside, static_cast<int64_t>(b->standalone.size()));
  std::vector<int> lane(b->standalone.size(), 0);
  {
    std::vector<size_t> order(b->standalone.size());
    for (size_t s = 0; s < order.size(); s++) order[s] = s;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t c) {
      return standalone_cost(inst[b->standalone[a]]) > standalone_cost(inst[b->standalone[c]]);
    });
    std::vector<double> load(static_cast<size_t>(std::max<int64_t>(1, nside)), 0.0);
    std::vector<int64_t> st2;
    std::vector<size_t> off2;
    std::vector<int> lane2;
    for (size_t s : order) {
      const size_t l = static_cast<size_t>(std::min_element(load.begin(), load.end()) - load.begin());
      load[l] += standalone_cost(inst[b->standalone[s]]);
      st2.push_back(b->standalone[s]);
      off2.push_back(ws_off[s]);
      lane2.push_back(static_cast<int>(l));
    }
    b->standalone.swap(st2);
    ws_off.swap(off2);
    lane.swap(lane2);
  }
  b->side_of.assign(static_cast<size_t>(count), -1);
  for (size_t s = 0; s < b->standalone.size(); s++) b->side_of[static_cast<size_t>(b->standalone[s])] = lane[s];

  // ---- capture one run as a graph ----
  BATCH_CUDA(cudaStreamCreateWithFlags(&b->s_main, cudaStreamNonBlocking));
  BATCH_CUDA(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming));
  for (int64_t l = 0; l < nside; l++) {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    BATCH_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    b->s_side.push_back(st);
    BATCH_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    b->ev_join.push_back(ev);
  }
  BATCH_CUDA(cudaStreamBeginCapture(b->s_main, cudaStreamCaptureModeThreadLocal));
  bool cap_ok = true;
  cap_ok &= cudaMemsetAsync(b->d_words, 0, 2 * sizeof(unsigned long long), b->s_main) == cudaSuccess;
  cap_ok &= cudaMemsetAsync(b->d_bad, 0, sizeof(unsigned long long) * std::max<int64_t>(1, count), b->s_main) ==
            cudaSuccess;
  if (nside > 0) {
    cap_ok &= cudaEventRecord(b->ev_fork, b->s_main) == cudaSuccess;
    for (int64_t l = 0; l < nside; l++) cap_ok &= cudaStreamWaitEvent(b->s_side[l], b->ev_fork, 0) == cudaSuccess;
    for (size_t s = 0; s < b->standalone.size() && cap_ok; s++) {
      const int64_t k = b->standalone[s];
      void *ws = static_cast<char *>(b->d_ws) + ws_off[s];
      cap_ok &= launch_standalone(inst[k], b->d_bad + k, ws, b->d_words + 2 + 4 * s, b->s_side[lane[s]]) == BALE_OK;
    }
    for (int64_t l = 0; l < nside; l++) cap_ok &= cudaEventRecord(b->ev_join[l], b->s_side[l]) == cudaSuccess;
  }
  cap_ok &= launch_queue(b->d_tasks, b->ntasks, b->d_inst, b->d_words, b->d_bad, blocks, b->s_main) == BALE_OK;
  for (int64_t l = 0; l < nside; l++) cap_ok &= cudaStreamWaitEvent(b->s_main, b->ev_join[l], 0) == cudaSuccess;
  cudaError_t ce = cudaStreamEndCapture(b->s_main, &b->graph);
  if (!cap_ok || ce != cudaSuccess || !b->graph) {
    set_error("bale_batch_create: graph capture failed: %s",
              cudaGetErrorString(ce != cudaSuccess ? ce : cudaGetLastError()));
    cudaGetLastError();
    destroy(b);
    return nullptr;
  }
  BATCH_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
#undef BATCH_CUDA
  return b;
}

int bale_batch_run(bale_batch_t *b, void *stream) {
  if (!b || !b->exec) {
    set_error("bale_batch_run: no batch");
    return BALE_EINVAL;
  }
  BALE_CUDA_OK(cudaGraphLaunch(b->exec, static_cast<cudaStream_t>(stream)));
  return BALE_OK;
}

int bale_batch_bad(bale_batch_t *b, int64_t *bad, int64_t count) {
  if (!b || !bad || count != b->count) {
    set_error("bale_batch_bad: bad arguments");
    return BALE_EINVAL;
  }
  if (count == 0) return BALE_OK;
  BALE_CUDA_OK(cudaMemcpy(bad, b->d_bad, sizeof(int64_t) * static_cast<size_t>(count), cudaMemcpyDeviceToHost));
  return BALE_OK;
}

int bale_batch_stats(bale_batch_t *b, int64_t *out, int n) {
  if (!b || !out || n <= 0) return BALE_EINVAL;
  const int64_t v[9] = {b->ntasks,
                        b->ntasks_kind[kHistoSmem],
                        b->ntasks_kind[kHistoL2],
                        b->ntasks_kind[kIgDirect],
                        b->ntasks_kind[kTriLight],
                        b->ntasks_kind[kTriHeavy],
                        static_cast<int64_t>(b->standalone.size()),
                        b->count,
                        static_cast<int64_t>(b->s_side.size())};
  for (int i = 0; i < n; i++) out[i] = i < 9 ? v[i] : -1;
  return BALE_OK;
}

int bale_batch_plan(bale_batch_t *b, int64_t *side, int64_t count) {
  if (!b || !side || count != b->count) {
    set_error("bale_batch_plan: bad arguments");
    return BALE_EINVAL;
  }
  for (int64_t k = 0; k < count; k++) side[k] = b->side_of[static_cast<size_t>(k)];
  return BALE_OK;
}

void bale_batch_destroy(bale_batch_t *b) { destroy(b); }

}  // extern "C"
