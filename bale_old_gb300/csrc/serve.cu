// serve.cu -- the serving loop: continuous batching of histo / ig / triangle
// requests against tables, counters and graphs kept resident in HBM.
//
// Objects (ig tables, histo counter arrays, CSR graphs) are registered once
// and stay in device memory; registration is refused (BALE_EBUSY) when free
// HBM would drop below a reserve.  bale_server_run then replays a trace of
// requests in real time:
//
//  * a request is admitted when it has arrived, a slot is free and its
//    buffers (index, output) fit in the server's preallocated arena; its
//    index array is uploaded on a copy stream while the GPU works;
//  * every admitted request is cut into the persistent queue kernel's tasks
//    (the batched form's planner) and the GPU runs "ticks": one queue launch
//    over a bounded slice of every active request's remaining tasks, so a
//    request that arrives while a long one is running joins at the next tick
//    instead of waiting for it to finish;
//  * a request large enough to fill the GPU by itself (the batched form's
//    standalone rule) skips the queue: it runs as its own specialised kernels
//    (region-partitioned ig / histo; for a graph, the wedge count kernel over
//    the prepared form built at registration, or beyond the wedge kernels'
//    32-bit limits the hybrid's heavy/light kernels over its resident column
//    copy) on one of a few express streams, concurrently with the ticks;
//  * when a request's last task has run, its result is copied back on a copy
//    stream (ig values, the triangle count) and its arena space is freed.
//    The express requests' uploads and downloads have copy streams of their
//    own, so a small request's copies do not queue behind a large one's
//    (they share the link, but a small copy finishes in microseconds).
//
// Latency is completion time minus arrival time.  Results are exactly the
// per-instance entry points': ig overwrites the caller's out, triangles write
// one int64, histo adds into the resident counters.  The host thread polls
// events and gives up with BALE_ETIMEDOUT if nothing progresses for 120 s.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <new>
#include <thread>
#include <vector>

#include "batch.cuh"

namespace {

using bale::q::Inst;
using bale::q::Planned;
using bale::q::Task;

struct Object {
  int32_t kind = -1;  // BALE_KIND_IG (table), BALE_KIND_HISTO (counts), BALE_KIND_TRIANGLES (graph)
  int64_t n = 0, m = 0;
  int64_t *d_a = nullptr;             // table / counts / row offsets
  int64_t *d_b = nullptr;             // graph nonzeros
  char *d_c = nullptr;                // graphs: the triangle kernels' prepared form
  bool wedge = false;                 // ... for the wedge kernels (else the hybrid's)
  uint32_t *col32 = nullptr, *heavy = nullptr;
  unsigned long long *nheavy = nullptr;
  std::vector<int64_t> host_offsets;  // graphs: for the planner
};

// First-fit allocator over one preallocated device arena (256-byte units).
class Arena {
 public:
  void init(char *base, size_t bytes) {
    base_ = base;
    free_.clear();
    if (bytes) free_[0] = bytes;
  }
  char *alloc(size_t bytes) {
    bytes = (bytes + 255) & ~size_t(255);
    if (bytes == 0) bytes = 256;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        const size_t off = it->first, rest = it->second - bytes;
        free_.erase(it);
        if (rest) free_[off + bytes] = rest;
        return base_ + off;
      }
    }
    return nullptr;
  }
  void release(char *p, size_t bytes) {
    bytes = (bytes + 255) & ~size_t(255);
    if (bytes == 0) bytes = 256;
    size_t off = static_cast<size_t>(p - base_);
    auto next = free_.lower_bound(off);
    if (next != free_.begin()) {
      auto prev = std::prev(next);
      if (prev->first + prev->second == off) {
        off = prev->first;
        bytes += prev->second;
        free_.erase(prev);
      }
    }
    next = free_.lower_bound(off);
    if (next != free_.end() && off + bytes == next->first) {
      bytes += next->second;
      free_.erase(next);
    }
    free_[off] = bytes;
  }

 private:
  char *base_ = nullptr;
  std::map<size_t, size_t> free_;
};

double now_s() {
  using namespace std::chrono;
  return duration_cast<duration<double>>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace

struct bale_server {
  int device = 0;
  std::vector<Object> objects;
  char *d_arena = nullptr;
  size_t arena_bytes = 0;
  int max_active = 64;
  int64_t reserve_bytes = int64_t(1) << 30;
  cudaStream_t s_compute = nullptr, s_up = nullptr, s_down = nullptr;
  // the large (express) requests' index uploads and result downloads, so
  // that a small request's copies never queue behind a gigabyte of them
  cudaStream_t s_up_big = nullptr, s_down_big = nullptr;
  static constexpr int kExpress = 4;
  cudaStream_t s_express[kExpress] = {};
};

namespace {

struct Active {
  ~Active() {
    if (uploaded) cudaEventDestroy(uploaded);
    if (downloaded) cudaEventDestroy(downloaded);
    if (xstart) cudaEventDestroy(xstart);
    if (xdone) cudaEventDestroy(xdone);
  }
  int64_t id = 0;
  char *buf = nullptr;
  size_t buf_bytes = 0;
  std::vector<Task> tasks;
  std::vector<double> cost;
  size_t next = 0;      // first task not yet launched
  size_t finished = 0;  // tasks whose tick completed
  cudaEvent_t uploaded = nullptr;
  cudaEvent_t downloaded = nullptr;
  bool downloading = false;
  // express requests: their own kernels on an express stream
  bool express = false, computed = false;
  int lane = 0;
  double xcost = 0;
  cudaEvent_t xstart = nullptr, xdone = nullptr;
};

void server_free(bale_server *s) {
  if (!s) return;
  for (auto &o : s->objects) {
    cudaFree(o.d_a);
    cudaFree(o.d_b);
    cudaFree(o.d_c);
  }
  cudaFree(s->d_arena);
  if (s->s_compute) cudaStreamDestroy(s->s_compute);
  if (s->s_up) cudaStreamDestroy(s->s_up);
  if (s->s_down) cudaStreamDestroy(s->s_down);
  if (s->s_up_big) cudaStreamDestroy(s->s_up_big);
  if (s->s_down_big) cudaStreamDestroy(s->s_down_big);
  for (auto st : s->s_express)
    if (st) cudaStreamDestroy(st);
  delete s;
}

// Admission by free HBM: an allocation must leave the reserve free.
int admit_alloc(bale_server *s, void **p, size_t bytes) {
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return BALE_ECUDA;
  const int64_t reserve = bale::knob_or("serve.reserve_bytes", s->reserve_bytes);  // read live
  if (static_cast<int64_t>(free_b) - static_cast<int64_t>(bytes) < reserve) {
    bale::set_error("bale_server: %zu bytes would leave less than the %lld-byte reserve of free HBM", bytes,
                    static_cast<long long>(reserve));
    return BALE_EBUSY;
  }
  if (cudaMalloc(p, bytes ? bytes : 256) != cudaSuccess) {
    cudaGetLastError();
    bale::set_error("bale_server: cudaMalloc(%zu) failed", bytes);
    return BALE_ENOMEM;
  }
  return BALE_OK;
}

int add_object(bale_server *s, Object &&o) {
  s->objects.push_back(std::move(o));
  return static_cast<int>(s->objects.size() - 1);
}

}  // namespace

using namespace bale;

extern "C" {

bale_server_t *bale_server_create(int64_t arena_bytes, int max_active) {
  bale_server *s = new (std::nothrow) bale_server();
  if (!s) return nullptr;
  if (cudaGetDevice(&s->device) != cudaSuccess) s->device = 0;
  s->max_active = max_active > 0 ? max_active : 64;
  if (arena_bytes <= 0) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      set_error("bale_server_create: cudaMemGetInfo failed");
      server_free(s);
      return nullptr;
    }
    arena_bytes = static_cast<int64_t>(free_b / 4);
  }
  void *p = nullptr;
  if (admit_alloc(s, &p, static_cast<size_t>(arena_bytes)) != BALE_OK) {
    server_free(s);
    return nullptr;
  }
  s->d_arena = static_cast<char *>(p);
  s->arena_bytes = static_cast<size_t>(arena_bytes);
  if (cudaStreamCreateWithFlags(&s->s_compute, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s->s_up, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s->s_down, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s->s_up_big, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s->s_down_big, cudaStreamNonBlocking) != cudaSuccess ||
      [&] {
        for (auto &st : s->s_express)
          if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return true;
        return false;
      }()) {
    set_error("bale_server_create: stream creation failed");
    server_free(s);
    return nullptr;
  }
  return s;
}

int bale_server_add_table(bale_server_t *s, const int64_t *host_table, int64_t n) {
  if (!s || n < 0 || (n > 0 && !host_table)) return -BALE_EINVAL;
  Object o;
  o.kind = BALE_KIND_IG;
  o.n = n;
  void *p = nullptr;
  int rc = admit_alloc(s, &p, static_cast<size_t>(n) * 8);
  if (rc != BALE_OK) return -rc;
  o.d_a = static_cast<int64_t *>(p);
  if (n && cudaMemcpy(o.d_a, host_table, static_cast<size_t>(n) * 8, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(o.d_a);
    set_error("bale_server_add_table: upload failed");
    return -BALE_ECUDA;
  }
  return add_object(s, std::move(o));
}

int bale_server_add_counts(bale_server_t *s, int64_t ncounts) {
  if (!s || ncounts < 0) return -BALE_EINVAL;
  Object o;
  o.kind = BALE_KIND_HISTO;
  o.n = ncounts;
  void *p = nullptr;
  int rc = admit_alloc(s, &p, static_cast<size_t>(ncounts) * 8);
  if (rc != BALE_OK) return -rc;
  o.d_a = static_cast<int64_t *>(p);
  if (cudaMemset(o.d_a, 0, static_cast<size_t>(ncounts) * 8) != cudaSuccess) {
    cudaFree(o.d_a);
    return -BALE_ECUDA;
  }
  return add_object(s, std::move(o));
}

int bale_server_add_graph(bale_server_t *s, const int64_t *offset, const int64_t *nonzero, int64_t numrows,
                          int64_t nnz) {
  if (!s || numrows < 0 || numrows >= 0xffffffffll || nnz < 0 || !offset || (nnz > 0 && !nonzero)) return -BALE_EINVAL;
  if (offset[numrows] != nnz) {
    set_error("bale_server_add_graph: offset[numrows] != nnz");
    return -BALE_EINVAL;
  }
  Object o;
  o.kind = BALE_KIND_TRIANGLES;
  o.n = numrows;
  o.m = nnz;
  // the CSR arrays plus the triangle kernels' prepared form, built once here:
  // the wedge kernels' column copy and transpose, or (beyond their 2^32
  // limits) the hybrid's column copy and heavy-row list
  o.wedge = tri_wedge_supported(numrows, nnz);
  const size_t hyb = (o.wedge ? tri_wedge_workspace_bytes(numrows, nnz) : tri_hybrid_workspace_bytes(numrows, nnz)) +
                     256;
  void *a = nullptr, *b = nullptr, *c = nullptr;
  int rc = admit_alloc(s, &a, static_cast<size_t>(numrows + 1) * 8 + static_cast<size_t>(nnz) * 8 + hyb + 256);
  if (rc != BALE_OK) return -rc;
  cudaFree(a);  // admitted: allocate the three arrays
  a = nullptr;
  if (cudaMalloc(&a, static_cast<size_t>(numrows + 1) * 8) != cudaSuccess ||
      cudaMalloc(&b, static_cast<size_t>(nnz > 0 ? nnz : 1) * 8) != cudaSuccess ||
      cudaMalloc(&c, hyb + 256) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(a);
    cudaFree(b);
    return -BALE_ENOMEM;
  }
  o.d_a = static_cast<int64_t *>(a);
  o.d_b = static_cast<int64_t *>(b);
  o.d_c = static_cast<char *>(c);
  unsigned long long *vbad = reinterpret_cast<unsigned long long *>(o.d_c + hyb);  // malformed entries
  o.col32 = reinterpret_cast<uint32_t *>(o.d_c);
  o.heavy = reinterpret_cast<uint32_t *>(o.d_c + ((static_cast<size_t>(nnz > 0 ? nnz : 1) * 4 + 255) & ~size_t(255)));
  o.nheavy = reinterpret_cast<unsigned long long *>(o.d_c + hyb - 256);
  unsigned long long h_bad = 0;
  const bool ok =
      cudaMemcpy(o.d_a, offset, static_cast<size_t>(numrows + 1) * 8, cudaMemcpyHostToDevice) == cudaSuccess &&
      (nnz == 0 || cudaMemcpy(o.d_b, nonzero, static_cast<size_t>(nnz) * 8, cudaMemcpyHostToDevice) == cudaSuccess) &&
      cudaMemsetAsync(vbad, 0, 8, s->s_compute) == cudaSuccess &&
      (o.wedge ? tri_wedge_prepare(o.d_a, o.d_b, numrows, nnz, o.d_c, vbad, s->s_compute)
               : tri_hybrid_prepare(o.d_a, o.d_b, numrows, nnz, o.col32, o.heavy, o.nheavy, s->s_compute)) ==
          BALE_OK &&
      cudaMemcpyAsync(&h_bad, vbad, 8, cudaMemcpyDeviceToHost, s->s_compute) == cudaSuccess &&
      cudaStreamSynchronize(s->s_compute) == cudaSuccess;
  if (!ok || h_bad) {
    cudaGetLastError();
    cudaFree(a);
    cudaFree(b);
    cudaFree(c);
    if (h_bad) {
      set_error("bale_server_add_graph: %llu malformed entries (rows must ascend inside [0,i))", h_bad);
      return -BALE_EINPUT;
    }
    return -BALE_ECUDA;
  }
  o.host_offsets.assign(offset, offset + numrows + 1);
  return add_object(s, std::move(o));
}

int bale_server_read_counts(bale_server_t *s, int object, int64_t *host_counts, int64_t ncounts) {
  if (!s || object < 0 || object >= static_cast<int>(s->objects.size())) return BALE_EINVAL;
  const Object &o = s->objects[static_cast<size_t>(object)];
  if (o.kind != BALE_KIND_HISTO || ncounts != o.n || (ncounts && !host_counts)) return BALE_EINVAL;
  BALE_CUDA_OK(cudaMemcpy(host_counts, o.d_a, static_cast<size_t>(ncounts) * 8, cudaMemcpyDeviceToHost));
  return BALE_OK;
}

int bale_server_run(bale_server_t *s, const bale_request_t *req, int64_t nreq, double *latency,
                    bale_serve_stats_t *stats) {
  if (!s || nreq < 0 || (nreq > 0 && (!req || !latency))) {
    set_error("bale_server_run: bad arguments");
    return BALE_EINVAL;
  }
  bale_serve_stats_t st;
  std::memset(&st, 0, sizeof(st));
  if (nreq == 0) {
    if (stats) *stats = st;
    return BALE_OK;
  }
  // validate every request before anything runs
  for (int64_t r = 0; r < nreq; r++) {
    const bale_request_t &x = req[r];
    const bool ok_obj = x.object >= 0 && x.object < static_cast<int32_t>(s->objects.size());
    const bool ok = ok_obj && s->objects[static_cast<size_t>(x.object)].kind == x.kind && x.n >= 0 &&
                    (x.kind == BALE_KIND_TRIANGLES ? x.out != nullptr
                                                    : (x.n == 0 || (x.index && (x.kind != BALE_KIND_IG || x.out)))) &&
                    (x.shift == 0 || x.shift == 16);
    if (!ok) {
      set_error("bale_server_run: request %lld is invalid", static_cast<long long>(r));
      return BALE_EINVAL;
    }
  }
  int rc = BALE_OK;
  // device arrays indexed by request id: instance records, bad counts, triangle counts
  Inst *d_inst = nullptr;
  unsigned long long *d_bad = nullptr, *d_tri = nullptr, *d_words = nullptr, *d_xwords = nullptr;
  constexpr int kSlots = 2;  // ticks in flight: the next one is queued while one runs
  Task *d_tasks[kSlots] = {nullptr, nullptr};
  Task *h_tasks[kSlots] = {nullptr, nullptr};
  cudaEvent_t tick_done[kSlots] = {nullptr, nullptr};
  cudaEvent_t tick_start[kSlots] = {nullptr, nullptr};
  Inst *h_inst = nullptr;
  int64_t task_cap = knob_or("serve.tick_tasks", 4096);
  const double tick_cost = static_cast<double>(knob_or("serve.tick_cost", int64_t(1) << 24));
  const double req_cost = static_cast<double>(knob_or("serve.request_cost", int64_t(1) << 22));  // floor
  const int64_t blocks = q::queue_blocks();
  const bool express_on = knob("serve.express") != 0;
  const int nlanes = static_cast<int>(
      std::min<int64_t>(bale_server::kExpress, std::max<int64_t>(1, knob_or("serve.express_streams", 2))));
  const int rows_per_fetch = static_cast<int>(knob_or("tri.rows_per_fetch", 8));
  // serve.copy_lanes 1: every copy on one upload and one download stream;
  // 2 (default): the express requests' copies on streams of their own
  const bool split_copies = knob_or("serve.copy_lanes", 2) != 1;
  cudaStream_t up_big = split_copies ? s->s_up_big : s->s_up;
  cudaStream_t down_big = split_copies ? s->s_down_big : s->s_down;
  double lane_load[bale_server::kExpress] = {0, 0, 0, 0};
#define SRV_CUDA(expr)                                                                 \
  do {                                                                                 \
    cudaError_t _e = (expr);                                                           \
    if (_e != cudaSuccess) {                                                           \
      set_error("bale_server_run: %s failed: %s", #expr, cudaGetErrorString(_e));      \
      cudaGetLastError();                                                              \
      rc = BALE_ECUDA;                                                                 \
      goto done;                                                                       \
    }                                                                                  \
  } while (0)
  {
    SRV_CUDA(cudaMalloc(&d_inst, sizeof(Inst) * static_cast<size_t>(nreq)));
    SRV_CUDA(cudaMalloc(&d_bad, sizeof(unsigned long long) * static_cast<size_t>(nreq)));
    SRV_CUDA(cudaMalloc(&d_tri, sizeof(unsigned long long) * static_cast<size_t>(nreq)));
    SRV_CUDA(cudaMalloc(&d_words, sizeof(unsigned long long) * 2));
    SRV_CUDA(cudaMalloc(&d_xwords, sizeof(unsigned long long) * 4 * static_cast<size_t>(nreq)));
    for (int k = 0; k < kSlots; k++) {
      SRV_CUDA(cudaMalloc(&d_tasks[k], sizeof(Task) * static_cast<size_t>(task_cap)));
      SRV_CUDA(cudaMallocHost(&h_tasks[k], sizeof(Task) * static_cast<size_t>(task_cap)));
      SRV_CUDA(cudaEventCreate(&tick_done[k]));
      SRV_CUDA(cudaEventCreate(&tick_start[k]));
    }
    SRV_CUDA(cudaMallocHost(&h_inst, sizeof(Inst) * static_cast<size_t>(nreq)));
    SRV_CUDA(cudaMemset(d_bad, 0, sizeof(unsigned long long) * static_cast<size_t>(nreq)));
    SRV_CUDA(cudaMemset(d_tri, 0, sizeof(unsigned long long) * static_cast<size_t>(nreq)));
    if (blocks < 1) {
      set_error("bale_server_run: the queue kernel cannot be configured");
      rc = BALE_ECUDA;
      goto done;
    }
    Arena arena;
    arena.init(s->d_arena, s->arena_bytes);
    // requests in arrival order
    std::vector<int64_t> order(static_cast<size_t>(nreq));
    for (int64_t r = 0; r < nreq; r++) order[static_cast<size_t>(r)] = r;
    std::stable_sort(order.begin(), order.end(),
                     [&](int64_t a, int64_t b) { return req[a].arrival < req[b].arrival; });
    std::deque<int64_t> pending;
    std::vector<std::unique_ptr<Active>> active;
    std::vector<std::pair<Active *, size_t>> in_tick[kSlots];  // request, tasks it has in that tick
    std::vector<bool> waited(static_cast<size_t>(nreq), false);
    size_t next_arrival = 0;
    int64_t done_count = 0;
    bool tick_running[kSlots] = {false, false};
    int tick_next = 0;  // slot of the next tick to launch (ticks complete in launch order)
    size_t rr = 0;  // round-robin start
    double items = 0;
    const double t0 = now_s();
    double last_progress = t0;
    while (done_count < nreq) {
      const double now = now_s();
      st.loop_iters++;
      bool progressed = false;
      while (next_arrival < order.size() && req[order[next_arrival]].arrival <= now - t0)
        pending.push_back(order[next_arrival++]);
      // ---- admission: a free slot and room in the arena ----
      while (!pending.empty() && static_cast<int>(active.size()) < s->max_active) {
        const int64_t id = pending.front();
        const bale_request_t &x = req[id];
        const Object &o = s->objects[static_cast<size_t>(x.object)];
        // the public instance, with the arena pointers filled in once allocated
        bale_instance_t inst;
        inst.kind = x.kind;
        inst.shift = x.shift;
        inst.n = x.kind == BALE_KIND_TRIANGLES ? o.n : x.n;
        inst.m = x.kind == BALE_KIND_TRIANGLES ? o.m : o.n;
        inst.in = inst.aux = nullptr;
        inst.out = nullptr;
        size_t io = x.kind == BALE_KIND_IG ? 16 * static_cast<size_t>(x.n)
                    : x.kind == BALE_KIND_HISTO ? 8 * static_cast<size_t>(x.n) : 0;
        io = (io + 255) & ~size_t(255);
        bool express = false;
        size_t ws = 0;
        if (express_on) {
          bale_instance_t probe = inst;  // any 256-aligned pointers decide the rule
          probe.in = probe.aux = reinterpret_cast<const int64_t *>(s->d_arena);
          probe.out = reinterpret_cast<int64_t *>(s->d_arena);
          express = x.kind == BALE_KIND_TRIANGLES
                        ? o.m > 0 && o.m >= knob_or("batch.standalone_min_edges", int64_t(1) << 21)
                        : q::goes_standalone(probe);
          if (express && x.kind != BALE_KIND_TRIANGLES) ws = q::standalone_ws(probe);
        }
        const size_t need = io + ws;
        char *buf = need ? arena.alloc(need) : nullptr;
        if (need && !buf) {
          if (!waited[static_cast<size_t>(id)]) st.admission_waits++;
          waited[static_cast<size_t>(id)] = true;
          break;  // FIFO: later requests wait behind it
        }
        pending.pop_front();
        active.emplace_back(new Active());
        Active *a = active.back().get();
        a->id = id;
        a->buf = buf;
        a->buf_bytes = need;
        a->express = express;
        SRV_CUDA(cudaEventCreateWithFlags(&a->uploaded, cudaEventDisableTiming));
        SRV_CUDA(cudaEventCreateWithFlags(&a->downloaded, cudaEventDisableTiming));
        if (x.kind == BALE_KIND_IG) {
          inst.in = reinterpret_cast<int64_t *>(buf);
          inst.out = reinterpret_cast<int64_t *>(buf) + x.n;
          inst.aux = o.d_a;
        } else if (x.kind == BALE_KIND_HISTO) {
          inst.in = reinterpret_cast<int64_t *>(buf);
          inst.out = o.d_a;
          inst.aux = nullptr;
        } else {
          inst.in = o.d_a;
          inst.aux = o.d_b;
          inst.out = reinterpret_cast<int64_t *>(d_tri + id);
        }
        if (x.kind != BALE_KIND_TRIANGLES && x.n)
          SRV_CUDA(cudaMemcpyAsync(buf, x.index, 8 * static_cast<size_t>(x.n), cudaMemcpyHostToDevice,
                                   express ? up_big : s->s_up));
        if (express) {
          SRV_CUDA(cudaEventRecord(a->uploaded, up_big));
          // the least loaded express stream runs it once its index is on the device
          int lane = 0;
          for (int l = 1; l < nlanes; l++)
            if (lane_load[l] < lane_load[lane]) lane = l;
          a->lane = lane;
          a->xcost = q::standalone_cost(inst);
          lane_load[lane] += a->xcost;
          cudaStream_t xs = s->s_express[lane];
          SRV_CUDA(cudaEventCreate(&a->xstart));
          SRV_CUDA(cudaEventCreate(&a->xdone));
          SRV_CUDA(cudaStreamWaitEvent(xs, a->uploaded, 0));
          SRV_CUDA(cudaEventRecord(a->xstart, xs));
          if (x.kind == BALE_KIND_TRIANGLES && o.wedge)
            rc = tri_wedge_run(o.d_a, o.d_c, o.n, o.m, d_tri + id, nullptr, d_xwords + 4 * id, xs);
          else if (x.kind == BALE_KIND_TRIANGLES)
            rc = tri_hybrid_run(o.d_a, o.col32, o.heavy, o.nheavy, o.n, o.m, d_tri + id, nullptr, d_bad + id,
                                d_xwords + 4 * id, rows_per_fetch, xs);
          else
            rc = q::launch_standalone(inst, d_bad + id, buf + io, d_xwords + 4 * id, xs);
          if (rc != BALE_OK) goto done;
          SRV_CUDA(cudaEventRecord(a->xdone, xs));
          st.express++;
        } else {
          h_inst[id] = q::make_inst(inst);
          SRV_CUDA(cudaMemcpyAsync(d_inst + id, h_inst + id, sizeof(Inst), cudaMemcpyHostToDevice, s->s_up));
          SRV_CUDA(cudaEventRecord(a->uploaded, s->s_up));
          std::vector<Planned> plan;
          q::plan_tasks(inst, static_cast<int32_t>(id), o.host_offsets.data(), plan);
          for (auto &p : plan) {
            a->tasks.push_back(p.t);
            a->cost.push_back(p.cost);
          }
        }
        items += static_cast<double>(x.kind == BALE_KIND_TRIANGLES ? o.m : x.n);
        st.max_active = std::max<int64_t>(st.max_active, static_cast<int64_t>(active.size()));
        progressed = true;
      }
      // ---- a finished tick: count the tasks that ran ----
      for (int k = 0; k < kSlots; k++) {
        if (!tick_running[k]) continue;
        cudaError_t e = cudaEventQuery(tick_done[k]);
        if (e == cudaSuccess) {
          tick_running[k] = false;
          float ms = 0.f;
          if (cudaEventElapsedTime(&ms, tick_start[k], tick_done[k]) == cudaSuccess) st.gpu_busy_s += ms * 1e-3;
          for (auto &p : in_tick[k]) p.first->finished += p.second;
          in_tick[k].clear();
          progressed = true;
        } else if (e != cudaErrorNotReady) {
          SRV_CUDA(e);
        }
      }
      // ---- express requests whose kernels finished ----
      for (auto &ap : active) {
        Active *a = ap.get();
        if (!a->express || a->computed) continue;
        cudaError_t e = cudaEventQuery(a->xdone);
        if (e == cudaSuccess) {
          a->computed = true;
          lane_load[a->lane] -= a->xcost;
          float ms = 0.f;
          if (cudaEventElapsedTime(&ms, a->xstart, a->xdone) == cudaSuccess) st.gpu_busy_s += ms * 1e-3;
          progressed = true;
        } else if (e != cudaErrorNotReady) {
          SRV_CUDA(e);
        }
      }
      // ---- requests whose tasks all ran: copy results back ----
      for (auto &ap : active) {
        Active *a = ap.get();
        if (a->downloading || (a->express ? !a->computed : a->finished < a->tasks.size())) continue;
        const bale_request_t &x = req[a->id];
        cudaStream_t down = a->express && x.kind == BALE_KIND_IG ? down_big : s->s_down;
        if (x.kind == BALE_KIND_IG && x.n)
          SRV_CUDA(cudaMemcpyAsync(x.out, a->buf + 8 * x.n, 8 * static_cast<size_t>(x.n), cudaMemcpyDeviceToHost,
                                   down));
        else if (x.kind == BALE_KIND_TRIANGLES)
          SRV_CUDA(cudaMemcpyAsync(x.out, d_tri + a->id, 8, cudaMemcpyDeviceToHost, down));
        SRV_CUDA(cudaEventRecord(a->downloaded, down));
        a->downloading = true;
        progressed = true;
      }
      // ---- completions ----
      for (size_t i = 0; i < active.size();) {
        Active *a = active[i].get();
        if (a->downloading) {
          cudaError_t e = cudaEventQuery(a->downloaded);
          if (e == cudaSuccess) {
            latency[a->id] = now_s() - t0 - req[a->id].arrival;
            if (a->buf) arena.release(a->buf, a->buf_bytes);
            active.erase(active.begin() + static_cast<long>(i));
            done_count++;
            progressed = true;
            continue;
          }
          if (e != cudaErrorNotReady) SRV_CUDA(e);
        }
        i++;
      }
      // ---- queue the next tick over a slice of every ready request ----
      if (!tick_running[tick_next] && !active.empty()) {
        const int slot = tick_next;
        int64_t nt = 0;
        const size_t na = active.size();
        size_t ready = 0;
        for (auto &ap : active)
          if (ap->next < ap->tasks.size() && cudaEventQuery(ap->uploaded) == cudaSuccess) ready++;
        // the tick's work is shared among the ready requests, each getting at
        // least req_cost, so a lone large request is not starved by the cap
        const double share = std::max(req_cost, tick_cost / static_cast<double>(std::max<size_t>(1, ready)));
        double budget = tick_cost;
        for (size_t k = 0; k < na && nt < task_cap && budget > 0; k++) {
          Active *a = active[(rr + k) % na].get();
          if (a->next >= a->tasks.size()) continue;
          if (cudaEventQuery(a->uploaded) != cudaSuccess) continue;
          double mine = 0;
          size_t took = 0;
          while (a->next < a->tasks.size() && nt < task_cap && mine < share && budget > 0) {
            h_tasks[slot][nt++] = a->tasks[a->next];
            mine += a->cost[a->next];
            budget -= a->cost[a->next];
            a->next++;
            took++;
          }
          if (took) in_tick[slot].push_back({a, took});
        }
        rr = (rr + 1) % std::max<size_t>(1, na);
        if (nt > 0) {
          SRV_CUDA(cudaEventRecord(tick_start[slot], s->s_compute));
          SRV_CUDA(cudaMemcpyAsync(d_tasks[slot], h_tasks[slot], sizeof(Task) * static_cast<size_t>(nt),
                                   cudaMemcpyHostToDevice, s->s_compute));
          SRV_CUDA(cudaMemsetAsync(d_words, 0, sizeof(unsigned long long) * 2, s->s_compute));
          rc = q::launch_queue(d_tasks[slot], nt, d_inst, d_words, d_bad, blocks, s->s_compute);
          if (rc != BALE_OK) goto done;
          SRV_CUDA(cudaEventRecord(tick_done[slot], s->s_compute));
          tick_running[slot] = true;
          tick_next = (slot + 1) % kSlots;
          st.ticks++;
          st.tasks += nt;
          progressed = true;
        }
      }
      if (progressed) {
        last_progress = now_s();
      } else {
        if (now_s() - last_progress > 120.0) {
          set_error("bale_server_run: no progress for 120 s");
          rc = BALE_ETIMEDOUT;
          goto done;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(20));
      }
    }
    SRV_CUDA(cudaStreamSynchronize(s->s_compute));
    for (int l = 0; l < nlanes; l++) SRV_CUDA(cudaStreamSynchronize(s->s_express[l]));
    st.makespan_s = now_s() - t0;
    st.items_per_s = st.makespan_s > 0 ? items / st.makespan_s : 0;
    {
      std::vector<int64_t> bad(static_cast<size_t>(nreq));
      SRV_CUDA(cudaMemcpy(bad.data(), d_bad, sizeof(int64_t) * static_cast<size_t>(nreq), cudaMemcpyDeviceToHost));
      for (int64_t v : bad) st.bad += v;
      std::vector<double> lat(latency, latency + nreq);
      std::sort(lat.begin(), lat.end());
      auto pct = [&](double p) { return lat[static_cast<size_t>(std::min<double>(p * (nreq - 1) + 0.5, nreq - 1))]; };
      st.p50_s = pct(0.50);
      st.p99_s = pct(0.99);
      double sum = 0;
      for (double v : lat) sum += v;
      st.mean_s = sum / static_cast<double>(nreq);
    }
  }
done:
#undef SRV_CUDA
  if (rc != BALE_OK) cudaDeviceSynchronize();
  for (int k = 0; k < kSlots; k++) {
    if (tick_done[k]) cudaEventDestroy(tick_done[k]);
    if (tick_start[k]) cudaEventDestroy(tick_start[k]);
  }
  cudaFree(d_inst);
  cudaFree(d_bad);
  cudaFree(d_tri);
  cudaFree(d_words);
  cudaFree(d_xwords);
  for (int k = 0; k < kSlots; k++) {
    cudaFree(d_tasks[k]);
    if (h_tasks[k]) cudaFreeHost(h_tasks[k]);
  }
  if (h_inst) cudaFreeHost(h_inst);
  if (stats) *stats = st;
  return rc;
}

void bale_server_destroy(bale_server_t *s) {
  if (s) cudaDeviceSynchronize();
  server_free(s);
}

}  // extern "C"
