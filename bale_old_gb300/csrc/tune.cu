// tune.cu -- named launch knobs shared by the kernels' launchers.
//
// Every knob defaults to -1 ("automatic": the launcher's own size-class
// rule).  The autotuner (bale_old_gb300/autotune.py) measures the variants of
// each kernel per size class and stores the winners; applications may also
// pin a knob directly.  Knobs only select among variants that compute the
// same result; none of them changes an output bit.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "common.cuh"

namespace bale {

namespace {
struct Knob {
  const char *name;
  int64_t value;
};

Knob g_knobs[] = {
    {"ig.mode", -1},            // 0 direct gather, 1 region-partitioned gather
    {"ig.skew_repeat_pct", -1}, // skewed streams to the direct gather: sample repeat share in %, 0 off
    {"ig.part_min_table_bytes", -1},   // automatic partitioning above this table size (96 MiB)
    {"ig.part_min_requests", -1},      // ... with at least this many requests (2^20)
    {"ig.unroll", -1},          // pairs of requests per thread per trip: 1, 2, 4, 8
    {"ig.threads", -1},         // threads per block: 128, 256, 512
    {"ig.blocks_per_sm", -1},   // resident blocks per SM to launch
    {"ig.table_policy", -1},    // 0 L1::no_allocate, 1 L2 evict_last, 2 L2 evict_first, 3 cached
    {"ig.l2_fetch", -1},        // cudaLimitMaxL2FetchGranularity in bytes (0..128)
    {"histo.part_min_table_bytes", -1},  // automatic partitioning above this table size (96 MiB)
    {"histo.part_min_updates", -1},      // ... with at least this many updates (2^20)
    {"histo.mode", -1},         // 0 shared-memory private, 1 warp-aggregated L2, 2 plain L2, 3 region-partitioned
    {"histo.unroll", -1},       // pairs per thread per trip (L2 modes): 1, 2, 4, 8
    {"histo.blocks_per_sm", -1},
    {"histo.smem_updates_per_counter", -1},  // updates per counter per block (shared-memory mode)
    {"tri.rows_per_fetch", -1}, // rows claimed per cursor increment
    {"batch.standalone", -1},   // 0: every instance in the work queue; -1/1: large instances run their own kernels
    {"batch.standalone_min", -1},        // histo/ig elements from which an instance runs standalone (2^23)
    {"batch.standalone_min_edges", -1},  // triangle nonzeros from which a graph runs standalone (2^21)
    {"batch.streams", -1},               // side streams for standalone instances (4)
    {"batch.queue_blocks", -1},          // blocks of the persistent queue kernel (one per SM)
    {"batch.histo_tile.small", -1},
    {"batch.histo_tile.medium", -1},
    {"batch.histo_tile.large", -1},
    {"batch.histo_l2_tile.small", -1},
    {"batch.histo_l2_tile.medium", -1},
    {"batch.histo_l2_tile.large", -1},
    {"batch.ig_tile.small", -1},
    {"batch.ig_tile.medium", -1},
    {"batch.ig_tile.large", -1},
    {"batch.tri_heavy_rows.small", -1},
    {"batch.tri_heavy_rows.medium", -1},
    {"batch.tri_heavy_rows.large", -1},
    {"batch.tri_light_rows.small", -1},
    {"batch.tri_light_rows.medium", -1},
    {"batch.tri_light_rows.large", -1},
    {"dropin.ig_chunk", -1},      // requests per chunk of the pipelined ig drop-in (2^24; 0 = one pass)
    {"serve.tick_cost", -1},      // work per tick (element-cost units, 2^24)
    {"serve.request_cost", -1},   // work one request may add to a tick (2^22)
    {"serve.tick_tasks", -1},     // tasks per tick (4096)
    {"serve.reserve_bytes", -1},  // free HBM a registration must leave (1 GiB)
    {"serve.express", -1},          // 0: every request goes through the queue kernel
    {"serve.express_streams", -1},  // express streams (2, at most 4)
    {"serve.copy_lanes", -1},       // 1: all copies on one upload and one download stream; 2: express ones apart
    {"sort.onesweep", -1},        // 0: every radix pass as histogram + scan + scatter (1: single sweep below 2^30 keys)
    {"sort.lookback_spins", -1},  // reads without progress before a sort pass's look-back gives up (2^22)
    {"sort.test_withhold", -1},   // 1: tile 0 of each sort pass publishes nothing (tests the bounded wait)
    {"tri.mode", -1},           // 0 warp-per-row merge, 1 bitmap/search hybrid, 2 wedge probes; -1 per graph
    {"tri.wedge_stage_max", -1}, // wedge mode: rows above 2^16 with at most this many columns are binary-searched (64)
    {"tri.wedge_pull_pct", -1},     // default mode: wedges when pulls >= this % of pushes (192)
    {"tri.wedge_push_per_nnz", -1}, // ... or when pushes >= this many per nonzero (no such clause)
    {"tri.choose_min_nnz", -1},     // the per-graph choice from this many nonzeros; wedges below (2^23)
    {"tri.dense", -1},              // wedge mode: 0 probes every prefix; dense pairs by bitmap AND otherwise
    {"tri.dense_ov", -1},           // ... a pair is dense when its prefix exceeds ceil(j/32) words by this (32)
};
std::mutex g_mu;
}  // namespace

int64_t knob(const char *name) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto &k : g_knobs)
    if (std::strcmp(k.name, name) == 0) return k.value;
  return -1;
}

int64_t knob_or(const char *name, int64_t dflt) {
  const int64_t v = knob(name);
  return v >= 0 ? v : dflt;
}

bool ig_auto_partition(int64_t n, int64_t table_len) {
  return table_len * 8 > knob_or("ig.part_min_table_bytes", int64_t(96) << 20) &&
         n >= knob_or("ig.part_min_requests", int64_t(1) << 20);
}

bool histo_auto_partition(int64_t n, int64_t ncounts) {
  return ncounts * 8 > knob_or("histo.part_min_table_bytes", int64_t(96) << 20) &&
         n >= knob_or("histo.part_min_updates", int64_t(1) << 20);
}



}  // namespace bale

extern "C" {

int bale_tune_set(const char *name, int64_t value) {
  if (!name) return BALE_EINVAL;
  std::lock_guard<std::mutex> lk(bale::g_mu);
  for (auto &k : bale::g_knobs)
    if (std::strcmp(k.name, name) == 0) {
      k.value = value;
      return BALE_OK;
    }
  bale::set_error("unknown tuning knob '%s'", name);
  return BALE_EINVAL;
}

int64_t bale_tune_get(const char *name) {
  if (!name) return -2;
  std::lock_guard<std::mutex> lk(bale::g_mu);
  for (auto &k : bale::g_knobs)
    if (std::strcmp(k.name, name) == 0) return k.value;
  return -2;
}

int bale_tune_load(const char *path) {
  if (!path) return -1;
  FILE *f = std::fopen(path, "r");
  if (!f) {
    bale::set_error("bale_tune_load: cannot open %s", path);
    return -1;
  }
  char line[256];
  int applied = 0;
  while (std::fgets(line, sizeof(line), f)) {
    char name[128];
    long long value = 0;
    if (line[0] == '#' || std::sscanf(line, "%127s %lld", name, &value) != 2) continue;
    if (bale_tune_set(name, static_cast<int64_t>(value)) == BALE_OK) applied++;
  }
  std::fclose(f);
  return applied;
}

int bale_tune_count(void) { return static_cast<int>(sizeof(bale::g_knobs) / sizeof(bale::g_knobs[0])); }

const char *bale_tune_name(int i) {
  if (i < 0 || i >= bale_tune_count()) return nullptr;
  return bale::g_knobs[i].name;
}

}  // extern "C"
