// batch.cuh -- the persistent work-queue kernel's task model, shared by the
// batched graph (batch.cu) and the serving loop (serve.cu).
#pragma once

#include <vector>

#include "tri_device.cuh"

namespace bale {
namespace q {

enum TaskKind : int32_t { kHistoSmem = 0, kHistoL2 = 1, kIgDirect = 2, kTriLight = 3, kTriHeavy = 4 };

struct Inst {
  int32_t kind, shift;
  int64_t n, m;
  int64_t *out;
  const int64_t *in;
  const int64_t *aux;
  int64_t bits;  // triangles: bitmap bits (power of two)
};

struct Task {
  int32_t kind, inst;
  int64_t lo, hi;
};

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
constexpr int64_t kSmemCounters = 24 * 1024;
constexpr size_t kSmemBytes = static_cast<size_t>(kSmemCounters) * sizeof(uint32_t);  // 96 KiB: two blocks per SM
static_assert(kSmemBytes >= static_cast<size_t>(tri::kHeavyBits / 8), "bitmap must fit");
static_assert(kSmemBytes >= static_cast<size_t>(kWarps) * tri::kLightCap * sizeof(uint32_t), "row slots must fit");

// A task with the planner's cost estimate (longest first).
struct Planned {
  Task t;
  double cost;
};

// Device record of a public instance.
Inst make_inst(const bale_instance_t &x);
// Cut one instance into queue tasks (tile sizes from the batch.* knobs per
// size class).  Triangles need the host copy of the row offsets (n+1).
void plan_tasks(const bale_instance_t &x, int32_t idx, const int64_t *host_off, std::vector<Planned> &out);
// Blocks of the queue kernel that fit the device (one per SM).
int64_t queue_blocks();
// Launch the queue kernel over d_tasks[0,ntasks); words[0] must be zero
// (the queue head) and words[1] accumulates the triangle work tally.
int launch_queue(const Task *d_tasks, int64_t ntasks, const Inst *d_inst, unsigned long long *words,
                 unsigned long long *bad, int64_t blocks, cudaStream_t stream);

// Large instances run as their own specialised kernels instead of queue
// tasks: the rule (batch.standalone* knobs and the partition thresholds),
// their workspace, a relative cost for stream balancing, and the launch
// (words: 4 zero-initialised device words of cursors).
bool partition_worthy(const bale_instance_t &x);
bool goes_standalone(const bale_instance_t &x);
size_t standalone_ws(const bale_instance_t &x);
double standalone_cost(const bale_instance_t &x);
int launch_standalone(const bale_instance_t &x, unsigned long long *bad, void *ws, unsigned long long *words,
                      cudaStream_t st);

}  // namespace q
}  // namespace bale
