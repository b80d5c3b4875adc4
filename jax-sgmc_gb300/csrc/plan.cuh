// Plans: multi-step drivers captured into CUDA graphs (not ABI).
//
// A plan owns an internal non-blocking stream, a device step counter and
// whatever buffers its steps need.  One block of G steps is enqueued by the
// plan's own enqueue(); the block reads the step index of each launch from
// the device counter and ends by advancing it by G, so one captured graph
// replays for every block.  plan_run orders the plan's stream after the
// caller's stream and back.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>

#include "internal.h"

struct gbsgmc_plan {
  virtual ~gbsgmc_plan();
  // Enqueues g steps (g <= G) on s, starting at the device counter.
  virtual int enqueue(int g, cudaStream_t s) = 0;
  // Kernel launches of one block of g steps.
  virtual int64_t launches_per_block(int g) const = 0;
  // plan_run's first step and step count must be multiples of this.
  virtual int step_multiple() const { return 1; }
  // Runs `full` blocks of G steps, then `rem` steps, on the plan's stream
  // (after plan_run has set the counter).  The default replays the captured
  // block and enqueues the remainder directly.
  virtual int run_blocks(int64_t full, int rem);

  int G = 0;
  bool use_graph = true;
  // Blocks run so far; the block graph is captured when the plan's second
  // block is about to run (a plan that runs one block launches it directly).
  int64_t blocks_run = 0;
  // External index source: the plan's index buffer [G, ext_per_step] int32
  // that gbsgmc_plan_set_indices fills (null when the plan draws its own).
  int32_t* ext_idx = nullptr;
  int64_t ext_per_step = 0;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  int64_t* base = nullptr;  // device step counter
};

namespace gbsgmc {

int cuda_err(cudaError_t e, const char* what);
// Stream, events and counter of a new plan with blocks of G steps.
int plan_init(gbsgmc_plan* p, int G);
// Waits for the plan's set-up work.  The block graph (enqueue(G) captured
// into p->exec, unless GBSGMC_NO_GRAPH=1) is captured later, when the
// plan's second block is about to run.
int plan_capture(gbsgmc_plan* p);
// Device memory of plans comes from one memory pool of the library per
// CUDA context: allocations and frees are ordered on the plan's stream, and
// freed blocks (up to a release threshold of 2 GiB) stay in the pool for the
// next plan instead of going back to the driver, so creating and destroying
// plans neither synchronises the device nor maps fresh memory each time.
// Every block handed out is zeroed on the plan's stream.
int plan_alloc(gbsgmc_plan* p, void** ptr, size_t bytes, const char* what);
template <class T>
int plan_alloc(gbsgmc_plan* p, T** ptr, size_t bytes, const char* what) {
  void* q = nullptr;
  const int rc = plan_alloc(p, &q, bytes, what);
  *ptr = static_cast<T*>(q);
  return rc;
}
// Returns plan memory to the pool, ordered after the plan's stream work.
void plan_free(gbsgmc_plan* p, void* ptr);
// Enqueues the one-thread launch that advances the counter by g.
int plan_advance(gbsgmc_plan* p, int g, cudaStream_t s);
// Captures what body() enqueues on s (and on streams it forks from s) into
// an executable graph; node_priority keeps the capturing streams' priorities
// on the kernel nodes.
int capture_graph(cudaStream_t s, const std::function<int()>& body,
                  cudaGraphExec_t* out, bool node_priority = false);

}  // namespace gbsgmc
