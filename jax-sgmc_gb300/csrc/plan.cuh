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
// Captures enqueue(G) into p->exec (unless GBSGMC_NO_GRAPH=1) and waits for
// the plan's stream.
int plan_capture(gbsgmc_plan* p);
// Enqueues the one-thread launch that advances the counter by g.
int plan_advance(gbsgmc_plan* p, int g, cudaStream_t s);
// Captures what body() enqueues on s (and on streams it forks from s) into
// an executable graph; node_priority keeps the capturing streams' priorities
// on the kernel nodes.
int capture_graph(cudaStream_t s, const std::function<int()>& body,
                  cudaGraphExec_t* out, bool node_priority = false);

}  // namespace gbsgmc
