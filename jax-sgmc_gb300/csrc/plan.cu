// Plans: the multi-step driver of the SGLD hot path on the GLM families, and
// the plan machinery shared with the network plans (plan.cuh).
//
// One block of G GLM steps is: index draw for G steps (numpy PCG64 streams,
// or Philox), G fused SGLD launches whose step index is read from the device
// counter (k = counter + j), and a one-thread launch that advances the
// counter by G.  The block is captured once into a CUDA graph and replayed,
// so a run of K steps costs K/G graph launches on the host.  The schedule
// tables (step size, temperature, keep slots) are read on the device at
// step k.  When the autotuner chooses one launch per block (one CTA per
// chain looping over the block's steps) and the indices come from PCG64
// streams, blocks are pipelined: the index draws of block b+1 run on a side
// stream into a second buffer while block b's launch runs.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <map>
#include <mutex>
#include <new>
#include <tuple>
#include <vector>

#include <cuda.h>

#include "common.cuh"
#include "internal.h"
#include "plan.cuh"

int gbsgmc_plan::run_blocks(int64_t full, int rem) {
  using namespace gbsgmc;
  int rc;
  if (use_graph && exec == nullptr && blocks_run + full >= 2) {
    rc = capture_graph(stream, [this]() { return enqueue(G, stream); }, &exec);
    if (rc) return rc;
  }
  blocks_run += full;
  for (int64_t b = 0; b < full; ++b) {
    if (exec != nullptr) {
      if ((rc = cuda_err(cudaGraphLaunch(exec, stream), "plan_run: graph"))) return rc;
    } else if ((rc = enqueue(G, stream))) {
      return rc;
    }
  }
  if (rem > 0 && (rc = enqueue(rem, stream))) return rc;
  return GBSGMC_OK;
}

gbsgmc_plan::~gbsgmc_plan() {
  if (stream != nullptr) cudaStreamSynchronize(stream);
  if (exec != nullptr) cudaGraphExecDestroy(exec);
  gbsgmc::plan_free(this, base);
  if (ev_in != nullptr) cudaEventDestroy(ev_in);
  if (ev_out != nullptr) cudaEventDestroy(ev_out);
  if (stream != nullptr) cudaStreamDestroy(stream);
}

namespace {

struct GlmPlan final : gbsgmc_plan {
  gbsgmc_glm model;
  int chains, n;
  float* w;
  float* v;
  float alpha, lmbd;
  gbsgmc_sched sched;
  gbsgmc_noise noise;
  gbsgmc_index_src isrc;
  double* U;
  double* lk_var;
  float* samples;
  double* sample_lik;
  int* status;
  gbsgmc::GlmTune tune;
  void* ws = nullptr;
  size_t ws_size = 0;
  int32_t* idx = nullptr;
  // Pipelined blocks (one launch per block, numpy PCG64 index streams): the
  // indices of block b+1 are drawn into the other buffer on a side stream
  // while block b runs.  g_pref[p] / g_last[p]: the block reading buffer p,
  // with and without the draw of the next block.
  bool pipelined = false;
  int32_t* idx2 = nullptr;
  cudaStream_t side = nullptr;
  cudaEvent_t e_fork = nullptr, e_join = nullptr;
  cudaGraphExec_t g_pref[2] = {nullptr, nullptr}, g_last[2] = {nullptr, nullptr};

  ~GlmPlan() override {
    if (stream != nullptr) cudaStreamSynchronize(stream);
    if (side != nullptr) cudaStreamSynchronize(side);
    for (int i = 0; i < 2; ++i) {
      if (g_pref[i] != nullptr) cudaGraphExecDestroy(g_pref[i]);
      if (g_last[i] != nullptr) cudaGraphExecDestroy(g_last[i]);
    }
    if (e_fork != nullptr) cudaEventDestroy(e_fork);
    if (e_join != nullptr) cudaEventDestroy(e_join);
    if (side != nullptr) cudaStreamDestroy(side);
    gbsgmc::plan_free(this, ws);
    gbsgmc::plan_free(this, idx);
    gbsgmc::plan_free(this, idx2);
  }
  int enqueue(int g, cudaStream_t s) override;
  int run_blocks(int64_t full, int rem) override;
  int draw(int g, int32_t* buf, cudaStream_t s);
  int steps_launch(int g, int32_t* buf, cudaStream_t s);
  int pipelined_block(int parity, bool prefetch, cudaStream_t s);
  int setup_pipeline();
  int64_t launches_per_block(int g) const override {
    return (tune.multistep ? 3 : g + 2) - (isrc.external ? 1 : 0);
  }
};

}  // namespace

namespace gbsgmc {

namespace {
__global__ void set_counter_kernel(int64_t* c, int64_t v) { *c = v; }
__global__ void advance_counter_kernel(int64_t* c, int64_t by) { *c += by; }
}  // namespace

int cuda_err(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return GBSGMC_OK;
  return set_error(GBSGMC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int plan_init(gbsgmc_plan* p, int G) {
  p->G = G;
  const char* env = std::getenv("GBSGMC_NO_GRAPH");
  p->use_graph = !(env != nullptr && env[0] == '1');
  int rc;
  if ((rc = cuda_err(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking),
                     "plan: stream")))
    return rc;
  if ((rc = cuda_err(cudaEventCreateWithFlags(&p->ev_in, cudaEventDisableTiming),
                     "plan: event")))
    return rc;
  if ((rc = cuda_err(cudaEventCreateWithFlags(&p->ev_out, cudaEventDisableTiming),
                     "plan: event")))
    return rc;
  if ((rc = plan_alloc(p, &p->base, sizeof(int64_t), "plan: counter"))) return rc;
  return cuda_err(cudaMemsetAsync(p->base, 0, sizeof(int64_t), p->stream), "plan: memset");
}

int plan_capture(gbsgmc_plan* p) {
  return cuda_err(cudaStreamSynchronize(p->stream), "plan: sync");
}

namespace {

// The library's memory pool of the current context, made on first use.
// Contexts are told apart by their process-unique ids (cuCtxGetId, resolved
// through the runtime), so a pool never outlives the context it belongs to
// in this table's eyes.
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* q = nullptr;
    cudaDriverEntryPointQueryResult r;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &q, 4000, cudaEnableDefault,
                                         &r) == cudaSuccess &&
        r == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(q);
    q = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &q, 12000, cudaEnableDefault,
                                         &r) == cudaSuccess &&
        r == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(q);
  });
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current != nullptr && get_id != nullptr && get_current(&ctx) == CUDA_SUCCESS &&
      ctx != nullptr && get_id(ctx, &id) == CUDA_SUCCESS)
    return id << 1;
  int dev = 0;
  cudaGetDevice(&dev);
  return (static_cast<unsigned long long>(dev) << 1) | 1ull;
}

constexpr uint64_t kPoolKeepBytes = 2ull << 30;
std::mutex g_pool_mutex;
std::vector<std::pair<unsigned long long, cudaMemPool_t>> g_pools;

int library_pool(cudaMemPool_t* out) {
  const unsigned long long key = current_context_id();
  std::lock_guard<std::mutex> lock(g_pool_mutex);
  for (const auto& e : g_pools)
    if (e.first == key) {
      *out = e.second;
      return GBSGMC_OK;
    }
  int dev = 0;
  int rc;
  if ((rc = cuda_err(cudaGetDevice(&dev), "plan: device"))) return rc;
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  cudaMemPool_t pool = nullptr;
  if ((rc = cuda_err(cudaMemPoolCreate(&pool, &props), "plan: memory pool"))) return rc;
  uint64_t keep = kPoolKeepBytes;
  if ((rc = cuda_err(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep),
                     "plan: memory pool"))) {
    cudaMemPoolDestroy(pool);
    return rc;
  }
  g_pools.emplace_back(key, pool);
  *out = pool;
  return GBSGMC_OK;
}

}  // namespace

int plan_alloc(gbsgmc_plan* p, void** ptr, size_t bytes, const char* what) {
  *ptr = nullptr;
  cudaMemPool_t pool = nullptr;
  int rc;
  if ((rc = library_pool(&pool))) return rc;
  if ((rc = cuda_err(cudaMallocFromPoolAsync(ptr, bytes, pool, p->stream), what)))
    return rc;
  // A pooled block may hold an earlier plan's data: start from zeros, as the
  // kernels' counters and partial sums expect of a fresh workspace.
  return cuda_err(cudaMemsetAsync(*ptr, 0, bytes, p->stream), what);
}

void plan_free(gbsgmc_plan* p, void* ptr) {
  if (ptr != nullptr) cudaFreeAsync(ptr, p->stream);
}

int plan_advance(gbsgmc_plan* p, int g, cudaStream_t s) {
  advance_counter_kernel<<<1, 1, 0, s>>>(p->base, g);
  return check_launch("plan: advance counter");
}

int capture_graph(cudaStream_t s, const std::function<int()>& body,
                  cudaGraphExec_t* out, bool node_priority) {
  int rc;
  if ((rc = cuda_err(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal),
                     "plan: begin capture")))
    return rc;
  rc = body();
  cudaGraph_t graph = nullptr;
  const cudaError_t e = cudaStreamEndCapture(s, &graph);
  if (rc != GBSGMC_OK) {
    if (graph != nullptr) cudaGraphDestroy(graph);
    return rc;
  }
  if ((rc = cuda_err(e, "plan: end capture"))) return rc;
  rc = cuda_err(cudaGraphInstantiate(
                    out, graph,
                    node_priority ? cudaGraphInstantiateFlagUseNodePriority : 0),
                "plan: instantiate");
  cudaGraphDestroy(graph);
  return rc;
}

namespace {

}  // namespace
}  // namespace gbsgmc

// Index draws of the next g steps into buf ([g, chains, n]).
int GlmPlan::draw(int g, int32_t* buf, cudaStream_t s) {
  using namespace gbsgmc;
  const int64_t cn = static_cast<int64_t>(chains) * n;
  const int64_t rows = model.n_rows > 0 ? model.n_rows : model.n_obs;
  if (isrc.external) return GBSGMC_OK;  // written by gbsgmc_plan_set_indices
  if (isrc.pcg_dev != nullptr)
    return gbsgmc_index_draw_pcg64(isrc.pcg_dev, chains, rows,
                                   static_cast<int64_t>(g) * n, n, buf, n, cn,
                                   status, s);
  return launch_philox_index(isrc.index_seed, isrc.chain_base, chains, base, 0,
                             g, n, rows, buf, n, cn, s);
}

// One launch running g steps from the index sets in buf, then the counter
// advance.
int GlmPlan::steps_launch(int g, int32_t* buf, cudaStream_t s) {
  using namespace gbsgmc;
  const int64_t cn = static_cast<int64_t>(chains) * n;
  gbsgmc_sched s0 = sched;
  s0.base_dev = base;
  s0.offset = 0;
  const int rc = glm_sgld_step(&model, chains, n, buf, n, w, v, alpha, lmbd, &s0,
                               &noise, U, lk_var, samples, sample_lik, ws,
                               ws_size, status, s, tune, g, cn);
  if (rc != GBSGMC_OK) return rc;
  return plan_advance(this, g, s);
}

int GlmPlan::pipelined_block(int parity, bool prefetch, cudaStream_t s) {
  using namespace gbsgmc;
  int32_t* cur = parity ? idx2 : idx;
  int32_t* nxt = parity ? idx : idx2;
  int rc;
  if (prefetch) {
    if ((rc = cuda_err(cudaEventRecord(e_fork, s), "plan: fork"))) return rc;
    if ((rc = cuda_err(cudaStreamWaitEvent(side, e_fork, 0), "plan: fork"))) return rc;
    if ((rc = draw(G, nxt, side))) return rc;
    if ((rc = cuda_err(cudaEventRecord(e_join, side), "plan: join"))) return rc;
  }
  if ((rc = steps_launch(G, cur, s))) return rc;
  if (prefetch && (rc = cuda_err(cudaStreamWaitEvent(s, e_join, 0), "plan: join")))
    return rc;
  return GBSGMC_OK;
}

int GlmPlan::setup_pipeline() {
  using namespace gbsgmc;
  int rc;
  const size_t bytes = sizeof(int32_t) * static_cast<size_t>(G) * chains * n;
  if ((rc = plan_alloc(this, &idx2, bytes, "plan_create: index buffer"))) return rc;
  // The block's launch runs at the greatest stream priority and the draws at
  // the least, so that the launch gets its CTAs onto the SMs first and the
  // draws fill the room it leaves.
  int least = 0, greatest = 0;
  if ((rc = cuda_err(cudaDeviceGetStreamPriorityRange(&least, &greatest),
                     "plan: priorities")))
    return rc;
  if ((rc = cuda_err(cudaStreamSynchronize(stream), "plan: sync"))) return rc;
  if ((rc = cuda_err(cudaStreamDestroy(stream), "plan: stream"))) return rc;
  stream = nullptr;
  if ((rc = cuda_err(cudaStreamCreateWithPriority(&stream, cudaStreamNonBlocking,
                                                  greatest),
                     "plan: stream")))
    return rc;
  if ((rc = cuda_err(cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, least),
                     "plan: stream")))
    return rc;
  if ((rc = cuda_err(cudaEventCreateWithFlags(&e_fork, cudaEventDisableTiming),
                     "plan: event")))
    return rc;
  if ((rc = cuda_err(cudaEventCreateWithFlags(&e_join, cudaEventDisableTiming),
                     "plan: event")))
    return rc;
  if (use_graph) {
    for (int par = 0; par < 2; ++par) {
      rc = capture_graph(stream, [this, par]() { return pipelined_block(par, true, stream); },
                         &g_pref[par], true);
      if (rc) return rc;
      rc = capture_graph(stream, [this, par]() { return pipelined_block(par, false, stream); },
                         &g_last[par], true);
      if (rc) return rc;
    }
  }
  pipelined = true;
  return GBSGMC_OK;
}

int GlmPlan::run_blocks(int64_t full, int rem) {
  using namespace gbsgmc;
  if (!pipelined) return gbsgmc_plan::run_blocks(full, rem);
  int rc;
  if (full > 0 && (rc = draw(G, idx, stream))) return rc;
  for (int64_t b = 0; b < full; ++b) {
    const int par = static_cast<int>(b & 1);
    const bool pref = b + 1 < full;
    if (use_graph) {
      if ((rc = cuda_err(cudaGraphLaunch(pref ? g_pref[par] : g_last[par], stream),
                         "plan_run: graph")))
        return rc;
    } else if ((rc = pipelined_block(par, pref, stream))) {
      return rc;
    }
  }
  if (rem > 0 && (rc = enqueue(rem, stream))) return rc;
  return GBSGMC_OK;
}

int GlmPlan::enqueue(int g, cudaStream_t s) {
  using namespace gbsgmc;
  int rc;
  GlmPlan* p = this;
  const int64_t cn = static_cast<int64_t>(p->chains) * p->n;
  if ((rc = draw(g, p->idx, s))) return rc;
  // One launch for the g steps: each CTA runs its chain's steps in turn.
  if (p->tune.multistep) return steps_launch(g, p->idx, s);
  for (int j = 0; j < g; ++j) {
    gbsgmc_sched sj = p->sched;
    sj.base_dev = p->base;
    sj.offset = j;
    rc = glm_sgld_step(&p->model, p->chains, p->n, p->idx + j * cn, p->n, p->w,
                       p->v, p->alpha, p->lmbd, &sj, &p->noise, p->U,
                       p->lk_var, p->samples, p->sample_lik, p->ws, p->ws_size,
                       p->status, s, p->tune);
    if (rc != GBSGMC_OK) return rc;
  }
  return plan_advance(p, g, s);
}

namespace gbsgmc {
namespace {

// Autotuner: times candidate launch shapes of the fused step (CTAs per chain
// and rows per warp) on scratch copies of the chain state and keeps the
// fastest.  The choice is cached per problem shape for the process, and
// direct step launches of that shape use it too.
int autotune(GlmPlan* p) {
  const char* env = std::getenv("GBSGMC_AUTOTUNE");
  if (env != nullptr && env[0] == '0') return GBSGMC_OK;
  if (glm_tune_lookup(p->chains, p->n, p->model.d, p->model.ld, &p->tune))
    return GBSGMC_OK;
  const int C = p->chains, n = p->n, d = p->model.d;
  const size_t wbytes = sizeof(float) * static_cast<size_t>(C) * d;
  float* w = nullptr;
  float* v = nullptr;
  int* status = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = GBSGMC_OK;
  std::vector<GlmTune> cands;
  {
    const double rows_per_cta = (384.0 * 1024.0) / (4.0 * std::max<int64_t>(p->model.ld, 1));
    const int base = std::max(1, static_cast<int>(std::ceil(n / rows_per_cta)));
    const int ss[] = {1, base / 2, base, base + 1, 2 * base};
    for (int s : ss) {
      if (s < 1 || s > 64 || (s > 1 && n / s < 32)) continue;
      bool dup = false;
      for (const GlmTune& t : cands) dup = dup || t.slices == s;
      if (dup) continue;
      if (d <= 256) {
        // (rows per warp, warps, prefetch)
        const int shapes[][3] = {{2, 8, 0}, {4, 8, 0}, {4, 8, 1}, {8, 8, 0},
                                 {2, 8, 1}, {2, 16, 0}, {4, 16, 0}, {4, 16, 1}};
        for (const auto& sh : shapes) cands.push_back(GlmTune{s, sh[0], sh[1], sh[2], 0});
      } else {
        for (int w : {8, 16}) cands.push_back(GlmTune{s, 0, w, 0, 0});
      }
    }
    // Dynamically scheduled kernel: items of n / ipc rows claimed by warps.
    if (d <= 256) {
      for (int ipc : {4, 8, 16}) {
        if (n / ipc < 32) continue;
        for (int rw : {4, 8}) cands.push_back(GlmTune{ipc, rw, 8, 0, 1, 0});
      }
    }
    // One CTA per chain running a block of steps per launch.
    if (n <= 1024 && p->G >= 6) {
      const size_t m = cands.size();
      for (size_t i = 0; i < m; ++i) {
        if (cands[i].slices != 1 || cands[i].dynamic) continue;
        GlmTune t = cands[i];
        t.multistep = 1;
        cands.push_back(t);
      }
    }
  }
  if (cands.size() <= 1) {
    if (!cands.empty()) p->tune = cands[0];
    return GBSGMC_OK;
  }
  do {
    if ((rc = cuda_err(cudaMalloc(&w, wbytes), "autotune: scratch"))) break;
    if ((rc = cuda_err(cudaMalloc(&v, wbytes), "autotune: scratch"))) break;
    if ((rc = cuda_err(cudaMalloc(&status, sizeof(int)), "autotune: scratch"))) break;
    if ((rc = cuda_err(cudaMemcpyAsync(w, p->w, wbytes, cudaMemcpyDeviceToDevice,
                                       p->stream), "autotune: copy")))
      break;
    if (p->v != nullptr &&
        (rc = cuda_err(cudaMemcpyAsync(v, p->v, wbytes, cudaMemcpyDeviceToDevice,
                                       p->stream), "autotune: copy")))
      break;
    if ((rc = cuda_err(cudaMemsetAsync(status, 0, sizeof(int), p->stream),
                       "autotune: memset")))
      break;
    if ((rc = cuda_err(cudaEventCreate(&e0), "autotune: event"))) break;
    if ((rc = cuda_err(cudaEventCreate(&e1), "autotune: event"))) break;
    const int64_t rows = p->model.n_rows > 0 ? p->model.n_rows : p->model.n_obs;
    const int trials = std::min(8, p->G);
    if ((rc = launch_philox_index(0x5EEDull, 0, C, nullptr, 0, trials, n, rows,
                                  p->idx, n, static_cast<int64_t>(C) * n,
                                  p->stream)))
      break;
    gbsgmc_sched sch = p->sched;
    sch.base_dev = nullptr;
    sch.keep_slot_dev = nullptr;
    sch.offset = 0;
    float best_ms = 1e30f;
    GlmTune best = cands[0];
    const char* vb = std::getenv("GBSGMC_AUTOTUNE_VERBOSE");
    const bool verbose = vb != nullptr && vb[0] == '1';
    for (const GlmTune& t : cands) {
      if (t.multistep) {
        // Two warm-up steps, then six steps in one launch.
        for (int rep = 0; rep < 2 && rc == GBSGMC_OK; ++rep)
          rc = glm_sgld_step(&p->model, C, n, p->idx, n, w,
                             p->v != nullptr ? v : nullptr, p->alpha, p->lmbd,
                             &sch, &p->noise, p->U, p->lk_var, nullptr, nullptr,
                             p->ws, p->ws_size, status, p->stream, t);
        if (rc == GBSGMC_OK) {
          cudaEventRecord(e0, p->stream);
          rc = glm_sgld_step(&p->model, C, n, p->idx, n, w,
                             p->v != nullptr ? v : nullptr, p->alpha, p->lmbd,
                             &sch, &p->noise, p->U, p->lk_var, nullptr, nullptr,
                             p->ws, p->ws_size, status, p->stream, t, 6,
                             static_cast<int64_t>(C) * n);
        }
      } else {
        for (int rep = 0; rep < 2 + 6 && rc == GBSGMC_OK; ++rep) {
          if (rep == 2) cudaEventRecord(e0, p->stream);
          const int j = rep % trials;
          rc = glm_sgld_step(&p->model, C, n, p->idx + static_cast<int64_t>(j) * C * n,
                             n, w, p->v != nullptr ? v : nullptr, p->alpha, p->lmbd,
                             &sch, &p->noise, p->U, p->lk_var, nullptr, nullptr,
                             p->ws, p->ws_size, status, p->stream, t);
        }
      }
      if (rc != GBSGMC_OK) break;
      cudaEventRecord(e1, p->stream);
      if ((rc = cuda_err(cudaEventSynchronize(e1), "autotune: sync"))) break;
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (verbose)
        std::fprintf(stderr,
                     "gbsgmc autotune: slices %d rows/warp %d warps %d prefetch %d "
                     "dynamic %d multistep %d: %.4f ms\n",
                     t.slices, t.rows_per_warp, t.warps, t.prefetch, t.dynamic,
                     t.multistep, ms / 6.0f);
      if (ms < best_ms) {
        best_ms = ms;
        best = t;
      }
    }
    if (rc != GBSGMC_OK) break;
    p->tune = best;
    glm_tune_store(p->chains, p->n, p->model.d, p->model.ld, best);
  } while (false);
  cudaStreamSynchronize(p->stream);
  if (e0 != nullptr) cudaEventDestroy(e0);
  if (e1 != nullptr) cudaEventDestroy(e1);
  if (w != nullptr) cudaFree(w);
  if (v != nullptr) cudaFree(v);
  if (status != nullptr) cudaFree(status);
  return rc;
}

}  // namespace
}  // namespace gbsgmc

using namespace gbsgmc;

extern "C" int gbsgmc_sgld_glm_plan_create(
    gbsgmc_plan** out, const gbsgmc_glm* model, int chains, int n,
    float* w_dev, float* v_dev, float alpha, float lmbd,
    const gbsgmc_sched* sched, const gbsgmc_noise* noise,
    const gbsgmc_index_src* index_src, double* U_dev, double* lk_var_dev,
    float* samples_dev, double* sample_lik_dev, int block_steps,
    int* status_dev) {
  if (out == nullptr || model == nullptr || sched == nullptr ||
      noise == nullptr || index_src == nullptr || w_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG, "plan_create: null argument");
  *out = nullptr;
  if (chains <= 0 || n <= 0 || block_steps <= 0 || block_steps > 100000)
    return set_error(GBSGMC_ERR_ARG, "plan_create: bad chains/n/block_steps");
  if (sched->keep_slot_dev != nullptr && samples_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG,
                     "plan_create: keep table given without sample buffer");
  GlmPlan* p = new (std::nothrow) GlmPlan();
  if (p == nullptr) return set_error(GBSGMC_ERR_ARG, "plan_create: out of memory");
  p->model = *model;
  p->chains = chains;
  p->n = n;
  p->w = w_dev;
  p->v = v_dev;
  p->alpha = alpha;
  p->lmbd = lmbd;
  p->sched = *sched;
  p->noise = *noise;
  p->isrc = *index_src;
  p->U = U_dev;
  p->lk_var = lk_var_dev;
  p->samples = samples_dev;
  p->sample_lik = sample_lik_dev;
  p->status = status_dev;
  int rc = GBSGMC_OK;
  do {
    if ((rc = plan_init(p, block_steps))) break;
    p->ws_size = glm_ws_bytes(chains, n, model->d);
    if ((rc = plan_alloc(p, &p->ws, p->ws_size, "plan_create: workspace"))) break;
    if ((rc = plan_alloc(p, &p->idx,
                         sizeof(int32_t) * static_cast<size_t>(block_steps) * chains * n,
                         "plan_create: index buffer")))
      break;
    if ((rc = cuda_err(cudaMemsetAsync(p->ws, 0, p->ws_size, p->stream),
                       "plan_create: memset")))
      break;
    if (p->isrc.external) {
      p->ext_idx = p->idx;
      p->ext_per_step = static_cast<int64_t>(chains) * n;
      if ((rc = cuda_err(cudaMemsetAsync(p->idx, 0, sizeof(int32_t) * block_steps *
                                                        p->ext_per_step, p->stream),
                         "plan_create: memset")))
        break;
    }
    if ((rc = glm_prepare())) break;
    if ((rc = autotune(p))) break;
    // GBSGMC_GLM_MULTISTEP=1/0 forces one launch per block of steps or one
    // launch per step, whatever the autotuner chose.
    if (const char* ms = std::getenv("GBSGMC_GLM_MULTISTEP"))
      if (ms[0] == '0' || ms[0] == '1') p->tune.multistep = ms[0] == '1';
    if ((rc = plan_capture(p))) break;
    // GBSGMC_PLAN_PIPELINE=1 overlaps the next block's index draws with this
    // block's launch when the block is one launch and the draws carry state
    // (PCG64 streams).  Off by default: on the 256-chain logistic workload
    // the overlapped draws slowed the block more than they saved.
    const char* pe = std::getenv("GBSGMC_PLAN_PIPELINE");
    const bool pipe_ok = pe != nullptr && pe[0] == '1';
    if (pipe_ok && p->tune.multistep && p->isrc.pcg_dev != nullptr)
      rc = p->setup_pipeline();
  } while (false);
  if (rc != GBSGMC_OK) {
    delete p;
    return rc;
  }
  *out = p;
  return GBSGMC_OK;
}

namespace {

// reSGLD pairs on a GLM potential (alias.re_sgld through solver.mcmc): 2P
// chains, normal chain p in slot p and its hot partner in slot P + p, plain
// SGLD (or SGLD + rms_prop) at the slot's temperature, and after every step
// the pairs' exchange on the device.  The chains' index streams and noise
// belong to chain identities that travel with exchanged states: identity i
// draws its own indices (buffer [G, 2P, n] by identity) and its own noise
// (chain id chain_base + i), and slot s runs identity ident[s].
struct GlmPairsPlan final : gbsgmc_plan {
  gbsgmc_glm model;
  int pairs = 0, n = 0;
  float* w = nullptr;
  float* v = nullptr;
  float alpha = 0.9f, lmbd = 1e-5f;
  gbsgmc_sched sched{};
  gbsgmc_noise noise{};
  gbsgmc_index_src isrc{};
  gbsgmc_tempering temp{};
  const int32_t* pair_chain = nullptr;
  int32_t* ident = nullptr;
  double* U = nullptr;
  double* lk_var = nullptr;
  float* samples = nullptr;
  double* sample_lik = nullptr;
  int* status = nullptr;
  gbsgmc::GlmTune tune;
  void* ws = nullptr;
  size_t ws_size = 0;
  int32_t* idx = nullptr;

  ~GlmPairsPlan() override {
    if (stream != nullptr) cudaStreamSynchronize(stream);
    gbsgmc::plan_free(this, ws);
    gbsgmc::plan_free(this, idx);
  }
  int64_t launches_per_block(int g) const override { return 2 + 2 * static_cast<int64_t>(g); }
  int enqueue(int g, cudaStream_t s) override {
    using namespace gbsgmc;
    const int chains = 2 * pairs;
    const int64_t cn = static_cast<int64_t>(chains) * n;
    const int64_t rows = model.n_rows > 0 ? model.n_rows : model.n_obs;
    int rc = gbsgmc_index_draw_pcg64(isrc.pcg_dev, chains, rows, static_cast<int64_t>(g) * n,
                                     n, idx, n, cn, status, s);
    if (rc != GBSGMC_OK) return rc;
    for (int j = 0; j < g; ++j) {
      gbsgmc_sched sj = sched;
      sj.base_dev = base;
      sj.offset = j;
      gbsgmc_sched step_sched = sj;
      step_sched.keep_slot_dev = nullptr;  // the exchange stores the samples
      rc = glm_sgld_step(&model, chains, n, idx + j * cn, n, w, v, alpha, lmbd, &step_sched,
                         &noise, U, lk_var, nullptr, nullptr, ws, ws_size, status, s, tune,
                         1, 0, ident);
      if (rc != GBSGMC_OK) return rc;
      rc = resgld_pairs_exchange(pairs, model.d, w, v, U, lk_var, ident, &sj, temp.F,
                                 temp.seed, pair_chain, temp.ssq_dev, temp.k_dev,
                                 temp.counts_dev, samples, sample_lik, s);
      if (rc != GBSGMC_OK) return rc;
    }
    return plan_advance(this, g, s);
  }
};

}  // namespace

extern "C" int gbsgmc_glm_resgld_plan_create(
    gbsgmc_plan** out, const gbsgmc_glm* model, int pairs, int n, float* x_dev,
    float* v_dev, float alpha, float lmbd, const gbsgmc_sched* sched,
    const gbsgmc_noise* noise, const gbsgmc_index_src* index_src,
    const gbsgmc_tempering* tempering, const int32_t* pair_chain_dev, int32_t* ident_dev,
    double* U_dev, double* lk_var_dev, float* samples_dev, double* sample_lik_dev,
    int block_steps, int* status_dev) {
  if (out == nullptr || model == nullptr || sched == nullptr || noise == nullptr ||
      index_src == nullptr || tempering == nullptr || x_dev == nullptr ||
      pair_chain_dev == nullptr || ident_dev == nullptr || U_dev == nullptr ||
      lk_var_dev == nullptr || status_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG, "glm_resgld_plan_create: null argument");
  *out = nullptr;
  if (pairs <= 0 || n <= 0 || block_steps <= 0 || block_steps > 100000 ||
      pairs > (1 << 20))
    return set_error(GBSGMC_ERR_ARG, "glm_resgld_plan_create: bad pairs/n/block_steps");
  if (index_src->pcg_dev == nullptr || index_src->external)
    return set_error(GBSGMC_ERR_ARG,
                     "glm_resgld_plan_create: needs PCG64 index streams (one per chain)");
  if (sched->chain_temperature_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG,
                     "glm_resgld_plan_create: needs the per-chain temperatures");
  if (tempering->ssq_dev == nullptr || tempering->k_dev == nullptr ||
      !(tempering->F != 0.0))
    return set_error(GBSGMC_ERR_ARG, "glm_resgld_plan_create: bad tempering state");
  if (sched->keep_slot_dev != nullptr && samples_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG,
                     "glm_resgld_plan_create: keep table given without sample buffer");
  GlmPairsPlan* p = new (std::nothrow) GlmPairsPlan();
  if (p == nullptr) return set_error(GBSGMC_ERR_ARG, "glm_resgld_plan_create: out of memory");
  p->model = *model;
  p->pairs = pairs;
  p->n = n;
  p->w = x_dev;
  p->v = v_dev;
  p->alpha = alpha;
  p->lmbd = lmbd;
  p->sched = *sched;
  p->noise = *noise;
  p->isrc = *index_src;
  p->temp = *tempering;
  p->pair_chain = pair_chain_dev;
  p->ident = ident_dev;
  p->U = U_dev;
  p->lk_var = lk_var_dev;
  p->samples = samples_dev;
  p->sample_lik = sample_lik_dev;
  p->status = status_dev;
  int rc = GBSGMC_OK;
  do {
    if ((rc = plan_init(p, block_steps))) break;
    const int chains = 2 * pairs;
    p->ws_size = glm_ws_bytes(chains, n, model->d);
    if ((rc = plan_alloc(p, &p->ws, p->ws_size, "glm_resgld_plan_create: workspace"))) break;
    if ((rc = plan_alloc(p, &p->idx,
                         sizeof(int32_t) * static_cast<size_t>(block_steps) * chains * n,
                         "glm_resgld_plan_create: index buffer")))
      break;
    if ((rc = glm_prepare())) break;
    // One launch per step (the exchange sits between steps): the cached
    // launch shape of this problem, or the library's default.
    glm_tune_lookup(chains, n, model->d, model->ld, &p->tune);
    p->tune.multistep = 0;
    rc = plan_capture(p);
  } while (false);
  if (rc != GBSGMC_OK) {
    delete p;
    return rc;
  }
  *out = p;
  return GBSGMC_OK;
}

extern "C" int gbsgmc_plan_run(gbsgmc_plan* p, int64_t first_step,
                               int64_t steps, gbsgmc_stream_t stream) {
  if (p == nullptr) return set_error(GBSGMC_ERR_ARG, "plan_run: null plan");
  if (first_step < 0 || steps < 0)
    return set_error(GBSGMC_ERR_ARG, "plan_run: negative step");
  const int m = p->step_multiple();
  if (first_step % m != 0 || steps % m != 0)
    return set_error(GBSGMC_ERR_ARG,
                     "plan_run: first_step and steps must be multiples of %d", m);
  if (steps == 0) return GBSGMC_OK;
  cudaStream_t us = static_cast<cudaStream_t>(stream);
  int rc;
  if ((rc = cuda_err(cudaEventRecord(p->ev_in, us), "plan_run: record"))) return rc;
  if ((rc = cuda_err(cudaStreamWaitEvent(p->stream, p->ev_in, 0), "plan_run: wait")))
    return rc;
  set_counter_kernel<<<1, 1, 0, p->stream>>>(p->base, first_step);
  if ((rc = check_launch("plan_run: set counter"))) return rc;
  const int64_t full = steps / p->G;
  const int rem = static_cast<int>(steps % p->G);
  if ((rc = p->run_blocks(full, rem))) return rc;
  if ((rc = cuda_err(cudaEventRecord(p->ev_out, p->stream), "plan_run: record")))
    return rc;
  return cuda_err(cudaStreamWaitEvent(us, p->ev_out, 0), "plan_run: wait");
}

extern "C" int gbsgmc_plan_set_indices(gbsgmc_plan* p, const int32_t* src, int steps,
                                       gbsgmc_stream_t stream) {
  if (p == nullptr || src == nullptr)
    return set_error(GBSGMC_ERR_ARG, "plan_set_indices: null argument");
  if (p->ext_idx == nullptr)
    return set_error(GBSGMC_ERR_ARG, "plan_set_indices: the plan draws its own indices");
  if (steps < 1 || steps > p->G)
    return set_error(GBSGMC_ERR_ARG, "plan_set_indices: steps %d outside [1, %d]", steps,
                     p->G);
  const size_t bytes = sizeof(int32_t) * static_cast<size_t>(steps) * p->ext_per_step;
  return cuda_err(cudaMemcpyAsync(p->ext_idx, src, bytes, cudaMemcpyDefault,
                                  static_cast<cudaStream_t>(stream)),
                  "plan_set_indices: copy");
}

extern "C" int gbsgmc_plan_launch_shape(const gbsgmc_plan* p, int* slices,
                                        int* rows_per_warp, int* warps, int* prefetch,
                                        int* dynamic, int* steps_per_launch) {
  if (p == nullptr || slices == nullptr || rows_per_warp == nullptr ||
      warps == nullptr || prefetch == nullptr || dynamic == nullptr ||
      steps_per_launch == nullptr)
    return set_error(GBSGMC_ERR_ARG, "plan_launch_shape: null argument");
  *slices = *rows_per_warp = *warps = *prefetch = *dynamic = 0;
  *steps_per_launch = 1;
  if (const GlmPlan* g = dynamic_cast<const GlmPlan*>(p)) {
    *slices = g->tune.slices;
    *rows_per_warp = g->tune.rows_per_warp;
    *warps = g->tune.warps;
    *prefetch = g->tune.prefetch;
    *dynamic = g->tune.dynamic;
    if (g->tune.multistep) *steps_per_launch = g->G;
  }
  return GBSGMC_OK;
}

extern "C" int64_t gbsgmc_plan_launches(const gbsgmc_plan* p, int64_t steps) {
  if (p == nullptr || steps <= 0) return 0;
  const int64_t full = steps / p->G;
  const int64_t rem = steps % p->G;
  return 1 + full * p->launches_per_block(p->G) +
         (rem > 0 ? p->launches_per_block(static_cast<int>(rem)) : 0);
}

extern "C" int gbsgmc_plan_destroy(gbsgmc_plan* p) {
  delete p;
  return GBSGMC_OK;
}
