// Plans over the network likelihoods (and the GLM families for OBABO and
// SGHMC): many chains of SGLD(+RMSprop), OBABO or SGHMC stepped together, one
// CUDA graph per block of steps.
//
// Per step: index draw(s) for all chains (one per minibatch the integrator
// consumes), the batched value-and-gradient of the network over all chains,
// and the integrator's elementwise kernels over [chains, P].  The integrator
// kernels read their step index from the plan's device counter, so the Philox
// noise of step k is the same whether the step runs inside a graph or alone.
#include <cstdlib>
#include <functional>
#include <new>

#include "common.cuh"
#include "internal.h"
#include "plan.cuh"

namespace gbsgmc {
namespace {

__global__ void mean_pair_kernel(int chains, double* a, const double* b) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < chains) a[c] = 0.5 * (a[c] + b[c]);
}

// Value and gradient over all chains:
// (idx, idx_stride, U, lk_var, gradient out [chains, P], stream).
using GradFn =
    std::function<int(const int32_t*, int64_t, double*, double*, float*, cudaStream_t)>;

struct NetPlan final : gbsgmc_plan {
  GradFn grad_fn;
  int chains = 0, n = 0;
  int64_t P = 0, rows = 0;
  gbsgmc_integrator integ{};
  float* x = nullptr;
  float* aux = nullptr;
  float* grad = nullptr;  // owned [chains, P]
  float* grad2 = nullptr; // owned [chains, P] (OBABO: the second gradient)
  gbsgmc_sched sched{};
  gbsgmc_noise noise{};
  gbsgmc_index_src isrc{};
  double* U = nullptr;
  double* U2 = nullptr;   // owned (OBABO)
  double* lk_var = nullptr;
  double* ke = nullptr;
  int* status = nullptr;
  int32_t* idx = nullptr;  // owned [G, chains, draws * n]
  void* ws = nullptr;      // owned
  size_t ws_size = 0;
  // Fused with the updates (network likelihoods that support it): the
  // updates add the prior's gradient, keep the BF16 weight mirror in the
  // workspace current and write the sums of squares the value needs.
  bool fused = false;
  UpdateFusion fz;          // the mirror and squares of the new positions
  float pf = 0.f;           // 1 / (s^2 T) of the prior, 0 for a flat prior
  double* sq = nullptr;     // owned [chains, update_blocks]

  int draws() const { return integ.kind == GBSGMC_INTEGRATOR_OBABO ? 2 : 1; }

  ~NetPlan() override {
    if (stream != nullptr) cudaStreamSynchronize(stream);
    plan_free(this, grad);
    plan_free(this, grad2);
    plan_free(this, U2);
    plan_free(this, idx);
    plan_free(this, ws);
    plan_free(this, sq);
  }

  int enqueue_fused(int g, cudaStream_t s);
  int enqueue_obabo(int g, const UpdateFusion& moving, const UpdateFusion& last,
                    cudaStream_t s);

  // With an external index source the caller writes the block's indices
  // (gbsgmc_plan_set_indices); until then the buffer holds index 0.
  int setup_external(const char* what) {
    if (!isrc.external) return GBSGMC_OK;
    ext_idx = idx;
    ext_per_step = static_cast<int64_t>(chains) * draws() * n;
    return cuda_err(cudaMemsetAsync(idx, 0, sizeof(int32_t) * G * ext_per_step, stream),
                    what);
  }

  // The gradient buffers: OBABO keeps two, because its second gradient of
  // step j and its first gradient of step j + 1 feed one update pass.
  int alloc_grads(const char* what) {
    const size_t bytes = sizeof(float) * static_cast<size_t>(chains) * P;
    int rc = plan_alloc(this, &grad, bytes, what);
    if (rc == GBSGMC_OK && integ.kind == GBSGMC_INTEGRATOR_OBABO)
      rc = plan_alloc(this, &grad2, bytes, what);
    return rc;
  }

  int step_multiple() const override {
    return integ.kind == GBSGMC_INTEGRATOR_SGHMC ? integ.leapfrog_steps : 1;
  }

  int64_t launches_per_block(int g) const override {
    // Kernels of one value-and-gradient call are counted by the caller.
    // Every block: the index draw (unless external), the step counter and,
    // fused, the mirror.
    const int64_t fixed = (fused ? 3 : 2) - (isrc.external ? 1 : 0);
    switch (integ.kind) {
      case GBSGMC_INTEGRATOR_OBABO: return fixed + 2 + static_cast<int64_t>(g);
      case GBSGMC_INTEGRATOR_SGHMC:
        return fixed + 2 * static_cast<int64_t>(g) + g / integ.leapfrog_steps;
      default: return fixed + static_cast<int64_t>(g);
    }
  }

  int enqueue(int g, cudaStream_t s) override {
    if (fused) return enqueue_fused(g, s);
    const int per = draws() * n;
    const int64_t cn = static_cast<int64_t>(chains) * per;
    int rc;
    if (isrc.external) {
      rc = GBSGMC_OK;  // written by gbsgmc_plan_set_indices
    } else if (isrc.pcg_dev != nullptr) {
      rc = gbsgmc_index_draw_pcg64(isrc.pcg_dev, chains, rows, static_cast<int64_t>(g) * per,
                                   per, idx, per, cn, status, s);
    } else {
      rc = launch_philox_index(isrc.index_seed, isrc.chain_base, chains, base, 0, g, per,
                               rows, idx, per, cn, s);
    }
    if (rc != GBSGMC_OK) return rc;
    if (integ.kind == GBSGMC_INTEGRATOR_OBABO) {
      if ((rc = enqueue_obabo(g, UpdateFusion{}, UpdateFusion{}, s))) return rc;
      return plan_advance(this, g, s);
    }
    for (int j = 0; j < g; ++j) {
      gbsgmc_sched sj = sched;
      sj.base_dev = base;
      sj.offset = j;
      const int32_t* ij = idx + j * cn;
      switch (integ.kind) {
        case GBSGMC_INTEGRATOR_SGLD:
          if ((rc = grad_fn(ij, per, U, lk_var, grad, s))) return rc;
          rc = gbsgmc_sgld_update(chains, P, x, grad, aux, integ.alpha, integ.lmbd, &sj,
                                  &noise, nullptr, s);
          break;
        default:  // SGHMC
          if (j % integ.leapfrog_steps == 0 &&
              (rc = gbsgmc_sghmc_resample(chains, P, aux, integ.mass_dev, &sj, &noise, s)))
            return rc;
          if ((rc = gbsgmc_sghmc_position(chains, P, x, aux, integ.mass_dev, nullptr,
                                          integ.friction, &sj, s)))
            return rc;
          if ((rc = grad_fn(ij, per, U, lk_var, grad, s))) return rc;
          rc = gbsgmc_sghmc_momentum(chains, P, aux, grad, nullptr, integ.friction, &sj,
                                     &noise, s);
          break;
      }
      if (rc != GBSGMC_OK) return rc;
    }
    return plan_advance(this, g, s);
  }
};

int NetPlan::enqueue_fused(int g, cudaStream_t s) {
  const int per = draws() * n;
  const int64_t cn = static_cast<int64_t>(chains) * per;
  int rc;
  if (isrc.external) {
    rc = GBSGMC_OK;  // written by gbsgmc_plan_set_indices
  } else if (isrc.pcg_dev != nullptr) {
    rc = gbsgmc_index_draw_pcg64(isrc.pcg_dev, chains, rows, static_cast<int64_t>(g) * per,
                                 per, idx, per, cn, status, s);
  } else {
    rc = launch_philox_index(isrc.index_seed, isrc.chain_base, chains, base, 0, g, per, rows,
                             idx, per, cn, s);
  }
  if (rc != GBSGMC_OK) return rc;
  // The positions may have changed since the last block: refresh the mirror
  // and the squares once per block; the updates keep them current after.
  if ((rc = mirror_fused(chains, P, x, fz, s))) return rc;
  UpdateFusion prior_only;
  prior_only.prior_pf = pf;
  UpdateFusion with_prior = fz;
  with_prior.prior_pf = pf;
  if (integ.kind == GBSGMC_INTEGRATOR_OBABO) {
    if ((rc = enqueue_obabo(g, with_prior, prior_only, s))) return rc;
    return plan_advance(this, g, s);
  }
  for (int j = 0; j < g; ++j) {
    gbsgmc_sched sj = sched;
    sj.base_dev = base;
    sj.offset = j;
    const int32_t* ij = idx + j * cn;
    switch (integ.kind) {
      case GBSGMC_INTEGRATOR_SGLD:
        if ((rc = grad_fn(ij, per, U, lk_var, grad, s))) return rc;
        rc = sgld_update_fused(chains, P, x, grad, aux, integ.alpha, integ.lmbd, &sj, &noise,
                               with_prior, s);
        break;
      default:  // SGHMC
        if (j % integ.leapfrog_steps == 0 &&
            (rc = gbsgmc_sghmc_resample(chains, P, aux, integ.mass_dev, &sj, &noise, s)))
          return rc;
        if ((rc = sghmc_position_fused(chains, P, x, aux, integ.mass_dev, integ.friction, &sj,
                                       fz, s)))
          return rc;
        if ((rc = grad_fn(ij, per, U, lk_var, grad, s))) return rc;
        rc = sghmc_momentum_fused(chains, P, x, aux, grad, integ.friction, &sj, &noise,
                                  prior_only, s);
        break;
    }
    if (rc != GBSGMC_OK) return rc;
  }
  return plan_advance(this, g, s);
}

// OBABO over the block's g steps (integrator.py:192-273), indices already
// drawn.  Step j's first half moves the positions; its second gradient and
// step j + 1's first gradient are both taken there, so step j's second half
// and step j + 1's first half run as one pass over the parameters.  The
// block's last step ends with its own second half, and the potential is the
// mean of that step's two minibatch values.  `moving` is the fusion of the
// passes that move x, `last` that of the final second half.
int NetPlan::enqueue_obabo(int g, const UpdateFusion& moving, const UpdateFusion& last,
                           cudaStream_t s) {
  const int per = draws() * n;
  const int64_t cn = static_cast<int64_t>(chains) * per;
  double* ke_start = ke;
  double* ke_end = ke != nullptr ? ke + chains : nullptr;
  gbsgmc_sched sj = sched;
  sj.base_dev = base;
  sj.offset = 0;
  int rc;
  if ((rc = grad_fn(idx, per, U, nullptr, grad, s))) return rc;
  if ((rc = obabo_first_fused(chains, P, x, aux, grad, integ.mass_dev, integ.friction,
                              ke_start, &sj, &noise, moving, s)))
    return rc;
  for (int j = 0; j + 1 < g; ++j) {
    const int32_t* ij = idx + j * cn;
    if ((rc = grad_fn(ij + n, per, U2, nullptr, grad2, s))) return rc;
    if ((rc = grad_fn(ij + cn, per, U, nullptr, grad, s))) return rc;
    sj.offset = j;
    if ((rc = obabo_second_first_fused(chains, P, x, aux, grad2, grad, integ.mass_dev,
                                       integ.friction, ke_end, ke_start, &sj, &noise, moving,
                                       s)))
      return rc;
  }
  sj.offset = g - 1;
  if ((rc = grad_fn(idx + (g - 1) * cn + n, per, U2, lk_var, grad2, s))) return rc;
  if ((rc = obabo_second_fused(chains, P, x, aux, grad2, integ.mass_dev, integ.friction,
                               ke_end, &sj, &noise, last, s)))
    return rc;
  mean_pair_kernel<<<(chains + 127) / 128, 128, 0, s>>>(chains, U, U2);
  return check_launch("plan: potential mean");
}

// reSGLD over R replicas with ragged minibatches and adjacent exchanges.
struct ResgldPlan final : gbsgmc_plan {
  GradFn grad_fn;
  int replicas = 0, n_max = 0;
  int64_t P = 0, rows = 0;
  float* x = nullptr;
  float* v = nullptr;
  float alpha = 0.9f, lmbd = 1e-5f;
  float* grad = nullptr;  // owned [R, P]
  gbsgmc_sched sched{};
  gbsgmc_noise noise{};
  gbsgmc_index_src isrc{};
  gbsgmc_tempering temp{};
  double* U = nullptr;
  double* lk_var = nullptr;
  double* var_own = nullptr;  // owned when the caller passes no lk_var buffer
  float* samples = nullptr;     // kept states of replica 0 [n_kept, P], or null
  double* sample_lik = nullptr; // their -U [n_kept]
  int* status = nullptr;
  int32_t* idx = nullptr;  // owned [G, R, n_max]
  void* ws = nullptr;      // owned
  size_t ws_size = 0;

  ~ResgldPlan() override {
    if (stream != nullptr) cudaStreamSynchronize(stream);
    plan_free(this, grad);
    plan_free(this, idx);
    plan_free(this, ws);
    plan_free(this, var_own);
  }

  int step_multiple() const override { return temp.every; }

  int64_t launches_per_block(int g) const override {
    return 2 + (samples != nullptr ? 3 : 2) * static_cast<int64_t>(g) + 3 * (g / temp.every);
  }

  int enqueue(int g, cudaStream_t s) override {
    const int64_t cn = static_cast<int64_t>(replicas) * n_max;
    int rc;
    if (isrc.pcg_dev != nullptr) {
      rc = gbsgmc_index_draw_pcg64(isrc.pcg_dev, replicas, rows,
                                   static_cast<int64_t>(g) * n_max, n_max, idx, n_max, cn,
                                   status, s);
    } else {
      rc = launch_philox_index(isrc.index_seed, isrc.chain_base, replicas, base, 0, g, n_max,
                               rows, idx, n_max, cn, s);
    }
    if (rc != GBSGMC_OK) return rc;
    for (int j = 0; j < g; ++j) {
      gbsgmc_sched sj = sched;
      sj.base_dev = base;
      sj.offset = j;
      gbsgmc_sched step_sched = sj;
      step_sched.keep_slot_dev = nullptr;  // kept samples are taken after the exchange
      if ((rc = grad_fn(idx + j * cn, n_max, U, lk_var, grad, s))) return rc;
      if ((rc = gbsgmc_sgld_update(replicas, P, x, grad, v, alpha, lmbd, &step_sched, &noise,
                                   nullptr, s)))
        return rc;
      if ((rc = gbsgmc_resgld_sa_update(replicas, lk_var, temp.ssq_dev, temp.k_dev, s)))
        return rc;
      if ((j + 1) % temp.every == 0 &&
          (rc = gbsgmc_resgld_exchange_adjacent(replicas, P, x, v, U, lk_var, &step_sched,
                                                temp.every, temp.ssq_dev, temp.F, temp.seed,
                                                nullptr, temp.flags_dev, temp.counts_dev,
                                                nullptr, s)))
        return rc;
      if (samples != nullptr &&
          (rc = keep_row(P, x, U, &sj, samples, sample_lik, s)))
        return rc;
    }
    return plan_advance(this, g, s);
  }
};

// alias.re_sgld on the dense network: `pairs` (normal, hot) pairs of SGLD
// chains and each pair's exchange after every step, as GlmPairsPlan runs them
// on a generalised-linear potential.  Row c of x holds the chain identity
// ident[c]: the minibatch rows are read from that identity's index stream
// and the noise is drawn as that chain, so streams travel with the states.
struct MlpPairsPlan final : gbsgmc_plan {
  gbsgmc_mlp model{};
  int pairs = 0, n = 0;
  int64_t P = 0, rows = 0;
  float* x = nullptr;
  float* v = nullptr;
  float alpha = 0.9f, lmbd = 1e-5f;
  float* grad = nullptr;  // owned [2 pairs, P]
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
  int32_t* idx = nullptr;  // owned [G, 2 pairs, n], by identity
  void* ws = nullptr;      // owned
  size_t ws_size = 0;

  ~MlpPairsPlan() override {
    if (stream != nullptr) cudaStreamSynchronize(stream);
    plan_free(this, grad);
    plan_free(this, idx);
    plan_free(this, ws);
  }

  // Per block the index draw and the step counter; per step the update and
  // the exchange (the value-and-gradient launches are counted by the caller).
  int64_t launches_per_block(int g) const override { return 2 + 2 * static_cast<int64_t>(g); }

  int enqueue(int g, cudaStream_t s) override {
    const int chains = 2 * pairs;
    const int64_t cn = static_cast<int64_t>(chains) * n;
    int rc = gbsgmc_index_draw_pcg64(isrc.pcg_dev, chains, rows, static_cast<int64_t>(g) * n, n,
                                     idx, n, cn, status, s);
    if (rc != GBSGMC_OK) return rc;
    UpdateFusion by_identity;
    by_identity.ident = ident;
    for (int j = 0; j < g; ++j) {
      gbsgmc_sched sj = sched;
      sj.base_dev = base;
      sj.offset = j;
      gbsgmc_sched step_sched = sj;
      step_sched.keep_slot_dev = nullptr;  // the exchange stores the samples
      if ((rc = mlp_value_and_grad_ident(&model, chains, n, idx + j * cn, n, ident, x, U, grad,
                                         lk_var, ws, ws_size, status, s)))
        return rc;
      if ((rc = sgld_update_fused(chains, P, x, grad, v, alpha, lmbd, &step_sched, &noise,
                                  by_identity, s)))
        return rc;
      if ((rc = resgld_pairs_exchange(pairs, static_cast<int>(P), x, v, U, lk_var, ident, &sj,
                                      temp.F, temp.seed, pair_chain, temp.ssq_dev, temp.k_dev,
                                      temp.counts_dev, samples, sample_lik, s)))
        return rc;
    }
    return plan_advance(this, g, s);
  }
};

int check_common(const gbsgmc_integrator* integ, int chains, int n, float* x, float* aux,
                 const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                 const gbsgmc_index_src* isrc, double* U, int block_steps, int* status) {
  if (integ == nullptr || x == nullptr || sched == nullptr || noise == nullptr ||
      isrc == nullptr || U == nullptr || status == nullptr)
    return set_error(GBSGMC_ERR_ARG, "net plan: null argument");
  if (chains <= 0 || n <= 0 || block_steps <= 0 || block_steps > 100000)
    return set_error(GBSGMC_ERR_ARG, "net plan: bad chains/n/block_steps");
  if (integ->kind < GBSGMC_INTEGRATOR_SGLD || integ->kind > GBSGMC_INTEGRATOR_SGHMC)
    return set_error(GBSGMC_ERR_ARG, "net plan: unknown integrator %d", integ->kind);
  if (integ->kind != GBSGMC_INTEGRATOR_SGLD && aux == nullptr)
    return set_error(GBSGMC_ERR_ARG, "net plan: OBABO and SGHMC need a momentum buffer");
  if (integ->kind == GBSGMC_INTEGRATOR_SGHMC &&
      (integ->leapfrog_steps < 1 || block_steps % integ->leapfrog_steps != 0))
    return set_error(GBSGMC_ERR_ARG,
                     "net plan: block_steps must be a multiple of leapfrog_steps");
  if (sched->keep_slot_dev != nullptr)
    return set_error(GBSGMC_ERR_UNSUPPORTED,
                     "net plan: samples are collected by the caller between runs");
  return GBSGMC_OK;
}

}  // namespace
}  // namespace gbsgmc

using namespace gbsgmc;

extern "C" int gbsgmc_mlp_plan_create(gbsgmc_plan** out, const gbsgmc_mlp* model,
                                      int chains, int n, const gbsgmc_integrator* integ,
                                      float* x_dev, float* aux_dev,
                                      const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                                      const gbsgmc_index_src* isrc, double* U_dev,
                                      double* lk_var_dev, double* ke_dev, int block_steps,
                                      int* status_dev) {
  if (out == nullptr) return set_error(GBSGMC_ERR_ARG, "mlp_plan_create: null plan");
  *out = nullptr;
  int rc = check_common(integ, chains, n, x_dev, aux_dev, sched, noise, isrc, U_dev,
                        block_steps, status_dev);
  if (rc != GBSGMC_OK) return rc;
  if (model == nullptr) return set_error(GBSGMC_ERR_ARG, "mlp_plan_create: null model");
  const size_t ws = gbsgmc_mlp_workspace_bytes(model, chains, n);
  if (ws == 0)
    return set_error(GBSGMC_ERR_SHAPE, "mlp_plan_create: unsupported shape (n %% 128)");
  NetPlan* p = new (std::nothrow) NetPlan();
  if (p == nullptr) return set_error(GBSGMC_ERR_ARG, "mlp_plan_create: out of memory");
  p->chains = chains;
  p->n = n;
  p->P = gbsgmc_mlp_param_count(model);
  p->rows = model->n_rows > 0 ? model->n_rows : model->n_obs;
  p->integ = *integ;
  p->x = x_dev;
  p->aux = aux_dev;
  p->sched = *sched;
  p->noise = *noise;
  p->isrc = *isrc;
  p->U = U_dev;
  p->lk_var = lk_var_dev;
  p->ke = ke_dev;
  p->status = status_dev;
  p->ws_size = ws;
  do {
    if ((rc = plan_init(p, block_steps))) break;
    const size_t ibytes = sizeof(int32_t) * static_cast<size_t>(block_steps) * chains *
                          p->draws() * n;
    if ((rc = p->alloc_grads("mlp_plan_create: gradient"))) break;
    if ((rc = plan_alloc(p, &p->U2, sizeof(double) * chains, "mlp_plan_create: U")))
      break;
    if ((rc = plan_alloc(p, &p->idx, ibytes, "mlp_plan_create: index buffer"))) break;
    if ((rc = plan_alloc(p, &p->ws, ws, "mlp_plan_create: workspace"))) break;
    const gbsgmc_mlp m = *model;
    void* wsp = p->ws;
    const float* x = x_dev;
    const char* env = std::getenv("GBSGMC_NO_STEP_FUSION");
    p->fused = !(env != nullptr && env[0] == '1') && integ->mass_dev == nullptr;
    if (p->fused) {
      const int nb = update_blocks(chains, p->P);
      if ((rc = plan_alloc(p, &p->sq, sizeof(double) * chains * nb, "mlp_plan_create: squares")))
        break;
      mlp_mirror_region(&m, chains, n, wsp, &p->fz.mirror, &p->fz.mirror_count,
                        &p->fz.mirror_stride);
      p->fz.sq_parts = p->sq;
      if (m.prior_scale > 0.f)
        p->pf = static_cast<float>(1.0 / (static_cast<double>(m.prior_scale) *
                                          m.prior_scale * m.temperature));
      const double* sqp = p->sq;
      p->grad_fn = [m, chains, n, x, wsp, ws, status_dev, sqp, nb](
                       const int32_t* idx, int64_t stride, double* U, double* var, float* grad,
                       cudaStream_t s) {
        return mlp_value_and_grad_fused(&m, chains, n, idx, stride, x, U, grad, var, wsp, ws,
                                        status_dev, s, sqp, nb);
      };
    } else {
      p->grad_fn = [m, chains, n, x, wsp, ws, status_dev](
                       const int32_t* idx, int64_t stride, double* U, double* var, float* grad,
                       cudaStream_t s) {
        return gbsgmc_mlp_value_and_grad(&m, chains, n, idx, stride, nullptr, x, U, grad,
                                         nullptr, var, wsp, ws, status_dev, s);
      };
    }
    if ((rc = p->setup_external("mlp_plan_create: index memset"))) break;
    rc = plan_capture(p);
  } while (false);
  if (rc != GBSGMC_OK) {
    delete p;
    return rc;
  }
  *out = p;
  return GBSGMC_OK;
}

extern "C" int gbsgmc_cnn_plan_create(gbsgmc_plan** out, const gbsgmc_cnn* model,
                                      int chains, int n, const gbsgmc_integrator* integ,
                                      float* x_dev, float* aux_dev,
                                      const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                                      const gbsgmc_index_src* isrc, double* U_dev,
                                      double* lk_var_dev, double* ke_dev, int block_steps,
                                      int* status_dev) {
  if (out == nullptr) return set_error(GBSGMC_ERR_ARG, "cnn_plan_create: null plan");
  *out = nullptr;
  int rc = check_common(integ, chains, n, x_dev, aux_dev, sched, noise, isrc, U_dev,
                        block_steps, status_dev);
  if (rc != GBSGMC_OK) return rc;
  if (model == nullptr) return set_error(GBSGMC_ERR_ARG, "cnn_plan_create: null model");
  const size_t ws = gbsgmc_cnn_workspace_bytes(chains, n);
  if (ws == 0) return set_error(GBSGMC_ERR_SHAPE, "cnn_plan_create: n must be even");
  NetPlan* p = new (std::nothrow) NetPlan();
  if (p == nullptr) return set_error(GBSGMC_ERR_ARG, "cnn_plan_create: out of memory");
  p->chains = chains;
  p->n = n;
  p->P = gbsgmc_cnn_param_count();
  p->rows = model->n_rows > 0 ? model->n_rows : model->n_obs;
  p->integ = *integ;
  p->x = x_dev;
  p->aux = aux_dev;
  p->sched = *sched;
  p->noise = *noise;
  p->isrc = *isrc;
  p->U = U_dev;
  p->lk_var = lk_var_dev;
  p->ke = ke_dev;
  p->status = status_dev;
  p->ws_size = ws;
  do {
    if ((rc = plan_init(p, block_steps))) break;
    const size_t ibytes = sizeof(int32_t) * static_cast<size_t>(block_steps) * chains *
                          p->draws() * n;
    if ((rc = p->alloc_grads("cnn_plan_create: gradient"))) break;
    if ((rc = plan_alloc(p, &p->U2, sizeof(double) * chains, "cnn_plan_create: U")))
      break;
    if ((rc = plan_alloc(p, &p->idx, ibytes, "cnn_plan_create: index buffer"))) break;
    if ((rc = plan_alloc(p, &p->ws, ws, "cnn_plan_create: workspace"))) break;
    const gbsgmc_cnn m = *model;
    void* wsp = p->ws;
    const float* x = x_dev;
    p->grad_fn = [m, chains, n, x, wsp, ws, status_dev](
                     const int32_t* idx, int64_t stride, double* U, double* var, float* grad,
                     cudaStream_t s) {
      return gbsgmc_cnn_value_and_grad(&m, chains, n, idx, stride, nullptr, x, U, grad,
                                       nullptr, var, wsp, ws, status_dev, s);
    };
    if ((rc = p->setup_external("cnn_plan_create: index memset"))) break;
    rc = plan_capture(p);
  } while (false);
  if (rc != GBSGMC_OK) {
    delete p;
    return rc;
  }
  *out = p;
  return GBSGMC_OK;
}

extern "C" int gbsgmc_mlp_resgld_plan_create(
    gbsgmc_plan** out, const gbsgmc_mlp* model, int replicas, int n_max, const int32_t* n_dev,
    float* x_dev, float* v_dev, float alpha, float lmbd, const gbsgmc_sched* sched,
    const gbsgmc_noise* noise, const gbsgmc_index_src* isrc, const gbsgmc_tempering* temp,
    double* U_dev, double* lk_var_dev, int block_steps, int* status_dev) {
  if (sched != nullptr && sched->keep_slot_dev != nullptr)
    return set_error(GBSGMC_ERR_UNSUPPORTED,
                     "mlp_resgld_plan_create: kept samples need "
                     "gbsgmc_mlp_resgld_plan_create_keep");
  return gbsgmc_mlp_resgld_plan_create_keep(out, model, replicas, n_max, n_dev, x_dev, v_dev,
                                            alpha, lmbd, sched, noise, isrc, temp, U_dev,
                                            lk_var_dev, nullptr, nullptr, block_steps,
                                            status_dev);
}

extern "C" int gbsgmc_mlp_resgld_plan_create_keep(
    gbsgmc_plan** out, const gbsgmc_mlp* model, int replicas, int n_max, const int32_t* n_dev,
    float* x_dev, float* v_dev, float alpha, float lmbd, const gbsgmc_sched* sched,
    const gbsgmc_noise* noise, const gbsgmc_index_src* isrc, const gbsgmc_tempering* temp,
    double* U_dev, double* lk_var_dev, float* samples_dev, double* sample_lik_dev,
    int block_steps, int* status_dev) {
  if (out == nullptr) return set_error(GBSGMC_ERR_ARG, "mlp_resgld_plan_create: null plan");
  *out = nullptr;
  if (model == nullptr || n_dev == nullptr || x_dev == nullptr || sched == nullptr ||
      noise == nullptr || isrc == nullptr || temp == nullptr || U_dev == nullptr ||
      status_dev == nullptr || temp->ssq_dev == nullptr || temp->k_dev == nullptr ||
      temp->flags_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG, "mlp_resgld_plan_create: null argument");
  if (replicas < 2 || replicas > 65535 || n_max <= 0 || block_steps <= 0 ||
      block_steps > 100000 || temp->every < 1 || block_steps % temp->every != 0 ||
      !(temp->F > 0))
    return set_error(GBSGMC_ERR_ARG,
                     "mlp_resgld_plan_create: bad replicas, sizes or exchange period "
                     "(block_steps must be a multiple of every)");
  if ((sched->keep_slot_dev != nullptr) != (samples_dev != nullptr))
    return set_error(GBSGMC_ERR_ARG,
                     "mlp_resgld_plan_create: a keep table and a sample buffer go together");
  if (isrc->external)
    return set_error(GBSGMC_ERR_UNSUPPORTED,
                     "mlp_resgld_plan_create: external index sources");
  const size_t ws = gbsgmc_mlp_workspace_bytes(model, replicas, n_max);
  if (ws == 0)
    return set_error(GBSGMC_ERR_SHAPE, "mlp_resgld_plan_create: unsupported shape (n_max %% 128)");
  ResgldPlan* p = new (std::nothrow) ResgldPlan();
  if (p == nullptr) return set_error(GBSGMC_ERR_ARG, "mlp_resgld_plan_create: out of memory");
  p->replicas = replicas;
  p->n_max = n_max;
  p->P = gbsgmc_mlp_param_count(model);
  p->rows = model->n_rows > 0 ? model->n_rows : model->n_obs;
  p->x = x_dev;
  p->v = v_dev;
  p->alpha = alpha;
  p->lmbd = lmbd;
  p->sched = *sched;
  p->noise = *noise;
  p->isrc = *isrc;
  p->temp = *temp;
  p->U = U_dev;
  p->lk_var = lk_var_dev;
  p->samples = samples_dev;
  p->sample_lik = sample_lik_dev;
  p->status = status_dev;
  p->ws_size = ws;
  int rc = GBSGMC_OK;
  do {
    if ((rc = plan_init(p, block_steps))) break;
    if (p->lk_var == nullptr) {
      if ((rc = plan_alloc(p, &p->var_own, sizeof(double) * replicas, "mlp_resgld_plan_create: var")))
        break;
      p->lk_var = p->var_own;
    }
    const size_t gbytes = sizeof(float) * static_cast<size_t>(replicas) * p->P;
    const size_t ibytes = sizeof(int32_t) * static_cast<size_t>(block_steps) * replicas * n_max;
    if ((rc = plan_alloc(p, &p->grad, gbytes, "mlp_resgld_plan_create: gradient")))
      break;
    if ((rc = plan_alloc(p, &p->idx, ibytes, "mlp_resgld_plan_create: index buffer")))
      break;
    if ((rc = plan_alloc(p, &p->ws, ws, "mlp_resgld_plan_create: workspace"))) break;
    const gbsgmc_mlp m = *model;
    void* wsp = p->ws;
    const float* x = x_dev;
    p->grad_fn = [m, replicas, n_max, n_dev, x, wsp, ws, status_dev](
                     const int32_t* idx, int64_t stride, double* U, double* var, float* grad,
                     cudaStream_t s) {
      return gbsgmc_mlp_value_and_grad_ragged(&m, replicas, n_max, n_dev, idx, stride, nullptr,
                                              x, U, grad, nullptr, var, wsp, ws, status_dev,
                                              s);
    };
    rc = plan_capture(p);
  } while (false);
  if (rc != GBSGMC_OK) {
    delete p;
    return rc;
  }
  *out = p;
  return GBSGMC_OK;
}

extern "C" int gbsgmc_mlp_resgld_pairs_plan_create(
    gbsgmc_plan** out, const gbsgmc_mlp* model, int pairs, int n, float* x_dev, float* v_dev,
    float alpha, float lmbd, const gbsgmc_sched* sched, const gbsgmc_noise* noise,
    const gbsgmc_index_src* index_src, const gbsgmc_tempering* tempering,
    const int32_t* pair_chain_dev, int32_t* ident_dev, double* U_dev, double* lk_var_dev,
    float* samples_dev, double* sample_lik_dev, int block_steps, int* status_dev) {
  if (out == nullptr)
    return set_error(GBSGMC_ERR_ARG, "mlp_resgld_pairs_plan_create: null plan");
  *out = nullptr;
  if (model == nullptr || sched == nullptr || noise == nullptr || index_src == nullptr ||
      tempering == nullptr || x_dev == nullptr || pair_chain_dev == nullptr ||
      ident_dev == nullptr || U_dev == nullptr || lk_var_dev == nullptr ||
      status_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG, "mlp_resgld_pairs_plan_create: null argument");
  if (pairs <= 0 || 2 * pairs > 65535 || n <= 0 || block_steps <= 0 || block_steps > 100000)
    return set_error(GBSGMC_ERR_ARG, "mlp_resgld_pairs_plan_create: bad pairs/n/block_steps");
  if (index_src->pcg_dev == nullptr || index_src->external)
    return set_error(GBSGMC_ERR_ARG,
                     "mlp_resgld_pairs_plan_create: needs PCG64 index streams (one per chain)");
  if (sched->chain_temperature_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG,
                     "mlp_resgld_pairs_plan_create: needs the per-chain temperatures");
  if (tempering->ssq_dev == nullptr || tempering->k_dev == nullptr || !(tempering->F != 0.0))
    return set_error(GBSGMC_ERR_ARG, "mlp_resgld_pairs_plan_create: bad tempering state");
  if (sched->keep_slot_dev != nullptr && samples_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG,
                     "mlp_resgld_pairs_plan_create: keep table given without sample buffer");
  const size_t ws = gbsgmc_mlp_workspace_bytes(model, 2 * pairs, n);
  if (ws == 0)
    return set_error(GBSGMC_ERR_SHAPE,
                     "mlp_resgld_pairs_plan_create: unsupported shape (n %% 128)");
  const int64_t P = gbsgmc_mlp_param_count(model);
  if (P <= 0 || P > (1ll << 31) - 1)
    return set_error(GBSGMC_ERR_SHAPE, "mlp_resgld_pairs_plan_create: parameter count");
  MlpPairsPlan* p = new (std::nothrow) MlpPairsPlan();
  if (p == nullptr)
    return set_error(GBSGMC_ERR_ARG, "mlp_resgld_pairs_plan_create: out of memory");
  p->model = *model;
  p->pairs = pairs;
  p->n = n;
  p->P = P;
  p->rows = model->n_rows > 0 ? model->n_rows : model->n_obs;
  p->x = x_dev;
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
  p->ws_size = ws;
  int rc = GBSGMC_OK;
  do {
    if ((rc = plan_init(p, block_steps))) break;
    const int chains = 2 * pairs;
    if ((rc = plan_alloc(p, &p->grad, sizeof(float) * static_cast<size_t>(chains) * P,
                         "mlp_resgld_pairs_plan_create: gradient")))
      break;
    if ((rc = plan_alloc(p, &p->idx,
                         sizeof(int32_t) * static_cast<size_t>(block_steps) * chains * n,
                         "mlp_resgld_pairs_plan_create: index buffer")))
      break;
    if ((rc = plan_alloc(p, &p->ws, ws, "mlp_resgld_pairs_plan_create: workspace"))) break;
    rc = plan_capture(p);
  } while (false);
  if (rc != GBSGMC_OK) {
    delete p;
    return rc;
  }
  *out = p;
  return GBSGMC_OK;
}

extern "C" int gbsgmc_glm_plan_create(gbsgmc_plan** out, const gbsgmc_glm* model,
                                      int chains, int n, const gbsgmc_integrator* integ,
                                      float* x_dev, float* aux_dev,
                                      const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                                      const gbsgmc_index_src* isrc, double* U_dev,
                                      double* lk_var_dev, double* ke_dev, int block_steps,
                                      int* status_dev) {
  if (out == nullptr) return set_error(GBSGMC_ERR_ARG, "glm_plan_create: null plan");
  *out = nullptr;
  int rc = check_common(integ, chains, n, x_dev, aux_dev, sched, noise, isrc, U_dev,
                        block_steps, status_dev);
  if (rc != GBSGMC_OK) return rc;
  if (model == nullptr) return set_error(GBSGMC_ERR_ARG, "glm_plan_create: null model");
  const size_t ws = gbsgmc_glm_workspace_bytes(chains, n, model->d);
  if (ws == 0) return set_error(GBSGMC_ERR_SHAPE, "glm_plan_create: bad shape");
  NetPlan* p = new (std::nothrow) NetPlan();
  if (p == nullptr) return set_error(GBSGMC_ERR_ARG, "glm_plan_create: out of memory");
  p->chains = chains;
  p->n = n;
  p->P = model->d;
  p->rows = model->n_rows > 0 ? model->n_rows : model->n_obs;
  p->integ = *integ;
  p->x = x_dev;
  p->aux = aux_dev;
  p->sched = *sched;
  p->noise = *noise;
  p->isrc = *isrc;
  p->U = U_dev;
  p->lk_var = lk_var_dev;
  p->ke = ke_dev;
  p->status = status_dev;
  p->ws_size = ws;
  do {
    if ((rc = plan_init(p, block_steps))) break;
    const size_t ibytes = sizeof(int32_t) * static_cast<size_t>(block_steps) * chains *
                          p->draws() * n;
    if ((rc = p->alloc_grads("glm_plan_create: gradient"))) break;
    if ((rc = plan_alloc(p, &p->U2, sizeof(double) * chains, "glm_plan_create: U")))
      break;
    if ((rc = plan_alloc(p, &p->idx, ibytes, "glm_plan_create: index buffer"))) break;
    if ((rc = plan_alloc(p, &p->ws, ws, "glm_plan_create: workspace"))) break;
    // The GLM workspace's tickets start at zero and are left at zero.
    if ((rc = cuda_err(cudaMemsetAsync(p->ws, 0, ws, p->stream), "glm_plan_create: memset")))
      break;
    if ((rc = glm_prepare())) break;
    const gbsgmc_glm m = *model;
    void* wsp = p->ws;
    const float* x = x_dev;
    p->grad_fn = [m, chains, n, x, wsp, ws, status_dev](
                     const int32_t* idx, int64_t stride, double* U, double* var, float* grad,
                     cudaStream_t s) {
      return gbsgmc_glm_value_and_grad(&m, chains, n, idx, stride, nullptr, x, U, grad,
                                       nullptr, var, wsp, ws, status_dev, s);
    };
    if ((rc = p->setup_external("glm_plan_create: index memset"))) break;
    rc = plan_capture(p);
  } while (false);
  if (rc != GBSGMC_OK) {
    delete p;
    return rc;
  }
  *out = p;
  return GBSGMC_OK;
}
