"""The fused many-chain SGLD driver.

``run_sgld_glm`` runs C chains of SGLD(+RMSprop) on a GLM potential as one
``gbsgmc_sgld_glm_plan``: per step ONE kernel launch for all chains (gather,
likelihood, adjoint, reduction, prior, RMSprop, noise, update, sample
store), with the index draws of a block of steps in one more launch and the
block replayed from a CUDA graph.  It replaces ``solver.mcmc``'s per-chain
``jit(lax.scan)`` over ``langevin_diffusion.update_fn``
(jax_sgmc/solver.py:152-171, jax_sgmc/integrator.py:860-922).
"""

from __future__ import annotations

from typing import List, NamedTuple

import numpy as np

from . import _lib, io, scheduler as sched_mod
from .data.core import RandomBatchFn, ShuffledFeed

DEFAULT_BLOCK_STEPS = 50

# When False, solver.mcmc steps every chain through the per-step C ABI calls
# instead of the fused plan (used to cross-check the two paths).
FUSED_ENABLED = True


class SgldRun(NamedTuple):
  w: object            # fp32 [C, d] final positions
  v: object            # fp32 [C, d] RMSprop state or None
  U: object            # fp64 [C] potential at the last pre-update position
  lk_var: object       # fp64 [C]
  samples: object      # fp32 [S, C, d]
  sample_lik: object   # fp64 [S, C]
  launches: int
  host: object = None  # [samples, likelihoods] host arrays, when copied
  early: object = None # what on_enqueued returned


# Device bytes the kept samples of a network plan may occupy with host
# saving; beyond that they pass through a ring of rows emptied to the host
# during the run.
RING_BYTES = 4 << 30

# Per-pair exchange counts ([P] int32, host) of the last reSGLD pairs run
# through try_fused_resgld, for inspection.
LAST_EXCHANGES = None


class _ExternalIndices:
  """Feeds a plan with an external index source: before each run of at
  most one block, the next steps' indices from a :class:`ShuffledFeed` go
  through one of two pinned host buffers into the plan
  (``gbsgmc_plan_set_indices``), so that the host prepares block b + 1
  while the GPU runs block b."""

  def __init__(self, feed, G, C, per_chain_step):
    import torch
    self.feed, self.G = feed, int(G)
    self.bufs = [torch.empty((self.G, C, per_chain_step), dtype=torch.int32,
                             pin_memory=True) for _ in range(2)]
    self.events = [None, None]
    self.turn = 0

  def run(self, handle, first_step, steps):
    import torch
    done = 0
    while done < steps:
      g = min(self.G, steps - done)
      i = self.turn
      self.turn ^= 1
      if self.events[i] is not None:
        self.events[i].synchronize()   # its previous copy has left the buffer
      self.feed.next(g, out=self.bufs[i].numpy())
      _lib.call("gbsgmc_plan_set_indices", handle, _lib.ptr(self.bufs[i]), g,
                _lib.stream_handle())
      ev = torch.cuda.Event()
      ev.record()
      self.events[i] = ev
      _lib.call("gbsgmc_plan_run", handle, int(first_step + done), g,
                _lib.stream_handle())
      done += g


def _plan_launches(handle, steps, external=None) -> int:
  """Launches of ``steps`` steps run by one plan_run, or, with external
  indices, by one plan_run per block."""
  f = _lib.load().gbsgmc_plan_launches
  if external is None:
    return int(f(handle, int(steps)))
  full, rem = divmod(int(steps), external.G)
  return full * int(f(handle, external.G)) + (int(f(handle, rem)) if rem else 0)


class SgldGlmPlan:
  """Owns a ``gbsgmc_plan`` and the device buffers baked into it."""

  def __init__(self, potential, dataset, W, V, alpha, lmbd, n, h_tab, t_tab,
               keep_tab, n_kept, index_src, noise_seed, chain_base=0,
               block_steps=DEFAULT_BLOCK_STEPS, noise_dev=None, feed=None):
    import torch
    self.potential = potential
    C, d = W.shape
    self.external = _ExternalIndices(feed, block_steps, C, n) \
        if index_src.external else None
    self.C, self.d, self.n = C, d, n
    self.model, self._keep_alive = potential.model(dataset)
    self.W = W
    self.V = V
    self.U = torch.zeros(C, dtype=torch.float64, device="cuda")
    self.lk_var = torch.zeros(C, dtype=torch.float64, device="cuda")
    self.samples = torch.empty((max(n_kept, 1), C, d), dtype=torch.float32,
                               device="cuda")
    self.sample_lik = torch.empty((max(n_kept, 1), C), dtype=torch.float64,
                                  device="cuda")
    self.n_kept = n_kept
    self.h_tab, self.t_tab, self.keep_tab = h_tab, t_tab, keep_tab
    self.status = torch.zeros(1, dtype=torch.int32, device="cuda")
    self.index_src = index_src
    self.sched = _lib.sched(step_size_dev=h_tab, temperature_dev=t_tab,
                            keep_slot_dev=keep_tab)
    self.noise = _lib.noise(noise_seed, chain_base)
    handle = _lib.C.c_void_p()
    _lib.call("gbsgmc_sgld_glm_plan_create", _lib.C.byref(handle), self.model,
              C, n, _lib.ptr(W), _lib.ptr(V), float(alpha), float(lmbd),
              self.sched, self.noise, index_src.struct, _lib.ptr(self.U),
              _lib.ptr(self.lk_var), _lib.ptr(self.samples),
              _lib.ptr(self.sample_lik), int(block_steps),
              _lib.ptr(self.status))
    self.handle = handle

  def run(self, first_step, steps):
    if self.external is not None:
      self.external.run(self.handle, int(first_step), int(steps))
      return
    _lib.call("gbsgmc_plan_run", self.handle, int(first_step), int(steps),
              _lib.stream_handle())

  def launch_shape(self):
    """(CTAs or row items per chain, rows per warp, warps per CTA,
    prefetch, dynamic scheduling, steps per launch) from the autotuner."""
    s, r, w, f, y, k = (_lib.C.c_int() for _ in range(6))
    _lib.call("gbsgmc_plan_launch_shape", self.handle, _lib.C.byref(s),
              _lib.C.byref(r), _lib.C.byref(w), _lib.C.byref(f),
              _lib.C.byref(y), _lib.C.byref(k))
    return s.value, r.value, w.value, f.value, y.value, k.value

  def launches(self, steps) -> int:
    return _plan_launches(self.handle, steps, self.external)

  def check_status(self):
    code = int(self.status.item())
    if code != 0:
      raise _lib.GbsgmcError(code, "device status of the SGLD plan")

  def close(self):
    if getattr(self, "handle", None):
      _lib.load().gbsgmc_plan_destroy(self.handle)
      self.handle = None

  def __del__(self):
    try:
      self.close()
    except Exception:  # pragma: no cover - interpreter shutdown
      pass


class IndexSource:
  """PCG64 streams (device [C] gbsgmc_pcg64, advanced in place), Philox, or
  ``external``: indices the host supplies block by block
  (:class:`ShuffledFeed`)."""

  def __init__(self, pcg=None, seed=0, chain_base=0, external=False):
    self.pcg = pcg
    self.external = bool(external)
    self.struct = _lib.IndexSrc(_lib.ptr(pcg), int(seed) & (2**64 - 1),
                                int(chain_base), int(self.external))


def run_sgld_glm(potential, dataset, W, V, n, iterations, h, t, keep, n_kept,
                 index_src, noise_seed=0, chain_base=0, alpha=0.9, lmbd=1e-5,
                 block_steps=None, feed=None, host=None,
                 on_enqueued=None) -> SgldRun:
  """Runs ``iterations`` fused SGLD steps for all chains (W, V updated in
  place) and returns the final state and the kept samples.  With ``host``
  (the kept samples' and likelihoods' host arrays, or a HostBuffers), the
  kept samples are copied there -- each block's while the next blocks run,
  or, for a run of one block, all at once after it -- and ``SgldRun.host``
  holds the filled arrays.  For a run of one block, ``on_enqueued(arrays)``
  is called with the host arrays once the block is enqueued and before
  they are filled (host work that overlaps the GPU's), and its value is
  ``SgldRun.early``."""
  import torch
  if block_steps is None:
    block_steps = min(DEFAULT_BLOCK_STEPS, max(1, iterations))
  h_tab = torch.from_numpy(np.asarray(h, np.float32)).cuda()
  t_tab = torch.from_numpy(np.asarray(t, np.float32)).cuda()
  k_tab = torch.from_numpy(np.asarray(keep, np.int32)).cuda()
  plan = SgldGlmPlan(potential, dataset, W, V, alpha, lmbd, n, h_tab, t_tab,
                     k_tab, n_kept, index_src, noise_seed, chain_base,
                     block_steps, feed=feed)
  try:
    filled = early = None
    if host is not None and n_kept > 0 and iterations <= block_steps \
        and plan.external is None:
      # One block: enqueue it, let the host work meanwhile, then copy.
      plan.run(0, iterations)
      launches = plan.launches(iterations)
      filled = host.get() if hasattr(host, "get") else host
      if on_enqueued is not None:
        early = on_enqueued(filled)
      torch.from_numpy(filled[0]).copy_(plan.samples[:n_kept])
      torch.from_numpy(filled[1]).copy_(plan.sample_lik[:n_kept])
    elif host is not None and n_kept > 0:
      # One run per block, so that each block's kept samples can leave
      # while the next block runs.
      drain = io.SampleDrain([plan.samples, plan.sample_lik], host)
      keep_np = np.asarray(keep)
      launches = 0
      try:
        for k0 in range(0, iterations, block_steps):
          g = min(block_steps, iterations - k0)
          plan.run(k0, g)
          launches += plan.launches(g)
          kept = keep_np[k0:k0 + g]
          kept = kept[kept >= 0]
          if kept.size:
            drain.filled(kept.min(), kept.max() + 1)
      finally:
        filled = drain.finish()
    else:
      plan.run(0, iterations)
      launches = plan.launches(iterations)
    plan.check_status()
    return SgldRun(W, V, plan.U, plan.lk_var, plan.samples[:n_kept],
                   plan.sample_lik[:n_kept], launches, filled, early)
  finally:
    plan.close()


class NetPlan:
  """Owns a network plan (``gbsgmc_mlp_plan_create``,
  ``gbsgmc_cnn_plan_create``, or ``gbsgmc_glm_plan_create`` for the GLM
  families): C chains of SGLD, OBABO or SGHMC, one CUDA graph per block of
  steps.  ``X`` [C, P] (positions) and ``AUX`` (rms_prop state, or momentum)
  are updated in place."""

  KINDS = {"langevin": _lib.INTEGRATOR_SGLD, "obabo": _lib.INTEGRATOR_OBABO,
           "sghmc": _lib.INTEGRATOR_SGHMC}

  def __init__(self, potential, dataset, X, AUX, n, kind, h_tab, t_tab,
               index_src, noise_seed, chain_base=0, block_steps=None,
               friction=0.0, leapfrog_steps=1, alpha=0.9, lmbd=1e-5,
               mass=None, observation_count=None, feed=None):
    import torch
    C, P = X.shape
    self.C, self.P, self.n, self.kind = C, P, n, kind
    self.model, self._keep_alive = potential.model(dataset, observation_count)
    self.X, self.AUX, self.mass = X, AUX, mass
    self.U = torch.zeros(C, dtype=torch.float64, device="cuda")
    self.lk_var = torch.zeros(C, dtype=torch.float64, device="cuda")
    self.ke = torch.zeros(2 * C, dtype=torch.float64, device="cuda")
    self.status = torch.zeros(1, dtype=torch.int32, device="cuda")
    self.h_tab, self.t_tab = h_tab, t_tab
    self.index_src = index_src
    self.sched = _lib.sched(step_size_dev=h_tab, temperature_dev=t_tab)
    self.noise = _lib.noise(noise_seed, chain_base)
    lf = int(leapfrog_steps) if kind == "sghmc" else 1
    if block_steps is None:
      block_steps = DEFAULT_BLOCK_STEPS
    block_steps = max(lf, block_steps // lf * lf)
    draws = 2 if kind == "obabo" else 1
    self.external = _ExternalIndices(feed, block_steps, C, draws * n) \
        if index_src.external else None
    self.integ = _lib.Integrator(self.KINDS[kind], lf, float(friction),
                                 float(alpha), float(lmbd), 0, _lib.ptr(mass))
    handle = _lib.C.c_void_p()
    # Kernel launches of one value-and-gradient call.
    self.launches_per_gradient = 30 if potential.is_cnn else \
        10 if potential.is_mlp else 1
    create = "gbsgmc_cnn_plan_create" if potential.is_cnn else \
        "gbsgmc_mlp_plan_create" if potential.is_mlp else \
        "gbsgmc_glm_plan_create"
    _lib.call(create, _lib.C.byref(handle), self.model, C, n,
              self.integ, _lib.ptr(X), _lib.ptr(AUX), self.sched, self.noise,
              index_src.struct, _lib.ptr(self.U), _lib.ptr(self.lk_var),
              _lib.ptr(self.ke), int(block_steps), _lib.ptr(self.status))
    self.handle = handle

  def run(self, first_step, steps):
    if self.external is not None:
      self.external.run(self.handle, int(first_step), int(steps))
      return
    _lib.call("gbsgmc_plan_run", self.handle, int(first_step), int(steps),
              _lib.stream_handle())

  def launches(self, steps) -> int:
    """Kernel launches of ``steps`` steps (value-and-gradient kernels
    included)."""
    per_grad = self.launches_per_gradient
    grads = {"obabo": 2}.get(self.kind, 1) * int(steps)
    return _plan_launches(self.handle, steps, self.external) + per_grad * grads

  def check_status(self):
    code = int(self.status.item())
    if code != 0:
      raise _lib.GbsgmcError(code, "device status of the network plan")

  def close(self):
    if getattr(self, "handle", None):
      _lib.load().gbsgmc_plan_destroy(self.handle)
      self.handle = None

  def __del__(self):
    try:
      self.close()
    except Exception:  # pragma: no cover - interpreter shutdown
      pass


class ResgldPlan:
  """Owns a reSGLD network plan (``gbsgmc_mlp_resgld_plan_create``): R
  replicas of SGLD(+RMSprop) on a dense-network potential at the temperature
  ladder ``ladder`` [R] (coldest first), minibatch rows[r] <= n_max for
  replica r, adjacent exchanges every ``every`` steps.  ``X`` [R, P] (and
  ``V``) are updated in place; ``U``, ``lk_var``, ``ssq``, ``counts`` and
  ``flags`` are readable device tensors."""

  def __init__(self, potential, dataset, X, V, rows, n_max, ladder, h_tab,
               t_tab, index_src, noise_seed, swap_seed, every=50, F=1.0,
               alpha=0.9, lmbd=1e-5, chain_base=0, block_steps=None,
               observation_count=None, keep_tab=None, n_kept=0):
    import torch
    R, P = X.shape
    self.R, self.P = R, P
    self.model, self._keep_alive = potential.model(dataset, observation_count)
    self.X, self.V = X, V
    self.rows = torch.as_tensor(rows, dtype=torch.int32).cuda().contiguous()
    self.ladder = torch.as_tensor(ladder, dtype=torch.float32).cuda().contiguous()
    self.U = torch.zeros(R, dtype=torch.float64, device="cuda")
    self.lk_var = torch.zeros(R, dtype=torch.float64, device="cuda")
    self.ssq = torch.zeros(R - 1, dtype=torch.float64, device="cuda")
    self.k = torch.zeros(1, dtype=torch.int64, device="cuda")
    self.counts = torch.zeros(R - 1, dtype=torch.int32, device="cuda")
    self.flags = torch.zeros(R - 1, dtype=torch.int32, device="cuda")
    self.status = torch.zeros(1, dtype=torch.int32, device="cuda")
    self.h_tab, self.t_tab, self.keep_tab = h_tab, t_tab, keep_tab
    self.index_src = index_src
    # Kept states of replica 0 (after each kept step's exchange attempt).
    self.samples = self.sample_lik = None
    if keep_tab is not None:
      self.samples = torch.empty((max(int(n_kept), 1), P), dtype=torch.float32, device="cuda")
      self.sample_lik = torch.empty(max(int(n_kept), 1), dtype=torch.float64, device="cuda")
    self.sched = _lib.sched(step_size_dev=h_tab, temperature_dev=t_tab,
                            keep_slot_dev=keep_tab, chain_temperature_dev=self.ladder)
    self.noise = _lib.noise(noise_seed, chain_base)
    self.temp = _lib.Tempering(int(every), 0, float(F), int(swap_seed) & (2**64 - 1),
                               _lib.ptr(self.ssq), _lib.ptr(self.k),
                               _lib.ptr(self.counts), _lib.ptr(self.flags))
    if block_steps is None:
      block_steps = every * max(1, DEFAULT_BLOCK_STEPS // every)
    handle = _lib.C.c_void_p()
    _lib.call("gbsgmc_mlp_resgld_plan_create_keep", _lib.C.byref(handle), self.model,
              R, int(n_max), _lib.ptr(self.rows), _lib.ptr(X), _lib.ptr(V),
              float(alpha), float(lmbd), self.sched, self.noise,
              index_src.struct, self.temp, _lib.ptr(self.U),
              _lib.ptr(self.lk_var), _lib.ptr(self.samples), _lib.ptr(self.sample_lik),
              int(block_steps), _lib.ptr(self.status))
    self.handle = handle

  def run(self, first_step, steps):
    _lib.call("gbsgmc_plan_run", self.handle, int(first_step), int(steps),
              _lib.stream_handle())

  def launches(self, steps) -> int:
    return int(_lib.load().gbsgmc_plan_launches(self.handle, int(steps))) + \
        10 * int(steps)

  def check_status(self):
    code = int(self.status.item())
    if code != 0:
      raise _lib.GbsgmcError(code, "device status of the reSGLD plan")

  def close(self):
    if getattr(self, "handle", None):
      _lib.load().gbsgmc_plan_destroy(self.handle)
      self.handle = None

  def __del__(self):
    try:
      self.close()
    except Exception:  # pragma: no cover - interpreter shutdown
      pass


def try_fused_net(solver, scheduler, states, schedulers, iterations, saving):
  """Runs sgmc chains of langevin_diffusion / obabo / friction_leapfrog
  through one :class:`NetPlan` (network potentials, and OBABO / SGHMC on the
  GLM families, whose SGLD has its own fused step); returns None when the
  chains do not qualify (the caller steps them one by one)."""
  import torch
  from .potential import StochasticPotential
  meta = getattr(solver, "meta", {})
  if not FUSED_ENABLED or meta.get("kind") != "sgmc" or schedulers:
    return None
  integ = meta.get("integrator")
  im = getattr(integ, "meta", {})
  kind = im.get("kind")
  if kind not in NetPlan.KINDS or im.get("noise_source") is not None \
      or im.get("noise_model") is not None:
    return None
  pot = im.get("potential")
  bfn = im.get("batch_fn")
  if not isinstance(pot, StochasticPotential) or not states:
    return None
  if not isinstance(bfn, tuple) or not isinstance(bfn[1], RandomBatchFn):
    return None
  rbf = bfn[1]
  if len({s.key for s in states}) != 1:
    return None
  chain_ids = [int(s.chain) for s in states]
  if chain_ids != list(range(chain_ids[0], chain_ids[0] + len(states))):
    return None
  if rbf.kind != "host":
    return None
  ds_list = [s.data_state for s in states]
  shuffled = ShuffledFeed.qualifies(rbf.loader, ds_list)
  if not shuffled and any(d.state is None or d.cached_batches is not None
                          for d in ds_list):
    return None
  steps = int(im.get("steps", 1)) if kind != "langevin" else 1
  if kind == "langevin":
    adapt = [s.adapt_state for s in states]
    if any(a is None for a in adapt) and not all(a is None for a in adapt):
      return None
    X = torch.stack([s.latent_variables for s in states]).contiguous().cuda()
    AUX = torch.stack([a.v for a in adapt]).contiguous().cuda() \
        if adapt[0] is not None else None
    kw = dict(alpha=adapt[0].alpha, lmbd=adapt[0].lmbd) \
        if adapt[0] is not None else {}
    if any(int(s.step) != 0 for s in states):
      return None
  else:
    X = torch.stack([s.positions for s in states]).contiguous()
    AUX = torch.stack([s.momentum for s in states]).contiguous()
    if im.get("const_mass") is not None or not np.isscalar(im.get("friction")):
      return None
    kw = dict(friction=float(im["friction"]), leapfrog_steps=steps)
    if any(int(s.step) != 0 for s in states):
      return None
  feed = pcg = None
  if shuffled:
    # Shuffled streams: the host loader draws them, the plan reads them.
    feed = ShuffledFeed(rbf.loader, ds_list, 2 if kind == "obabo" else 1)
    index_src = IndexSource(chain_base=chain_ids[0], external=True)
  else:
    pcg = torch.stack([d.state for d in ds_list]).contiguous().cuda()
    index_src = IndexSource(pcg=pcg, chain_base=chain_ids[0])
  dataset = rbf.loader.device_dataset()
  h, t, keep, n_kept, _ = sched_mod.tables(scheduler, iterations)
  # One solver iteration is `steps` integrator steps with the same schedule.
  h_tab = torch.from_numpy(np.repeat(np.asarray(h, np.float32), steps)).cuda()
  t_tab = torch.from_numpy(np.repeat(np.asarray(t, np.float32), steps)).cuda()
  plan = NetPlan(pot, dataset, X, AUX, rbf.mb_size, kind, h_tab, t_tab,
                 index_src, states[0].key, chain_ids[0], feed=feed, **kw)
  C, P = len(states), X.shape[1]
  extra = torch.empty((max(n_kept, 1), C), dtype=torch.float64, device="cuda")
  # Kept samples: all on the device (device saving), streamed into FP64
  # moments (moments saving), or through a ring of device rows that a
  # SampleDrain empties to the host while the chains run (host saving).
  mom = drain = None
  kind_saving = saving.kind if saving is not None else "device"
  ring = max(n_kept, 1)
  if kind_saving == "moments":
    mom = io.DeviceMoments(C, P)
    samples = None
  else:
    if kind_saving == "memory":
      ring = max(1, min(ring, RING_BYTES // max(1, 4 * C * P)))
    samples = torch.empty((ring, C, P), dtype=torch.float32, device="cuda")
    if kind_saving == "memory" and ring < n_kept:
      drain = io.SampleDrain([samples], io.HostBuffers(
          [((n_kept, C, P), np.float32)]), ring=ring)
  drained = None
  try:
    done = 0
    try:
      for k in np.nonzero(np.asarray(keep) >= 0)[0]:
        plan.run(done * steps, (k + 1 - done) * steps)
        done = k + 1
        slot = int(keep[k])
        if mom is not None:
          mom.add(X)
        else:
          if drain is not None and slot >= ring:
            drain.wait_copied(slot - ring)   # the row's last sample has left
          samples[slot % ring] = X
          if drain is not None:
            drain.filled(slot, slot + 1)
        extra[slot] = -plan.U if kind == "langevin" else plan.U
      if done < iterations:
        plan.run(done * steps, (iterations - done) * steps)
    finally:
      if drain is not None:
        drained = drain.finish()
    plan.check_status()
  finally:
    plan.close()
    if feed is not None:
      feed.close()
  if pcg is not None:
    host = pcg.cpu()   # the streams advanced on the device
    for c, s in enumerate(states):
      dst = s.data_state.state
      dst.copy_(pcg[c] if dst.is_cuda else host[c])
  key = "likelihood" if kind == "langevin" else "energy"
  treedefs = [s.treedef for s in states]
  model_states = [s.model_state for s in states]
  if mom is not None:
    return io.moment_results(n_kept, mom, treedefs, {key: extra[:n_kept]},
                             model_states)
  if drained is not None:
    return io.postprocess_chains(saving, n_kept, samples, treedefs,
                                 {key: extra[:n_kept]}, model_states,
                                 host=[drained[0], extra[:n_kept].cpu().numpy()],
                                 host_filled=True)
  return io.postprocess_chains(saving or io.no_save(), n_kept,
                               samples[:n_kept], treedefs,
                               {key: extra[:n_kept]}, model_states)


def try_fused_sgld(solver, scheduler, states, schedulers, iterations, saving):
  """Runs the chains through :func:`run_sgld_glm` when they qualify;
  returns None otherwise (the caller then steps chain by chain).  Chains
  made together (:class:`~gbsgmc.integrator.LangevinChains`) move as whole
  [C, ...] tensors, and their result dicts are assembled while the GPU
  runs."""
  import torch
  from .integrator import LangevinChains
  from .potential import StochasticPotential
  meta = getattr(solver, "meta", {})
  if not FUSED_ENABLED or meta.get("kind") != "sgmc" or schedulers:
    return None
  integ = meta.get("integrator")
  im = getattr(integ, "meta", {})
  if im.get("kind") != "langevin" or im.get("noise_source") is not None:
    return None
  pot = im.get("potential")
  bfn = im.get("batch_fn")
  if not isinstance(pot, StochasticPotential) or pot.is_network or not len(states):
    return None
  if not isinstance(bfn, tuple) or not isinstance(bfn[1], RandomBatchFn):
    return None
  rbf = bfn[1]
  C = len(states)
  feed = None
  if isinstance(states, LangevinChains):
    # Fresh chains made together: consecutive ids, one key, step 0.
    if rbf.kind != "host" or states.pipelines.loader is not rbf.loader:
      return None
    chain_base, key = int(states.chain_ids[0]), states.key
    W = states.positions.cuda()
    V = None if states.rms_v is None else states.rms_v.cuda()
    alpha, lmbd = states.alpha, states.lmbd
    index_src = IndexSource(pcg=states.pipelines.pcg.cuda(), chain_base=chain_base)
    treedefs = [states.treedef] * C
    model_states = [states.model_state] * C
  else:
    keys = {s.key for s in states}
    if len(keys) != 1:
      return None
    key = states[0].key
    adapt = [s.adapt_state for s in states]
    if any(a is None for a in adapt) and not all(a is None for a in adapt):
      return None
    chain_ids = [int(s.chain) for s in states]
    if chain_ids != list(range(chain_ids[0], chain_ids[0] + C)):
      return None
    chain_base = chain_ids[0]
    if rbf.kind == "host":
      ds_list = [s.data_state for s in states]
      if ShuffledFeed.qualifies(rbf.loader, ds_list):
        # Shuffled streams: the host loader draws them, the plan reads them.
        feed = ShuffledFeed(rbf.loader, ds_list, 1)
        index_src = IndexSource(chain_base=chain_base, external=True)
      elif any(d.state is None or d.cached_batches is not None for d in ds_list):
        return None   # draws already consumed
      else:
        pcg = torch.stack([d.state for d in ds_list]).contiguous().cuda()
        index_src = IndexSource(pcg=pcg, chain_base=chain_base)
    else:
      seeds = {s.data_state.state[0] for s in states}
      if len(seeds) != 1 or any(s.data_state.state[1] != 0 for s in states):
        return None
      index_src = IndexSource(seed=seeds.pop(), chain_base=chain_base)
    W = torch.stack([s.latent_variables for s in states]).contiguous().cuda()
    if adapt[0] is not None:
      V = torch.stack([a.v for a in adapt]).contiguous().cuda()
      alpha, lmbd = adapt[0].alpha, adapt[0].lmbd
    else:
      V, alpha, lmbd = None, 0.9, 1e-5
    treedefs = [s.treedef for s in states]
    model_states = [s.model_state for s in states]
  dataset = rbf.loader.device_dataset()
  if W.shape[1] != pot.dim(dataset):
    if feed is not None:
      feed.close()
    return None
  h, t, keep, n_kept, _ = sched_mod.tables(scheduler, iterations)
  block = min(rbf.cached_batches_count, DEFAULT_BLOCK_STEPS, max(iterations, 1))
  outbuf = None
  early = None
  if saving is not None and saving.kind == "memory":
    outbuf = io.HostBuffers([((n_kept, C, W.shape[1]), np.float32),
                             ((n_kept, C), np.float64)])
    if getattr(saving.collector, "_dir", None) is None:
      # Collectors that write nothing take views of the host arrays, so the
      # result dicts can be built before the samples arrive.
      def early(arrays):
        return io.postprocess_chains(saving, n_kept, arrays[0], treedefs,
                                     {"likelihood": arrays[1]}, model_states,
                                     host=arrays, host_filled=True)
  try:
    res = run_sgld_glm(pot, dataset, W, V, rbf.mb_size, iterations, h, t, keep,
                       n_kept, index_src, noise_seed=key, chain_base=chain_base,
                       alpha=alpha, lmbd=lmbd, block_steps=block, feed=feed,
                       host=outbuf, on_enqueued=early)
  finally:
    if feed is not None:
      feed.close()
  if isinstance(states, LangevinChains):
    # The streams advanced on the device: every chain's stream words are a
    # row of the pipelines' host tensor.
    states.pipelines.pcg.copy_(index_src.pcg)
  elif rbf.kind == "host" and feed is None:
    # The streams advanced on the device; states still holding their
    # initial host words get them back in one copy.
    host = index_src.pcg.cpu()
    for c, s in enumerate(states):
      dst = s.data_state.state
      dst.copy_(index_src.pcg[c] if dst.is_cuda else host[c])
  if res.early is not None:
    return res.early
  return io.postprocess_chains(saving or io.no_save(), n_kept, res.samples,
                               treedefs, {"likelihood": res.sample_lik},
                               model_states, host=res.host,
                               host_filled=res.host is not None)


class ResgldPairsPlan:
  """Owns a ``gbsgmc_glm_resgld_plan`` (or, on the MLP likelihood,
  ``gbsgmc_mlp_resgld_pairs_plan``): P (normal, hot) pairs of SGLD chains
  with the pairs' exchange after every step on the device (alias.re_sgld).
  X [2P, d] holds the normal chains in rows [0, P) and their hot partners in
  rows [P, 2P); ``ident`` [2P] maps each row to the chain identity (index
  stream ``pcg[i]``, noise chain id chain_base + i) it holds after the
  exchanges so far."""

  def __init__(self, potential, dataset, X, V, alpha, lmbd, n, h_tab, t_tab,
               keep_tab, ladder, n_kept, pcg, ident, pair_chain, ssq, k, F,
               swap_seed, noise_seed, chain_base, block_steps):
    import torch
    P2, d = X.shape
    self.pairs = P2 // 2
    self.model, self._keep_alive = potential.model(dataset)
    self.X, self.V, self.pcg, self.ident = X, V, pcg, ident
    self.pair_chain, self.ssq, self.k = pair_chain, ssq, k
    self.U = torch.zeros(P2, dtype=torch.float64, device="cuda")
    self.lk_var = torch.zeros(P2, dtype=torch.float64, device="cuda")
    self.counts = torch.zeros(self.pairs, dtype=torch.int32, device="cuda")
    self.samples = torch.empty((max(n_kept, 1), self.pairs, d), dtype=torch.float32,
                               device="cuda")
    self.sample_lik = torch.empty((max(n_kept, 1), self.pairs), dtype=torch.float64,
                                  device="cuda")
    self.status = torch.zeros(1, dtype=torch.int32, device="cuda")
    self.tabs = (h_tab, t_tab, keep_tab, ladder)
    self.sched = _lib.sched(step_size_dev=h_tab, temperature_dev=t_tab,
                            keep_slot_dev=keep_tab, chain_temperature_dev=ladder)
    self.noise = _lib.noise(noise_seed, chain_base)
    self.isrc = _lib.IndexSrc(_lib.ptr(pcg), 0, int(chain_base), 0)
    self.temp = _lib.Tempering(1, 0, float(F), int(swap_seed) & (2**64 - 1),
                               _lib.ptr(ssq), _lib.ptr(k), _lib.ptr(self.counts), None)
    handle = _lib.C.c_void_p()
    self.network = bool(potential.is_mlp)
    fn = "gbsgmc_mlp_resgld_pairs_plan_create" if self.network else \
        "gbsgmc_glm_resgld_plan_create"
    _lib.call(fn, _lib.C.byref(handle), self.model,
              self.pairs, int(n), _lib.ptr(X), _lib.ptr(V), float(alpha), float(lmbd),
              self.sched, self.noise, self.isrc, self.temp, _lib.ptr(pair_chain),
              _lib.ptr(ident), _lib.ptr(self.U), _lib.ptr(self.lk_var),
              _lib.ptr(self.samples), _lib.ptr(self.sample_lik), int(block_steps),
              _lib.ptr(self.status))
    self.handle = handle

  def run(self, first_step, steps):
    _lib.call("gbsgmc_plan_run", self.handle, int(first_step), int(steps),
              _lib.stream_handle())

  def launches(self, steps) -> int:
    # The MLP plan counts its value-and-gradient calls here: prep, gather,
    # four GEMMs and the dW1 GEMM, the output pass and the finalisation.
    extra = 9 * int(steps) if self.network else 0
    return int(_lib.load().gbsgmc_plan_launches(self.handle, int(steps))) + extra

  def check_status(self):
    code = int(self.status.item())
    if code != 0:
      raise _lib.GbsgmcError(code, "device status of the reSGLD pairs plan")

  def close(self):
    if getattr(self, "handle", None):
      _lib.load().gbsgmc_plan_destroy(self.handle)
      self.handle = None

  def __del__(self):
    try:
      self.close()
    except Exception:  # pragma: no cover - interpreter shutdown
      pass


def try_fused_resgld(solver, scheduler, states, schedulers, iterations, saving):
  """Runs alias.re_sgld's pairs (solver.parallel_tempering over
  langevin_diffusion, solver.py:220-299) on a GLM or MLP potential as one
  :class:`ResgldPairsPlan`: every pair steps, exchanges and keeps its normal
  chain's samples on the device, and the chains' index streams and noise
  are the per-pair path's, so the samples are the same.  Returns None when
  the pairs do not qualify: fresh pairs of one key and one F whose chains
  have consecutive ids (normal, hot, normal, hot, ...), fresh numpy PCG64
  pipelines, one hot schedule whose temperatures are the normal schedule's
  times a constant factor and whose step sizes are the same, no injected
  noise; on the MLP, minibatches of a multiple of 128 rows."""
  import torch
  from .integrator import LangevinState, key_to_seed
  from .potential import StochasticPotential
  meta = getattr(solver, "meta", {})
  if not FUSED_ENABLED or meta.get("kind") != "parallel_tempering":
    return None
  if not schedulers or len(schedulers) != 1 or not len(states):
    return None
  im = getattr(meta.get("integrator"), "meta", {})
  if im.get("kind") != "langevin" or im.get("noise_source") is not None:
    return None
  pot, bfn = im.get("potential"), im.get("batch_fn")
  if not isinstance(pot, StochasticPotential) or pot.is_cnn:
    return None
  if not isinstance(bfn, tuple) or not isinstance(bfn[1], RandomBatchFn) \
      or bfn[1].kind != "host":
    return None
  rbf = bfn[1]
  if pot.is_mlp and rbf.mb_size % 128 != 0:
    return None
  P = len(states)
  chains = []
  for s in states:
    chains += [s.normal, s.hot]
  if not all(isinstance(c, LangevinState) and c.step == 0 for c in chains):
    return None
  seeds = {int(s.seed) for s in states}
  if len(seeds) != 1 or len({float(s.F) for s in states}) != 1:
    return None
  seed = seeds.pop()
  if any(c.key != seed for c in chains):
    return None
  ids = [int(c.chain) for c in chains]
  if ids != list(range(ids[0], ids[0] + 2 * P)):
    return None
  if any(int(s.pair_chain) != int(s.normal.chain) for s in states):
    return None
  ds = [c.data_state for c in chains]
  if any(d.state is None or d.cached_batches is not None for d in ds):
    return None
  adapt = [c.adapt_state for c in chains]
  if any(a is None for a in adapt) != all(a is None for a in adapt):
    return None
  h, t, keep, n_kept, _ = sched_mod.tables(scheduler, iterations)
  h2, t2, _, _, _ = sched_mod.tables(scheduler, iterations, **schedulers[0])
  if not np.array_equal(h, h2) or iterations == 0 or not (t[0] > 0):
    return None
  f = np.float32(t2[0] / t[0])
  if not np.array_equal((t * f).astype(np.float32), t2):
    return None
  dataset = rbf.loader.device_dataset()
  normals = [s.normal for s in states]
  hots = [s.hot for s in states]
  X = torch.stack([c.latent_variables for c in normals + hots]).contiguous().cuda()
  if X.shape[1] != pot.dim(dataset):
    return None
  if adapt[0] is not None:
    V = torch.stack([c.adapt_state.v for c in normals + hots]).contiguous().cuda()
    alpha, lmbd = adapt[0].alpha, adapt[0].lmbd
  else:
    V, alpha, lmbd = None, 0.9, 1e-5
  pcg = torch.stack([d.state for d in ds]).contiguous().cuda()   # by identity
  ident = torch.from_numpy(np.concatenate([np.arange(0, 2 * P, 2),
                                           np.arange(1, 2 * P, 2)]).astype(np.int32)).cuda()
  pair_chain = torch.tensor([int(s.pair_chain) for s in states], dtype=torch.int32,
                            device="cuda")
  ssq = torch.cat([s.ssq.reshape(1).to(torch.float64) for s in states]).cuda()
  k = torch.cat([s.step.reshape(1).to(torch.int64) for s in states]).cuda()
  ladder = torch.from_numpy(np.concatenate([np.ones(P, np.float32),
                                            np.full(P, f, np.float32)])).cuda()
  tabs = [torch.from_numpy(np.ascontiguousarray(a)).cuda()
          for a in (np.asarray(h, np.float32), np.asarray(t, np.float32),
                    np.asarray(keep, np.int32))]
  block = min(rbf.cached_batches_count, DEFAULT_BLOCK_STEPS, max(iterations, 1))
  plan = ResgldPairsPlan(pot, dataset, X, V, alpha, lmbd, rbf.mb_size, *tabs, ladder,
                         n_kept, pcg, ident, pair_chain, ssq, k, float(states[0].F),
                         seed, seed, ids[0], block)
  global LAST_EXCHANGES
  try:
    plan.run(0, iterations)
    plan.check_status()
    samples, lik = plan.samples[:n_kept], plan.sample_lik[:n_kept]
    LAST_EXCHANGES = plan.counts.cpu().numpy()
  finally:
    plan.close()
  host = pcg.cpu()   # the identities' streams advanced on the device
  for i, d in enumerate(ds):
    d.state.copy_(pcg[i] if d.state.is_cuda else host[i])
  return io.postprocess_chains(saving or io.no_save(), n_kept, samples,
                               [s.normal.treedef for s in states],
                               {"likelihood": lik},
                               [s.normal.model_state for s in states])


def try_fused_mh(solver, scheduler, states, schedulers, iterations, saving):
  """Runs AMAGOLD / SGGMC chains batched (solver.py:301-577): each MH
  iteration proposes for all chains at once with the [C, P] kernels (the
  batched value and gradient, the leapfrog or OBABO updates), evaluates the
  full-data potential of all proposals in one pass over the ordered chunks
  and decides all chains in one MH launch.  The per-chain streams are the
  per-chain path's (numpy PCG64 index draws, Philox noise and MH uniforms
  keyed by chain id), so the samples are the same.  Returns None when the
  chains do not qualify: a static schedule (no adaptive step size), one key,
  consecutive chain ids, fresh numpy PCG64 pipelines, no mass adaption, no
  constant mass or per-parameter friction, no injected noise."""
  import torch
  from .potential import StochasticPotential
  meta = getattr(solver, "meta", {})
  kind = meta.get("kind")
  if not FUSED_ENABLED or kind not in ("amagold", "sggmc") or schedulers:
    return None
  if meta.get("mass_adaption") is not None:
    return None
  integ = meta.get("integrator")
  im = getattr(integ, "meta", {})
  if im.get("noise_source") is not None or im.get("const_mass") is not None:
    return None
  if not np.isscalar(im.get("friction")):
    return None
  want = "reversible_leapfrog" if kind == "amagold" else "obabo"
  if im.get("kind") != want:
    return None
  pot, bfn, full = im.get("potential"), im.get("batch_fn"), meta.get("full_potential")
  fmap = meta.get("full_data_map")
  if not isinstance(pot, StochasticPotential) or full is None or not states:
    return None
  if not isinstance(bfn, tuple) or not isinstance(bfn[1], RandomBatchFn) \
      or bfn[1].kind != "host":
    return None
  comps = getattr(scheduler, "components", None)
  if comps is None or any(getattr(comps[k], "table", None) is None
                          for k in ("step_size", "temperature", "burn_in", "thinning")):
    return None
  if len({int(s.key) for s in states}) != 1 or any(s.mh_step != 0 for s in states):
    return None
  ists = [s.integrator_state for s in states]
  chain_ids = [int(i.chain) for i in ists]
  if chain_ids != list(range(chain_ids[0], chain_ids[0] + len(states))):
    return None
  if any(int(i.step) != 0 for i in ists) or len({int(i.key) for i in ists}) != 1:
    return None
  ds_list = [i.data_state for i in ists]
  if any(d.state is None or d.cached_batches is not None for d in ds_list):
    return None
  loader = getattr(fmap[1], "loader", None) if isinstance(fmap, tuple) else None
  if loader is None or loader is not bfn[1].loader:
    return None
  rbf = bfn[1]
  C, n = len(states), rbf.mb_size
  ds = loader.device_dataset()
  N = ds.observation_count
  steps, f = int(im["steps"]), float(im["friction"])
  X = torch.stack([i.positions for i in ists]).contiguous()
  Pm = torch.stack([i.momentum for i in ists]).contiguous()
  P = X.shape[1]
  U_old = torch.cat([s.potential.reshape(1) for s in states]).to(torch.float64)
  pcg = torch.stack([d.state for d in ds_list]).contiguous().cuda()
  status = torch.zeros(1, dtype=torch.int32, device="cuda")
  seed, noise_key = int(states[0].key), int(ists[0].key)
  noise = _lib.noise(noise_key, chain_ids[0])
  h, t, keep, n_kept, _ = sched_mod.tables(scheduler, iterations)
  per = steps * (2 if kind == "sggmc" else 1)
  idx = torch.empty((per, C, n), dtype=torch.int32, device="cuda")
  samples = torch.empty((max(n_kept, 1), C, P), dtype=torch.float32, device="cuda")
  extra = torch.empty((max(n_kept, 1), C), dtype=torch.float64, device="cuda")
  accept = torch.empty(C, dtype=torch.int32, device="cuda")
  ratio = torch.empty(C, dtype=torch.float64, device="cuda")
  U_keep = torch.empty(C, dtype=torch.float64, device="cuda")
  rows = loader.static_information["observation_count"]
  s = _lib.stream_handle()
  step = 0
  for k in range(iterations):
    hk, tk = float(h[k]), float(t[k])

    def sch(kk):
      return _lib.sched(step_size=hk, temperature=tk, offset=kk)

    x_old, p_old = X.clone(), Pm.clone()
    _lib.call("gbsgmc_index_draw_pcg64", _lib.ptr(pcg), C, rows, per * n, n,
              _lib.ptr(idx), n, C * n, _lib.ptr(status), s)
    if kind == "amagold":
      # Reversible leapfrog (integrator.py:349-560), as integrator.reversible_leapfrog.
      energy = torch.zeros(C, dtype=torch.float64, device="cuda")
      _lib.call("gbsgmc_leapfrog_position", C, P, _lib.ptr(X), _lib.ptr(Pm), None,
                0.5, sch(step), s)
      for j in range(steps):
        if j > 0:
          _lib.call("gbsgmc_leapfrog_position", C, P, _lib.ptr(X), _lib.ptr(Pm),
                    None, 1.0, sch(step), s)
        r = pot.evaluate(X, idx[j], ds, grad=True, observation_count=N)
        _lib.call("gbsgmc_amagold_momentum", C, P, _lib.ptr(Pm), _lib.ptr(r.grad),
                  None, f, _lib.ptr(energy), sch(step), noise, s)
        step += 1
      _lib.call("gbsgmc_leapfrog_position", C, P, _lib.ptr(X), _lib.ptr(Pm), None,
                0.5, sch(step), s)
      stat = energy
      ke0 = ke1 = None
    else:
      # OBABO (integrator.py:138-346); the kinetic energies restart at 0
      # after each correction (solver.py:536-537).
      ke0 = torch.zeros(C, dtype=torch.float64, device="cuda")
      ke1 = torch.zeros(C, dtype=torch.float64, device="cuda")
      energy = None
      for j in range(steps):
        r1 = pot.evaluate(X, idx[2 * j], ds, grad=True, observation_count=N)
        _lib.call("gbsgmc_obabo_first", C, P, _lib.ptr(X), _lib.ptr(Pm),
                  _lib.ptr(r1.grad), None, f, _lib.ptr(ke0), sch(step), noise, s)
        r2 = pot.evaluate(X, idx[2 * j + 1], ds, grad=True, observation_count=N)
        _lib.call("gbsgmc_obabo_second", C, P, _lib.ptr(Pm), _lib.ptr(r2.grad), None,
                  f, _lib.ptr(ke1), sch(step), noise, s)
        step += 1
      stat = 0.5 * (r1.U + r2.U)
    U_new, _ = full.value_and_grad_all(X, ds)
    U_new = U_new.to(torch.float64).contiguous()
    _lib.call("gbsgmc_mh_accept", C,
              _lib.MH_AMAGOLD if kind == "amagold" else _lib.MH_SGGMC,
              _lib.ptr(U_old), _lib.ptr(U_new), _lib.ptr(energy), _lib.ptr(ke0),
              _lib.ptr(ke1), _lib.sched(step_size=hk, temperature=tk, offset=k),
              None, seed, chain_ids[0], _lib.ptr(accept), _lib.ptr(ratio),
              _lib.ptr(U_keep), s)
    _lib.call("gbsgmc_mh_select", C, P, _lib.ptr(accept), _lib.ptr(X),
              _lib.ptr(x_old), _lib.ptr(Pm), _lib.ptr(p_old),
              -1.0 if kind == "amagold" else 1.0, s)
    U_old = U_keep.clone()
    if keep[k] >= 0:
      samples[keep[k]] = X
      extra[keep[k]] = stat
  code = int(status.item())
  if code != 0:
    raise _lib.GbsgmcError(code, "device status of the batched MH chains")
  pot.check_status()
  full._unit.check_status()
  full._flat.check_status()
  host = pcg.cpu()   # the streams advanced on the device
  for c, d in enumerate(ds_list):
    d.state.copy_(pcg[c] if d.state.is_cuda else host[c])
  return io.postprocess_chains(saving or io.no_save(), n_kept, samples[:n_kept],
                               [i.treedef for i in ists], {"energy": extra[:n_kept]},
                               [i.model_state for i in ists])
