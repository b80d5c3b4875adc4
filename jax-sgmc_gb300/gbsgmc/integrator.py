"""Integrators (mirrors jax_sgmc/integrator.py) driving the CUDA kernels.

Each factory returns the reference's ``(init_fn, update_fn, get_fn)`` triplet
for ONE chain, stepping through the C ABI: index draw -> GLM value and
adjoint -> elementwise integrator kernel.  Chain parameters are flat fp32
device vectors updated in place (a state passed to ``update_fn`` must not be
reused afterwards).  ``solver.mcmc`` runs many chains of
``langevin_diffusion`` in one fused, graph-captured plan instead
(:mod:`gbsgmc.engine`).

Noise: Philox4x32-10 normals keyed by the chain's ``key`` and indexed by
(chain id, chain-step counter, stream tag), replacing JAX's threefry
``random_tree`` (integrator.py:119-135).  ``noise_source(step, chain, tag)``
may inject explicit normals instead (used to compare trajectories with the
oracle on identical noise).
"""

from __future__ import annotations

from collections.abc import Sequence
from typing import Any, Callable, NamedTuple

import numpy as np

from . import _lib, util
from .adaption import AdaptionStrategy, MassMatrix, RmsPropState

PyTree = Any


class IntegratorTriplet(tuple):
  """``(init_fn, update_fn, get_fn)`` plus what the fused driver needs."""

  def __new__(cls, init_fn, update_fn, get_fn, **meta):
    obj = super().__new__(cls, (init_fn, update_fn, get_fn))
    obj.meta = meta
    return obj


class LangevinState(NamedTuple):
  latent_variables: Any      # fp32 device [P]
  model_state: Any
  key: Any                   # Philox seed (int)
  adapt_state: Any           # RmsPropState or None
  data_state: Any
  potential: Any             # fp64 device scalar
  variance: Any              # fp64 device scalar
  step: int = 0              # chain-steps taken (noise counter)
  chain: int = 0             # chain index in the noise counter
  treedef: Any = None


class ObaboState(NamedTuple):
  positions: Any
  momentum: Any
  potential: Any
  model_state: Any
  data_state: Any
  key: Any
  kinetic_energy_start: Any
  kinetic_energy_end: Any
  step: int = 0
  chain: int = 0
  treedef: Any = None


class LeapfrogState(NamedTuple):
  positions: Any
  momentum: Any
  potential: Any
  model_state: Any
  data_state: Any
  key: Any
  extra_fields: Any = None
  step: int = 0
  chain: int = 0
  treedef: Any = None


def key_to_seed(key) -> int:
  """An int seed, or a JAX-style 2-word key, as the 64-bit Philox key."""
  if key is None:
    return 0
  a = np.asarray(key).ravel()
  seed = 0
  for k in a:
    seed = ((seed << 32) | (int(k) & 0xFFFFFFFF)) & ((1 << 64) - 1)
  return seed


def _flat(sample):
  import torch
  flat, tdef = util.ravel(sample)
  return torch.from_numpy(flat).cuda(), tdef


def _flat_host(sample):
  """Flat fp32 host tensor of a sample (a copy).  The first step moves it to
  the device; fused runs of many chains move all chains' in one copy."""
  import torch
  flat, tdef = util.ravel(sample)
  return torch.from_numpy(flat), tdef


def _dev(t):
  return t if t is None or t.is_cuda else t.cuda()


def _flat_tree_like(tree, P, fill=None):
  """Mass / friction pytree (or scalar) -> fp32 device [P] or None."""
  import torch
  if tree is None:
    return None
  if np.isscalar(tree):
    return torch.full((P,), float(tree), dtype=torch.float32, device="cuda")
  flat, _ = util.ravel(tree)
  if flat.size != P:
    raise ValueError(f"tree has {flat.size} entries, sample has {P}")
  return torch.from_numpy(flat).cuda()


def _mass_vector(mass, const_mass, P):
  """The diagonal mass M [P] the update kernels take (they use 1/M and
  sqrt(M)): an adapted mass -- a flat device vector M, or a ``MassMatrix``
  whose inverse is inverted -- else ``const_mass``, else None (unit mass)."""
  import torch
  if mass is None:
    return _flat_tree_like(const_mass, P)
  if isinstance(mass, MassMatrix):
    inv = mass.inv
    inv = inv.reshape(-1) if hasattr(inv, "is_cuda") else _flat_tree_like(inv, P)
    return torch.reciprocal(_dev(inv).to(torch.float32))
  m = _dev(mass.reshape(-1).to(torch.float32)) if hasattr(mass, "is_cuda") else \
      _flat_tree_like(mass, P)
  if m.numel() != P:
    raise ValueError(f"mass has {m.numel()} entries, sample has {P}")
  return m


def _dense_mass(mass):
  """(inverse mass [P, P], root mass [P, P]) fp32 device matrices when
  ``mass`` is a dense MassMatrix (mass_matrix(diagonal=False)), else None."""
  if isinstance(mass, MassMatrix) and hasattr(mass.inv, "dim") and mass.inv.dim() == 2:
    import torch
    inv = _dev(mass.inv).to(torch.float32).contiguous()
    sq = _dev(mass.sqrt).to(torch.float32).contiguous()
    return inv, sq
  return None


def _noise(seed, chain, buf=None):
  if buf is not None:
    return _lib.noise(seed, chain, noise_dev=buf, noise_stride=buf.numel())
  return _lib.noise(seed, chain)


def _injected(noise_source, step, chain, tag):
  if noise_source is None:
    return None
  import torch
  z = noise_source(step, chain, tag)
  return torch.as_tensor(z, dtype=torch.float32).reshape(-1).cuda().contiguous()


def _eval(potential_fn, w, batch, info, want_grad=True):
  ds = batch.dataset
  n_obs = info.observation_count if info is not None else ds.observation_count
  mask = None
  return potential_fn.evaluate(w.view(1, -1), batch.indices.view(1, -1), ds,
                               mask=mask, grad=want_grad,
                               observation_count=n_obs)


class LangevinChains(Sequence):
  """The initial states of C chains of :func:`langevin_diffusion` made
  together (``init_fn.many``), held as whole host tensors: positions
  [C, P], RMSprop ``v`` [C, P] (or None) and the chains' data pipelines
  (:class:`gbsgmc.data.core.RandomPipelines`, whose stream words are one
  [C, 5] tensor).  Indexing gives chain i's :class:`LangevinState`, whose
  tensors are row views of these (made on first access and kept), so the
  sequence stands for the list of states; the fused driver moves each
  whole tensor in one copy instead."""

  def __init__(self, positions, rms_v, alpha, lmbd, pipelines, key,
               model_state, treedef):
    self.positions, self.rms_v = positions, rms_v
    self.alpha, self.lmbd = float(alpha), float(lmbd)
    self.pipelines = pipelines
    self.key = key
    self.model_state = model_state
    self.treedef = treedef
    self._states = [None] * int(positions.shape[0])

  @property
  def chain_ids(self):
    return self.pipelines.chain_ids

  def __len__(self):
    return len(self._states)

  def __getitem__(self, i):
    if isinstance(i, slice):
      return [self[j] for j in range(*i.indices(len(self)))]
    if i < 0:
      i += len(self)
    st = self._states[i]   # raises IndexError past the end
    if st is None:
      import torch
      from .adaption import RmsPropState
      adapt = None if self.rms_v is None else \
          RmsPropState(self.rms_v[i], self.alpha, self.lmbd)
      st = LangevinState(
          latent_variables=self.positions[i], model_state=self.model_state,
          key=self.key, adapt_state=adapt, data_state=self.pipelines.state(i),
          potential=torch.zeros((), dtype=torch.float64),
          variance=torch.ones((), dtype=torch.float64), step=0,
          chain=int(self.pipelines.chain_ids[i]), treedef=self.treedef)
      self._states[i] = st
    return st


def langevin_diffusion(potential_fn, batch_fn, adaption: AdaptionStrategy = None,
                       noise_source: Callable = None):
  """SGLD with optional RMSprop (integrator.py:767-924)."""
  if adaption is not None and getattr(adaption, "kind", "rms_prop") != "rms_prop":
    raise NotImplementedError("langevin_diffusion adapts its manifold with "
                              "rms_prop only")
  batch_init, batch_get, _ = batch_fn

  def init_fn(init_sample, key=0, adaption_kwargs=None, batch_kwargs=None,
              init_model_state=None):
    import torch
    adaption_kwargs = adaption_kwargs or {}
    batch_kwargs = batch_kwargs or {}
    # The state starts on the host; update_fn (or a fused run) moves it.
    w, tdef = _flat_host(init_sample)
    adapt_state = None if adaption is None else adaption.init(w, **adaption_kwargs)
    data_state = batch_init(**batch_kwargs)
    chain = int(data_state.chain_id or 0)
    return LangevinState(
        latent_variables=w, model_state=init_model_state,
        key=key_to_seed(key), adapt_state=adapt_state, data_state=data_state,
        potential=torch.zeros((), dtype=torch.float64),
        variance=torch.ones((), dtype=torch.float64),
        step=0, chain=chain, treedef=tdef)

  def init_many(init_samples, key=0, adaption_kwargs=None, batch_kwargs=None,
                init_model_state=None):
    """``[init_fn(s, key, ...) for s in init_samples]`` in bulk.  With host
    random pipelines that register in bulk, the chains come back as one
    :class:`LangevinChains` (the samples raveled into one [C, P] tensor, the
    RMSprop states and the pipelines' stream words made for all chains at
    once); otherwise as a list of states made one by one."""
    import torch
    adaption_kwargs = adaption_kwargs or {}
    batch_kwargs = batch_kwargs or {}
    many = getattr(batch_init, "many", None)
    if adaption is not None and getattr(adaption.init, "many", None) is None:
      many = None
    if many is None:
      return [init_fn(s, key, adaption_kwargs, batch_kwargs, init_model_state)
              for s in init_samples]
    flat, tdef = util.ravel_many(init_samples)
    pipelines = many(len(init_samples), **batch_kwargs)
    if pipelines is None:
      return [init_fn(s, key, adaption_kwargs, batch_kwargs, init_model_state)
              for s in init_samples]
    W = torch.from_numpy(flat)
    V, alpha, lmbd = None, 0.9, 1e-5
    if adaption is not None:
      V, alpha, lmbd = adaption.init.many(W, **adaption_kwargs)
    return LangevinChains(W, V, alpha, lmbd, pipelines, key_to_seed(key),
                          init_model_state, tdef)

  init_fn.many = init_many

  def get_fn(state: LangevinState):
    return {"variables": state.latent_variables,
            "likelihood": -state.potential,
            "model_state": state.model_state}

  def update_fn(state: LangevinState, parameters):
    data_state, (batch, info) = batch_get(state.data_state, information=True)
    w = _dev(state.latent_variables)
    r = _eval(potential_fn, w, batch, info)
    adapt_state = state.adapt_state
    if adapt_state is not None and not adapt_state.v.is_cuda:
      adapt_state = adapt_state._replace(v=adapt_state.v.cuda())
    v = None if adapt_state is None else adapt_state.v
    alpha = 0.9 if state.adapt_state is None else state.adapt_state.alpha
    lmbd = 1e-5 if state.adapt_state is None else state.adapt_state.lmbd
    buf = _injected(noise_source, state.step, state.chain, _lib.TAG_SGLD)
    sch = _lib.sched(step_size=float(parameters.step_size),
                     temperature=float(parameters.temperature),
                     offset=state.step)
    _lib.call("gbsgmc_sgld_update", 1, w.numel(), _lib.ptr(w),
              _lib.ptr(r.grad), _lib.ptr(v), alpha, lmbd, sch,
              _noise(state.key, state.chain, buf), None, _lib.stream_handle())
    return state._replace(latent_variables=w, adapt_state=adapt_state,
                          data_state=data_state, potential=r.U[0],
                          variance=r.lk_var[0], step=state.step + 1)

  return IntegratorTriplet(init_fn, update_fn, get_fn, kind="langevin",
                           potential=potential_fn, batch_fn=batch_fn,
                           adaption=adaption, noise_source=noise_source)


def init_mass(mass) -> MassMatrix:
  """Diagonal mass (integrator.py:99-116): inverse and square root."""
  return MassMatrix(inv=1.0 / mass, sqrt=mass ** 0.5)


def obabo(potential_fn, batch_fn, steps=10, friction=1.0, const_mass=None,
          noise_source: Callable = None):
  """OBABO integrator with two minibatches per step (integrator.py:138-346)."""
  init_data, get_data, _ = batch_fn

  def init_fn(init_sample, key=None, batch_kwargs=None, init_model_state=None):
    import torch
    batch_kwargs = batch_kwargs or {}
    data_state = init_data(**batch_kwargs)
    w, tdef = _flat(init_sample)
    return ObaboState(
        positions=w, momentum=torch.zeros_like(w),
        potential=torch.zeros((), dtype=torch.float64, device="cuda"),
        model_state=init_model_state, data_state=data_state,
        key=key_to_seed(key),
        kinetic_energy_start=torch.zeros(1, dtype=torch.float64, device="cuda"),
        kinetic_energy_end=torch.zeros(1, dtype=torch.float64, device="cuda"),
        step=0, chain=int(data_state.chain_id or 0), treedef=tdef)

  def integrate(state: ObaboState, parameters, mass=None):
    x, p = state.positions, state.momentum
    P = x.numel()
    dense = _dense_mass(mass)
    m = None if dense is not None else _mass_vector(mass, const_mass, P)
    if dense is not None and noise_source is not None:
      raise NotImplementedError("injected noise with a dense mass")
    data_state = state.data_state
    step = state.step
    pot = state.potential
    for _ in range(steps):
      sch = _lib.sched(step_size=float(parameters.step_size),
                       temperature=float(parameters.temperature), offset=step)
      data_state, (b1, i1) = get_data(data_state, information=True)
      r1 = _eval(potential_fn, x, b1, i1)
      buf1 = _injected(noise_source, step, state.chain, _lib.TAG_OBABO_1)
      if dense is not None:
        _lib.call("gbsgmc_obabo_first_dense", 1, P, _lib.ptr(x), _lib.ptr(p),
                  _lib.ptr(r1.grad), _lib.ptr(dense[0]), _lib.ptr(dense[1]),
                  float(friction), _lib.ptr(state.kinetic_energy_start), sch,
                  _noise(state.key, state.chain), _lib.stream_handle())
      else:
        _lib.call("gbsgmc_obabo_first", 1, P, _lib.ptr(x), _lib.ptr(p),
                  _lib.ptr(r1.grad), _lib.ptr(m), float(friction),
                  _lib.ptr(state.kinetic_energy_start), sch,
                  _noise(state.key, state.chain, buf1), _lib.stream_handle())
      data_state, (b2, i2) = get_data(data_state, information=True)
      r2 = _eval(potential_fn, x, b2, i2)
      buf2 = _injected(noise_source, step, state.chain, _lib.TAG_OBABO_2)
      if dense is not None:
        _lib.call("gbsgmc_obabo_second_dense", 1, P, _lib.ptr(p), _lib.ptr(r2.grad),
                  _lib.ptr(dense[0]), _lib.ptr(dense[1]), float(friction),
                  _lib.ptr(state.kinetic_energy_end), sch,
                  _noise(state.key, state.chain), _lib.stream_handle())
      else:
        _lib.call("gbsgmc_obabo_second", 1, P, _lib.ptr(p), _lib.ptr(r2.grad),
                  _lib.ptr(m), float(friction),
                  _lib.ptr(state.kinetic_energy_end), sch,
                  _noise(state.key, state.chain, buf2), _lib.stream_handle())
      pot = 0.5 * (r1.U[0] + r2.U[0])
      step += 1
    return state._replace(potential=pot, data_state=data_state, step=step)

  def get_fn(state):
    return {"variables": state.positions, "energy": state.potential,
            "model_state": state.model_state}

  return IntegratorTriplet(init_fn, integrate, get_fn, kind="obabo",
                           potential=potential_fn, batch_fn=batch_fn,
                           steps=steps, friction=friction,
                           const_mass=const_mass, noise_source=noise_source)


def friction_leapfrog(potential_fn, batch_fn, steps=10, friction=0.25,
                      const_mass=None, noise_model=None,
                      noise_source: Callable = None):
  """Original SGHMC leapfrog (integrator.py:563-765).  With a noise model
  (``adaption.fisher_information``) the injected noise of each step is
  sqrt(2h) cb_diff_sqrt xi, cb_diff_sqrt from the step's minibatch at the
  new positions (integrator.py:630-647), instead of friction sqrt(2h) xi."""
  if noise_model is not None and getattr(noise_model, "kind", None) != \
      "fisher_information":
    raise NotImplementedError("the SGHMC noise model is fisher_information")
  init_data, get_data, _ = batch_fn

  def init_fn(init_sample, key=None, batch_kwargs=None, init_model_state=None):
    import torch
    batch_kwargs = batch_kwargs or {}
    data_state = init_data(**batch_kwargs)
    w, tdef = _flat(init_sample)
    return LeapfrogState(
        positions=w, momentum=w.clone(),
        potential=torch.zeros((), dtype=torch.float64, device="cuda"),
        model_state=init_model_state, data_state=data_state,
        key=key_to_seed(key), step=0, chain=int(data_state.chain_id or 0),
        treedef=tdef)

  def integrate(state: LeapfrogState, parameters, mass=None):
    x, p = state.positions, state.momentum
    P = x.numel()
    m = _flat_tree_like(const_mass, P)
    scalar_friction = np.isscalar(friction)
    fric = None if scalar_friction else _flat_tree_like(friction, P)
    f = float(friction) if scalar_friction else 0.0
    step = state.step
    sch0 = _lib.sched(step_size=float(parameters.step_size),
                      temperature=float(parameters.temperature), offset=step)
    buf = _injected(noise_source, step, state.chain, _lib.TAG_SGHMC_RESAMPLE)
    _lib.call("gbsgmc_sghmc_resample", 1, P, _lib.ptr(p), _lib.ptr(m), sch0,
              _noise(state.key, state.chain, buf), _lib.stream_handle())
    data_state = state.data_state
    pot = state.potential
    for _ in range(steps):
      sch = _lib.sched(step_size=float(parameters.step_size),
                       temperature=float(parameters.temperature), offset=step)
      _lib.call("gbsgmc_sghmc_position", 1, P, _lib.ptr(x), _lib.ptr(p),
                _lib.ptr(m), _lib.ptr(fric), f, sch, _lib.stream_handle())
      data_state, (b, i) = get_data(data_state, information=True)
      r = _eval(potential_fn, x, b, i)
      buf = _injected(noise_source, step, state.chain, _lib.TAG_SGHMC_STEP)
      if noise_model is not None:
        nm = noise_model.get(None, x, r.grad, friction if scalar_friction else fric,
                             mini_batch=(b, i),
                             step_size=float(parameters.step_size))
        _lib.call("gbsgmc_sghmc_momentum_noise_model", 1, P, _lib.ptr(p),
                  _lib.ptr(r.grad), _lib.ptr(nm.cb_diff_sqrt), sch,
                  _noise(state.key, state.chain, buf), _lib.stream_handle())
      else:
        _lib.call("gbsgmc_sghmc_momentum", 1, P, _lib.ptr(p), _lib.ptr(r.grad),
                  _lib.ptr(fric), f, sch, _noise(state.key, state.chain, buf),
                  _lib.stream_handle())
      pot = r.U[0]
      step += 1
    return state._replace(potential=pot, data_state=data_state, step=step)

  def get_fn(state):
    return {"variables": state.positions, "energy": state.potential,
            "model_state": state.model_state}

  return IntegratorTriplet(init_fn, integrate, get_fn, kind="sghmc",
                           potential=potential_fn, batch_fn=batch_fn,
                           steps=steps, friction=friction,
                           const_mass=const_mass, noise_source=noise_source,
                           noise_model=noise_model)


def reversible_leapfrog(potential_fn, batch_fn, steps: int = 10,
                        friction: float = 0.25, const_mass=None,
                        noise_source: Callable = None):
  """Time-reversible leapfrog of AMAGOLD (integrator.py:349-560): a half
  position step, ``steps`` momentum steps (each but the first after a full
  position step) with the friction-implicit update
  ``p' = ((1 - h f) p - h g + sqrt(4 f h) sqrt(M) xi) / (1 + h f)``, and a
  final half position step.  The state's ``potential`` is the energy the
  MH test needs, ``sum 0.5 h (p + p') . M^-1 g`` over the steps (fp64,
  accumulated on the device).  The initial momentum is ``sqrt(M) xi``
  (Philox tag GBSGMC_TAG_AMAGOLD_INIT).  ``noise_source(step, chain, tag)``
  injects the normals (tests)."""
  if not np.isscalar(friction):
    raise NotImplementedError("per-parameter friction is not supported by the "
                              "reversible leapfrog kernels")
  init_data, get_data, _ = batch_fn
  f = float(friction)

  def init_fn(init_sample, key=None, batch_kwargs=None, init_model_state=None,
              mass=None):
    import torch
    batch_kwargs = batch_kwargs or {}
    data_state = init_data(**batch_kwargs)
    w, tdef = _flat(init_sample)
    P = w.numel()
    chain = int(data_state.chain_id or 0)
    seed = key_to_seed(key)
    buf = _injected(noise_source, 0, chain, _lib.TAG_AMAGOLD_INIT)
    if buf is not None:
      p = buf.clone()
    else:
      p = torch.empty(P, dtype=torch.float32, device="cuda")
      _lib.call("gbsgmc_philox_normal", seed, chain, 1, 0,
                _lib.TAG_AMAGOLD_INIT, P, _lib.ptr(p), P, _lib.stream_handle())
    dense = _dense_mass(mass)
    if dense is not None:
      q = torch.empty_like(p)
      _lib.call("gbsgmc_dense_matvec", 1, P, _lib.ptr(dense[1]), _lib.ptr(p),
                _lib.ptr(q), _lib.stream_handle())
      p = q
    else:
      m = _mass_vector(mass, const_mass, P)
      if m is not None:
        p = p * m.sqrt()
    return LeapfrogState(
        positions=w, momentum=p,
        potential=torch.zeros(1, dtype=torch.float64, device="cuda"),
        model_state=init_model_state, data_state=data_state, key=seed,
        step=0, chain=chain, treedef=tdef)

  def integrate(state: LeapfrogState, parameters, mass=None):
    import torch
    x, p = state.positions, state.momentum
    P = x.numel()
    dense = _dense_mass(mass)
    m = None if dense is not None else _mass_vector(mass, const_mass, P)
    if dense is not None and noise_source is not None:
      raise NotImplementedError("injected noise with a dense mass")
    step = state.step
    energy = torch.zeros(1, dtype=torch.float64, device="cuda")

    def sch(k):
      return _lib.sched(step_size=float(parameters.step_size),
                        temperature=float(parameters.temperature), offset=k)

    def position(scale, k):
      if dense is not None:
        _lib.call("gbsgmc_leapfrog_position_dense", 1, P, _lib.ptr(x), _lib.ptr(p),
                  _lib.ptr(dense[0]), scale, sch(k), _lib.stream_handle())
      else:
        _lib.call("gbsgmc_leapfrog_position", 1, P, _lib.ptr(x), _lib.ptr(p),
                  _lib.ptr(m), scale, sch(k), _lib.stream_handle())

    position(0.5, step)
    data_state = state.data_state
    for j in range(steps):
      if j > 0:
        position(1.0, step)
      data_state, (b, i) = get_data(data_state, information=True)
      r = _eval(potential_fn, x, b, i)
      if dense is not None:
        _lib.call("gbsgmc_amagold_momentum_dense", 1, P, _lib.ptr(p),
                  _lib.ptr(r.grad), _lib.ptr(dense[0]), _lib.ptr(dense[1]), f,
                  _lib.ptr(energy), sch(step), _noise(state.key, state.chain),
                  _lib.stream_handle())
      else:
        buf = _injected(noise_source, step, state.chain, _lib.TAG_AMAGOLD)
        _lib.call("gbsgmc_amagold_momentum", 1, P, _lib.ptr(p), _lib.ptr(r.grad),
                  _lib.ptr(m), f, _lib.ptr(energy), sch(step),
                  _noise(state.key, state.chain, buf), _lib.stream_handle())
      step += 1
    position(0.5, step)
    return state._replace(potential=energy, data_state=data_state, step=step)

  def get_fn(state):
    return {"variables": state.positions, "energy": state.potential,
            "model_state": state.model_state}

  return IntegratorTriplet(init_fn, integrate, get_fn, kind="reversible_leapfrog",
                           potential=potential_fn, batch_fn=batch_fn,
                           steps=steps, friction=friction,
                           const_mass=const_mass, noise_source=noise_source)
