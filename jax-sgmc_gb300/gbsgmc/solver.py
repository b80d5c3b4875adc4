"""Solvers and the MCMC driver (mirrors jax_sgmc/solver.py).

``mcmc(solver, scheduler, strategy, saving)`` returns ``run(*states,
schedulers=None, iterations)``.  The reference runs each chain's
``jit(lax.scan)`` in turn (solver.py:152-171).  Here, when every chain is an
SGLD chain on a kernel-backed GLM potential, all chains run together in one
fused, CUDA-graph-captured plan (:func:`gbsgmc.engine.run_sgld_glm`);
otherwise each chain steps through the per-step C ABI calls.  Results have
the reference's per-chain format either way.
"""

from __future__ import annotations

from typing import Any, NamedTuple

import numpy as np

from . import _lib, engine, io, scheduler as sched_mod


class SolverTriplet(tuple):

  def __new__(cls, init, update, get, **meta):
    obj = super().__new__(cls, (init, update, get))
    obj.meta = meta
    return obj


def sgmc(integrator):
  """Plain SG-MCMC: integrate without MH step or tempering (solver.py:188-217)."""
  init_integrator, update_integrator, get_integrator = integrator

  def init(*args, **kwargs):
    return init_integrator(*args, **kwargs)

  many = getattr(init_integrator, "many", None)
  if many is not None:
    init.many = many

  def update(state, schedule):
    return update_integrator(state, schedule), None

  def get(state):
    return get_integrator(state)

  return SolverTriplet(init, update, get, kind="sgmc", integrator=integrator)


class TemperingState(NamedTuple):
  normal: Any
  hot: Any
  ssq: Any        # fp64 device [1]
  F: float
  step: Any       # int64 device [1]
  key: int        # the exchange uniforms' Philox key: (seed << 32) | pair chain
  seed: int = 0   # the user's key
  pair_chain: int = 0   # chain id of the pair's first normal chain


def parallel_tempering(integrator, sa_schedule=None):
  """reSGLD: a normal and a hot chain exchanging states (solver.py:220-299).

  The exchange test runs in FP64 on the device (``gbsgmc_resgld_swap_f64``)
  with the reference's rule: the pair keeps its states when
  ``log u < log s`` and exchanges them otherwise (solver.py:283-291).
  Only the reference's stochastic-approximation schedule 1/n is supported.
  """
  if sa_schedule is not None:
    probe = [sa_schedule(n) for n in (1, 2, 7)]
    if not np.allclose(probe, [1.0, 0.5, 1 / 7]):
      raise NotImplementedError("only sa_schedule = 1/n is implemented")
  init_integrator, update_integrator, get_integrator = integrator

  def init(normal_sample, tempered_sample, ssq_init=0.0, key=0, F=1.0,
           **kwargs):
    import torch
    from .integrator import key_to_seed
    seed = int(np.asarray(key).ravel()[-1]) if key is not None else 0
    # Both chains draw their noise with the pair's key; their own chain ids
    # (their data pipelines') keep the streams apart, and the streams move
    # with the states when the pair exchanges them.  Chains without distinct
    # ids (pipelines that carry none) get distinct keys instead.
    normal = init_integrator(normal_sample, key=seed, **kwargs)
    hot = init_integrator(tempered_sample, key=seed, **kwargs)
    if normal.chain == hot.chain:
      normal = normal._replace(key=key_to_seed((seed, 1)))
      hot = hot._replace(key=key_to_seed((seed, 2)))
    return TemperingState(
        normal, hot,
        torch.full((1,), float(ssq_init), dtype=torch.float64, device="cuda"),
        float(F), torch.zeros(1, dtype=torch.int64, device="cuda"),
        key_to_seed((seed, normal.chain)), seed, int(normal.chain))

  def update(state: TemperingState, normal_schedule, hot_schedule,
             uniform=None):
    import torch
    normal = update_integrator(state.normal, normal_schedule)
    hot = update_integrator(state.hot, hot_schedule)
    # Every buffer is bound to a name until the launch is enqueued.
    temps = torch.tensor([float(normal_schedule.temperature),
                          float(hot_schedule.temperature)],
                         dtype=torch.float64, device="cuda")
    perm = torch.zeros(1, dtype=torch.int32, device="cuda")
    u = None if uniform is None else torch.tensor(
        [float(uniform)], dtype=torch.float64, device="cuda")
    Un = normal.potential.reshape(1)
    Uh = hot.potential.reshape(1)
    var = normal.variance.reshape(1)
    step = int(normal.step)
    _lib.call("gbsgmc_resgld_swap_f64", 1, _lib.ptr(Un), _lib.ptr(Uh),
              _lib.ptr(var), _lib.ptr(temps[0:1]), _lib.ptr(temps[1:2]),
              state.F, _lib.ptr(state.ssq), _lib.ptr(state.step), _lib.ptr(u),
              state.key, step, None, _lib.ptr(perm), _lib.stream_handle())
    if int(perm.item()) == 1:
      normal, hot = hot, normal
    return state._replace(normal=normal, hot=hot), None

  def get(state: TemperingState):
    return get_integrator(state.normal)

  return SolverTriplet(init, update, get, kind="parallel_tempering",
                       integrator=integrator)


class MHState(NamedTuple):
  """State of a solver with a full-data MH correction (AMAGOLD, SGGMC)."""
  integrator_state: Any
  potential: Any          # fp64 device [1]: full potential of the current sample
  full_data_state: Any
  key: int
  acceptance_ratio: Any   # fp64 device [1]
  step_size: float
  mh_step: int            # MH corrections done (the Philox counter of u)
  mass_state: Any = None


# The reference's state names for the two MH solvers (solver.py:27-64);
# both share one layout here.
AMAGOLDState = MHState
SGGMCState = MHState


def _mh_solver(kind, integrator, full_potential_fn, full_data_map,
               mass_adaption, reject_sign):
  init_integrator, update_integrator, get_integrator = integrator
  init_full_data, full_data_map_fn, _ = full_data_map
  if mass_adaption is not None:
    init_mass, update_mass, get_mass = tuple(mass_adaption)[:3]

  def current_mass(mass_state):
    # The device adaption keeps the kernels' mass vector itself; any other
    # adaption triplet gives a MassMatrix.
    m = getattr(mass_state, "mass", None)
    return m if m is not None else get_mass(mass_state)

  def init(init_sample, key=0, initial_mass=None, full_data_kwargs=None,
           **kwargs):
    import torch
    mass_state = mass = None
    if mass_adaption is not None:
      mass_state = init_mass(init_sample, initial_mass)
      mass = current_mass(mass_state)
    elif initial_mass is not None:
      raise ValueError("initial_mass needs a mass_adaption")
    full_data_state = init_full_data(**(full_data_kwargs or {}))
    U, (full_data_state, model_state) = full_potential_fn(
        init_sample, full_data_state, full_data_map_fn,
        state=kwargs.get("init_model_state"))
    kwargs["init_model_state"] = model_state
    seed = int(np.asarray(key).ravel()[-1]) if key is not None else 0
    if kind == _lib.MH_AMAGOLD and mass is not None:
      # The initial momentum is drawn with the initial mass (solver.py:352).
      kwargs["mass"] = mass
    integrator_state = init_integrator(init_sample, key=(seed, 1), **kwargs)
    return MHState(integrator_state=integrator_state,
                   potential=U.reshape(1).to(torch.float64).clone(),
                   full_data_state=full_data_state, key=seed,
                   acceptance_ratio=torch.zeros(1, dtype=torch.float64,
                                                device="cuda"),
                   step_size=0.0, mh_step=0, mass_state=mass_state)

  def update(state: MHState, schedule):
    import torch
    ist = state.integrator_state
    x_old = ist.positions.clone()
    p_old = ist.momentum.clone()
    if mass_adaption is not None:
      proposal = update_integrator(ist, schedule,
                                   mass=current_mass(state.mass_state))
    else:
      proposal = update_integrator(ist, schedule)
    U_new, (full_data_state, model_state) = full_potential_fn(
        proposal.positions, state.full_data_state, full_data_map_fn,
        state=proposal.model_state)
    U_new = U_new.reshape(1).to(torch.float64)
    accept = torch.empty(1, dtype=torch.int32, device="cuda")
    ratio = torch.empty(1, dtype=torch.float64, device="cuda")
    U_keep = torch.empty(1, dtype=torch.float64, device="cuda")
    sch = _lib.sched(step_size=float(schedule.step_size),
                     temperature=float(schedule.temperature),
                     offset=state.mh_step)
    if kind == _lib.MH_AMAGOLD:
      energy, ke0, ke1 = proposal.potential, None, None
    else:
      energy, ke0, ke1 = None, proposal.kinetic_energy_start, \
          proposal.kinetic_energy_end
    _lib.call("gbsgmc_mh_accept", 1, kind, _lib.ptr(state.potential),
              _lib.ptr(U_new), _lib.ptr(energy), _lib.ptr(ke0), _lib.ptr(ke1),
              sch, None, state.key, int(ist.chain), _lib.ptr(accept),
              _lib.ptr(ratio), _lib.ptr(U_keep), _lib.stream_handle())
    P = proposal.positions.numel()
    _lib.call("gbsgmc_mh_select", 1, P, _lib.ptr(accept),
              _lib.ptr(proposal.positions), _lib.ptr(x_old),
              _lib.ptr(proposal.momentum), _lib.ptr(p_old), float(reject_sign),
              _lib.stream_handle())
    new_ist = proposal
    if kind == _lib.MH_SGGMC:
      # The kinetic energies restart at 0 after each correction
      # (solver.py:536-537).
      new_ist = proposal._replace(
          kinetic_energy_start=torch.zeros(1, dtype=torch.float64, device="cuda"),
          kinetic_energy_end=torch.zeros(1, dtype=torch.float64, device="cuda"))
    mass_state = state.mass_state
    if mass_adaption is not None:
      # Adapted on the sample the correction kept (solver.py:409-412).
      mass_state = update_mass(mass_state, new_ist.positions)
    new_state = state._replace(integrator_state=new_ist, potential=U_keep,
                               full_data_state=full_data_state,
                               acceptance_ratio=ratio,
                               step_size=float(schedule.step_size),
                               mh_step=state.mh_step + 1,
                               mass_state=mass_state)
    return new_state, {"acceptance_ratio": ratio}

  def get(state: MHState):
    out = dict(get_integrator(state.integrator_state))
    out["acceptance_ratio"] = state.acceptance_ratio
    out["step_size"] = state.step_size
    if kind == _lib.MH_SGGMC:
      out["potential"] = state.potential
    return out

  return init, update, get


def amagold(integrator_fn, full_potential_fn, full_data_map,
            mass_adaption=None):
  """AMAGOLD (solver.py:301-432): reversible-leapfrog proposals with an
  amortised full-data MH correction, log a = U_old - U_new + E (E the
  proposal's accumulated energy); a rejected proposal returns to the old
  sample with the momentum flipped.  The decision runs in FP64 on the device
  (``gbsgmc_mh_accept``); u comes from Philox (tag GBSGMC_TAG_MH) where the
  reference splits a JAX key."""
  init, update, get = _mh_solver(_lib.MH_AMAGOLD, integrator_fn,
                                 full_potential_fn, full_data_map,
                                 mass_adaption, -1.0)
  return SolverTriplet(init, update, get, kind="amagold",
                       integrator=integrator_fn, full_potential=full_potential_fn,
                       full_data_map=full_data_map, mass_adaption=mass_adaption)


def sggmc(integrator_fn, full_potential_fn, full_data_map, mass_adaption=None):
  """SGGMC (solver.py:434-577): OBABO proposals with a full-data MH
  correction, log a = -(U_new - U_old + KE_end - KE_start) / T; a rejected
  proposal returns to the old sample and momentum.  FP64 decision on the
  device as for :func:`amagold`."""
  init, update, get = _mh_solver(_lib.MH_SGGMC, integrator_fn,
                                 full_potential_fn, full_data_map,
                                 mass_adaption, 1.0)
  return SolverTriplet(init, update, get, kind="sggmc",
                       integrator=integrator_fn, full_potential=full_potential_fn,
                       full_data_map=full_data_map, mass_adaption=mass_adaption)


def _flat_of(sample_dict):
  v = sample_dict["variables"]
  return v.reshape(-1)


def mcmc(solver, scheduler, strategy="map", saving=None, loading=None):
  """Runs the solver for multiple chains and collects the samples."""
  if strategy not in ("map", "vmap", "pmap"):
    raise NotImplementedError(f"Strategy {strategy} is unknown. ")
  _, solver_update, solver_get = solver

  def run_single(state, iterations, schedulers):
    import torch
    main_kwargs = {}
    h, t, keep, n_kept, static = sched_mod.tables(scheduler, iterations,
                                                  **main_kwargs)
    init_fn, update_fn, get_fn = scheduler
    states = [init_fn(iterations)[0]]
    for kw in (schedulers or []):
      states.append(init_fn(iterations, **kw)[0])
    probe = solver_get(state)
    P = _flat_of(probe).numel()
    samples = torch.empty((n_kept, P), dtype=torch.float32, device="cuda")
    extra_key = "likelihood" if "likelihood" in probe else "energy"
    extra = torch.empty((n_kept,), dtype=torch.float64, device="cuda")
    for k in range(iterations):
      schedules = [get_fn(s) for s in states]
      state, stats = solver_update(state, *schedules)
      if keep[k] >= 0:
        got = solver_get(state)
        samples[keep[k]] = _flat_of(got)
        extra[keep[k]] = got[extra_key].reshape(())
      # The solver's statistics (the MH acceptance ratio) feed the schedule,
      # as in solver.py:113-121.
      states = [update_fn(s, **(stats or {})) for s in states]
    treedef = _treedef_of(state)
    return io.postprocess(saving or io.no_save(), n_kept, samples, treedef,
                          {extra_key: extra})

  def run_chains(states, schedulers=None, iterations=100000):
    """``run(*states)`` over a sequence of chain states, such as the
    :class:`~gbsgmc.integrator.LangevinChains` of a bulk initialisation
    (which the fused driver moves as whole tensors)."""
    iterations = int(iterations)
    if loading is not None:
      raise NotImplementedError("Loading of checkpoints is currently not "
                                "supported.")
    fused = engine.try_fused_resgld(solver, scheduler, states, schedulers,
                                    iterations, saving)
    if fused is None:
      fused = engine.try_fused_sgld(solver, scheduler, states, schedulers,
                                    iterations, saving)
    if fused is None:
      fused = engine.try_fused_net(solver, scheduler, states, schedulers,
                                   iterations, saving)
    if fused is None:
      fused = engine.try_fused_mh(solver, scheduler, states, schedulers,
                                  iterations, saving)
    if fused is not None:
      return fused
    return [run_single(s, iterations, schedulers) for s in states]

  def run(*states, schedulers=None, iterations=100000):
    return run_chains(list(states), schedulers, iterations)

  run.run_chains = run_chains
  return run


def _treedef_of(state):
  for name in ("treedef",):
    if hasattr(state, name) and getattr(state, name) is not None:
      return getattr(state, name)
  if hasattr(state, "normal"):
    return _treedef_of(state.normal)
  if hasattr(state, "integrator_state"):
    return _treedef_of(state.integrator_state)
  raise ValueError("state carries no sample tree definition")
