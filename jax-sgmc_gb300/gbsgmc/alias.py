"""Ready-to-use samplers (mirrors jax_sgmc/alias.py).

Same factory signatures and defaults as the reference; each returns
``run_fn(*init_samples, init_model_state=None, iterations=1000)`` producing
one result dict per chain.  ``sgld`` chains on a GLM potential run as one
fused GPU plan; the other presets step each chain through the C ABI.
"""

from __future__ import annotations

from functools import partial
from typing import Any, Union

from . import adaption, data, integrator, io, scheduler, solver

Pytree = Any


def _schedule(first_step_size, last_step_size, burn_in, accepted_samples,
              progress_bar, temperature=None):
  step_size_schedule = scheduler.polynomial_step_size_first_last(
      first=first_step_size, last=last_step_size)
  burn_in_schedule = scheduler.initial_burn_in(burn_in)
  random_thinning_schedule = scheduler.random_thinning(
      step_size_schedule, burn_in_schedule, selections=accepted_samples)
  return scheduler.init_scheduler(step_size=step_size_schedule,
                                  burn_in=burn_in_schedule,
                                  thinning=random_thinning_schedule,
                                  temperature=temperature,
                                  progress_bar=progress_bar)


def _init_states(solver_init, init, init_samples, **kwargs):
  """``[init(s) for s in init_samples]``, or for several chains whose
  samples have one structure the solver's bulk initialisation
  (``solver_init.many``): a sequence of the same states."""
  many = getattr(solver_init, "many", None)
  if many is not None and len(init_samples) > 1:
    try:
      return many(list(init_samples), **kwargs)
    except ValueError:
      pass   # samples of different structures: one by one
  return [init(s) for s in init_samples]


def sgld(potential_fn, data_loader, cache_size: int = 512,
         batch_size: int = 32, first_step_size: float = 0.05,
         last_step_size: float = 0.001, burn_in: int = 0,
         accepted_samples: int = 1000, rms_prop: bool = False,
         alpha: float = 0.9, lmbd: float = 1e-5, save_to_numpy: bool = True,
         progress_bar: bool = True):
  """Stochastic Gradient Langevin Dynamics (alias.py:30-120)."""
  random_data = data.random_reference_data(data_loader, cache_size, batch_size)
  rms = adaption.rms_prop() if rms_prop else None
  rms_integrator = integrator.langevin_diffusion(potential_fn, random_data,
                                                 adaption=rms)
  schedule = _schedule(first_step_size, last_step_size, burn_in,
                       accepted_samples, progress_bar)
  saving = io.save(io.MemoryCollector()) if save_to_numpy else None
  sgld_solver = solver.sgmc(rms_integrator)
  mcmc = solver.mcmc(sgld_solver, schedule, strategy='map', saving=saving)

  def run_fn(*init_samples, init_model_state: Pytree = None, iterations=1000):
    init = partial(sgld_solver[0],
                   adaption_kwargs={'alpha': alpha, 'lmbd': lmbd},
                   init_model_state=init_model_state)
    states = _init_states(sgld_solver[0], init, init_samples,
                          adaption_kwargs={'alpha': alpha, 'lmbd': lmbd},
                          init_model_state=init_model_state)
    return mcmc.run_chains(states, iterations=iterations)

  return run_fn


def re_sgld(potential_fn, data_loader, cache_size: int = 512,
            batch_size: int = 32, temperature: float = 1000.0,
            first_step_size: float = 0.05, last_step_size: float = 0.001,
            burn_in: int = 0, accepted_samples: int = 100,
            save_to_numpy: bool = True, progress_bar: bool = True):
  """Replica-exchange SGLD with one hot helper chain (alias.py:122-208)."""
  del progress_bar
  random_data = data.random_reference_data(data_loader, cache_size, batch_size)
  resgld_integrator = integrator.langevin_diffusion(potential_fn, random_data)
  schedule = _schedule(first_step_size, last_step_size, burn_in,
                       accepted_samples, False,
                       temperature=scheduler.constant_temperature(1.0))
  saving = io.save(io.MemoryCollector()) if save_to_numpy else None
  resgld_solver = solver.parallel_tempering(resgld_integrator)
  mcmc = solver.mcmc(resgld_solver, schedule, strategy='map', saving=saving)

  def run_fn(*init_samples, init_model_state: Pytree = None, iterations=1000):
    init = partial(resgld_solver[0], init_model_state=init_model_state)
    states = [init(*pair) for pair in init_samples]
    return mcmc(*states, iterations=iterations,
                schedulers=[{'temperature': {'tau': temperature}}])

  return run_fn


def re_sgld_ladder(potential_fn, data_loader, temperatures,
                   batch_sizes=None, batch_size: int = 32,
                   exchange_every: int = 1, F: float = 1.0,
                   first_step_size: float = 0.05, last_step_size: float = 0.001,
                   burn_in: int = 0, accepted_samples: int = 100,
                   rms_prop: bool = False, alpha: float = 0.9,
                   lmbd: float = 1e-5, save_to_numpy: bool = True,
                   seed: int = 0):
  """Replica-exchange SGLD over a ladder of R >= 2 temperatures: the
  generalisation of :func:`re_sgld`'s (normal, hot) pair (alias.py:122-208,
  solver.py:220-299) to R replicas at ``temperatures`` (coldest first; the
  first is the sampled chain, usually 1), each with its own minibatch size
  (``batch_sizes``, default ``batch_size`` for all), in which adjacent
  replicas attempt the reference's FP64 exchange every ``exchange_every``
  steps (pair parity alternating), each pair keeping its own stochastic-
  approximation variance estimate.  SGLD, with RMSprop when ``rms_prop``.
  No reference counterpart beyond R = 2.  On the MLP likelihood the ladder
  runs as one graph-captured plan (``gbsgmc_mlp_resgld_plan_create_keep``);
  ``run_fn(init_sample, iterations=K)`` starts every replica at
  ``init_sample`` (or at ``init_samples`` given one per replica) and
  returns one result dict, the kept samples of the coldest replica, in the
  reference's format.  K must be a multiple of ``exchange_every``.  Index
  streams are the loader's numpy pipelines, one per replica, each drawing
  ``max(batch_sizes)`` rounded up to 128 rows per step of which the replica
  uses its own count."""
  import numpy as np
  from . import engine, util
  from . import scheduler as sched_mod
  temps = np.asarray(temperatures, np.float32).reshape(-1)
  R = temps.size
  if R < 2:
    raise ValueError("a ladder needs at least two temperatures")
  if not getattr(potential_fn, "is_mlp", False):
    raise NotImplementedError("the replica ladder runs on the MLP likelihood")
  rows = np.full(R, batch_size, np.int32) if batch_sizes is None else \
      np.asarray(batch_sizes, np.int32).reshape(-1)
  if rows.size != R or (rows < 1).any():
    raise ValueError("one positive minibatch size per temperature")
  n_max = int((rows.max() + 127) // 128 * 128)
  every = int(exchange_every)
  if every < 1:
    raise ValueError("exchange_every must be positive")
  schedule = _schedule(first_step_size, last_step_size, burn_in,
                       accepted_samples, False)

  def run_fn(*init_samples, iterations=1000):
    import torch
    if iterations % every != 0:
      raise ValueError(f"iterations ({iterations}) must be a multiple of "
                       f"exchange_every ({every})")
    if len(init_samples) not in (1, R):
      raise ValueError(f"one initial sample, or one per replica ({R})")
    flats = [util.ravel(s) for s in init_samples]
    tdef = flats[0][1]
    Xh = np.stack([f[0] for f in flats]).astype(np.float32)
    if Xh.shape[0] == 1:
      Xh = np.repeat(Xh, R, axis=0)
    ds = data_loader.device_dataset()
    if Xh.shape[1] != potential_fn.dim(ds):
      raise ValueError(f"samples have {Xh.shape[1]} parameters, the network "
                       f"{potential_fn.dim(ds)}")
    ids, words = data_loader.register_random_pipelines(R, cache_size=1,
                                                       mb_size=n_max)
    pcg = torch.from_numpy(np.ascontiguousarray(words).view(np.int64)).cuda()
    h, t, keep, n_kept, _ = sched_mod.tables(schedule, iterations)
    tabs = [torch.from_numpy(np.ascontiguousarray(a)).cuda()
            for a in (np.asarray(h, np.float32), np.asarray(t, np.float32),
                      np.asarray(keep, np.int32))]
    X = torch.from_numpy(Xh).cuda()
    V = torch.ones_like(X) if rms_prop else None
    plan = engine.ResgldPlan(potential_fn, ds, X, V, rows, n_max, temps, tabs[0],
                             tabs[1], engine.IndexSource(pcg=pcg, chain_base=int(ids[0])),
                             noise_seed=seed, swap_seed=seed, every=every, F=F,
                             alpha=alpha, lmbd=lmbd, chain_base=int(ids[0]),
                             keep_tab=tabs[2], n_kept=n_kept)
    try:
      if iterations:
        plan.run(0, iterations)
      plan.check_status()
      samples = plan.samples[:n_kept].reshape(n_kept, 1, -1)
      lik = plan.sample_lik[:n_kept].reshape(n_kept, 1)
      run_fn.exchanges = plan.counts.cpu().numpy()
    finally:
      plan.close()
    return io.postprocess_chains(io.save(io.MemoryCollector()) if save_to_numpy
                                 else io.no_save(), n_kept, samples, [tdef],
                                 {"likelihood": lik}, [None])

  run_fn.exchanges = None
  return run_fn


def sghmc(potential_fn, data_loader, cache_size: int = 512,
          batch_size: int = 32, integration_steps: int = 10,
          friction: Union[float, Pytree] = 1.0, mass: Pytree = None,
          first_step_size: float = 0.05, last_step_size: float = 0.001,
          burn_in: int = 0, accepted_samples: int = 1000,
          adapt_noise_model: bool = False, diagonal_noise: bool = True,
          save_to_numpy: bool = True, progress_bar: bool = True):
  """Stochastic Gradient Hamiltonian Monte Carlo (alias.py:451-540)."""
  if adapt_noise_model:
    noise_model = adaption.fisher_information(minibatch_potential=potential_fn,
                                              diagonal=diagonal_noise)
  else:
    noise_model = None
  random_data = data.random_reference_data(data_loader, cache_size, batch_size)
  leapfrog = integrator.friction_leapfrog(potential_fn, random_data,
                                          friction=friction, const_mass=mass,
                                          steps=integration_steps,
                                          noise_model=noise_model)
  schedule = _schedule(first_step_size, last_step_size, burn_in,
                       accepted_samples, progress_bar)
  saving = io.save(io.MemoryCollector()) if save_to_numpy else None
  sghmc_solver = solver.sgmc(leapfrog)
  mcmc = solver.mcmc(sghmc_solver, schedule, strategy='map', saving=saving)

  def run_fn(*init_samples, init_model_state: Pytree = None, iterations=1000):
    init = partial(sghmc_solver[0], init_model_state=init_model_state)
    states = [init(s) for s in init_samples]
    return mcmc(*states, iterations=iterations)

  return run_fn


def obabo(potential_fn, data_loader, cache_size: int = 512,
          batch_size: int = 32, integration_steps: int = 10,
          friction: Union[float, Pytree] = 1.0, mass: Pytree = None,
          first_step_size: float = 0.05, last_step_size: float = 0.001,
          burn_in: int = 0, accepted_samples: int = 1000,
          save_to_numpy: bool = True, progress_bar: bool = True):
  """Langevin Monte Carlo with partial momentum refreshment (alias.py:542-619)."""
  random_data = data.random_reference_data(data_loader, cache_size, batch_size)
  obabo_integrator = integrator.obabo(potential_fn=potential_fn,
                                      batch_fn=random_data,
                                      steps=integration_steps,
                                      friction=friction, const_mass=mass)
  schedule = _schedule(first_step_size, last_step_size, burn_in,
                       accepted_samples, progress_bar)
  saving = io.save(io.MemoryCollector()) if save_to_numpy else None
  obabo_solver = solver.sgmc(obabo_integrator)
  mcmc = solver.mcmc(obabo_solver, schedule, strategy='map', saving=saving)

  def run_fn(*init_samples, init_model_state: Pytree = None, iterations=1000):
    init = partial(obabo_solver[0], init_model_state=init_model_state)
    states = [init(s) for s in init_samples]
    return mcmc(*states, iterations=iterations)

  return run_fn


def _mh_schedule(first_step_size, last_step_size, adaptive_step_size,
                 stabilization_constant, decay_constant, speed_constant,
                 target_acceptance_rate, burn_in, accepted_samples,
                 progress_bar):
  """The schedule of alias.amagold / alias.sggmc (alias.py:281-312)."""
  burn_in_schedule = scheduler.initial_burn_in(burn_in)
  if adaptive_step_size:
    step_size_schedule = scheduler.adaptive_step_size(
        burn_in=burn_in, initial_step_size=first_step_size,
        stabilization_constant=stabilization_constant,
        decay_constant=decay_constant, speed_constant=speed_constant,
        target_acceptance_rate=target_acceptance_rate)
    thinning = None
    assert accepted_samples is None, ("Thinning currently not supported for"
                                      " adaptive step size.")
  else:
    step_size_schedule = scheduler.polynomial_step_size_first_last(
        first=first_step_size, last=last_step_size)
    thinning = None if accepted_samples is None else scheduler.random_thinning(
        step_size_schedule, burn_in_schedule, selections=accepted_samples)
  return scheduler.init_scheduler(step_size=step_size_schedule,
                                  burn_in=burn_in_schedule, thinning=thinning,
                                  progress_bar=progress_bar)


def amagold(stochastic_potential_fn, full_potential_fn, data_loader,
            cache_size: int = 512, batch_size: int = 32,
            integration_steps: int = 10, friction: float = 0.25,
            first_step_size: float = 0.001, last_step_size: float = 0.001,
            adaptive_step_size: bool = False, stabilization_constant: int = 10,
            decay_constant: float = 0.75, speed_constant: float = 0.05,
            target_acceptance_rate: float = 0.25, burn_in: int = 0,
            accepted_samples: Union[int, None] = None, mass: Pytree = None,
            save_to_numpy: bool = True, progress_bar: bool = True):
  """AMAGOLD: reversible leapfrog with amortised full-data MH corrections
  (alias.py:210-327)."""
  random_data = data.random_reference_data(data_loader, cache_size, batch_size)
  full_data_map = data.full_reference_data(data_loader, cache_size, batch_size)
  leapfrog = integrator.reversible_leapfrog(
      stochastic_potential_fn, random_data, integration_steps, friction, mass)
  amagold_solver = solver.amagold(leapfrog, full_potential_fn, full_data_map)
  schedule = _mh_schedule(first_step_size, last_step_size, adaptive_step_size,
                          stabilization_constant, decay_constant,
                          speed_constant, target_acceptance_rate, burn_in,
                          accepted_samples, progress_bar)
  saving = io.save(io.MemoryCollector()) if save_to_numpy else None
  mcmc = solver.mcmc(amagold_solver, schedule, strategy='map', saving=saving)

  def run_fn(*init_samples, init_model_state: Pytree = None, iterations=1000):
    init = partial(amagold_solver[0], init_model_state=init_model_state)
    states = [init(s) for s in init_samples]
    return mcmc(*states, iterations=iterations)

  return run_fn


def sggmc(stochastic_potential_fn, full_potential_fn, data_loader,
          cache_size: int = 512, batch_size: int = 32,
          integration_steps: int = 10, friction_coefficient: float = 1.0,
          first_step_size: float = 0.001, last_step_size: float = 0.001,
          adaptive_step_size: bool = False, stabilization_constant: int = 10,
          decay_constant: float = 0.75, speed_constant: float = 0.05,
          target_acceptance_rate: float = 0.25, burn_in: int = 0,
          accepted_samples: Union[int, None] = None, mass: Pytree = None,
          save_to_numpy: bool = True, progress_bar: bool = True):
  """SGGMC: OBABO proposals with full-data MH corrections
  (alias.py:330-448)."""
  random_data = data.random_reference_data(data_loader, cache_size, batch_size)
  full_data_map = data.full_reference_data(data_loader, cache_size, batch_size)
  obabo_integrator = integrator.obabo(stochastic_potential_fn, random_data,
                                      integration_steps, friction_coefficient,
                                      mass)
  sggmc_solver = solver.sggmc(obabo_integrator, full_potential_fn,
                              full_data_map)
  schedule = _mh_schedule(first_step_size, last_step_size, adaptive_step_size,
                          stabilization_constant, decay_constant,
                          speed_constant, target_acceptance_rate, burn_in,
                          accepted_samples, progress_bar)
  saving = io.save(io.MemoryCollector()) if save_to_numpy else None
  mcmc = solver.mcmc(sggmc_solver, schedule, strategy='map', saving=saving)

  def run_fn(*init_samples, init_model_state: Pytree = None, iterations=1000):
    init = partial(sggmc_solver[0], init_model_state=init_model_state)
    states = [init(s) for s in init_samples]
    return mcmc(*states, iterations=iterations)

  return run_fn
