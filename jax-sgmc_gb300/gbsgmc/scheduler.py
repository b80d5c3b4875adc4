"""Schedules for step size, temperature, burn-in and thinning.

Mirrors jax_sgmc/scheduler.py: the same ``(init, update, get)`` triplets,
evaluated on the host (the values are tiny).  The fused driver turns a
scheduler into device tables (:func:`tables`): step size [K], temperature
[K] and the sample slot of each kept step [K].

``random_thinning`` draws its selection with numpy
(``Generator.choice(replace=False, p=...)``) instead of ``jax.random.choice``
(scheduler.py:599-666); the selection rule (probability proportional to step
size times burn-in) is the reference's, the random stream is not.
"""

from __future__ import annotations

from collections import namedtuple
from typing import Callable, Tuple

import numpy as np

specific_scheduler = namedtuple("specific_scheduler", ["init", "update", "get"])


class _Specific(specific_scheduler):
  """A specific scheduler that can also produce its whole table at once."""

  def __new__(cls, init, update, get, table=None):
    obj = super().__new__(cls, init, update, get)
    obj.table = table  # table(state, iterations) -> np.ndarray, or None
    return obj


class SchedulerTriplet(tuple):
  """``(init_fn, update_fn, get_fn)`` with the component schedulers."""

  def __new__(cls, init_fn, update_fn, get_fn, components):
    obj = super().__new__(cls, (init_fn, update_fn, get_fn))
    obj.components = components
    return obj


schedule = namedtuple("schedule", ["step_size", "temperature", "burn_in",
                                   "accept"])
scheduler_state = namedtuple("scheduler_state",
                             ["state", "step_size_state", "temperature_state",
                              "burn_in_state", "thinning_state",
                              "progress_bar_state"])
static_information = namedtuple("static_information", ["samples_collected"])


def init_scheduler(step_size: specific_scheduler = None,
                   temperature: specific_scheduler = None,
                   burn_in: specific_scheduler = None,
                   thinning: specific_scheduler = None,
                   progress_bar: bool = True,
                   progress_bar_steps=20) -> Tuple[Callable, Callable, Callable]:
  """Combines the specific schedulers (scheduler.py:93-237)."""
  del progress_bar_steps
  if step_size is None:
    step_size = polynomial_step_size(a=1.0, b=1.0, gamma=0.0)
  if temperature is None:
    temperature = constant_temperature(tau=1.0)
  if burn_in is None:
    burn_in = initial_burn_in(n=0)
  if thinning is None:
    thinning = _Specific(lambda iterations: (None, iterations),
                         lambda *args, **kwargs: None,
                         lambda *args, **kwargs: True,
                         lambda state, its: np.ones(its, bool))

  def init_fn(iterations: int, **scheduler_kwargs):
    state = (0, iterations)
    thinning_state, total_samples = thinning.init(
        iterations, **scheduler_kwargs.get('thinning', {}))
    burn_in_state, collected_samples = burn_in.init(
        iterations, **scheduler_kwargs.get('burn_in', {}))
    total_samples = min(total_samples, collected_samples)
    init_state = scheduler_state(
        state=state,
        step_size_state=step_size.init(iterations,
                                       **scheduler_kwargs.get('step_size', {})),
        temperature_state=temperature.init(
            iterations, **scheduler_kwargs.get('temperature', {})),
        burn_in_state=burn_in_state,
        thinning_state=thinning_state,
        progress_bar_state=None)
    return init_state, static_information(samples_collected=total_samples)

  def update_fn(state, **kwargs):
    iteration, total_iterations = state.state
    return scheduler_state(
        state=(iteration + 1, total_iterations),
        step_size_state=step_size.update(state.step_size_state, iteration,
                                         **kwargs),
        temperature_state=temperature.update(state.temperature_state,
                                             iteration, **kwargs),
        burn_in_state=burn_in.update(state.burn_in_state, iteration, **kwargs),
        thinning_state=thinning.update(state.thinning_state, iteration,
                                       **kwargs),
        progress_bar_state=None)

  def get_fn(state, **kwargs):
    iteration, _ = state.state
    return schedule(
        step_size=np.float32(step_size.get(state.step_size_state, iteration,
                                           **kwargs)),
        temperature=np.float32(temperature.get(state.temperature_state,
                                               iteration, **kwargs)),
        burn_in=np.float32(burn_in.get(state.burn_in_state, iteration,
                                       **kwargs)),
        accept=bool(thinning.get(state.thinning_state, iteration, **kwargs)))

  return SchedulerTriplet(init_fn, update_fn, get_fn,
                          dict(step_size=step_size, temperature=temperature,
                               burn_in=burn_in, thinning=thinning))


def _vector_tables(scheduler, state, iterations):
  comps = getattr(scheduler, "components", None)
  if comps is None:
    return None
  arrays = {}
  for name, field in (("step_size", "step_size_state"),
                      ("temperature", "temperature_state"),
                      ("burn_in", "burn_in_state"),
                      ("thinning", "thinning_state")):
    table = getattr(comps[name], "table", None)
    if table is None:
      return None
    arrays[name] = np.broadcast_to(
        np.asarray(table(getattr(state, field), iterations)), (iterations,))
  return arrays


def tables(scheduler, iterations: int, **scheduler_kwargs):
  """Evaluates a scheduler for all iterations.

  Returns ``(step_size[K] f32, temperature[K] f32, keep_slot[K] i32,
  n_kept)``: ``keep_slot[k]`` is the index of step k's sample in the sample
  buffer, or -1 when step k is not kept (burn-in or thinning), exactly the
  ``keep = burn_in and accept`` rule of solver.mcmc (solver.py:103-104).
  """
  init_fn, update_fn, get_fn = scheduler
  # Tables of the component schedulers' own (vectorised) tables depend on
  # the iteration count alone: a scheduler keeps the last few it made.
  cache = getattr(scheduler, "__dict__", {}).setdefault("_tables", {}) \
      if not scheduler_kwargs else None
  if cache is not None and iterations in cache:
    h, t, keep, n, static = cache[iterations]
    return h.copy(), t.copy(), keep.copy(), n, static
  state, static = init_fn(iterations, **scheduler_kwargs)
  vec = _vector_tables(scheduler, state, iterations)
  if vec is not None:
    h = vec["step_size"].astype(np.float32)
    t = vec["temperature"].astype(np.float32)
    kept = (vec["burn_in"] > 0) & vec["thinning"].astype(bool)
    keep = np.full(iterations, -1, np.int32)
    keep[kept] = np.arange(int(kept.sum()), dtype=np.int32)
    if cache is not None:
      if len(cache) >= 8:
        cache.pop(next(iter(cache)))
      cache[iterations] = (h.copy(), t.copy(), keep.copy(), int(kept.sum()), static)
    return h, t, keep, int(kept.sum()), static
  h = np.empty(iterations, np.float32)
  t = np.empty(iterations, np.float32)
  keep = np.full(iterations, -1, np.int32)
  slot = 0
  for k in range(iterations):
    s = get_fn(state)
    h[k] = s.step_size
    t[k] = s.temperature
    if bool(s.burn_in) and bool(s.accept):
      keep[k] = slot
      slot += 1
    state = update_fn(state)
  return h, t, keep, slot, static


def constant_temperature(tau=1.0) -> specific_scheduler:
  """Scales the added noise with an unchanged constant (scheduler.py:245-278)."""

  def init_fn(iterations, tau=tau):
    del iterations
    return tau

  def update_fn(state, iteration, **kwargs):
    return state

  def get_fn(state, iteration, **kwargs):
    return state

  return _Specific(init_fn, update_fn, get_fn,
                   lambda state, its: np.full(its, state, np.float32))


def cyclic_temperature(beta=1.0, k: int = 1) -> specific_scheduler:
  raise NotImplementedError


def adaptive_step_size(burn_in=0, initial_step_size=0.05,
                       stabilization_constant=100, decay_constant=0.75,
                       speed_constant=0.05, target_acceptance_rate=0.02):
  """Dual averaging step size (scheduler.py:376-444)."""

  def init(iterations, burn_in=burn_in, initial_step_size=initial_step_size,
           stabilization_constant=stabilization_constant,
           decay_constant=decay_constant, speed_constant=speed_constant,
           target_acceptance_rate=target_acceptance_rate):
    del iterations
    return (burn_in, float(np.log(initial_step_size)), 0.0,
            target_acceptance_rate, stabilization_constant, decay_constant,
            speed_constant, float(np.log(10 * initial_step_size)))

  def update(state, iteration, acceptance_ratio=0.0, **kwargs):
    burn_in, x_bar, h_bar, alpha, t0, kappa, gamma, mu = state
    acceptance_ratio = float(acceptance_ratio)  # a device scalar from the MH step
    m = iteration + 1
    h_bar *= (1 - 1 / (m + t0))
    h_bar += 1 / (m + t0) * (alpha - acceptance_ratio)
    x = mu - np.sqrt(m) / gamma * h_bar
    lr = m ** (-kappa)
    x_bar_old = x_bar
    x_bar = x_bar * (1 - lr) + lr * x
    x_bar = x_bar if iteration < burn_in else x_bar_old
    return burn_in, x_bar, h_bar, alpha, t0, kappa, gamma, mu

  def get(state, iteration, **kwargs):
    return np.exp(state[1])

  return specific_scheduler(init, update, get)


def polynomial_step_size(a=1.0, b=1.0, gamma=0.33) -> specific_scheduler:
  """eps_n = a (b + n)^(-gamma) (scheduler.py:447-491), as an fp32 table."""

  def init_fn(iterations, a=a, b=b, gamma=gamma):
    assert gamma >= 0, f"Gamma must be positive: gamma = {gamma}"
    assert a > 0, f"a must be positive: a = {a}"
    assert b > 0, f"b must be greater than zero: b = {b}"
    n = np.arange(iterations, dtype=np.float32)
    unscaled = np.power(np.float32(b) + n, np.float32(-gamma), dtype=np.float32)
    return np.multiply(np.float32(a), unscaled, dtype=np.float32)

  def update_fn(state, iteration, **kwargs):
    return state

  def get_fn(state, iteration, **kwargs):
    return state[iteration]

  return _Specific(init_fn, update_fn, get_fn, lambda state, its: state[:its])


def _find_ab(its, gamma, first, last):
  """a, b with a b^-gamma = first and a (b + its - 1)^-gamma = last
  (scheduler.py:512-519), in fp32 like the reference."""
  f32 = np.float32
  ginv = np.power(f32(gamma), f32(-1.0))
  fpow = np.power(f32(first), -ginv)
  lpow = np.power(f32(last), -ginv)
  apow = np.divide(lpow - fpow, f32(its - 1))
  a = np.power(apow, f32(-gamma))
  b = np.power(np.divide(f32(first), a), -ginv)
  return a, b


def polynomial_step_size_first_last(first=1.0, last=1.0,
                                    gamma=0.33) -> specific_scheduler:
  """Polynomial schedule defined by the first and last step (scheduler.py:494-542)."""

  def init_fn(iterations, first=first, last=last, gamma=gamma):
    assert gamma > 0, f"Gamma must be bigger than 0, is {gamma}"
    assert first >= last, (f"The first step size must be larger than the "
                           f"last: {first} !>= {last}")
    a, b = _find_ab(iterations, gamma, first, last)
    return polynomial_step_size(a=a, b=b, gamma=gamma).init(iterations)

  def update_fn(state, iteration, **kwargs):
    return state

  def get_fn(state, iteration, **kwargs):
    return state[iteration]

  return _Specific(init_fn, update_fn, get_fn, lambda state, its: state[:its])


def cyclic_burn_in(beta=1.0, k: int = 1):
  raise NotImplementedError


def initial_burn_in(n=0) -> specific_scheduler:
  """Discards the first n steps (scheduler.py:567-589)."""

  def init_fn(iterations, n=n):
    return n, iterations - n

  def update_fn(state, iteration, **kwargs):
    return state

  def get_fn(state, iteration, **kwargs):
    return 1.0 if state <= iteration else 0.0

  return _Specific(init_fn, update_fn, get_fn,
                   lambda state, its: (np.arange(its) >= state).astype(np.float32))


def random_thinning(step_size_schedule: specific_scheduler,
                    burn_in_schedule: specific_scheduler, selections: int,
                    key=None) -> specific_scheduler:
  """Random thinning weighted by the step size (scheduler.py:599-666)."""

  def init_fn(iterations, step_size_schedule=step_size_schedule,
              burn_in_schedule=burn_in_schedule, selections=selections,
              key=key):
    seed = 0 if key is None else int(np.asarray(key, dtype=np.uint64).ravel()[-1])
    ss_state = step_size_schedule.init(iterations)
    bi_state, _ = burn_in_schedule.init(iterations)
    ss_tab = getattr(step_size_schedule, "table", None)
    bi_tab = getattr(burn_in_schedule, "table", None)
    if ss_tab is not None and bi_tab is not None:
      probs = (np.asarray(ss_tab(ss_state, iterations), np.float64)
               * np.asarray(bi_tab(bi_state, iterations), np.float64))
    else:
      probs = np.empty(iterations, np.float64)
      for it in range(iterations):
        probs[it] = (float(step_size_schedule.get(ss_state, it))
                     * float(burn_in_schedule.get(bi_state, it)))
        ss_state = step_size_schedule.update(ss_state, it)
        bi_state = burn_in_schedule.update(bi_state, it)
    assert np.count_nonzero(probs) >= selections, "Cannot select enough values"
    rng = np.random.default_rng(seed)
    accepted = rng.choice(np.arange(iterations), size=(selections,),
                          replace=False, p=probs / probs.sum())
    return np.sort(accepted), selections

  def update_fn(state, iteration, **kwargs):
    return state

  def get_fn(state, iteration, **kwargs):
    return bool(np.any(iteration == state))

  def table(state, its):
    out = np.zeros(its, bool)
    out[np.asarray(state)[np.asarray(state) < its]] = True
    return out

  return _Specific(init_fn, update_fn, get_fn, table)
