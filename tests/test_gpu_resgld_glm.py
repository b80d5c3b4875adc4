"""alias.re_sgld on a generalised-linear potential through the fused pairs
plan (gbsgmc_glm_resgld_plan_create): P (normal, hot) pairs step, exchange
and keep their samples on the device, replayed from CUDA graphs.

With the launch shape of the GLM kernel fixed (one CTA per chain, four rows
per warp, no autotuning), the plan and the per-pair path (one chain at a
time through the C ABI, solver.parallel_tempering's host loop) run the same
arithmetic on the same index streams, noise and exchange uniforms, so they
must give the same samples bit for bit -- exchanges included.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(seed=3, N=3000, d=12):
  rng = np.random.default_rng(seed)
  X = rng.normal(size=(N, d)).astype(np.float32)
  y = (X @ rng.normal(size=d) + 0.5 * rng.normal(size=N)).astype(np.float32)
  return X, y


def _run(pairs, iterations, fused, temperature=1000.0, rms=False):
  from gbsgmc import alias, data, engine, likelihoods as L, potential
  X, y = _problem()
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = potential.minibatch_potential(L.GaussianPrior(10.0), L.LinearGaussian(sigma=0.5))
  run = alias.re_sgld(pot, loader, cache_size=16, batch_size=32,
                      temperature=temperature, first_step_size=2e-4,
                      last_step_size=2e-5, burn_in=20, accepted_samples=40)
  rng = np.random.default_rng(1)
  inits = [({"w": (0.1 * rng.normal(size=12)).astype(np.float32)},
            {"w": (0.1 * rng.normal(size=12)).astype(np.float32)})
           for _ in range(pairs)]
  engine.FUSED_ENABLED = fused
  try:
    return run(*inits, iterations=iterations)
  finally:
    engine.FUSED_ENABLED = True


def test_fused_pairs_equal_per_pair_path(lib, monkeypatch):
  from gbsgmc import engine
  monkeypatch.setenv("GBSGMC_AUTOTUNE", "0")
  monkeypatch.setenv("GBSGMC_GLM_SLICES", "1")
  monkeypatch.setenv("GBSGMC_GLM_RW", "4")
  used = []
  real = engine.try_fused_resgld

  def spy(*args, **kwargs):
    out = real(*args, **kwargs)
    used.append(out is not None)
    return out

  monkeypatch.setattr(engine, "try_fused_resgld", spy)
  engine.LAST_EXCHANGES = None
  fused = _run(5, 120, True)
  swaps = engine.LAST_EXCHANGES
  stepped = _run(5, 120, False)
  assert used == [True, False]
  # The pairs exchanged states many times.
  assert swaps is not None and swaps.min() > 5, swaps
  for a, b in zip(fused, stepped):
    assert a["sample_count"] == b["sample_count"] == 40
    wa = np.asarray(a["samples"]["variables"]["w"])
    wb = np.asarray(b["samples"]["variables"]["w"])
    assert np.isfinite(wa).all()
    np.testing.assert_array_equal(wa, wb)
    np.testing.assert_array_equal(a["samples"]["likelihood"], b["samples"]["likelihood"])


def test_fused_pairs_run_many_pairs_fast(lib):
  """512 pairs (1,024 chains) for 500 steps in one plan: finite samples in
  the reference's format, and every pair exchanged."""
  import time
  from gbsgmc import engine
  t0 = time.perf_counter()
  res = _run(512, 500, True)
  dt = time.perf_counter() - t0
  assert len(res) == 512
  W = np.stack([r["samples"]["variables"]["w"] for r in res])
  assert W.shape == (512, 40, 12) and np.isfinite(W).all()
  assert engine.LAST_EXCHANGES.min() > 0
  assert dt < 30, dt
