"""alias.re_sgld on the MLP likelihood through the fused pairs plan
(gbsgmc_mlp_resgld_pairs_plan_create): P (normal, hot) pairs step, exchange
and keep their samples on the device, replayed from CUDA graphs.

A chain's GEMM tiles do not depend on the other chains of a batch, and the
plan reads each row's minibatch and noise through its chain identity, so
the plan and the per-pair path (one chain at a time through the C ABI,
solver.parallel_tempering's host loop) run the same arithmetic on the same
index streams, noise and exchange uniforms: the samples must agree bit for
bit, exchanges included.
"""

import numpy as np
import pytest

import test_gpu_mlp as M

pytestmark = pytest.mark.gpu


def _run(pairs, iterations, fused, temperature=100.0):
  from gbsgmc import alias, data, engine, likelihoods as L, potential
  lik = L.MLPGaussian(d_in=64, h1=256, h2=256, sigma=M.SIGMA)
  X, y, w_star, rng = M.teacher_data(lik, 2000, seed=41)
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), lik)
  run = alias.re_sgld(pot, loader, cache_size=8, batch_size=128,
                      temperature=temperature, first_step_size=2e-6,
                      last_step_size=1e-6, burn_in=10, accepted_samples=20)
  W = M.chains_near(w_star, 2 * pairs, rng, spread=0.05)
  inits = [(lik.unravel(W[2 * i]), lik.unravel(W[2 * i + 1])) for i in range(pairs)]
  engine.FUSED_ENABLED = fused
  try:
    return run(*inits, iterations=iterations), lik
  finally:
    engine.FUSED_ENABLED = True


def test_fused_mlp_pairs_equal_per_pair_path(lib, monkeypatch):
  from gbsgmc import engine
  used = []
  real = engine.try_fused_resgld

  def spy(*args, **kwargs):
    out = real(*args, **kwargs)
    used.append(out is not None)
    return out

  monkeypatch.setattr(engine, "try_fused_resgld", spy)
  engine.LAST_EXCHANGES = None
  fused, lik = _run(3, 30, True)
  swaps = engine.LAST_EXCHANGES
  stepped, _ = _run(3, 30, False)
  assert used == [True, False]
  assert swaps is not None and swaps.sum() > 0, swaps
  for a, b in zip(fused, stepped):
    assert a["sample_count"] == b["sample_count"] == 20
    for name in lik.shapes():
      wa = np.asarray(a["samples"]["variables"][name])
      wb = np.asarray(b["samples"]["variables"][name])
      assert np.isfinite(wa).all()
      np.testing.assert_array_equal(wa, wb)
    np.testing.assert_array_equal(a["samples"]["likelihood"], b["samples"]["likelihood"])
