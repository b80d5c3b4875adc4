"""End-to-end runs through the reference-shaped API (gbsgmc.alias).

* Config-1 problem (Bayesian linear regression, N=10,000, d=32, n=128):
  alias.sgld with RMSprop reaches the closed-form posterior mean and the
  per-weight variances within 2 % relative error (bench.CFG1_PHASES).
* The fused many-chain plan and the per-step path give the same samples
  (1e-4 relative), and the plan reproduces the oracle trajectory driven by
  the same index stream and Philox normals.
* sghmc / obabo / re_sgld return the reference's result format.
"""

import numpy as np
import pytest

from oracle import sgmc_oracle as O

pytestmark = pytest.mark.gpu


def linreg(N=10_000, d=32, seed=20261204):
  rng = np.random.default_rng(seed)
  X = rng.normal(size=(N, d)).astype(np.float32)
  y = (X @ rng.normal(size=d) + 0.5 * rng.normal(size=N)).astype(np.float32)
  return X, y


def sgld_run(X, y, iterations, chains=1, burn_in=0, accepted=100, first=0.05,
             last=0.001, batch=128):
  from gbsgmc import alias, data, likelihoods as L, potential
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = potential.minibatch_potential(L.GaussianPrior(10.0),
                                      L.LinearGaussian(sigma=0.5),
                                      strategy="vmap")
  run = alias.sgld(pot, loader, cache_size=512, batch_size=batch,
                   first_step_size=first, last_step_size=last, burn_in=burn_in,
                   accepted_samples=accepted, rms_prop=True)
  d = X.shape[1]
  return run(*[{"w": np.zeros(d, np.float32)} for _ in range(chains)],
             iterations=iterations)


def test_config1_posterior_moments_within_2_percent(lib):
  """Bayesian linear regression with a closed-form posterior (N = 10,000,
  d = 32, sigma 0.5, prior N(0, 10^2 I), minibatch 128): alias.sgld with
  RMSprop (alpha 0.999), 16,384 chains run as the bench's three calls (travel
  from w = 0, shrink the spread, sample), reaches the posterior mean AND the
  per-weight posterior variances within 2 % relative L2 error.  At the
  default alpha 0.9 the reference's rms_prop (v updated with the current
  gradient before scaling it) widens the variance by about 11 %, whatever
  the step size; that is checked on the restated algorithm in
  tests/test_oracle.py."""
  import bench
  m = bench.config1_moment_error(chains=16384)
  assert m["mean"] < 0.02, m
  assert m["var"] < 0.02, m


def test_fused_plan_equals_per_step_path(lib):
  from gbsgmc import engine
  X, y = linreg(N=3000, d=12, seed=3)
  fused = sgld_run(X, y, 300, chains=3, accepted=50, batch=64)
  engine.FUSED_ENABLED = False
  try:
    stepped = sgld_run(X, y, 300, chains=3, accepted=50, batch=64)
  finally:
    engine.FUSED_ENABLED = True
  for a, b in zip(fused, stepped):
    assert a["sample_count"] == b["sample_count"] == 50
    np.testing.assert_allclose(a["samples"]["variables"]["w"],
                               b["samples"]["variables"]["w"], rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(a["samples"]["likelihood"],
                               b["samples"]["likelihood"], rtol=1e-5, atol=1e-2)


def test_plan_reproduces_oracle_over_many_steps(lib):
  """1000 steps of the linear-regression workload (N = 10,000, d = 32,
  minibatch 128) with the reference loader's index stream (seed = chain id
  0) and the production Philox noise, against the oracle."""
  from gbsgmc import engine, likelihoods as L, potential, data
  X, y = linreg()
  N, d, n, K = 10_000, 32, 128, 1000
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = potential.minibatch_potential(L.GaussianPrior(10.0), L.LinearGaussian(sigma=0.5))
  h = O.polynomial_first_last(0.05, 0.001, 0.33, K).astype(np.float32)
  T = np.ones(K, np.float32)
  keep = np.arange(K, dtype=np.int32)
  import torch
  st = O.loader_rng(0).bit_generator.state
  s, inc = st["state"]["state"], st["state"]["inc"]
  m = (1 << 64) - 1
  pcg = torch.from_numpy(np.array([[(s >> 64) & m, s & m, (inc >> 64) & m, inc & m, 0]],
                                  np.uint64).view(np.int64)).cuda()
  W = torch.zeros((1, d), dtype=torch.float32, device="cuda")
  V = torch.ones((1, d), dtype=torch.float32, device="cuda")
  run = engine.run_sgld_glm(pot, loader.device_dataset(), W, V, n, K, h, T, keep,
                            K, engine.IndexSource(pcg=pcg), noise_seed=0)
  idx = O.loader_draws(O.loader_rng(0), N, n, K)[:, None, :]
  xi = np.stack([O.philox_normals(0, 0, k, 0, d) for k in range(K)])[:, None, :]
  Ws, Us, _ = O.sgld_glm_trajectory(X, y, np.zeros((1, d), np.float32), idx,
                                    xi.astype(np.float32), h, T,
                                    O.LINEAR_GAUSSIAN, 0.5, 10.0)
  got = run.samples.cpu().numpy()[:, 0]
  ref = Ws[1:, 0]
  scale = np.sqrt(np.diag(O.linear_posterior(X, y, 0.5, 10.0)[1]))
  # Differences stay a small fraction of a posterior standard deviation.
  assert np.max(np.abs(got - ref) / scale) < 0.05


def test_other_presets_return_reference_format(lib):
  from gbsgmc import alias, data, likelihoods as L, potential
  X, y = linreg(N=2000, d=8, seed=5)
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = potential.minibatch_potential(L.GaussianPrior(10.0), L.LinearGaussian(sigma=0.5))
  sample = {"w": np.zeros(8, np.float32)}
  for preset, kw in ((alias.sghmc, dict(integration_steps=3, friction=1.0)),
                     (alias.obabo, dict(integration_steps=3, friction=1.0))):
    run = preset(pot, loader, cache_size=16, batch_size=32, first_step_size=1e-4,
                 last_step_size=1e-5, accepted_samples=10, **kw)
    res = run(sample, sample, iterations=40)
    assert len(res) == 2
    for r in res:
      assert r["sample_count"] == 10
      assert r["samples"]["variables"]["w"].shape == (10, 8)
      assert np.all(np.isfinite(r["samples"]["variables"]["w"]))
      assert r["samples"]["energy"].shape == (10,)
  run = alias.re_sgld(pot, loader, cache_size=16, batch_size=32, temperature=10.0,
                      first_step_size=1e-5, last_step_size=1e-6,
                      accepted_samples=10)
  res = run((sample, sample), iterations=40)
  assert res[0]["sample_count"] == 10
  assert np.all(np.isfinite(res[0]["samples"]["variables"]["w"]))


def test_bulk_initialisation_equals_one_by_one(lib, monkeypatch):
  """alias.sgld initialises many chains in bulk (one ChainGroup: stacked
  samples, RMSprop states and PCG64 words computed for all chains at once);
  its samples and advanced index streams must equal those of chains
  initialised one by one, bit for bit."""
  from gbsgmc import alias
  X, y = linreg(N=4000, d=16, seed=9)
  bulk = sgld_run(X, y, 120, chains=7, accepted=30, batch=64)
  monkeypatch.setattr(alias, "_init_states",
                      lambda solver_init, init, samples, **kw:
                      [init(s) for s in samples])
  single = sgld_run(X, y, 120, chains=7, accepted=30, batch=64)
  for a, b in zip(bulk, single):
    np.testing.assert_array_equal(a["samples"]["variables"]["w"],
                                  b["samples"]["variables"]["w"])
    np.testing.assert_array_equal(a["samples"]["likelihood"],
                                  b["samples"]["likelihood"])
