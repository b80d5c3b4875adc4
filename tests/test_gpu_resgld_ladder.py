"""The replica ladder with kept samples (gbsgmc_mlp_resgld_plan_create_keep)
and its reference-shaped entry point alias.re_sgld_ladder.

The kept sample of a step is replica 0's state after that step's exchange
attempt: a plan that keeps every step must hold, bit for bit, what the same
plan without a keep table leaves in replica 0 after each single step (the
plan is keyed by its device step counter, so stepping one at a time runs
the same arithmetic).
"""

import numpy as np
import pytest

import test_gpu_resgld_mlp as RM

pytestmark = pytest.mark.gpu


def _problem(R):
  from gbsgmc import likelihoods as L, potential
  from gbsgmc.data import NumpyDataLoader
  lik = L.MLPGaussian(d_in=64, h1=256, h2=256, sigma=0.1)
  rng = np.random.default_rng(32)
  N = 2000
  X = rng.normal(size=(N, 64)).astype(np.float32)
  y = (np.tanh(X[:, 1]) + 0.1 * rng.normal(size=N)).astype(np.float32)
  loader = NumpyDataLoader(x=X, y=y)
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), lik)
  W0 = np.stack([lik.init(np.random.default_rng(60 + r)) for r in range(R)])
  return lik, loader, pot, W0


def test_ladder_keeps_replica_zero_after_each_exchange(lib):
  import torch
  from gbsgmc import engine
  R, n_max, steps, every = 4, 256, 12, 1
  lik, loader, pot, W0 = _problem(R)
  ds = loader.device_dataset()
  rows = np.array([256, 200, 130, 64], np.int32)
  ladder = np.array([1.0, 4.0, 16.0, 64.0], np.float32)
  h = torch.full((steps,), 2e-6, dtype=torch.float32, device="cuda")
  t = torch.ones(steps, dtype=torch.float32, device="cuda")
  keep = torch.arange(steps, dtype=torch.int32, device="cuda")   # every step kept

  Xa = torch.from_numpy(W0).cuda()
  plan = engine.ResgldPlan(pot, ds, Xa, torch.ones_like(Xa), rows, n_max, ladder, h, t,
                           engine.IndexSource(pcg=RM.pcg_states(R)), noise_seed=9,
                           swap_seed=77, every=every, keep_tab=keep, n_kept=steps)
  plan.run(0, steps)
  plan.check_status()
  kept = plan.samples.cpu().numpy()
  kept_lik = plan.sample_lik.cpu().numpy()
  swaps = plan.counts.cpu().numpy()
  plan.close()

  Xb = torch.from_numpy(W0).cuda()
  planb = engine.ResgldPlan(pot, ds, Xb, torch.ones_like(Xb), rows, n_max, ladder, h, t,
                            engine.IndexSource(pcg=RM.pcg_states(R)), noise_seed=9,
                            swap_seed=77, every=every, block_steps=1)
  for k in range(steps):
    planb.run(k, 1)
    np.testing.assert_array_equal(kept[k], Xb[0].cpu().numpy())
    assert kept_lik[k] == -planb.U[0].item()
  planb.check_status()
  planb.close()
  assert np.isfinite(kept).all()
  assert swaps.sum() > 0, swaps


def test_alias_re_sgld_ladder_runs_in_the_reference_format(lib):
  from gbsgmc import alias
  R = 4
  lik, loader, pot, W0 = _problem(R)
  run = alias.re_sgld_ladder(pot, loader, temperatures=[1.0, 3.0, 9.0, 27.0],
                             batch_sizes=[128, 128, 96, 64], exchange_every=2,
                             first_step_size=2e-6, last_step_size=1e-6, burn_in=10,
                             accepted_samples=15, rms_prop=True, seed=5)
  out = run(lik.unravel(W0[0]), iterations=40)
  assert len(out) == 1 and out[0]["sample_count"] == 15
  for name, shp in lik.shapes().items():
    w = np.asarray(out[0]["samples"]["variables"][name])
    assert w.shape == (15,) + shp and np.isfinite(w).all()
  assert np.isfinite(np.asarray(out[0]["samples"]["likelihood"])).all()
  assert run.exchanges is not None and run.exchanges.sum() > 0
  with pytest.raises(ValueError):
    run(lik.unravel(W0[0]), iterations=41)       # not a multiple of exchange_every
  with pytest.raises(NotImplementedError):
    from gbsgmc import likelihoods as L, potential
    alias.re_sgld_ladder(potential.minibatch_potential(L.FlatPrior(), L.Logistic()),
                         loader, temperatures=[1.0, 2.0])
