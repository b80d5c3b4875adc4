"""Shuffled index streams (NumpyDataLoader shuffle=True, with and without
in_epochs, jax_sgmc/data/numpy_loader.py:391-460) in the fused many-chain
plans: the host loader draws each chain's permutations (numpy itself, so
the streams are numpy's), ``ShuffledFeed`` hands them to a plan with an
external index source block by block (``gbsgmc_plan_set_indices``), and the samples equal
the per-chain path's, which takes the same batches one call at a time: bit
for bit for OBABO and SGHMC (the same kernels run), and within 1e-4
relative for SGLD on a GLM (the fused step kernel rounds its update
differently from the per-chain gradient + update kernels, as with the
PCG64 streams).
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, D, n, CHAINS = 900, 10, 32, 3


def _run(kind, fused, iterations=60, accepted=20, cache=7, shuffle=True,
         in_epochs=False):
  from gbsgmc import adaption, alias, data, engine, integrator, io, solver
  from gbsgmc import likelihoods as L, potential
  rng = np.random.default_rng(3)
  X = rng.normal(size=(N, D)).astype(np.float32)
  y = (rng.random(N) < 1 / (1 + np.exp(-X @ rng.normal(size=D)))).astype(np.float32)
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), L.Logistic())
  rd = data.random_reference_data(loader, cache, n)
  if kind == "sgld":
    integ = integrator.langevin_diffusion(pot, rd, adaption=adaption.rms_prop())
  elif kind == "obabo":
    integ = integrator.obabo(pot, rd, 3, 1.0)
  else:
    integ = integrator.friction_leapfrog(pot, rd, 2, 0.5)
  s = solver.sgmc(integ)
  sched = alias._schedule(1e-3, 1e-4, 10, accepted, False)
  run = solver.mcmc(s, sched, saving=io.save())
  kw = {"shuffle": shuffle, "in_epochs": in_epochs} if in_epochs else {"shuffle": shuffle}
  states = [s[0]({"w": np.zeros(D, np.float32)}, batch_kwargs=kw)
            for _ in range(CHAINS)]
  engine.FUSED_ENABLED = fused
  try:
    return run(*states, iterations=iterations), loader
  finally:
    engine.FUSED_ENABLED = True


@pytest.mark.parametrize("in_epochs", [False, True])
@pytest.mark.parametrize("kind", ["sgld", "obabo", "sghmc"])
def test_fused_shuffled_streams_equal_per_chain_path(lib, kind, in_epochs, monkeypatch):
  from gbsgmc.data import core
  # One CTA per chain, a fixed row tiling and no autotuned shape (a plan's
  # autotuner stores its choice for later calls of the same shape): a
  # chain's GLM arithmetic then does not depend on how many chains share the
  # launch.
  monkeypatch.setenv("GBSGMC_AUTOTUNE", "0")
  monkeypatch.setenv("GBSGMC_GLM_SLICES", "1")
  monkeypatch.setenv("GBSGMC_GLM_RW", "4")
  calls = []
  orig = core.ShuffledFeed.next

  def spy(self, steps, out=None):
    calls.append(steps)
    return orig(self, steps, out)

  monkeypatch.setattr(core.ShuffledFeed, "next", spy)
  a, la = _run(kind, fused=True, in_epochs=in_epochs)
  fused_calls = len(calls)
  b, lb = _run(kind, fused=False, in_epochs=in_epochs)
  assert fused_calls > 1 and len(calls) == fused_calls   # only the fused run
  assert len(a) == len(b) == CHAINS
  for ra, rb in zip(a, b):
    assert ra["sample_count"] == rb["sample_count"] == 20
    wa = np.asarray(ra["samples"]["variables"]["w"])
    wb = np.asarray(rb["samples"]["variables"]["w"])
    assert np.isfinite(wa).all()
    if kind == "sgld":
      np.testing.assert_allclose(wa, wb, rtol=1e-4, atol=1e-5)
    else:
      np.testing.assert_array_equal(wa, wb)
  # The loaders' chains end where the per-chain calls leave them.
  for ca, cb in zip(la._chains, lb._chains):
    assert (ca["draws"], ca["remaining_samples"]) == (cb["draws"], cb["remaining_samples"])
    assert ca["in_epochs"] == in_epochs
    assert ca["rng"].bit_generator.state == cb["rng"].bit_generator.state
    np.testing.assert_array_equal(ca["random_indices"], cb["random_indices"])


def test_shuffled_streams_differ_from_replacement_draws_and_between_chains(lib):
  a, _ = _run("sgld", fused=True)
  b, _ = _run("sgld", fused=True, shuffle=False)
  wa = np.asarray(a[0]["samples"]["variables"]["w"])
  wb = np.asarray(b[0]["samples"]["variables"]["w"])
  assert not np.array_equal(wa, wb)
  assert not np.array_equal(wa, np.asarray(a[1]["samples"]["variables"]["w"]))


def test_set_indices_needs_an_external_source(lib):
  import torch
  from gbsgmc import _lib, data, engine, likelihoods as L, potential
  rng = np.random.default_rng(0)
  X = rng.normal(size=(N, D)).astype(np.float32)
  y = (rng.random(N) < 0.5).astype(np.float32)
  ds = data.NumpyDataLoader(x=X, y=y).device_dataset()
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), L.Logistic())
  W = torch.zeros((2, D), dtype=torch.float32, device="cuda")
  h = torch.full((8,), 1e-3, dtype=torch.float32, device="cuda")
  t = torch.ones(8, dtype=torch.float32, device="cuda")
  idx = torch.zeros((8, 2, n), dtype=torch.int32, device="cuda")
  own = engine.NetPlan(pot, ds, W, torch.zeros_like(W), n, "sghmc", h, t,
                       engine.IndexSource(seed=1), noise_seed=1, block_steps=4,
                       friction=0.5)
  with pytest.raises(_lib.GbsgmcError):
    _lib.call("gbsgmc_plan_set_indices", own.handle, _lib.ptr(idx), 4, None)
  own.close()
  ext = engine.NetPlan(pot, ds, W, torch.zeros_like(W), n, "sghmc", h, t,
                       engine.IndexSource(external=True), noise_seed=1,
                       block_steps=4, friction=0.5)
  with pytest.raises(_lib.GbsgmcError):
    _lib.call("gbsgmc_plan_set_indices", ext.handle, _lib.ptr(idx), 5, None)
  _lib.call("gbsgmc_plan_set_indices", ext.handle, _lib.ptr(idx), 4, None)
  ext.close()
