"""Many chains of OBABO / SGHMC / SGLD on the tanh network through one
network plan (gbsgmc_mlp_plan_create) against the per-chain step path.

Both paths draw the same numpy PCG64 index streams, the same Philox noise
(keyed by chain and step) and run the same kernels per chain (a chain's
GEMM tiles do not depend on the other chains in the batch), so the samples
agree bit for bit.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

D, H1, H2, N, n = 64, 256, 256, 3000, 128


def problem(seed=11):
  from gbsgmc import likelihoods as L
  rng = np.random.default_rng(seed)
  lik = L.MLPGaussian(d_in=D, h1=H1, h2=H2, sigma=0.1)
  X = rng.normal(size=(N, D)).astype(np.float32)
  y = (np.tanh(X[:, 0]) + 0.1 * rng.normal(size=N)).astype(np.float32)
  inits = [lik.init(np.random.default_rng(100 + c)) for c in range(3)]
  return lik, X, y, inits


def run(kind, fused, iterations=6, accepted=3):
  from gbsgmc import alias, data, engine, likelihoods as L, potential
  lik, X, y, inits = problem()
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), lik)
  common = dict(cache_size=64, batch_size=n, first_step_size=1e-6,
                last_step_size=1e-7, burn_in=0, accepted_samples=accepted)
  if kind == "obabo":
    r = alias.obabo(pot, loader, integration_steps=3, friction=10.0, **common)
  elif kind == "sghmc":
    r = alias.sghmc(pot, loader, integration_steps=2, friction=0.5, **common)
  else:
    r = alias.sgld(pot, loader, rms_prop=True, **common)
  engine.FUSED_ENABLED = fused
  try:
    return r(*[lik.unravel(w) for w in inits], iterations=iterations)
  finally:
    engine.FUSED_ENABLED = True


@pytest.mark.parametrize("kind", ["obabo", "sghmc", "sgld"])
def test_network_plan_equals_per_chain_steps(lib, kind):
  a = run(kind, fused=True)
  b = run(kind, fused=False)
  assert len(a) == len(b) == 3
  for ra, rb in zip(a, b):
    assert ra["sample_count"] == rb["sample_count"] == 3
    for leaf in ("W1", "W2", "W3", "b1", "b2", "b3"):
      va = np.asarray(ra["samples"]["variables"][leaf])
      vb = np.asarray(rb["samples"]["variables"][leaf])
      assert va.shape == vb.shape
      assert np.isfinite(va).all()
      np.testing.assert_array_equal(va, vb)


def test_network_plan_moves_chains_and_keeps_them_distinct(lib):
  a = run("obabo", fused=True, iterations=4, accepted=2)
  w0 = [np.asarray(r["samples"]["variables"]["W2"][-1]) for r in a]
  _, _, _, inits = problem()
  from gbsgmc import likelihoods as L
  lik = L.MLPGaussian(d_in=D, h1=H1, h2=H2, sigma=0.1)
  for c in range(3):
    start = lik.unravel(inits[c])["W2"]
    assert not np.array_equal(w0[c], start)
  assert not np.array_equal(w0[0], w0[1])


def test_kept_samples_through_a_device_ring_equal_the_full_buffer(lib, monkeypatch):
  """With host saving and more kept samples than the ring holds, the
  network plan keeps two device rows and a SampleDrain empties them to the
  host during the run; the samples equal those kept in a full buffer."""
  from gbsgmc import engine
  from gbsgmc.likelihoods import MLPGaussian
  full = run("obabo", fused=True, iterations=8, accepted=5)
  P = MLPGaussian(d_in=D, h1=H1, h2=H2, sigma=0.1).param_count
  monkeypatch.setattr(engine, "RING_BYTES", 2 * 3 * P * 4)
  ringed = run("obabo", fused=True, iterations=8, accepted=5)
  for a, b in zip(full, ringed):
    assert a["sample_count"] == b["sample_count"] == 5
    for leaf in ("W1", "W2", "b3"):
      np.testing.assert_array_equal(np.asarray(a["samples"]["variables"][leaf]),
                                    np.asarray(b["samples"]["variables"][leaf]))
    np.testing.assert_array_equal(a["samples"]["energy"], b["samples"]["energy"])


def test_moments_saving_streams_from_the_network_plan(lib, monkeypatch):
  """io.moments() on the network plan: each kept sample goes into the FP64
  sums as it is taken; the moments equal those of the saved samples."""
  from gbsgmc import io
  from oracle import sgmc_oracle as O
  saved = run("obabo", fused=True, iterations=8, accepted=5)
  monkeypatch.setattr(io, "save", lambda *args, **kwargs: io.moments())
  mom = run("obabo", fused=True, iterations=8, accepted=5)
  for a, b in zip(saved, mom):
    assert b["sample_count"] == 5
    for leaf in ("W2", "b1"):
      mean, var = O.sample_moments(np.asarray(a["samples"]["variables"][leaf]))
      np.testing.assert_allclose(b["moments"]["mean"][leaf], mean, rtol=1e-12,
                                 atol=1e-14)
      np.testing.assert_allclose(b["moments"]["variance"][leaf], var, rtol=1e-9,
                                 atol=1e-14)
