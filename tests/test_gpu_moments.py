"""Sample statistics on the device: FP64 posterior moments of kept samples
(``gbsgmc_moments_accumulate`` / ``_finalize``, ``io.moments()``) and the
diagonal mass adaption of the MH samplers (``gbsgmc_mass_adapt``,
``adaption.mass_matrix``, the reference's adaption.py:296-368).

Tolerances: moments against numpy's float64 two-pass mean and variance
1e-12 relative (+1e-14 absolute; the kernels' differences are exact and
only fp64 additions round); the mass adaption bit for bit (fp32 in the
reference's operation order on both sides); sampling checks by KS test.
"""

import numpy as np
import pytest

from oracle import sgmc_oracle as O

pytestmark = pytest.mark.gpu


def cuda(a):
  import torch
  return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_moments_kernels_match_numpy_in_chunks_and_strided(lib):
  import torch
  from gbsgmc import io
  rng = np.random.default_rng(5)
  K, C, P = 9, 4, 1001
  # Large common offsets and small spreads: the shifted sums must not lose
  # the variance to cancellation.
  base = rng.normal(size=(1, C, P)) * 100.0
  buf = (base + rng.normal(size=(K, C, P)) * 1e-2).astype(np.float32)
  dev = cuda(buf)
  m = io.DeviceMoments(C, P)
  m.add(dev[:3]).add(dev[3]).add(dev[4:])
  mean, var = m.finalize()
  want_mean, want_var = O.sample_moments(buf)
  np.testing.assert_allclose(mean.cpu().numpy(), want_mean, rtol=1e-12, atol=1e-14)
  np.testing.assert_allclose(var.cpu().numpy(), want_var, rtol=1e-10, atol=1e-14)
  # A chain slice of the buffer: slot stride C * P, chain stride P.
  sub = io.DeviceMoments(2, P).add(dev[:, 1:3])
  mean2, var2 = sub.finalize()
  wm, wv = O.sample_moments(buf[:, 1:3])
  np.testing.assert_allclose(mean2.cpu().numpy(), wm, rtol=1e-12, atol=1e-14)
  np.testing.assert_allclose(var2.cpu().numpy(), wv, rtol=1e-10, atol=1e-14)
  # One sample: zero variance, the sample as the mean.
  one = io.DeviceMoments(C, P).add(dev[0])
  m1, v1 = one.finalize()
  np.testing.assert_array_equal(m1.cpu().numpy(), buf[0].astype(np.float64))
  assert not v1.any()
  with pytest.raises(ValueError):
    io.DeviceMoments(C, P).finalize()
  with pytest.raises(ValueError):
    io.DeviceMoments(C, P + 1).add(dev)
  assert torch.cuda.is_available()


def test_mass_adapt_kernel_matches_oracle_bit_for_bit(lib):
  import torch
  from gbsgmc import _lib
  rng = np.random.default_rng(8)
  P, burn_in, iters = 1003, 5, 8
  xs = (rng.normal(size=(iters, P)) * rng.uniform(0.1, 3.0, size=P)).astype(np.float32)
  cov = rng.uniform(0.5, 2.0, size=P).astype(np.float32)
  st = O.mass_adapt_init(xs[0], cov)
  mean = torch.zeros(P, dtype=torch.float32, device="cuda")
  ssq = torch.zeros_like(mean)
  inv = cuda(st.inv)
  sq = cuda(st.sqrt)
  mass = cuda((1.0 / cov).astype(np.float32))
  mass0 = mass.cpu().numpy()
  ssq_at_burn_in = None
  for i in range(iters):
    x = cuda(xs[i])
    _lib.call("gbsgmc_mass_adapt", P, i + 1, burn_in, _lib.ptr(x), _lib.ptr(mean),
              _lib.ptr(ssq), _lib.ptr(inv), _lib.ptr(sq), _lib.ptr(mass), None)
    st = O.mass_adapt_update(st, xs[i], burn_in)
    np.testing.assert_array_equal(mean.cpu().numpy(), st.mean)
    np.testing.assert_array_equal(ssq.cpu().numpy(), st.ssq)
    np.testing.assert_array_equal(inv.cpu().numpy(), st.inv)
    np.testing.assert_array_equal(sq.cpu().numpy(), st.sqrt)
    if i + 1 < burn_in:
      np.testing.assert_array_equal(mass.cpu().numpy(), mass0)
    if i + 1 == burn_in:
      ssq_at_burn_in = st.ssq
  # The mass is set once, at burn-in; later updates move only mean and ssq.
  np.testing.assert_array_equal(mass.cpu().numpy(), np.float32(burn_in) / ssq_at_burn_in)


def _gaussian(sigmas):
  """U(w) = sum 0.5 (w_j / sigma_j)^2: one observation per coordinate of a
  linear-Gaussian likelihood with a flat prior (x_j = e_j / sigma_j, y = 0,
  noise sd 1)."""
  from gbsgmc import data, likelihoods as L, potential
  d = len(sigmas)
  X = np.diag(1.0 / np.asarray(sigmas, np.float64)).astype(np.float32)
  loader = data.NumpyDataLoader(x=X, y=np.zeros(d, np.float32))
  lik = L.LinearGaussian(sigma=1.0)
  return (loader, potential.minibatch_potential(L.FlatPrior(), lik),
          potential.full_potential(L.FlatPrior(), lik))


@pytest.mark.parametrize("name", ["amagold", "sggmc"])
def test_mh_solver_adapts_the_mass_on_kept_samples(lib, name):
  """The solver feeds each sample the MH correction keeps to the adaption
  (solver.py:409-412, :552-556); the state's inverse mass, root and mass
  equal the oracle's adaption over the recorded samples."""
  from gbsgmc import adaption, data, integrator, solver
  sigmas = [0.3, 1.0, 2.0]
  loader, pot, full = _gaussian(sigmas)
  rd = data.random_reference_data(loader, 4, 3)
  fm = data.full_reference_data(loader, 4, 3)
  burn_in = 12
  if name == "amagold":
    integ = integrator.reversible_leapfrog(pot, rd, 5, 0.25)
    s = solver.amagold(integ, full, fm, mass_adaption=adaption.mass_matrix(
        burn_in=burn_in))
  else:
    integ = integrator.obabo(pot, rd, 5, 1.0)
    s = solver.sggmc(integ, full, fm, mass_adaption=adaption.mass_matrix(
        burn_in=burn_in))
  init, update, _ = s
  st = init({"w": np.array([0.1, -0.2, 0.3], np.float32)}, key=3)

  class Sched:
    step_size, temperature = np.float32(0.1), np.float32(1.0)

  oracle = O.mass_adapt_init(np.zeros(3, np.float32))
  accepted, ssq_at_burn_in = 0, None
  for k in range(burn_in + 4):
    st, stats = update(st, Sched())
    accepted += stats["acceptance_ratio"].item() > 0
    x = st.integrator_state.positions.cpu().numpy()
    oracle = O.mass_adapt_update(oracle, x, burn_in)
    if k + 1 == burn_in:
      ssq_at_burn_in = oracle.ssq
  ms = st.mass_state
  assert ms.iteration == burn_in + 4
  np.testing.assert_array_equal(ms.mean.cpu().numpy(), oracle.mean)
  np.testing.assert_array_equal(ms.inv.cpu().numpy(), oracle.inv)
  np.testing.assert_array_equal(ms.sqrt.cpu().numpy(), oracle.sqrt)
  np.testing.assert_array_equal(ms.mass.cpu().numpy(),
                                np.float32(burn_in) / ssq_at_burn_in)
  # The adapted inverse mass is the per-coordinate sample variance, largest
  # for the widest coordinate.
  assert oracle.inv[2] > oracle.inv[0]
  assert accepted > 0


@pytest.mark.parametrize("name", ["amagold", "sggmc"])
def test_mh_samplers_with_adapted_mass_sample_the_gaussian(lib, name):
  """The reference's 1-D Gaussian check (tests/test_alias.py:166-201) with
  the diagonal mass adapted over the first 50 kept samples."""
  from scipy import stats
  from gbsgmc import adaption, alias, data, integrator, io, solver
  loader, pot, full = _gaussian([0.5])
  rd = data.random_reference_data(loader, 1, 1)
  fm = data.full_reference_data(loader, 1, 1)
  if name == "amagold":
    integ = integrator.reversible_leapfrog(pot, rd, 10, 0.25)
    s = solver.amagold(integ, full, fm, mass_adaption=adaption.mass_matrix(burn_in=50))
  else:
    integ = integrator.obabo(pot, rd, 10, 1.0)
    s = solver.sggmc(integ, full, fm, mass_adaption=adaption.mass_matrix(burn_in=50))
  sched = alias._mh_schedule(0.5, 0.1, False, 10, 0.75, 0.05, 0.25, 100, None, False)
  run = solver.mcmc(s, sched, saving=io.save())
  out = run(s[0]({"w": np.array([0.3], np.float32)}), iterations=500)
  w = np.asarray(out[0]["samples"]["variables"]["w"]).reshape(-1)
  assert w.size == 400 and np.isfinite(w).all()
  res = stats.kstest(w, stats.norm(0.0, 0.5).cdf)
  assert res.pvalue > 0.01, res


def _sgld_run(saving, chains=3, iterations=120):
  """Fused GLM SGLD of `chains` chains through solver.mcmc (fresh loader, so
  the chain ids and streams are the same for every call)."""
  from gbsgmc import adaption, alias, data, integrator, likelihoods as L, potential, solver
  rng = np.random.default_rng(21)
  N, d = 2000, 12
  X = rng.normal(size=(N, d)).astype(np.float32)
  y = (X @ rng.normal(size=d) + 0.5 * rng.normal(size=N)).astype(np.float32)
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = potential.minibatch_potential(L.GaussianPrior(10.0), L.LinearGaussian(sigma=0.5))
  rdata = data.random_reference_data(loader, 64, 32)
  integ = integrator.langevin_diffusion(pot, rdata, adaption=adaption.rms_prop())
  s = solver.sgmc(integ)
  sched = alias._schedule(0.05, 0.001, 20, 60, False)
  run = solver.mcmc(s, sched, saving=saving)
  states = [s[0]({"w": np.zeros(d, np.float32)}) for _ in range(chains)]
  return run(*states, iterations=iterations)


def test_moments_saving_equals_moments_of_the_saved_samples(lib):
  from gbsgmc import io
  full = _sgld_run(io.save())
  mom = _sgld_run(io.moments())
  assert len(full) == len(mom) == 3
  for a, b in zip(full, mom):
    assert a["sample_count"] == b["sample_count"] == 60
    w = np.asarray(a["samples"]["variables"]["w"])
    mean, var = O.sample_moments(w)
    np.testing.assert_allclose(b["moments"]["mean"]["w"], mean, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(b["moments"]["variance"]["w"], var, rtol=1e-10,
                               atol=1e-14)
    np.testing.assert_array_equal(b["samples"]["likelihood"],
                                  a["samples"]["likelihood"])
