"""AMAGOLD and SGGMC: the reversible-leapfrog and MH kernels against the
oracle, the integrator against the oracle trajectory, and the samplers'
distributions (the reference's tests/test_alias.py:166-201 on a 1-D
Gaussian, as a kernel-backed linear-Gaussian potential).

Tolerances: elementwise fp32 updates 1e-6 relative (+1e-6 absolute);
energies (fp64 sums of fp32 products) 1e-5 relative; MH decisions exact;
trajectories with GPU gradients (fp32) against fp64 ones 1e-4 relative.
"""

import numpy as np
import pytest

from oracle import sgmc_oracle as O

pytestmark = pytest.mark.gpu


def cuda(a, dtype=None):
  import torch
  t = torch.from_numpy(np.ascontiguousarray(a))
  return (t.to(dtype) if dtype is not None else t).cuda()


@pytest.mark.parametrize("with_mass", [False, True])
def test_leapfrog_kernels_match_oracle(lib, with_mass):
  import torch
  from gbsgmc import _lib
  rng = np.random.default_rng(3)
  C, P = 3, 1003
  x = rng.normal(size=(C, P)).astype(np.float32)
  p = rng.normal(size=(C, P)).astype(np.float32)
  g = rng.normal(size=(C, P)).astype(np.float32)
  xi = rng.normal(size=(C, P)).astype(np.float32)
  mass = rng.uniform(0.5, 2.0, size=P).astype(np.float32) if with_mass else None
  h, f = 0.01, 0.3
  sch = _lib.sched(step_size=h, offset=4)
  # Every device buffer stays bound to a name until its launch is enqueued
  # (a temporary would return its memory to the allocator first).
  xd, pd, gd, xid = cuda(x), cuda(p), cuda(g), cuda(xi)
  md = cuda(mass) if with_mass else None
  _lib.call("gbsgmc_leapfrog_position", C, P, _lib.ptr(xd), _lib.ptr(pd),
            _lib.ptr(md), 0.5, sch, None)
  want = O.leapfrog_position(x, p, h, 0.5, mass)
  np.testing.assert_allclose(xd.cpu().numpy(), want, rtol=1e-6, atol=1e-6)
  energy = torch.zeros(C, dtype=torch.float64, device="cuda")
  _lib.call("gbsgmc_amagold_momentum", C, P, _lib.ptr(pd), _lib.ptr(gd),
            _lib.ptr(md), f, _lib.ptr(energy), sch,
            _lib.noise(noise_dev=xid, noise_stride=P), None)
  for c in range(C):
    pn, e = O.amagold_momentum(p[c], g[c], xi[c], h, f, mass)
    np.testing.assert_allclose(pd[c].cpu().numpy(), pn, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(energy[c].item(), e, rtol=1e-5)
  # Production noise: Philox normals of tag GBSGMC_TAG_AMAGOLD at step 4.
  pd = cuda(p)
  _lib.call("gbsgmc_amagold_momentum", C, P, _lib.ptr(pd), _lib.ptr(gd),
            _lib.ptr(md), f, None, sch, _lib.noise(seed=77, chain_base=10), None)
  for c in range(C):
    xi_c = O.philox_normals(77, 10 + c, 4, _lib.TAG_AMAGOLD, P).astype(np.float32)
    pn, _ = O.amagold_momentum(p[c], g[c], xi_c, h, f, mass)
    np.testing.assert_allclose(pd[c].cpu().numpy(), pn, rtol=1e-5, atol=1e-5)


def test_mh_accept_and_select_match_oracle(lib):
  import torch
  from gbsgmc import _lib
  U_old = np.array([1.0, 2.0, -3.0, 5.0, 0.5, 1e3])
  U_new = np.array([1.5, 1.0, -2.0, 5.5, 0.5, 1e3 + 40])
  energy = np.array([0.2, -0.3, 0.9, 0.1, 0.0, 1.0])
  ke0 = np.array([0.1, 0.4, 1.0, 2.0, 0.0, 0.3])
  ke1 = np.array([0.3, 0.2, 0.5, 2.1, 0.0, 0.1])
  C = U_old.size
  T = 1.7
  u = np.array([0.5, 0.9, 0.1, 0.99, 0.3, 0.5])
  Uo, Un, En, K0, K1, Ud = (cuda(a) for a in (U_old, U_new, energy, ke0, ke1, u))
  for kind, name in ((_lib.MH_AMAGOLD, "amagold"), (_lib.MH_SGGMC, "sggmc")):
    for injected in (True, False):
      acc = torch.empty(C, dtype=torch.int32, device="cuda")
      ratio = torch.empty(C, dtype=torch.float64, device="cuda")
      keepU = torch.empty(C, dtype=torch.float64, device="cuda")
      sch = _lib.sched(temperature=T, offset=12)
      _lib.call("gbsgmc_mh_accept", C, kind, _lib.ptr(Uo), _lib.ptr(Un),
                _lib.ptr(En), _lib.ptr(K0), _lib.ptr(K1), sch,
                _lib.ptr(Ud) if injected else None, 99, 5, _lib.ptr(acc),
                _lib.ptr(ratio), _lib.ptr(keepU), None)
      for c in range(C):
        # The schedule carries the temperature as fp32.
        la = O.mh_log_alpha(name, U_old[c], U_new[c], energy[c], ke0[c], ke1[c],
                            float(np.float32(T)))
        uc = u[c] if injected else O.mh_uniform(99, 5 + c, 12)
        a = 1 if np.log(uc) < la else 0
        assert acc[c].item() == a, (name, injected, c)
        np.testing.assert_allclose(ratio[c].item(), np.exp(la), rtol=1e-14)
        assert keepU[c].item() == (U_new[c] if a else U_old[c])
  # Select: rejected chains return to (x_old, -p_old).
  rng = np.random.default_rng(0)
  P = 37
  x, xo, p, po = (rng.normal(size=(C, P)).astype(np.float32) for _ in range(4))
  accept = np.array([1, 0, 1, 0, 0, 1], np.int32)
  xd, pd, ad, xod, pod = cuda(x), cuda(p), cuda(accept), cuda(xo), cuda(po)
  _lib.call("gbsgmc_mh_select", C, P, _lib.ptr(ad), _lib.ptr(xd), _lib.ptr(xod),
            _lib.ptr(pd), _lib.ptr(pod), -1.0, None)
  for c in range(C):
    np.testing.assert_array_equal(xd[c].cpu().numpy(), x[c] if accept[c] else xo[c])
    np.testing.assert_array_equal(pd[c].cpu().numpy(), p[c] if accept[c] else -po[c])


def test_reversible_leapfrog_matches_oracle_trajectory(lib):
  """One integrate call on a linear-Gaussian potential with injected noise,
  against the oracle's trajectory fed the same minibatches (the loader's
  PCG64 stream) and fp64 gradients."""
  from gbsgmc import data, integrator, likelihoods as L, potential
  rng = np.random.default_rng(4)
  N, d, n, steps = 400, 6, 32, 5
  X = rng.normal(size=(N, d)).astype(np.float32)
  y = (X @ rng.normal(size=d) + 0.5 * rng.normal(size=N)).astype(np.float32)
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = potential.minibatch_potential(L.GaussianPrior(3.0), L.LinearGaussian(sigma=0.5))
  batch = data.random_reference_data(loader, 16, n)
  noises = {}

  def noise_source(step, chain, tag):
    key = (step, chain, tag)
    if key not in noises:
      noises[key] = np.random.default_rng(hash(key) % 2**32).normal(size=d).astype(
          np.float32)
    return noises[key]

  h, f = 0.002, 0.4
  integ = integrator.reversible_leapfrog(pot, batch, steps=steps, friction=f,
                                         noise_source=noise_source)
  w0 = (0.1 * rng.normal(size=d)).astype(np.float32)
  st = integ[0]({"w": w0}, key=5)
  p0 = st.momentum.cpu().numpy()
  np.testing.assert_array_equal(p0, noise_source(0, st.chain, 8))

  class Sched:
    step_size, temperature = np.float32(h), np.float32(1.0)

  out = integ[1](st, Sched())
  idx = O.loader_draws(O.loader_rng(st.chain), N, n, steps)

  def grad_fn(x, j):
    r = O.glm_potential(x[None], X, y, idx[j][None], N, O.LINEAR_GAUSSIAN, 0.5, 3.0)
    return r.grad[0].astype(np.float32)

  xis = [noise_source(j, st.chain, 7) for j in range(steps)]
  xw, pw, ew = O.reversible_leapfrog(w0, p0, grad_fn, xis, h, f)
  np.testing.assert_allclose(out.positions.cpu().numpy(), xw, rtol=1e-4, atol=1e-5)
  np.testing.assert_allclose(out.momentum.cpu().numpy(), pw, rtol=1e-4, atol=1e-4)
  np.testing.assert_allclose(out.potential.item(), ew, rtol=1e-3, atol=1e-6)
  assert out.step == steps


def _gaussian_1d(sigma=0.5):
  """U(w) = 0.5 (w / sigma)^2 + const: one observation x = 1, y = 0 of a
  linear-Gaussian likelihood with noise sigma and a flat prior."""
  from gbsgmc import data, likelihoods as L, potential
  loader = data.NumpyDataLoader(x=np.ones((1, 1), np.float32),
                                y=np.zeros(1, np.float32))
  lik = L.LinearGaussian(sigma=sigma)
  return (loader, potential.minibatch_potential(L.FlatPrior(), lik),
          potential.full_potential(L.FlatPrior(), lik))


@pytest.mark.parametrize("name", ["amagold", "sggmc"])
def test_mh_samplers_sample_the_gaussian(lib, name):
  """tests/test_alias.py:166-201 of the reference: 200 iterations, step size
  0.5 -> 0.1, burn-in 100 on a 1-D Gaussian (sd 0.5); here checked against
  the exact distribution (KS p > 0.01) with 400 kept samples."""
  from scipy import stats
  from gbsgmc import alias
  loader, pot, full = _gaussian_1d()
  make = alias.amagold if name == "amagold" else alias.sggmc
  run = make(pot, full, loader, cache_size=1, batch_size=1, first_step_size=0.5,
             last_step_size=0.1, burn_in=100)
  out = run({"w": np.array([0.3], np.float32)}, iterations=500)
  w = np.asarray(out[0]["samples"]["variables"]["w"]).reshape(-1)
  assert out[0]["sample_count"] == 400 and np.isfinite(w).all()
  res = stats.kstest(w, stats.norm(0.0, 0.5).cdf)
  assert res.pvalue > 0.01, res
  assert abs(np.std(w) - 0.5) < 0.1


def test_amagold_rejects_flip_momentum_and_adaptive_step_size_runs(lib):
  """A step size far too large makes AMAGOLD reject; the adaptive schedule
  (dual averaging on the acceptance ratio, scheduler.py:376-444) then shrinks
  the step size during burn-in."""
  from gbsgmc import alias
  loader, pot, full = _gaussian_1d()
  run = alias.amagold(pot, full, loader, cache_size=1, batch_size=1,
                      first_step_size=3.0, adaptive_step_size=True,
                      burn_in=60, target_acceptance_rate=0.6)
  out = run({"w": np.array([0.2], np.float32)}, iterations=120)
  w = np.asarray(out[0]["samples"]["variables"]["w"]).reshape(-1)
  assert np.isfinite(w).all() and w.size == 60
  assert np.std(w) > 0.05


@pytest.mark.parametrize("name", ["amagold", "sggmc"])
def test_batched_mh_chains_equal_per_chain_runs(lib, name, monkeypatch):
  """Several AMAGOLD / SGGMC chains run batched (engine.try_fused_mh: one
  [C, P] proposal, one full-data pass and one MH launch per iteration for
  all chains) give the per-chain path's samples bit for bit: the same index
  streams, noise and MH uniforms per chain, and (one CTA per chain, fixed
  row tiling) the same arithmetic per chain."""
  from gbsgmc import alias, data, engine, likelihoods as L, potential
  monkeypatch.setenv("GBSGMC_AUTOTUNE", "0")
  monkeypatch.setenv("GBSGMC_GLM_SLICES", "1")
  monkeypatch.setenv("GBSGMC_GLM_RW", "4")
  rng = np.random.default_rng(13)
  N, d, n, C = 700, 9, 32, 3
  X = rng.normal(size=(N, d)).astype(np.float32)
  y = (rng.random(N) < 1 / (1 + np.exp(-X @ rng.normal(size=d)))).astype(np.float32)
  pot = potential.minibatch_potential(L.GaussianPrior(2.0), L.Logistic())
  full = potential.full_potential(L.GaussianPrior(2.0), L.Logistic())
  inits = [{"w": (0.1 * rng.normal(size=d)).astype(np.float32)} for _ in range(C)]
  used = []
  real = engine.try_fused_mh

  def spy(*args, **kwargs):
    out = real(*args, **kwargs)
    used.append(out is not None)
    return out

  monkeypatch.setattr(engine, "try_fused_mh", spy)
  outs = []
  for fused in (True, False):
    loader = data.NumpyDataLoader(x=X, y=y)
    make = alias.amagold if name == "amagold" else alias.sggmc
    run = make(pot, full, loader, cache_size=16, batch_size=n, integration_steps=4,
               first_step_size=0.02, last_step_size=0.01, burn_in=5)
    engine.FUSED_ENABLED = fused
    try:
      outs.append(run(*inits, iterations=30))
    finally:
      engine.FUSED_ENABLED = True
  assert used == [True, False]
  for a, b in zip(*outs):
    assert a["sample_count"] == b["sample_count"] == 25
    wa = np.asarray(a["samples"]["variables"]["w"])
    wb = np.asarray(b["samples"]["variables"]["w"])
    assert np.isfinite(wa).all()
    np.testing.assert_array_equal(wa, wb)
    np.testing.assert_array_equal(np.asarray(a["samples"]["energy"]),
                                  np.asarray(b["samples"]["energy"]))
  # The chains moved and stayed distinct.
  w0 = np.asarray(outs[0][0]["samples"]["variables"]["w"])
  w1 = np.asarray(outs[0][1]["samples"]["variables"]["w"])
  assert not np.array_equal(w0, w1)
