"""Dense mass matrices of the MH samplers (mass_matrix(diagonal=False),
jax_sgmc/adaption.py:296-368, and the integrators' tensor_matmul with an
ndim-2 Tensor, jax_sgmc/util/tree_util.py:38-56): the dense integrator
kernels, the dense adaption and the solvers that use them, against the
oracle.

Tolerances: the kernels' row dot products (fp32, one warp per row) against
fp64 products 1e-5 relative + 1e-5 absolute; kinetic energies and AMAGOLD
energies (fp64 sums of fp32 terms) 1e-5 relative; the adaption's mean, ssq
and inverse mass bit for bit (fp32 in the reference's operation order); the
adapted root (an fp32 Jacobi eigendecomposition against fp64 LAPACK) 2e-4
of its largest entry.
"""

import numpy as np
import pytest

from oracle import sgmc_oracle as O

pytestmark = pytest.mark.gpu


def cuda(a, dtype=None):
  import torch
  t = torch.from_numpy(np.ascontiguousarray(a))
  return (t.to(dtype) if dtype is not None else t).cuda()


def _matrices(rng, P):
  """A symmetric positive definite inverse mass and an unsymmetric root (the
  kernels do not assume the reference's root to be symmetric)."""
  A = rng.normal(size=(P, P)) / np.sqrt(P)
  minv = (A @ A.T + 0.5 * np.eye(P)).astype(np.float32)
  msqrt = (np.eye(P) + 0.3 * rng.normal(size=(P, P)) / np.sqrt(P)).astype(np.float32)
  return minv, msqrt


def _close(got, want, tol=1e-5):
  np.testing.assert_allclose(got, want, rtol=tol, atol=tol)


@pytest.mark.parametrize("P", [1, 7, 100, 1003])
def test_dense_leapfrog_kernels_match_oracle(lib, P):
  import torch
  from gbsgmc import _lib
  rng = np.random.default_rng(P)
  C = 3
  x, p, g = (rng.normal(size=(C, P)).astype(np.float32) for _ in range(3))
  minv, msqrt = _matrices(rng, P)
  h, f, seed, base, k = 0.01, 0.3, 19, 4, 6
  sch = _lib.sched(step_size=h, offset=k)
  xd, pd, gd, mid, msd = cuda(x), cuda(p), cuda(g), cuda(minv), cuda(msqrt)
  _lib.call("gbsgmc_leapfrog_position_dense", C, P, _lib.ptr(xd), _lib.ptr(pd),
            _lib.ptr(mid), 0.5, sch, None)
  _close(xd.cpu().numpy(), O.dense_leapfrog_position(x, p, h, 0.5, minv))
  energy = torch.zeros(C, dtype=torch.float64, device="cuda")
  _lib.call("gbsgmc_amagold_momentum_dense", C, P, _lib.ptr(pd), _lib.ptr(gd),
            _lib.ptr(mid), _lib.ptr(msd), f, _lib.ptr(energy), sch,
            _lib.noise(seed=seed, chain_base=base), None)
  xi = np.stack([O.philox_normals(seed, base + c, k, _lib.TAG_AMAGOLD, P)
                 for c in range(C)]).astype(np.float32)
  pn, e = O.dense_amagold_momentum(p, g, xi, h, f, minv, msqrt)
  _close(pd.cpu().numpy(), pn)
  np.testing.assert_allclose(energy.cpu().numpy(), e, rtol=1e-5, atol=1e-7)
  y = torch.empty_like(xd)
  _lib.call("gbsgmc_dense_matvec", C, P, _lib.ptr(msd), _lib.ptr(gd), _lib.ptr(y), None)
  _close(y.cpu().numpy(), g.astype(np.float64) @ msqrt.T.astype(np.float64))


@pytest.mark.parametrize("P", [1, 9, 128, 517])
def test_dense_obabo_kernels_match_oracle(lib, P):
  import torch
  from gbsgmc import _lib
  rng = np.random.default_rng(100 + P)
  C = 2
  x, p, g1, g2 = (rng.normal(size=(C, P)).astype(np.float32) for _ in range(4))
  minv, msqrt = _matrices(rng, P)
  h, T, f, seed, k = 0.02, 0.8, 0.7, 23, 3
  sch = _lib.sched(step_size=h, temperature=T, offset=k)
  xd, pd, g1d, g2d, mid, msd = (cuda(a) for a in (x, p, g1, g2, minv, msqrt))
  ke0 = torch.zeros(C, dtype=torch.float64, device="cuda")
  ke1 = torch.zeros(C, dtype=torch.float64, device="cuda")
  _lib.call("gbsgmc_obabo_first_dense", C, P, _lib.ptr(xd), _lib.ptr(pd),
            _lib.ptr(g1d), _lib.ptr(mid), _lib.ptr(msd), f, _lib.ptr(ke0), sch,
            _lib.noise(seed=seed), None)
  xi1 = np.stack([O.philox_normals(seed, c, k, _lib.TAG_OBABO_1, P) for c in range(C)])
  xr, pr, kr0 = O.dense_obabo_first(x, p, g1, xi1.astype(np.float32), h, T, f,
                                    minv, msqrt)
  _close(xd.cpu().numpy(), xr)
  _close(pd.cpu().numpy(), pr)
  np.testing.assert_allclose(ke0.cpu().numpy(), kr0, rtol=1e-5)
  # The second half continues from the kernel's own momentum.
  p1 = pd.cpu().numpy()
  _lib.call("gbsgmc_obabo_second_dense", C, P, _lib.ptr(pd), _lib.ptr(g2d),
            _lib.ptr(mid), _lib.ptr(msd), f, _lib.ptr(ke1), sch,
            _lib.noise(seed=seed), None)
  xi2 = np.stack([O.philox_normals(seed, c, k, _lib.TAG_OBABO_2, P) for c in range(C)])
  pr2, kr1 = O.dense_obabo_second(p1, g2, xi2.astype(np.float32), h, T, f, minv, msqrt)
  _close(pd.cpu().numpy(), pr2)
  np.testing.assert_allclose(ke1.cpu().numpy(), kr1, rtol=1e-5)


def test_dense_kernels_reject_bad_arguments(lib):
  import torch
  from gbsgmc import _lib
  P = 4
  a = torch.zeros((2, P), dtype=torch.float32, device="cuda")
  m = torch.eye(P, dtype=torch.float32, device="cuda")
  sch = _lib.sched(step_size=0.1)
  with pytest.raises(_lib.GbsgmcError):   # injected noise
    _lib.call("gbsgmc_amagold_momentum_dense", 2, P, _lib.ptr(a), _lib.ptr(a),
              _lib.ptr(m), _lib.ptr(m), 0.1, None, sch,
              _lib.noise(noise_dev=a, noise_stride=P), None)
  with pytest.raises(_lib.GbsgmcError):   # no matrix
    _lib.call("gbsgmc_leapfrog_position_dense", 2, P, _lib.ptr(a), _lib.ptr(a),
              None, 1.0, sch, None)
  with pytest.raises(_lib.GbsgmcError):   # too many parameters to adapt
    big = torch.zeros(129, dtype=torch.float32, device="cuda")
    _lib.call("gbsgmc_mass_adapt_dense", 129, 1, 5, _lib.ptr(big), _lib.ptr(big),
              _lib.ptr(big), _lib.ptr(big), _lib.ptr(big), None, None, None)
  # No chains is a no-op.
  _lib.call("gbsgmc_dense_matvec", 0, P, _lib.ptr(m), _lib.ptr(a), _lib.ptr(a), None)


@pytest.mark.parametrize("P,burn_in", [(1, 4), (6, 30), (64, 200)])
def test_dense_mass_adaption_matches_oracle(lib, P, burn_in):
  """gbsgmc_mass_adapt_dense against the oracle's restatement: the running
  mean and ssq and the inverse mass bit for bit, the root V^T diag(sqrt w) V
  (adaption.py:314-317, eigenvalues distinct: more samples than parameters)
  within 2e-4 of its largest entry; the matrices change only at burn-in."""
  import torch
  from gbsgmc import _lib
  rng = np.random.default_rng(7 * P)
  iters = burn_in + 3
  scales = rng.uniform(0.2, 3.0, size=P)
  mix = np.eye(P) + 0.4 * rng.normal(size=(P, P)) / np.sqrt(P)
  xs = ((rng.normal(size=(iters, P)) * scales) @ mix.T).astype(np.float32)
  cov = rng.uniform(0.5, 2.0, size=P).astype(np.float32)
  st = O.dense_mass_adapt_init(xs[0], cov)
  mean = torch.zeros(P, dtype=torch.float32, device="cuda")
  ssq = torch.zeros((P, P), dtype=torch.float32, device="cuda")
  inv, sq = cuda(st.inv), cuda(st.sqrt)
  w = torch.zeros(P, dtype=torch.float32, device="cuda")
  V = torch.zeros((P, P), dtype=torch.float32, device="cuda")
  for i in range(iters):
    x = cuda(xs[i])
    _lib.call("gbsgmc_mass_adapt_dense", P, i + 1, burn_in, _lib.ptr(x),
              _lib.ptr(mean), _lib.ptr(ssq), _lib.ptr(inv), _lib.ptr(sq),
              _lib.ptr(w), _lib.ptr(V), None)
    st = O.dense_mass_adapt_update(st, xs[i], burn_in)
    np.testing.assert_array_equal(mean.cpu().numpy(), st.mean)
    np.testing.assert_array_equal(ssq.cpu().numpy(), st.ssq)
    np.testing.assert_array_equal(inv.cpu().numpy(), st.inv)
    if i + 1 < burn_in:
      np.testing.assert_array_equal(sq.cpu().numpy(), np.diag(1.0 / np.sqrt(cov)).astype(
          np.float32))
    else:
      got, want = sq.cpu().numpy(), st.sqrt
      assert np.max(np.abs(got - want)) <= 2e-4 * np.max(np.abs(want)), \
          np.max(np.abs(got - want))


def _gaussian(sigmas):
  """U(w) = sum 0.5 (w_j / sigma_j)^2: one observation per coordinate of a
  linear-Gaussian likelihood with a flat prior (x_j = e_j / sigma_j, y = 0,
  noise sd 1); a minibatch of all d observations gives the exact gradient
  w / sigma^2."""
  from gbsgmc import data, likelihoods as L, potential
  d = len(sigmas)
  X = np.diag(1.0 / np.asarray(sigmas, np.float64)).astype(np.float32)
  loader = data.NumpyDataLoader(x=X, y=np.zeros(d, np.float32))
  lik = L.LinearGaussian(sigma=1.0)
  return (loader, potential.minibatch_potential(L.FlatPrior(), lik),
          potential.full_potential(L.FlatPrior(), lik))


@pytest.mark.parametrize("name", ["reversible_leapfrog", "obabo"])
def test_dense_mass_integrators_match_oracle_trajectory(lib, name):
  """reversible_leapfrog and obabo integrate with a dense MassMatrix on a
  linear-Gaussian potential: the initial momentum M^1/2 xi and one integrate
  call against the oracle's dense restatement fed the loader's minibatches
  (its PCG64 stream), fp64 gradients and the library's Philox noise."""
  from gbsgmc import _lib, data, integrator, likelihoods as L, potential
  from gbsgmc.adaption import MassMatrix
  rng = np.random.default_rng(5)
  N, d, n, steps = 300, 5, 24, 4
  X = rng.normal(size=(N, d)).astype(np.float32)
  y = (X @ rng.normal(size=d) + 0.5 * rng.normal(size=N)).astype(np.float32)
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = potential.minibatch_potential(L.GaussianPrior(3.0), L.LinearGaussian(sigma=0.5))
  rd = data.random_reference_data(loader, 16, n)
  minv, msqrt = _matrices(rng, d)
  minv *= np.float32(0.05)
  mass = MassMatrix(cuda(minv), cuda(msqrt))
  w0 = (0.1 * rng.normal(size=d)).astype(np.float32)
  h, f = 0.01, 0.6

  class Sched:
    step_size, temperature = np.float32(h), np.float32(1.0)

  if name == "reversible_leapfrog":
    integ = integrator.reversible_leapfrog(pot, rd, steps=steps, friction=f)
    st = integ[0]({"w": w0}, key=11, mass=mass)
    xi0 = O.philox_normals(st.key, st.chain, 0, _lib.TAG_AMAGOLD_INIT, d)
    p0 = xi0.astype(np.float32).astype(np.float64) @ msqrt.T.astype(np.float64)
    _close(st.momentum.cpu().numpy(), p0)
    p0 = st.momentum.cpu().numpy()
    out = integ[1](st, Sched(), mass=mass)
    idx = O.loader_draws(O.loader_rng(st.chain), N, n, steps)
  else:
    integ = integrator.obabo(pot, rd, steps=steps, friction=f)
    st = integ[0]({"w": w0}, key=11)
    p0 = st.momentum.cpu().numpy()
    out = integ[1](st, Sched(), mass=mass)
    idx = O.loader_draws(O.loader_rng(st.chain), N, n, 2 * steps)

  def grad(x, j):
    r = O.glm_potential(np.asarray(x)[None], X, y, idx[j][None], N,
                        O.LINEAR_GAUSSIAN, 0.5, 3.0)
    return r.grad[0].astype(np.float32)

  def normals(j, tag):
    return O.philox_normals(st.key, st.chain, j, tag, d).astype(np.float32)

  if name == "reversible_leapfrog":
    x = O.dense_leapfrog_position(w0, p0, h, 0.5, minv)
    p, energy = p0.astype(np.float64), 0.0
    for j in range(steps):
      if j > 0:
        x = O.dense_leapfrog_position(x, p, h, 1.0, minv)
      p, e = O.dense_amagold_momentum(p, grad(x, j), normals(j, _lib.TAG_AMAGOLD), h, f,
                                      minv, msqrt)
      energy += e
    x = O.dense_leapfrog_position(x, p, h, 0.5, minv)
    np.testing.assert_allclose(out.potential.item(), energy, rtol=1e-4, atol=1e-6)
  else:
    x, p, k0, k1 = w0.astype(np.float64), p0.astype(np.float64), 0.0, 0.0
    for j in range(steps):
      x, p, ke = O.dense_obabo_first(x, p, grad(x, 2 * j), normals(j, _lib.TAG_OBABO_1),
                                     h, 1.0, f, minv, msqrt)
      k0 += ke
      p, ke = O.dense_obabo_second(p, grad(x, 2 * j + 1), normals(j, _lib.TAG_OBABO_2),
                                   h, 1.0, f, minv, msqrt)
      k1 += ke
    np.testing.assert_allclose(out.kinetic_energy_start.item(), k0, rtol=1e-4)
    np.testing.assert_allclose(out.kinetic_energy_end.item(), k1, rtol=1e-4)
  np.testing.assert_allclose(out.positions.cpu().numpy(), x, rtol=1e-4, atol=1e-5)
  np.testing.assert_allclose(out.momentum.cpu().numpy(), p, rtol=1e-4, atol=1e-4)
  assert out.step == steps


@pytest.mark.parametrize("name", ["amagold", "sggmc"])
def test_mh_solver_adapts_the_dense_mass_on_kept_samples(lib, name):
  """The solvers with mass_matrix(diagonal=False): each kept sample updates
  the dense adaption, whose state equals the oracle's over the recorded
  samples (mean, ssq and inverse mass bit for bit, the root to the
  eigensolver's tolerance); the integrator then runs with the adapted
  matrices (the chain stays finite and keeps accepting)."""
  from gbsgmc import adaption, data, integrator, solver
  sigmas = [0.3, 1.0, 2.0]
  loader, pot, full = _gaussian(sigmas)
  rd = data.random_reference_data(loader, 4, 3)
  fm = data.full_reference_data(loader, 4, 3)
  burn_in = 12
  strat = adaption.mass_matrix(diagonal=False, burn_in=burn_in)
  if name == "amagold":
    s = solver.amagold(integrator.reversible_leapfrog(pot, rd, 5, 0.25), full, fm,
                       mass_adaption=strat)
  else:
    s = solver.sggmc(integrator.obabo(pot, rd, 5, 1.0), full, fm, mass_adaption=strat)
  init, update, _ = s
  st = init({"w": np.array([0.1, -0.2, 0.3], np.float32)}, key=3)

  class Sched:
    step_size, temperature = np.float32(0.1), np.float32(1.0)

  oracle = O.dense_mass_adapt_init(np.zeros(3, np.float32))
  accepted = 0
  for _ in range(burn_in + 10):
    st, stats = update(st, Sched())
    accepted += stats["acceptance_ratio"].item() > 0
    oracle = O.dense_mass_adapt_update(oracle, st.integrator_state.positions.cpu().numpy(),
                                       burn_in)
  ms = st.mass_state
  assert ms.iteration == burn_in + 10
  np.testing.assert_array_equal(ms.mean.cpu().numpy(), oracle.mean)
  np.testing.assert_array_equal(ms.ssq.cpu().numpy(), oracle.ssq)
  np.testing.assert_array_equal(ms.inv.cpu().numpy(), oracle.inv)
  got = ms.sqrt.cpu().numpy()
  assert np.max(np.abs(got - oracle.sqrt)) <= 2e-4 * np.max(np.abs(oracle.sqrt))
  assert np.isfinite(st.integrator_state.positions.cpu().numpy()).all()
  assert accepted > 0


@pytest.mark.parametrize("name", ["amagold", "sggmc"])
def test_dense_and_diagonal_initial_mass_agree(lib, name):
  """Before burn-in the dense adaption's matrices are diag(init_cov) and
  diag(1 / sqrt(init_cov)): the dense kernels then sample what the diagonal
  ones do, up to fp32 rounding of M^-1 p (a product against 1 / m), so a
  short run's samples agree closely."""
  from gbsgmc import adaption, data, integrator, solver
  cov = np.array([0.25, 2.0], np.float32)
  runs = []
  for diagonal in (True, False):
    # A fresh loader per run: its pipelines then have the same chain ids.
    loader, pot, full = _gaussian([0.5, 1.5])
    rd = data.random_reference_data(loader, 4, 2)
    fm = data.full_reference_data(loader, 4, 2)
    strat = adaption.mass_matrix(diagonal=diagonal, burn_in=1000)
    if name == "amagold":
      s = solver.amagold(integrator.reversible_leapfrog(pot, rd, 3, 0.5), full, fm,
                         mass_adaption=strat)
    else:
      s = solver.sggmc(integrator.obabo(pot, rd, 3, 1.0), full, fm, mass_adaption=strat)
    init, update, _ = s
    st = init({"w": np.array([0.2, -0.4], np.float32)}, key=8,
              initial_mass={"w": cov})

    class Sched:
      step_size, temperature = np.float32(0.2), np.float32(1.0)

    xs = []
    for _ in range(8):
      st, _stats = update(st, Sched())
      xs.append(st.integrator_state.positions.cpu().numpy().copy())
    runs.append(np.stack(xs))
  np.testing.assert_allclose(runs[1], runs[0], rtol=1e-4, atol=1e-5)
