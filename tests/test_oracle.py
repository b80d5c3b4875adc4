"""Pins the CPU oracle against the reference's own call sites, known-answer
tests and the golden fixtures (CPU only)."""

import itertools
import json
import math
from pathlib import Path

import numpy as np
import pytest

from oracle import sgmc_oracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"


def words_to_state(w):
  w = [int(x) for x in w]
  return {"bit_generator": "PCG64",
          "state": {"state": (w[0] << 64) | w[1], "inc": (w[2] << 64) | w[3]},
          "has_uint32": w[4], "uinteger": w[5]}


@pytest.fixture(scope="module")
def streams():
  return np.load(GOLDEN / "index_streams.npz")


@pytest.mark.parametrize("seed,N,n", itertools.product(range(8), (10_000, 1_000_000),
                                                       (128, 1024)))
def test_golden_streams_match_reference_loader(streams, seed, N, n):
  """The fixture is the reference loader's own draw (numpy_loader.py:382-389)."""
  key = f"s{seed}_N{N}_n{n}"
  rng = O.loader_rng(seed)
  np.testing.assert_array_equal(O.loader_draws(rng, N, n, 3), streams[key + "_idx"])


@pytest.mark.parametrize("seed,N,n", [(0, 10_000, 128), (3, 1_000_000, 1024),
                                      (7, 1_000_000, 128), (5, 10_000, 1024)])
def test_pcg64_restatement_matches_golden(streams, seed, N, n):
  key = f"s{seed}_N{N}_n{n}"
  before = words_to_state(streams[key + "_before"])
  idx, after = O.pcg64_bounded(before, N, 3 * n)
  np.testing.assert_array_equal(idx.reshape(3, n), streams[key + "_idx"])
  want = words_to_state(streams[key + "_after"])
  assert after["state"] == want["state"]
  assert after["has_uint32"] == want["has_uint32"]
  assert after["uinteger"] == want["uinteger"]


@pytest.mark.parametrize("N", [1, 2, 3, 10, 12345677, 2**31 - 1, 3 * 10**9])
def test_pcg64_restatement_edge_ranges(N):
  rng = O.loader_rng(11)
  st = rng.bit_generator.state
  want = rng.integers(0, N, 777, dtype=np.int64)
  got, new = O.pcg64_bounded(st, N, 777)
  np.testing.assert_array_equal(got, want)
  assert new["state"] == rng.bit_generator.state["state"]


def test_seeding_and_cache_size_order():
  """Same seed -> same draws (test_data.py:255-274); the cache size does not
  change the order (test_data.py:281-297): the stream is consecutive draws."""
  a = O.loader_draws(O.loader_rng(1), 50, 2, 5)
  b = O.loader_draws(O.loader_rng(1), 50, 2, 3)
  c = O.loader_draws(O.loader_rng(2), 50, 2, 3)
  np.testing.assert_array_equal(a[:3], b)
  assert not np.array_equal(b, c)


def test_philox_kat():
  for case in json.loads((GOLDEN / "philox_kat.json").read_text()):
    out = O.philox4x32_10(np.array([case["ctr"]], np.uint64), case["key"])[0]
    assert [int(x) for x in out] == case["out"]


def test_philox_normals_are_standard():
  z = O.philox_normals(1234, 3, 9, 0, 200_000)
  assert abs(z.mean()) < 0.01 and abs(z.std() - 1) < 0.01


def test_philox_indices_in_range():
  idx = O.philox_indices(7, 2, 5, 1001, 999_983)
  assert idx.min() >= 0 and idx.max() < 999_983 and idx.size == 1001


@pytest.mark.parametrize("case", json.loads((GOLDEN / "potential_kat.json").read_text()))
def test_linear_potential_closed_form(case):
  """tests/test_potential.py:66-92 restated: lk = sum(sample * x)."""
  obs, dim = case["obs"], case["dim"]
  X = np.tile(np.arange(4.0), (dim, 1))
  pot = O.glm_potential(np.ones(4), X, np.zeros(dim), np.arange(dim)[None],
                        obs, O.LINEAR)
  assert pot.U[0] == pytest.approx(case["U_flat_prior"], rel=1e-12)
  # the reference's prior sum(sample) = 4 enters as -4
  assert pot.U[0] - 4.0 == pytest.approx(case["U_sum_prior"], rel=1e-12)


@pytest.mark.parametrize("obs,dim", list(itertools.product([7, 11], [3, 5])))
def test_zero_potential(obs, dim):
  """tests/test_potential.py:95-122: zero likelihood gives exactly -0.0."""
  rng = np.random.default_rng(0)
  X = rng.exponential(size=(obs, dim))
  pot = O.glm_potential(np.zeros(dim), X, np.zeros(obs), np.arange(obs)[None],
                        obs, O.LINEAR)
  assert pot.U[0] == 0.0
  assert np.all(pot.grad == -1.0 * X.sum(0))  # -N/n * sum x_i


@pytest.mark.parametrize("family", [O.LINEAR_GAUSSIAN, O.LOGISTIC])
def test_gradient_finite_differences(family):
  rng = np.random.default_rng(5)
  X = rng.normal(size=(50, 6))
  y = rng.integers(0, 2, 50).astype(float) if family == O.LOGISTIC else rng.normal(size=50)
  w = rng.normal(size=(1, 6)) * 0.3
  idx = rng.integers(0, 50, (1, 20))
  pot = O.glm_potential(w, X, y, idx, 50, family, 0.7, 2.0, 1.3)
  eps = 1e-6
  for j in range(6):
    wp, wm = w.copy(), w.copy()
    wp[0, j] += eps
    wm[0, j] -= eps
    fd = (O.glm_potential(wp, X, y, idx, 50, family, 0.7, 2.0, 1.3).U[0]
          - O.glm_potential(wm, X, y, idx, 50, family, 0.7, 2.0, 1.3).U[0]) / (2 * eps)
    assert fd == pytest.approx(pot.grad[0, j], rel=1e-6, abs=1e-6)


@pytest.mark.parametrize("obs,dim,mb", list(itertools.product([7, 11], [3, 5], [2, 3])))
def test_full_equals_minibatch_over_all(obs, dim, mb):
  """tests/test_potential.py:299-333: full potential == minibatch potential
  over all observations."""
  rng = np.random.default_rng(obs * dim)
  X = rng.exponential(size=(obs, dim))
  y = rng.normal(size=obs)
  w = rng.normal(size=dim)
  mb_pot = O.glm_potential(w, X, y, np.arange(obs)[None], obs,
                           O.LINEAR_GAUSSIAN, 0.5, 3.0)
  U, g = O.full_potential(w, X, y, O.LINEAR_GAUSSIAN, 0.5, 3.0)
  assert U == pytest.approx(mb_pot.U[0], rel=1e-12)
  np.testing.assert_allclose(g, mb_pot.grad[0], rtol=1e-12)


def test_variance_matches_single_observation_evaluations():
  """tests/test_potential.py:336-367."""
  rng = np.random.default_rng(3)
  X = rng.normal(size=(9, 4))
  y = rng.normal(size=9)
  w = rng.normal(size=4)
  pot = O.glm_potential(w, X, y, np.arange(9)[None], 9, O.LINEAR_GAUSSIAN, 0.5)
  singles = [O.glm_potential(w, X, y, np.array([[i]]), 1, O.LINEAR_GAUSSIAN,
                             0.5).lk[0, 0] for i in range(9)]
  assert pot.var[0] == pytest.approx(np.var(singles), rel=1e-12)


@pytest.mark.parametrize("first,last,gamma,its",
                         itertools.product([1.0, 0.05], [0.01, 0.0009],
                                           [0.33, 0.55], [100, 14723]))
def test_step_size_first_last(first, last, gamma, its):
  """tests/test_scheduler.py:83-102 (rtol 1e-5)."""
  h = O.polynomial_first_last(first, last, gamma, its)
  assert h[0] == pytest.approx(first, rel=1e-5)
  assert h[-1] == pytest.approx(last, rel=1e-5)


def test_sgld_rmsprop_step_against_formula():
  rng = np.random.default_rng(0)
  x, g, xi = rng.normal(size=(3, 8)).astype(np.float32)
  v = np.ones(8, np.float32)
  x1, v1 = O.sgld_step(x, g, v, xi, 1e-3, 1.0, 0.9, 1e-5, True)
  v_ref = 0.9 * v + 0.1 * g * g
  G = 1 / (1e-5 + np.sqrt(v_ref))
  x_ref = x - 1e-3 * G * g + np.sqrt(G) * np.sqrt(2e-3) * xi
  np.testing.assert_allclose(v1, v_ref, rtol=1e-6)
  np.testing.assert_allclose(x1, x_ref, rtol=1e-5, atol=1e-6)


def test_swap_rule_follows_reference_cond():
  """solver.py:283-291: lax.cond(log_u < log_s, keep, exchange)."""
  sw, ssq, k, log_s = O.resgld_swap(10.0, 12.0, 0.5, 1.0, 10.0, 0.0, 0, 0.5)
  assert k == 1 and ssq == pytest.approx(0.5)
  assert log_s == pytest.approx(0.9 * (10.0 - 12.0 - 0.9 * 0.5))
  assert sw == (not (math.log(0.5) < log_s))


def test_linear_posterior_is_the_normal_equations():
  rng = np.random.default_rng(1)
  X = rng.normal(size=(200, 3))
  y = X @ np.array([1.0, -2.0, 0.5]) + 0.1 * rng.normal(size=200)
  mu, cov = O.linear_posterior(X, y, 0.1, 1e6)
  np.testing.assert_allclose(mu, np.linalg.lstsq(X, y, rcond=None)[0], rtol=1e-6)
  assert np.all(np.linalg.eigvalsh(cov) > 0)


def test_reversible_leapfrog_oracle_is_time_reversible():
  """With friction 0 (no noise) and a deterministic gradient, running the
  leapfrog back from (x', -p') returns to (x, -p) -- the property AMAGOLD's
  MH correction rests on (integrator.py:349-360) -- and the capped MH
  log-acceptances follow solver.py:381-383 / 518-524."""
  rng = np.random.default_rng(0)
  d, steps, h = 7, 12, 0.05
  A = rng.normal(size=(d, d))
  A = (A @ A.T / d + np.eye(d)).astype(np.float32)
  grad = lambda x, j: (A @ x).astype(np.float32)
  x0 = rng.normal(size=d).astype(np.float32)
  p0 = rng.normal(size=d).astype(np.float32)
  xis = [np.zeros(d, np.float32)] * steps
  x1, p1, _ = O.reversible_leapfrog(x0, p0, grad, xis, h, 0.0)
  x2, p2, _ = O.reversible_leapfrog(x1, -p1, grad, xis, h, 0.0)
  np.testing.assert_allclose(x2, x0, rtol=1e-4, atol=1e-5)
  np.testing.assert_allclose(-p2, p0, rtol=1e-4, atol=1e-5)
  assert O.mh_log_alpha("amagold", 1.0, 0.5, 0.1) == 0.0
  assert O.mh_log_alpha("amagold", 1.0, 2.0, 0.25) == -0.75
  assert np.isnan(O.mh_log_alpha("amagold", 1.0, np.nan, 0.0))
  assert O.mh_log_alpha("sggmc", 1.0, np.nan) == 0.0
  assert O.mh_log_alpha("sggmc", 1.0, 3.0, 0.0, 0.5, 1.0, 2.0) == -1.25
  u = O.mh_uniform(7, 3, 11)
  assert 0.0 < u < 1.0 and u != O.mh_uniform(7, 3, 12)


def test_mass_adaption_oracle_is_the_sample_variance():
  """mass_matrix(diagonal=True) (adaption.py:296-368): after burn_in
  updates the inverse mass is the population variance of the samples seen
  and its root's reciprocal sqrt(burn_in / ssq); before burn-in and after it
  the matrix does not move."""
  rng = np.random.default_rng(2)
  B, P = 40, 9
  xs = (rng.normal(size=(B + 5, P)) * rng.uniform(0.2, 4.0, size=P) + 3.0).astype(
      np.float32)
  st = O.mass_adapt_init(xs[0])
  for k in range(B + 5):
    st = O.mass_adapt_update(st, xs[k], B)
    if k + 1 < B:
      np.testing.assert_array_equal(st.inv, np.ones(P, np.float32))
    if k + 1 == B:
      at_burn_in = st
  assert st.iteration == B + 5
  np.testing.assert_array_equal(st.inv, at_burn_in.inv)
  np.testing.assert_allclose(at_burn_in.inv, xs[:B].astype(np.float64).var(axis=0),
                             rtol=1e-4)
  np.testing.assert_allclose(at_burn_in.sqrt, 1.0 / np.sqrt(at_burn_in.inv), rtol=1e-6)
  np.testing.assert_allclose(st.mean, xs.astype(np.float64).mean(axis=0), rtol=1e-5)


def test_sample_moments_oracle():
  a = np.arange(12, dtype=np.float32).reshape(4, 3)
  m, v = O.sample_moments(a)
  np.testing.assert_array_equal(m, [4.5, 5.5, 6.5])
  np.testing.assert_array_equal(v, [11.25, 11.25, 11.25])


@pytest.mark.parametrize("family", [O.LOGISTIC, O.LINEAR_GAUSSIAN, O.LINEAR])
def test_fisher_oracle_matches_finite_differences(family):
  """fisher_variance's per-observation gradients (lk'(z_i) x_i) against
  central differences of the per-observation log-likelihoods, and
  fisher_noise's replacement rule: corrections <= 0 take the smallest
  positive one (adaption.py:437-448)."""
  rng = np.random.default_rng(4)
  N, d, n = 50, 6, 12
  X = rng.normal(size=(N, d))
  y = (rng.random(N) < 0.5).astype(float) if family == O.LOGISTIC else rng.normal(size=N)
  w = 0.3 * rng.normal(size=d)
  idx = rng.integers(0, N, size=n)
  grad = rng.normal(size=d)
  sigma = 0.7
  eps = 1e-6
  per_obs = np.empty((n, d))
  for j in range(d):
    e = np.zeros(d)
    e[j] = eps
    lp, _ = O.glm_lk(family, X[idx] @ (w + e), y[idx], sigma)
    lm, _ = O.glm_lk(family, X[idx] @ (w - e), y[idx], sigma)
    per_obs[:, j] = (lp - lm) / (2 * eps)
  want = np.sum((per_obs - grad / N) ** 2, axis=0) / (n - 1)
  np.testing.assert_allclose(O.fisher_variance(w, X, y, idx, grad, N, family, sigma),
                             want, rtol=1e-6, atol=1e-9)
  v = O.fisher_variance(w, X, y, idx, grad, N, family, sigma)
  f = 1.0
  h = 2.0 * f / np.median(v)
  cb, bs = O.fisher_noise(w, X, y, idx, grad, N, family, sigma, f, h)
  corr = f - 0.5 * h * v
  smallest = corr[corr > 0].min()
  np.testing.assert_allclose(cb ** 2, np.where(corr <= 0, smallest, corr), rtol=1e-12)
  np.testing.assert_allclose(bs ** 2 + cb ** 2, f, rtol=1e-12)


@pytest.mark.parametrize("alpha,low,high", [(0.9, 0.07, 0.16), (0.999, -0.02, 0.03)])
def test_rms_prop_sgld_variance_excess_is_set_by_alpha(alpha, low, high):
  """The restated SGLD + rms_prop update (integrator.py:882-912 with
  adaption.py:254-291: v is updated with the current gradient before
  G = 1 / (lmbd + sqrt v) scales it) on a Gaussian potential whose
  stochastic gradient is g = A x + eps (A = 4e4, Var eps = 3.125e6: the
  config-1 linear regression at minibatch 128).  The larger a gradient,
  the more it raises v and the less of it moves x: the restoring drift is
  weaker than the noise scale assumes, and the stationary variance exceeds
  1 / A by about 11 % at alpha 0.9, whatever the step size, but by about
  1 % at alpha 0.999 -- the setting of the config-1 moment check."""
  A, S, h, C = 4e4, 3.125e6, 1e-5, 4000
  rng = np.random.default_rng(3)
  x = (rng.normal(size=C) / np.sqrt(A)).astype(np.float32)
  v = np.full(C, S, np.float32)
  acc = []
  for k in range(16000):
    g = (A * x + np.sqrt(S) * rng.normal(size=C)).astype(np.float32)
    x, v = O.sgld_step(x, g, v, rng.normal(size=C).astype(np.float32), 1e-5, 1.0,
                       alpha=alpha)
    if k >= 8000 and k % 50 == 0:
      acc.append(float(np.var(x.astype(np.float64))))
  excess = np.mean(acc) * A - 1.0
  assert low < excess < high, excess


def test_cpu_baseline_steps_compute_the_potential_and_variance():
  """The timed CPU loop computes, like update_fn every step
  (integrator.py:875-880), U and var(lk) at the pre-update position: they
  equal the FP64 restatement on the same draws (float32 likelihoods)."""
  rng = np.random.default_rng(4)
  N, d, C, n = 500, 6, 3, 16
  X = rng.normal(size=(N, d)).astype(np.float32)
  y = (rng.random(N) < 0.5).astype(np.float32)
  W = (0.1 * rng.normal(size=(C, d))).astype(np.float32)
  W0 = W.copy()
  V = np.ones_like(W)
  _, _, U, var = O.sgld_glm_cpu_steps(X, y, W, V, [O.loader_rng(c) for c in range(C)],
                                      (1, n), np.full(1, 1e-4), np.ones(1), O.LOGISTIC,
                                      prior_scale=1.0)
  idx = np.stack([O.loader_draws(O.loader_rng(c), N, n, 1)[0] for c in range(C)])
  ref = O.glm_potential(W0, X, y, idx, N, O.LOGISTIC, 1.0, 1.0)
  np.testing.assert_allclose(U, ref.U, rtol=1e-5)
  np.testing.assert_allclose(var, ref.var, rtol=1e-4)


def test_sym_eig_convention_and_dense_fisher_restatement():
  """The oracle's eigendecomposition reconstructs its input and follows the
  library's sign convention; with a scalar friction the dense noise model's
  two matrices share eigenvectors, and b_sqrt's singular values are b's
  eigenvalues."""
  rng = np.random.default_rng(8)
  M = rng.normal(size=(7, 7))
  A = M + M.T
  w, V = O.sym_eig(A)
  np.testing.assert_allclose(V @ np.diag(w) @ V.T, A, atol=1e-12)
  assert np.all(np.diff(w) >= 0)
  k = np.argmax(np.abs(V), axis=0)
  assert np.all(V[k, np.arange(7)] > 0)
  N, d, n = 400, 5, 32
  X = rng.normal(size=(N, d)).astype(np.float32)
  y = (rng.random(N) < 0.5).astype(np.float32)
  wv = 0.3 * rng.normal(size=d)
  idx = rng.integers(0, N, n)
  g = O.glm_potential(wv[None], X, y, idx[None], N, O.LOGISTIC, 1.0, 1.0).grad[0]
  cb, bs = O.fisher_noise_dense(wv, X, y, idx, g, N, O.LOGISTIC, 1.0, 2.0, 1e-2)
  Xb = X[idx].astype(np.float64)
  dz = y[idx] - 1 / (1 + np.exp(-(Xb @ wv)))
  D = dz[:, None] * Xb - g / N
  b = 0.5e-2 / (n - 1) * D.T @ D
  lam, U = O.sym_eig(b)
  np.testing.assert_allclose(bs, U @ np.sqrt(np.abs(lam)), rtol=1e-9)
  lam2, U2 = O.sym_eig(2.0 * np.eye(d) - b)
  np.testing.assert_allclose(np.sort(lam2), np.sort(2.0 - lam), rtol=1e-10)
  np.testing.assert_allclose(cb, U2 @ np.sqrt(np.abs(lam2)), rtol=1e-9)


def test_dense_mass_oracle_reduces_to_the_diagonal_one():
  """With diagonal matrices diag(1/m) and diag(sqrt m) the dense restatements
  are the diagonal ones; the dense adaption's mean, diagonal of ssq and
  inverse mass are the diagonal adaption's, and its root after burn-in is
  V^T diag(sqrt w) V of the sample covariance (for a diagonal covariance
  with distinct entries: diag(sqrt of the variances))."""
  rng = np.random.default_rng(0)
  P, C = 5, 2
  x, p, g, xi, xi2 = (rng.normal(size=(C, P)).astype(np.float32) for _ in range(5))
  m = rng.uniform(0.5, 2.0, size=P).astype(np.float32)
  minv = np.diag(1.0 / m.astype(np.float64))
  msq = np.diag(np.sqrt(m.astype(np.float64)))
  np.testing.assert_allclose(O.dense_leapfrog_position(x, p, 0.1, 0.5, minv),
                             O.leapfrog_position(x, p, 0.1, 0.5, m), rtol=1e-6)
  pn, e = O.dense_amagold_momentum(p, g, xi, 0.1, 0.3, minv, msq)
  for c in range(C):
    pw, ew = O.amagold_momentum(p[c], g[c], xi[c], 0.1, 0.3, m)
    np.testing.assert_allclose(pn[c], pw, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(e[c], ew, rtol=1e-5)
  xd, pd, k0 = O.dense_obabo_first(x, p, g, xi, 0.1, 0.9, 0.4, minv, msq)
  xw, pw, kw = O.obabo_first(x, p, g, xi, 0.1, 0.9, 0.4, m)
  np.testing.assert_allclose(xd, xw, rtol=1e-5, atol=1e-6)
  np.testing.assert_allclose(pd, pw, rtol=1e-5, atol=1e-6)
  np.testing.assert_allclose(k0, kw, rtol=1e-5)
  pd2, k1 = O.dense_obabo_second(pd, g, xi2, 0.1, 0.9, 0.4, minv, msq)
  pw2, kw1 = O.obabo_second(pw, g, xi2, 0.1, 0.9, 0.4, m)
  np.testing.assert_allclose(pd2, pw2, rtol=1e-5, atol=1e-6)
  np.testing.assert_allclose(k1, kw1, rtol=1e-5)
  # Adaption: samples with independent coordinates of distinct scales.
  xs = (rng.normal(size=(400, 3)) * np.array([0.5, 1.0, 2.0])).astype(np.float32)
  dn, dg = O.dense_mass_adapt_init(xs[0]), O.mass_adapt_init(xs[0])
  for s in xs:
    dn = O.dense_mass_adapt_update(dn, s, 400)
    dg = O.mass_adapt_update(dg, s, 400)
  np.testing.assert_array_equal(dn.mean, dg.mean)
  np.testing.assert_allclose(np.diag(dn.ssq), dg.ssq, rtol=1e-6)
  np.testing.assert_allclose(np.diag(dn.inv), dg.inv, rtol=1e-6)
  # The scales are in ascending order, so V is close to the identity and
  # the root close to diag(0.5, 1, 2).
  np.testing.assert_allclose(np.diag(dn.sqrt), [0.5, 1.0, 2.0], rtol=0.15)
  assert np.max(np.abs(dn.sqrt - np.diag(np.diag(dn.sqrt)))) < 0.2
