"""SGHMC's empirical-Fisher noise model (fisher_information(diagonal=True),
jax_sgmc/adaption.py:371-457) on the generalised-linear likelihoods:
``gbsgmc_glm_fisher_noise`` against the oracle's float64 restatement, the
noise-model momentum update, and alias.sghmc(adapt_noise_model=True).

Tolerances: the noise scales are fp32 sums over the minibatch against
float64 (1e-4 relative); the momentum update is elementwise fp32 (1e-6).
"""

import numpy as np
import pytest

from oracle import sgmc_oracle as O

pytestmark = pytest.mark.gpu

N, D, n = 500, 37, 64


def cuda(a):
  import torch
  return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _setup(family, seed):
  from gbsgmc import data, likelihoods as L, potential
  rng = np.random.default_rng(seed)
  X = rng.normal(size=(N, D)).astype(np.float32)
  w = (0.3 * rng.normal(size=D)).astype(np.float32)
  if family == O.LOGISTIC:
    lik, sigma = L.Logistic(), 1.0
    y = (rng.random(N) < 1 / (1 + np.exp(-X @ w))).astype(np.float32)
  elif family == O.LINEAR_GAUSSIAN:
    lik, sigma = L.LinearGaussian(sigma=0.5), 0.5
    y = (X @ w + 0.5 * rng.normal(size=N)).astype(np.float32)
  else:
    lik, sigma = L.Linear(), 1.0
    y = np.zeros(N, np.float32)
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), lik)
  ds = data.NumpyDataLoader(x=X, y=y).device_dataset()
  idx = rng.integers(0, N, size=n).astype(np.int32)
  grad = O.glm_potential(w[None], X, y, idx[None], N, family, sigma, 1.0).grad[0]
  return pot, ds, X, y, w, idx, grad.astype(np.float32), sigma, rng


@pytest.mark.parametrize("family", [O.LOGISTIC, O.LINEAR_GAUSSIAN, O.LINEAR])
@pytest.mark.parametrize("per_param", [False, True])
@pytest.mark.parametrize("regime", ["all_positive", "some_replaced"])
def test_fisher_noise_matches_oracle(lib, family, per_param, regime):
  import torch
  from gbsgmc import _lib
  pot, ds, X, y, w, idx, grad, sigma, rng = _setup(family, 7 + family)
  fric = rng.uniform(0.5, 1.5, size=D).astype(np.float32) if per_param else None
  f = 0.0 if per_param else 0.8
  friction = fric if per_param else f
  # b = 0.5 h v: a small step leaves every correction positive; a step at
  # the scale of the median variance replaces about half of them.
  v = O.fisher_variance(w, X, y, idx, grad, N, family, sigma)
  fb = np.broadcast_to(np.asarray(friction, np.float64), v.shape)
  if regime == "all_positive":
    h = 1e-4 / max(v.max(), 1e-12)
  else:
    base = 2.0 * np.median(fb) / max(np.median(v), 1e-12)
    for mult in (1.0, 0.93, 1.07, 0.87, 1.13, 0.8, 1.2):
      h = base * mult
      corr = fb - 0.5 * h * v
      # Both signs, and no correction close enough to 0 for fp32 rounding
      # to flip its sign.
      if ((corr <= 0).any() and (corr > 0).any()
          and np.min(np.abs(corr)) > 1e-4 * np.max(np.abs(corr))):
        break
    else:
      pytest.fail("no step size separates the corrections")
  want_cb, want_bs = O.fisher_noise(w, X, y, idx, grad, N, family, sigma, friction, h)
  m, keep = pot.model(ds, N)
  wd, gd, idd = cuda(w), cuda(grad), cuda(idx)
  fd = cuda(fric) if per_param else None
  cb = torch.empty(D, dtype=torch.float32, device="cuda")
  bs = torch.empty(D, dtype=torch.float32, device="cuda")
  status = torch.zeros(1, dtype=torch.int32, device="cuda")
  _lib.call("gbsgmc_glm_fisher_noise", m, 1, n, _lib.ptr(idd), n, _lib.ptr(wd),
            _lib.ptr(gd), _lib.ptr(fd), f, float(h), _lib.ptr(cb), _lib.ptr(bs),
            _lib.ptr(status), None)
  assert status.item() == 0
  np.testing.assert_allclose(cb.cpu().numpy(), want_cb, rtol=1e-4, atol=1e-6)
  np.testing.assert_allclose(bs.cpu().numpy(), want_bs, rtol=1e-3, atol=1e-5)
  del keep


def test_noise_model_momentum_matches_oracle(lib):
  import torch
  from gbsgmc import _lib
  rng = np.random.default_rng(2)
  C, P, h = 2, 1001, 0.01
  p, g, cb, xi = (rng.normal(size=(C, P)).astype(np.float32) for _ in range(4))
  cb = np.abs(cb)
  pd, gd, cbd, xid = cuda(p), cuda(g), cuda(cb), cuda(xi)
  _lib.call("gbsgmc_sghmc_momentum_noise_model", C, P, _lib.ptr(pd), _lib.ptr(gd),
            _lib.ptr(cbd), _lib.sched(step_size=h),
            _lib.noise(noise_dev=xid, noise_stride=P), None)
  hf = np.float32(h)
  want = (p + (-hf) * g) + np.float32(np.sqrt(np.float32(2) * hf)) * (cb * xi)
  np.testing.assert_allclose(pd.cpu().numpy(), want, rtol=1e-6, atol=1e-6)
  assert torch.cuda.is_available()


def test_sghmc_with_fisher_noise_model_samples_the_posterior(lib):
  """alias.sghmc(adapt_noise_model=True) on Bayesian linear regression: the
  chain mean approaches the closed-form posterior mean."""
  from gbsgmc import alias, data, likelihoods as L, potential
  rng = np.random.default_rng(11)
  Nn, d, sigma = 2000, 5, 0.5
  X = rng.normal(size=(Nn, d)).astype(np.float32)
  w_true = rng.normal(size=d)
  y = (X @ w_true + sigma * rng.normal(size=Nn)).astype(np.float32)
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = potential.minibatch_potential(L.GaussianPrior(10.0), L.LinearGaussian(sigma=sigma))
  run = alias.sghmc(pot, loader, cache_size=64, batch_size=64, integration_steps=5,
                    friction=5.0, first_step_size=1e-3, last_step_size=5e-4,
                    burn_in=200, accepted_samples=300, adapt_noise_model=True)
  out = run({"w": np.zeros(d, np.float32)}, iterations=600)
  wv = np.asarray(out[0]["samples"]["variables"]["w"])
  assert wv.shape == (300, d) and np.isfinite(wv).all()
  mu, cov = O.linear_posterior(X, y, sigma, 10.0)
  sd = np.sqrt(np.diag(cov))
  assert np.all(np.abs(wv.mean(0) - mu) < 10 * sd + 1e-3), (wv.mean(0), mu, sd)
