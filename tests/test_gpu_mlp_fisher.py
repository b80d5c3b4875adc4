"""The empirical-Fisher noise model on the MLP likelihood
(fisher_information(diagonal=True), jax_sgmc/adaption.py:371-457;
``gbsgmc_mlp_fisher_noise``) against the oracle's float64 restatement, and
alias.sghmc(adapt_noise_model=True) on the network.

Tolerances.  The sums of the per-observation gradients come from the BF16
adjoint GEMMs and the sums of their squares from GEMMs on the squared BF16
operands, so b = 0.5 h ssq / (n - 1) inherits the relative error of the
residuals that the network's gradient has (a few percent near the teacher,
see test_gpu_mlp.py): per leaf, b's relative L2 error <= 1.2e-1 and cosine
>= 0.99; cb_diff_sqrt^2 = friction - b elementwise to 2e-2 of friction.
The corrections' own rule (a replaced entry takes the chain's smallest
positive correction; cb^2 + b_sqrt^2 = friction) holds to fp32 rounding.
"""

import numpy as np
import pytest

from oracle import sgmc_oracle as O
import test_gpu_mlp as M

pytestmark = pytest.mark.gpu


def _fisher(lik, ds, pot, Wd, idxd, grad, friction_dev, friction, h):
  import torch
  from gbsgmc import _lib
  C, P = Wd.shape
  n = idxd.shape[1]
  m, keep = pot.model(ds)
  ws = pot.fisher_workspace(C, n, m)
  cb = torch.empty((C, P), dtype=torch.float32, device="cuda")
  bs = torch.empty_like(cb)
  gd = torch.from_numpy(np.ascontiguousarray(grad, np.float32)).cuda()
  _lib.call("gbsgmc_mlp_fisher_noise", m, C, n, _lib.ptr(idxd), n, _lib.ptr(Wd),
            _lib.ptr(gd), _lib.ptr(friction_dev), friction, h, _lib.ptr(cb), _lib.ptr(bs),
            _lib.ptr(ws), ws.numel(), _lib.ptr(pot.status()), None)
  pot.check_status()
  del keep
  return cb.cpu().numpy().astype(np.float64), bs.cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("shape", [(64, 256, 256, 2000, 2, 256),
                                   (128, 512, 256, 3000, 1, 384)])
@pytest.mark.parametrize("per_param", [False, True])
def test_mlp_fisher_noise_matches_oracle(lib, shape, per_param):
  import torch
  D, H1, H2, N, C, n = shape
  lik, X, y, W, idx, ds, pot, Wd, idxd = M.setup(D, H1, H2, N, C, n, seed=21)
  P = lik.param_count
  ref = O.mlp_potential(W, X, y, idx, N, D, H1, H2, M.SIGMA, prior_scale=1.0)
  rng = np.random.default_rng(5)
  fric = rng.uniform(0.5, 1.5, size=P).astype(np.float32) if per_param else None
  f = fric.astype(np.float64) if per_param else 1.0
  S1, S2 = O.mlp_fisher_sums(W, X, y, idx, D, H1, H2, M.SIGMA)
  gbar = ref.grad / N
  ssq = np.maximum(S2 - 2 * gbar * S1 + n * gbar ** 2, 0.0)
  # A step size that puts the largest b at half the friction.
  h = float(np.float32(0.5 * np.min(f) * (n - 1) / (0.5 * ssq.max())))
  fd = None if fric is None else torch.from_numpy(fric).cuda()
  cb, bs = _fisher(lik, ds, pot, Wd, idxd, ref.grad, fd, 1.0, h)
  wcb, wbs = O.mlp_fisher_noise(W, X, y, idx, ref.grad, N, D, H1, H2, M.SIGMA, f, h)
  assert np.isfinite(cb).all() and np.isfinite(bs).all()
  b, bref = bs ** 2, wbs ** 2
  for name in lik.shapes():
    a = lik.unravel(b)[name].reshape(C, -1)
    r = lik.unravel(bref)[name].reshape(C, -1)
    rel = np.linalg.norm(a - r, axis=1) / (np.linalg.norm(r, axis=1) + 1e-30)
    cos = np.sum(a * r, 1) / (np.linalg.norm(a, axis=1) * np.linalg.norm(r, axis=1) + 1e-30)
    assert rel.max() <= 1.2e-1 and cos.min() >= 0.99, (name, rel, cos)
  ff = np.broadcast_to(f, (C, P))
  assert np.all(np.abs(cb ** 2 - wcb ** 2) <= 2e-2 * ff)
  np.testing.assert_allclose(cb ** 2 + bs ** 2, ff, rtol=2e-6, atol=1e-6)


def test_mlp_fisher_noise_replaces_non_positive_corrections(lib):
  """With a step size that makes b exceed the friction for some parameters,
  those take the chain's smallest positive correction (adaption.py:439-442):
  the replaced entries all hold min(cb) and b_sqrt^2 = friction - cb^2."""
  D, H1, H2, N, C, n = 64, 256, 256, 2000, 2, 256
  lik, X, y, W, idx, ds, pot, Wd, idxd = M.setup(D, H1, H2, N, C, n, seed=22)
  ref = O.mlp_potential(W, X, y, idx, N, D, H1, H2, M.SIGMA, prior_scale=1.0)
  S1, S2 = O.mlp_fisher_sums(W, X, y, idx, D, H1, H2, M.SIGMA)
  gbar = ref.grad / N
  ssq = np.maximum(S2 - 2 * gbar * S1 + n * gbar ** 2, 0.0)
  f = 1.0
  h = float(np.float32(4.0 * f * (n - 1) / (0.5 * ssq.max())))
  cb, bs = _fisher(lik, ds, pot, Wd, idxd, ref.grad, None, f, h)
  wcb, _ = O.mlp_fisher_noise(W, X, y, idx, ref.grad, N, D, H1, H2, M.SIGMA, f, h)
  for c in range(C):
    b_ref = 0.5 * h * ssq[c] / (n - 1)
    clearly = b_ref > 1.3 * f           # replaced in any rounding
    assert clearly.any()
    np.testing.assert_allclose(cb[c][clearly], cb[c].min(), rtol=0, atol=0)
    np.testing.assert_allclose(cb[c].min(), wcb[c].min(), rtol=0.15)
    np.testing.assert_allclose(cb[c] ** 2 + bs[c] ** 2, f, rtol=2e-6)


def test_sghmc_with_mlp_fisher_noise_model_runs(lib):
  """alias.sghmc(adapt_noise_model=True) on the MLP regression: the noise
  model is evaluated every step on the device and the chain stays finite
  and moves towards lower potential than its start."""
  from gbsgmc import alias, data, likelihoods as L, potential
  lik = L.MLPGaussian(d_in=64, h1=256, h2=256, sigma=M.SIGMA)
  X, y, w_star, rng = M.teacher_data(lik, 2000, seed=23)
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), lik)
  run = alias.sghmc(pot, loader, cache_size=8, batch_size=128, integration_steps=3,
                    friction=10.0, first_step_size=2e-5, last_step_size=1e-5,
                    burn_in=10, accepted_samples=10, adapt_noise_model=True)
  w0 = M.chains_near(w_star, 1, rng, spread=0.3)[0]
  out = run(lik.unravel(w0), iterations=20)
  ws = np.stack([np.concatenate([np.asarray(out[0]["samples"]["variables"][k])[i].reshape(-1)
                                 for k in lik.shapes()]) for i in range(10)])
  assert np.isfinite(ws).all()
  full = O.mlp_potential(np.stack([w0, ws[-1]]).astype(np.float64), X, y,
                         np.tile(np.arange(2000), (2, 1)), 2000, 64, 256, 256, M.SIGMA,
                         prior_scale=1.0).U
  assert full[1] < full[0], full
