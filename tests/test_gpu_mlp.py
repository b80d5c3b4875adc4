"""The tanh-network potential (BF16 tcgen05 GEMMs, fp32 accumulation) vs the
FP64 oracle and a torch fp32 autograd reference, through the C ABI.

The inputs are the MLP regression workload's: X ~ N(0, 1), targets from a
random teacher network plus N(0, 0.1^2) noise, chains near the teacher.

Tolerances.  BF16 operands carry 8 significant bits, so the network output
is off by |d| <= t = 5e-3 max|out_ref| (measured: about 1e-3 of max|out|).
That moves lk_i by at most e_i = (|r_i| t + t^2 / 2) / sigma^2, r = y - out:
  lk            |lk_i - lk_ref_i| <= e_i, row by row
  U             |U - U_ref| <= (N/n sum_i m_i e_i) / T + 1e-6 |U_ref|
  var(lk)       5e-2 relative
The gradient inherits the relative error of the residuals r_i (sigma = 0.1
puts chains near the teacher at |r| ~ 0.1, where d / r is a few percent):
  each leaf     relative L2 error <= 6e-2 and cosine >= 0.998
(measured on these inputs: 1.2e-2 to 4.3e-2 and >= 0.99944).
"""

import numpy as np
import pytest

from oracle import sgmc_oracle as O

pytestmark = pytest.mark.gpu

SIGMA = 0.1


def teacher_data(lik, N, seed):
  rng = np.random.default_rng(seed)
  X = rng.normal(size=(N, lik.d_in)).astype(np.float32)
  w_star = lik.init(rng, scale=1.5)
  w_star[lik.param_count - 1] = 0.3
  f, _, _ = O.mlp_forward(w_star[None].astype(np.float64),
                          X[None].astype(np.float64), lik.d_in, lik.h1, lik.h2)
  y = (f[0] + SIGMA * rng.normal(size=N)).astype(np.float32)
  return X, y, w_star, rng


def chains_near(w_star, C, rng, spread=0.05):
  W = w_star[None] + spread * rng.normal(size=(C, w_star.size)) * \
      (np.abs(w_star[None]) + 0.02)
  return W.astype(np.float32)


def setup(D, H1, H2, N, C, n, seed, prior=1.0, T=1.0):
  import torch
  from gbsgmc import likelihoods as L, potential
  from gbsgmc.data import NumpyDataLoader
  lik = L.MLPGaussian(d_in=D, h1=H1, h2=H2, sigma=SIGMA)
  X, y, w_star, rng = teacher_data(lik, N, seed)
  W = chains_near(w_star, C, rng)
  idx = rng.integers(0, N, size=(C, n)).astype(np.int32)
  ds = NumpyDataLoader(x=X, y=y).device_dataset()
  pr = L.GaussianPrior(prior) if prior else L.FlatPrior()
  pot = potential.minibatch_potential(pr, lik, temperature=T)
  return lik, X, y, W, idx, ds, pot, torch.from_numpy(W).cuda(), \
      torch.from_numpy(idx).cuda()


def leaf_errors(lik, g, ref):
  out = {}
  for name in lik.shapes():
    a = lik.unravel(g)[name].reshape(g.shape[0], -1).astype(np.float64)
    b = lik.unravel(ref)[name].reshape(g.shape[0], -1)
    rel = np.linalg.norm(a - b, axis=1) / (np.linalg.norm(b, axis=1) + 1e-30)
    cos = np.sum(a * b, 1) / (np.linalg.norm(a, axis=1) * np.linalg.norm(b, axis=1) + 1e-30)
    out[name] = (rel.max(), cos.min())
  return out


def lk_bounds(lik, W, X, y, idx):
  out, _, _ = O.mlp_forward(W.astype(np.float64),
                            X[idx][..., :lik.d_in].astype(np.float64),
                            lik.d_in, lik.h1, lik.h2)
  res = np.abs(y[idx] - out)
  t = 5e-3 * np.abs(out).max()
  return (res * t + 0.5 * t * t) / SIGMA ** 2 + 1e-4


def check_grad(lik, g, ref_grad):
  errs = leaf_errors(lik, g, ref_grad)
  for name, (rel, cos) in errs.items():
    assert rel <= 6e-2 and cos >= 0.998, (name, rel, cos, errs)


def check(lik, r, ref, W, X, y, idx, n_obs, mask=None, T=1.0):
  e = lk_bounds(lik, W, X, y, idx)
  m = np.ones_like(e) if mask is None else mask
  U = r.U.cpu().numpy()
  u_tol = (n_obs / idx.shape[1]) * np.sum(m * e, 1) / T + 1e-6 * np.abs(ref.U)
  assert np.all(np.abs(U - ref.U) <= u_tol), (U, ref.U, u_tol)
  if r.lk is not None:
    lk = r.lk.cpu().numpy()
    assert np.all(np.abs(lk - ref.lk) <= e), np.max(np.abs(lk - ref.lk) / e)
  np.testing.assert_allclose(r.lk_var.cpu().numpy(), ref.var, rtol=5e-2)
  if r.grad is not None:
    check_grad(lik, r.grad.cpu().numpy(), ref.grad)


@pytest.mark.parametrize("shape", [(64, 256, 256, 2000, 3, 128),
                                   (128, 512, 256, 3000, 2, 256),
                                   (64, 256, 2304, 700, 1, 128),
                                   (64, 1024, 1024, 8192, 2, 2048)])
def test_mlp_matches_oracle(lib, shape):
  D, H1, H2, N, C, n = shape
  lik, X, y, W, idx, ds, pot, Wd, idxd = setup(D, H1, H2, N, C, n, seed=D + H1)
  r = pot.evaluate(Wd, idxd, ds, grad=True, lk=True, observation_count=N)
  pot.check_status()
  ref = O.mlp_potential(W, X, y, idx, N, D, H1, H2, SIGMA, prior_scale=1.0)
  check(lik, r, ref, W, X, y, idx, N)


def test_mlp_value_only_equals_value_of_gradient_call(lib):
  lik, X, y, W, idx, ds, pot, Wd, idxd = setup(64, 256, 512, 1000, 2, 256, 3)
  a = pot.evaluate(Wd, idxd, ds, grad=True, lk=True)
  b = pot.evaluate(Wd, idxd, ds, grad=False, lk=True)
  pot.check_status()
  assert b.grad is None
  assert np.array_equal(a.U.cpu().numpy(), b.U.cpu().numpy())
  assert np.array_equal(a.lk.cpu().numpy(), b.lk.cpu().numpy())


def test_mlp_mask_flat_prior_temperature(lib):
  import torch
  lik, X, y, W, idx, ds, pot, Wd, idxd = setup(64, 256, 256, 1500, 3, 384, 4,
                                               prior=None, T=2.5)
  mask = (np.random.default_rng(9).random(idx.shape) < 0.6).astype(np.float32)
  md = torch.from_numpy(mask).cuda()
  r = pot.evaluate(Wd, idxd, ds, mask=md, grad=True, lk=True,
                   observation_count=50_000)
  pot.check_status()
  ref = O.mlp_potential(W, X, y, idx, 50_000, 64, 256, 256, SIGMA,
                        prior_scale=0.0, temperature=2.5, mask=mask)
  check(lik, r, ref, W, X, y, idx, 50_000, mask=mask, T=2.5)


def test_mlp_matches_torch_fp32_autograd(lib):
  """The same potential in plain torch fp32 on the GPU, differentiated by
  autograd."""
  import torch
  lik, X, y, W, idx, ds, pot, Wd, idxd = setup(64, 1024, 1024, 6000, 2, 1024, 5)
  r = pot.evaluate(Wd, idxd, ds, grad=True, lk=True, observation_count=6000)
  pot.check_status()
  w = Wd.clone().requires_grad_(True)
  p = lik.unravel(w)
  Xb = torch.from_numpy(X).cuda()[idxd.long()]
  yb = torch.from_numpy(y).cuda()[idxd.long()]
  z1 = torch.tanh(Xb @ p["W1"] + p["b1"][:, None])
  z2 = torch.tanh(z1 @ p["W2"] + p["b2"][:, None])
  out = (z2 @ p["W3"])[..., 0] + p["b3"]
  lk = torch.distributions.Normal(out, SIGMA).log_prob(yb)
  lp = torch.distributions.Normal(0.0, 1.0).log_prob(w).sum(-1)
  U = -(6000 / idx.shape[1]) * lk.sum(-1) - lp
  U.sum().backward()
  Ut = U.detach().double().cpu().numpy()
  e = lk_bounds(lik, W, X, y, idx)
  u_tol = (6000 / idx.shape[1]) * e.sum(1) + 1e-5 * np.abs(Ut)
  assert np.all(np.abs(r.U.cpu().numpy() - Ut) <= u_tol)
  check_grad(lik, r.grad.cpu().numpy(), w.grad.double().cpu().numpy())


def test_mlp_index_out_of_range_sets_status(lib):
  import torch
  from gbsgmc import _lib
  lik, X, y, W, idx, ds, pot, Wd, idxd = setup(64, 256, 256, 500, 1, 128, 6)
  bad = idxd.clone()
  bad[0, 17] = 500
  pot.evaluate(Wd, bad, ds, grad=True)
  torch.cuda.synchronize()
  with pytest.raises(_lib.GbsgmcError):
    pot.check_status()


def test_mlp_full_potential_pads_ragged_chunks(lib):
  from gbsgmc import likelihoods as L, potential
  lik, X, y, W, idx, ds, pot, Wd, idxd = setup(64, 256, 256, 1000, 2, 128, 7)
  full = potential.full_potential(L.GaussianPrior(1.0), lik)
  full.CHUNK = 384
  U, g = full.value_and_grad_all(Wd, ds)
  ref = O.mlp_potential(W, X, y, np.tile(np.arange(1000), (2, 1)), 1000, 64,
                        256, 256, SIGMA, prior_scale=1.0)
  e = lk_bounds(lik, W, X, y, np.tile(np.arange(1000), (2, 1)))
  assert np.all(np.abs(U.cpu().numpy() - ref.U) <= e.sum(1) + 1e-6 * np.abs(ref.U))
  check_grad(lik, g.cpu().numpy(), ref.grad)


def test_mlp_rows_are_independent_and_deterministic(lib):
  """Each row's lk depends on that row alone: permuting the minibatch permutes
  lk bit for bit, and a repeated call gives identical bits."""
  import torch
  lik, X, y, W, idx, ds, pot, Wd, idxd = setup(64, 256, 256, 900, 2, 256, 8)
  a = pot.evaluate(Wd, idxd, ds, grad=True, lk=True)
  perm = torch.randperm(256, device="cuda")
  b = pot.evaluate(Wd, idxd[:, perm].contiguous(), ds, grad=True, lk=True)
  c = pot.evaluate(Wd, idxd, ds, grad=True, lk=True)
  pot.check_status()
  assert torch.equal(a.lk[:, perm], b.lk)
  assert torch.equal(a.U, c.U) and torch.equal(a.grad, c.grad)
