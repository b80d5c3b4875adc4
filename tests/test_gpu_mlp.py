"""The tanh-network potential (BF16 tcgen05 GEMMs, fp32 accumulation) vs the
FP64 oracle and a torch fp32 autograd reference, through the C ABI.

The inputs are the MLP regression workload's: X ~ N(0, 1), targets from a
random teacher network plus N(0, 0.1^2) noise, chains near the teacher.

Tolerances (BF16 operands carry 8 significant bits):
  U             |U - U_ref| <= 5e-3 |U_ref|
  lk            max |lk - lk_ref| <= 2e-2 max |lk_ref| + 1e-3
  var(lk)       2e-2 relative
  each leaf of the gradient: relative L2 error <= 3e-2 and cosine >= 0.999.
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


def check(lik, r, ref):
  U = r.U.cpu().numpy()
  assert np.all(np.abs(U - ref.U) <= 5e-3 * np.abs(ref.U)), (U, ref.U)
  if r.lk is not None:
    lk = r.lk.cpu().numpy()
    assert np.abs(lk - ref.lk).max() <= 2e-2 * np.abs(ref.lk).max() + 1e-3
  np.testing.assert_allclose(r.lk_var.cpu().numpy(), ref.var, rtol=2e-2)
  if r.grad is not None:
    errs = leaf_errors(lik, r.grad.cpu().numpy(), ref.grad)
    for name, (rel, cos) in errs.items():
      assert rel <= 3e-2 and cos >= 0.999, (name, rel, cos, errs)


@pytest.mark.parametrize("shape", [(64, 256, 256, 2000, 3, 128),
                                   (128, 512, 256, 3000, 2, 256),
                                   (64, 1024, 1024, 8192, 2, 2048)])
def test_mlp_matches_oracle(lib, shape):
  D, H1, H2, N, C, n = shape
  lik, X, y, W, idx, ds, pot, Wd, idxd = setup(D, H1, H2, N, C, n, seed=D + H1)
  r = pot.evaluate(Wd, idxd, ds, grad=True, lk=True, observation_count=N)
  pot.check_status()
  ref = O.mlp_potential(W, X, y, idx, N, D, H1, H2, SIGMA, prior_scale=1.0)
  check(lik, r, ref)


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
  check(lik, r, ref)


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
  assert np.all(np.abs(r.U.cpu().numpy() - Ut) <= 5e-3 * np.abs(Ut))
  errs = leaf_errors(lik, r.grad.cpu().numpy(), w.grad.double().cpu().numpy())
  for name, (rel, cos) in errs.items():
    assert rel <= 3e-2 and cos >= 0.999, (name, rel, cos, errs)


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
  assert np.all(np.abs(U.cpu().numpy() - ref.U) <= 5e-3 * np.abs(ref.U))
  errs = leaf_errors(lik, g.cpu().numpy(), ref.grad)
  for name, (rel, cos) in errs.items():
    assert rel <= 3e-2 and cos >= 0.999, (name, rel, cos)
