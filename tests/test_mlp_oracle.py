"""The tanh-network potential of the oracle against torch autograd (float64)
and central finite differences: the reference obtains this gradient with
jax.value_and_grad (jax_sgmc/integrator.py:166,593,792), so the oracle's
hand-written adjoint must be the exact derivative of its potential.

Tolerances: autograd 1e-9 relative; finite differences 1e-6 relative to
the largest gradient entry (step 1e-6, float64).
"""

import numpy as np
import pytest

from oracle import sgmc_oracle as O

SHAPES = [(3, 5, 4, 7, 2), (8, 16, 6, 33, 3)]


def problem(D, H1, H2, n, C, seed):
  rng = np.random.default_rng(seed)
  _, P = O.mlp_offsets(D, H1, H2)
  W = rng.normal(size=(C, P)) * 0.7
  X = rng.normal(size=(50, D))
  y = rng.normal(size=50)
  idx = rng.integers(0, 50, size=(C, n))
  mask = (rng.random((C, n)) < 0.8).astype(np.float64)
  return W, X, y, idx, mask


def torch_potential(W, X, y, idx, n_obs, D, H1, H2, sigma, prior, T, mask):
  torch = pytest.importorskip("torch")
  w = torch.tensor(W, dtype=torch.float64, requires_grad=True)
  W1, W2, W3, b1, b2, b3 = O.mlp_unravel(w, D, H1, H2)
  Xb = torch.tensor(np.asarray(X)[idx])
  yb = torch.tensor(np.asarray(y)[idx])
  out = (torch.tanh(torch.tanh(Xb @ W1 + b1[:, None]) @ W2 + b2[:, None])
         @ W3[..., None])[..., 0] + b3[:, None]
  lk = torch.distributions.Normal(out, sigma).log_prob(yb)
  m = torch.tensor(mask)
  n = idx.shape[-1]
  lp = torch.distributions.Normal(0.0, prior).log_prob(w).sum(-1)
  U = (-(n_obs / n) * (m * lk).sum(-1) - lp) / T
  U.sum().backward()
  return U.detach().numpy(), w.grad.numpy(), lk.detach().numpy()


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("masked", [False, True])
def test_mlp_oracle_matches_autograd(shape, masked):
  D, H1, H2, n, C = shape
  W, X, y, idx, mask = problem(D, H1, H2, n, C, seed=n)
  m = mask if masked else np.ones_like(mask)
  ref = O.mlp_potential(W, X, y, idx, 1000, D, H1, H2, 0.3, prior_scale=2.0,
                        temperature=1.7, mask=mask if masked else None)
  U, g, lk = torch_potential(W, X, y, idx, 1000, D, H1, H2, 0.3, 2.0, 1.7, m)
  np.testing.assert_allclose(ref.U, U, rtol=1e-9)
  np.testing.assert_allclose(ref.lk, lk, rtol=1e-9)
  np.testing.assert_allclose(ref.grad, g, rtol=1e-9, atol=1e-9 * np.abs(g).max())
  np.testing.assert_allclose(ref.var, np.var(lk, axis=-1), rtol=1e-9)


def test_mlp_oracle_central_differences():
  D, H1, H2, n, C = SHAPES[1]
  W, X, y, idx, _ = problem(D, H1, H2, n, 1, seed=5)
  args = (X, y, idx, 400, D, H1, H2, 0.5)
  ref = O.mlp_potential(W, *args, prior_scale=1.5, temperature=0.9)
  rng = np.random.default_rng(1)
  h = 1e-6
  for j in rng.choice(W.shape[1], size=40, replace=False):
    e = np.zeros_like(W)
    e[0, j] = h
    up = O.mlp_potential(W + e, *args, prior_scale=1.5, temperature=0.9).U[0]
    dn = O.mlp_potential(W - e, *args, prior_scale=1.5, temperature=0.9).U[0]
    fd = (up - dn) / (2 * h)
    assert abs(fd - ref.grad[0, j]) <= 1e-6 * np.abs(ref.grad).max(), (j, fd, ref.grad[0, j])


def test_mlp_offsets_follow_sorted_ravel():
  offs, P = O.mlp_offsets(64, 1024, 1024)
  assert P == 1_117_185
  assert offs == [0, 65536, 65536 + 1048576, 65536 + 1048576 + 1024,
                  65536 + 1048576 + 2048, 65536 + 1048576 + 3072]


@pytest.mark.parametrize("shape", SHAPES)
def test_mlp_fisher_oracle_matches_per_observation_gradients(shape):
  """mlp_fisher_sums and mlp_fisher_noise against per-observation gradients
  taken one row at a time from mlp_potential (n = 1, N = 1, no prior: the
  gradient is -d lk_i / d w), the reference's vmap over grad of
  likelihoods[i] (adaption.py:420-437) written as a loop."""
  D, H1, H2, n, C = shape
  W, X, y, idx, _ = problem(D, H1, H2, n, C, seed=11)
  sigma, N, h = 0.7, 500, 0.02
  S1, S2 = O.mlp_fisher_sums(W, X, y, idx, D, H1, H2, sigma)
  grad = O.mlp_potential(W, X, y, idx, N, D, H1, H2, sigma, prior_scale=2.0).grad
  rng = np.random.default_rng(3)
  friction = rng.uniform(0.5, 2.0, size=W.shape[1])
  cb, bs = O.mlp_fisher_noise(W, X, y, idx, grad, N, D, H1, H2, sigma, friction, h)
  for c in range(C):
    d = np.stack([-O.mlp_potential(W[c:c + 1], X, y, idx[c:c + 1, i:i + 1], 1, D, H1, H2,
                                   sigma).grad[0] for i in range(n)])
    np.testing.assert_allclose(S1[c], d.sum(0), rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(S2[c], (d ** 2).sum(0), rtol=1e-10, atol=1e-12)
    ssq = ((d - grad[c] / N) ** 2).sum(0)
    wcb, wbs = O.fisher_noise_from_ssq(ssq, n, friction, h)
    np.testing.assert_allclose(cb[c], wcb, rtol=1e-9)
    np.testing.assert_allclose(bs[c], wbs, rtol=1e-9, atol=1e-12)
