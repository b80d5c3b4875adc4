"""The classifier potential of the oracle against torch float64 autograd and
central finite differences (the reference differentiates its user
likelihood with jax.value_and_grad, integrator.py:166,593,792).

Tolerances: autograd 1e-9 relative; finite differences 1e-5 of max|g|.
"""

import numpy as np
import pytest

from oracle import sgmc_oracle as O


def problem(n, seed):
  rng = np.random.default_rng(seed)
  _, P = O.cnn_offsets()
  w = rng.normal(size=P) * 0.2
  images = rng.normal(size=(40, 32, 32, 3))
  labels = rng.integers(0, 10, size=40)
  idx = rng.integers(0, 40, size=n)
  return w, images, labels, idx


def torch_potential(w, images, labels, idx, n_obs, prior, T):
  torch = pytest.importorskip("torch")
  F = torch.nn.functional
  off, P = O.cnn_offsets()
  wt = torch.tensor(w, dtype=torch.float64, requires_grad=True)
  get = lambda k: wt[off[k][0]:off[k][1]]
  h = torch.tensor(images[idx], dtype=torch.float64).permute(0, 3, 1, 2)
  for l in range(3):
    ci, co = O.CNN_CHANNELS[l], O.CNN_CHANNELS[l + 1]
    k = get(f"W{l + 1}").reshape(3, 3, ci, co).permute(3, 2, 0, 1)
    h = F.max_pool2d(F.relu(F.conv2d(h, k, get(f"b{l + 1}"), padding=1)), 2)
  flat = h.permute(0, 2, 3, 1).reshape(len(idx), -1)
  logits = flat @ get("Wd").reshape(-1, 10) + get("bd")
  lk = -F.cross_entropy(logits, torch.tensor(labels[idx]), reduction="none")
  lp = torch.distributions.Normal(0.0, prior).log_prob(wt).sum()
  U = (-(n_obs / len(idx)) * lk.sum() - lp) / T
  U.backward()
  return U.item(), wt.grad.numpy(), lk.detach().numpy()


def test_cnn_oracle_matches_autograd():
  w, images, labels, idx = problem(6, 1)
  ref = O.cnn_potential(w, images, labels, idx, 500, prior_scale=2.0, temperature=1.3)
  U, g, lk = torch_potential(w, images, labels, idx, 500, 2.0, 1.3)
  np.testing.assert_allclose(ref.U[0], U, rtol=1e-9)
  np.testing.assert_allclose(ref.lk[0], lk, rtol=1e-9, atol=1e-12)
  np.testing.assert_allclose(ref.grad[0], g, rtol=1e-8, atol=1e-9 * np.abs(g).max())


def test_cnn_oracle_central_differences():
  w, images, labels, idx = problem(3, 2)
  ref = O.cnn_potential(w, images, labels, idx, 100, prior_scale=1.0)
  off, _ = O.cnn_offsets()
  rng = np.random.default_rng(3)
  picks = [int(rng.integers(a, b)) for a, b in off.values() for _ in range(3)]
  h = 1e-5
  for j in picks:
    e = np.zeros_like(w)
    e[j] = h
    fd = (O.cnn_potential(w + e, images, labels, idx, 100, prior_scale=1.0).U[0] -
          O.cnn_potential(w - e, images, labels, idx, 100, prior_scale=1.0).U[0]) / (2 * h)
    assert abs(fd - ref.grad[0, j]) <= 1e-5 * np.abs(ref.grad).max(), (j, fd, ref.grad[0, j])


def test_cnn_parameter_count():
  off, P = O.cnn_offsets()
  assert P == 113_738
  assert list(off) == ["b1", "W1", "b2", "W2", "b3", "W3", "bd", "Wd"]


def test_bf16_pooling_would_reroute_gradients():
  """Why the kernels keep the pre-pool ReLU outputs in fp32: rounding them to
  BF16 before the 2x2 max creates ties and moves the first layer's gradient
  by about 10 % on these inputs."""
  w, images, labels, idx = problem(16, 16)
  exact = O.cnn_potential(w, images, labels, idx, 500, prior_scale=1.0)
  rounded = O.cnn_potential(w, images, labels, idx, 500, prior_scale=1.0,
                            activations=O.round_bf16)
  off, _ = O.cnn_offsets()
  a, b = off["W1"]
  x, y = rounded.grad[0, a:b], exact.grad[0, a:b]
  assert np.linalg.norm(x - y) / np.linalg.norm(y) > 0.02
  np.testing.assert_allclose(rounded.U, exact.U, rtol=1e-3)


def test_round_bf16_is_round_to_nearest_even():
  x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.0e38])
  r = O.round_bf16(x)
  assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -7
  assert r[3] == -2.5 and np.isfinite(r[4])
