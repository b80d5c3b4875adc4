"""The dense empirical-Fisher noise model of SGHMC
(fisher_information(diagonal=False), jax_sgmc/adaption.py:441-452) and the
batched symmetric eigendecomposition it rests on, against the FP64 oracle
with the same eigenvector sign convention (LAPACK's is unspecified).

Tolerances (fp32 rotations, whose rounding grows with the order P):
eigenvalues within 5e-7 P of the largest |eigenvalue|; eigenvectors
(well-separated spectra) within 2e-4; reconstructions within 5e-7 P
relative; the noise vectors within 5e-4 relative (fp32 accumulation of the
d x d sums over the minibatch as well).
"""

import numpy as np
import pytest

from oracle import sgmc_oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("P", [1, 2, 3, 7, 32, 64, 127, 128])
def test_sym_eig_matches_oracle(lib, P):
  import torch
  from gbsgmc import _lib
  rng = np.random.default_rng(P)
  B = 5
  M = rng.normal(size=(B, P, P))
  A = (M + M.transpose(0, 2, 1)).astype(np.float32)
  Ad = torch.from_numpy(A).cuda()
  w = torch.empty((B, P), dtype=torch.float32, device="cuda")
  V = torch.empty((B, P, P), dtype=torch.float32, device="cuda")
  _lib.call("gbsgmc_sym_eig", B, P, _lib.ptr(Ad), _lib.ptr(w), _lib.ptr(V),
            _lib.stream_handle())
  torch.cuda.synchronize()
  w, V = w.cpu().numpy().astype(np.float64), V.cpu().numpy().astype(np.float64)
  for b in range(B):
    wr, Vr = O.sym_eig(A[b].astype(np.float64))
    scale = np.abs(wr).max()
    np.testing.assert_allclose(w[b], wr, atol=5e-7 * P * scale)
    rec = V[b] @ np.diag(w[b]) @ V[b].T
    assert np.linalg.norm(rec - A[b]) <= 5e-7 * P * np.linalg.norm(A[b])
    gaps = np.diff(wr)
    if P > 1 and gaps.min() > 1e-2 * scale:
      np.testing.assert_allclose(V[b], Vr, atol=2e-4)


def test_sym_eig_of_degenerate_and_zero_matrices(lib):
  import torch
  from gbsgmc import _lib
  A = np.stack([np.eye(6), np.zeros((6, 6)), np.diag([3.0, 1, 1, 1, 2, 2])]).astype(np.float32)
  Ad = torch.from_numpy(A).cuda()
  w = torch.empty((3, 6), dtype=torch.float32, device="cuda")
  V = torch.empty((3, 6, 6), dtype=torch.float32, device="cuda")
  _lib.call("gbsgmc_sym_eig", 3, 6, _lib.ptr(Ad), _lib.ptr(w), _lib.ptr(V),
            _lib.stream_handle())
  torch.cuda.synchronize()
  np.testing.assert_allclose(w.cpu().numpy(), [[1] * 6, [0] * 6, [1, 1, 1, 2, 2, 3]])
  for b in range(3):
    Vb = V[b].cpu().numpy()
    np.testing.assert_allclose(Vb.T @ Vb, np.eye(6), atol=1e-6)


@pytest.mark.parametrize("family,d", [(O.LOGISTIC, 4), (O.LOGISTIC, 12),
                                      (O.LINEAR_GAUSSIAN, 33), (O.LOGISTIC, 96)])
@pytest.mark.parametrize("vector_friction", [False, True])
def test_dense_fisher_noise_matches_oracle(lib, family, d, vector_friction):
  import torch
  from gbsgmc import _lib, data, likelihoods as L, potential
  rng = np.random.default_rng(d)
  N, C, n = 2000, 3, 4 * d + 40
  X = rng.normal(size=(N, d)).astype(np.float32)
  wt = rng.normal(size=d) / np.sqrt(d)
  if family == O.LOGISTIC:
    y = (rng.random(N) < 1 / (1 + np.exp(-X @ wt))).astype(np.float32)
    lik, sigma = L.Logistic(), 1.0
  else:
    y = (X @ wt + 0.5 * rng.normal(size=N)).astype(np.float32)
    lik, sigma = L.LinearGaussian(sigma=0.5), 0.5
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), lik)
  m, keep = pot.model(data.NumpyDataLoader(x=X, y=y).device_dataset())
  W = (0.3 * rng.normal(size=(C, d))).astype(np.float32)
  idx = rng.integers(0, N, (C, n)).astype(np.int32)
  G = np.stack([O.glm_potential(W[c:c + 1], X, y, idx[c:c + 1], N, family, sigma,
                                1.0).grad[0] for c in range(C)]).astype(np.float32)
  h = 1e-3
  fric = (0.5 + rng.random(d)).astype(np.float32) if vector_friction else None
  dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
  Wd, Gd, idxd = dev(W), dev(G), dev(idx)
  fd = dev(fric) if fric is not None else None
  cb = torch.empty((C, d), dtype=torch.float32, device="cuda")
  bs = torch.empty((C, d), dtype=torch.float32, device="cuda")
  status = torch.zeros(1, dtype=torch.int32, device="cuda")
  _lib.call("gbsgmc_glm_fisher_noise_dense", m, C, n, _lib.ptr(idxd), n, _lib.ptr(Wd),
            _lib.ptr(Gd), _lib.ptr(fd), 0.75, h, _lib.ptr(cb), _lib.ptr(bs),
            _lib.ptr(status), _lib.stream_handle())
  torch.cuda.synchronize()
  assert int(status.item()) == 0
  for c in range(C):
    f = fric.astype(np.float64) if fric is not None else 0.75
    cref, bref = O.fisher_noise_dense(W[c], X, y, idx[c], G[c].astype(np.float64), N,
                                      family, sigma, f, h)
    np.testing.assert_allclose(cb[c].cpu().numpy(), cref, rtol=5e-4,
                               atol=5e-4 * np.abs(cref).max())
    np.testing.assert_allclose(bs[c].cpu().numpy(), bref, rtol=5e-4,
                               atol=5e-4 * np.abs(bref).max())


def test_dense_fisher_rejects_large_models(lib):
  from gbsgmc import _lib
  m = _lib.Glm(_lib.GLM_LOGISTIC, 200, 1000, 200, 16, 16, 1.0, 1.0, 1.0, 0, 1000)
  rc = lib.gbsgmc_glm_fisher_noise_dense(m, 1, 64, 16, 64, 16, 16, None, 1.0, 1e-3,
                                         16, None, 16, None)
  assert rc == _lib.ERR_SHAPE and b"d <= 128" in lib.gbsgmc_last_error()


def test_alias_sghmc_with_dense_noise_model(lib):
  """The reference's alias.sghmc linear-regression test
  (tests/test_alias.py:356-378: adapt_noise_model=True,
  diagonal_noise=False, friction 0.5, five leapfrog steps) with the noise sd
  known (0.5) and steps small enough for that posterior (2e-3 -> 2e-4
  instead of 0.05 -> 0.001): the mean of the kept samples is within 5 % of
  the closed-form posterior mean."""
  from gbsgmc import alias, data, likelihoods as L, potential
  import test_gpu_alias_linreg as LR
  X, y, mu = LR._problem()
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = potential.minibatch_potential(L.FlatPrior(), L.LinearGaussian(sigma=0.5),
                                      strategy="vmap")
  res = alias.sghmc(pot, loader, cache_size=512, batch_size=10, integration_steps=5,
                    first_step_size=2e-3, last_step_size=2e-4, friction=0.5,
                    burn_in=5000, adapt_noise_model=True, diagonal_noise=False)(
                        {"w": np.zeros(4, np.float32)}, iterations=10000)
  LR._check(res, mu)
