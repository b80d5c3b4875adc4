"""The GLM potential kernel vs the FP64 oracle and the reference's
known-answer tests (tests/test_potential.py), through the C ABI.

Tolerances: U within 1e-5 relative (+1e-3 absolute); gradients within 2e-4
of max|grad| per chain (fp32 accumulation over up to 4096 observations);
closed-form and zero cases exact.
"""

import itertools
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import sgmc_oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def make_data(N, d, family, seed=0):
  rng = np.random.default_rng(seed)
  X = rng.normal(size=(N, d)).astype(np.float32)
  if family == O.LOGISTIC:
    w = rng.normal(size=d) / np.sqrt(d)
    y = (rng.random(N) < 1 / (1 + np.exp(-(X @ w)))).astype(np.float32)
  else:
    y = (X @ rng.normal(size=d) + 0.5 * rng.normal(size=N)).astype(np.float32)
  return X, y


def potential_for(family, sigma=0.5, prior=3.0, temperature=1.0):
  from gbsgmc import likelihoods as L, potential
  lik = {O.LOGISTIC: L.Logistic(), O.LINEAR_GAUSSIAN: L.LinearGaussian(sigma=sigma),
         O.LINEAR: L.Linear()}[family]
  pr = L.GaussianPrior(prior) if prior else L.FlatPrior()
  return potential.minibatch_potential(pr, lik, temperature=temperature)


def dataset(X, y):
  from gbsgmc.data import NumpyDataLoader
  return NumpyDataLoader(x=X, y=y).device_dataset()


def check(pot_gpu, ref, rtol_g=2e-4):
  U = pot_gpu.U.cpu().numpy()
  np.testing.assert_allclose(U, ref.U, rtol=1e-5, atol=1e-3)
  if pot_gpu.grad is not None:
    g = pot_gpu.grad.cpu().numpy()
    scale = np.abs(ref.grad).max(axis=1, keepdims=True) + 1e-6
    assert np.all(np.abs(g - ref.grad) <= rtol_g * scale), \
        np.abs(g - ref.grad).max()
  np.testing.assert_allclose(pot_gpu.lk_var.cpu().numpy(), ref.var, rtol=1e-4,
                             atol=1e-4)


CASES = list(itertools.product([O.LINEAR_GAUSSIAN, O.LOGISTIC],
                               [1, 3, 5, 32, 256, 300],
                               [(1, 1), (3, 7), (2, 128), (4, 1024)]))


@pytest.mark.parametrize("family,d,cn", CASES)
def test_value_and_grad_matches_oracle(lib, family, d, cn):
  import torch
  C, n = cn
  N = 2000
  X, y = make_data(N, d, family, seed=d)
  ds = dataset(X, y)
  pot = potential_for(family, temperature=1.7)
  rng = np.random.default_rng(1)
  W = (rng.normal(size=(C, d)) / np.sqrt(d)).astype(np.float32)
  idx = rng.integers(0, N, (C, n)).astype(np.int32)
  r = pot.evaluate(torch.from_numpy(W).cuda(), torch.from_numpy(idx).cuda(), ds,
                   lk=True)
  ref = O.glm_potential(W, X, y, idx, N, family, 0.5, 3.0, 1.7)
  check(r, ref)
  np.testing.assert_allclose(r.lk.cpu().numpy(), ref.lk, rtol=1e-4, atol=1e-4)
  pot.check_status()


@pytest.mark.parametrize("C,n,d", [(256, 1024, 256), (64, 4096, 64), (7, 2048, 1024),
                                   (1, 128, 32), (300, 33, 8)])
def test_large_shapes_and_slices(lib, C, n, d):
  import torch
  N = 50_000
  X, y = make_data(N, d, O.LOGISTIC, seed=3)
  ds = dataset(X, y)
  pot = potential_for(O.LOGISTIC, prior=1.0)
  rng = np.random.default_rng(2)
  W = (rng.normal(size=(C, d)) / np.sqrt(d)).astype(np.float32)
  idx = rng.integers(0, N, (C, n)).astype(np.int32)
  r = pot.evaluate(torch.from_numpy(W).cuda(), torch.from_numpy(idx).cuda(), ds)
  ref = O.glm_potential(W, X, y, idx, N, O.LOGISTIC, 1.0, 1.0, 1.0)
  check(r, ref, rtol_g=3e-4)
  # Deterministic: a second launch gives bit-identical results.
  r2 = pot.evaluate(torch.from_numpy(W).cuda(), torch.from_numpy(idx).cuda(), ds)
  assert torch.equal(r.U, r2.U) and torch.equal(r.grad, r2.grad)


def test_masked_potential(lib):
  import torch
  N, d, C, n = 300, 12, 3, 50
  X, y = make_data(N, d, O.LINEAR_GAUSSIAN)
  ds = dataset(X, y)
  pot = potential_for(O.LINEAR_GAUSSIAN)
  rng = np.random.default_rng(4)
  W = rng.normal(size=(C, d)).astype(np.float32)
  idx = rng.integers(0, N, (C, n)).astype(np.int32)
  mask = (rng.random((C, n)) < 0.6).astype(np.float32)
  r = pot.evaluate(torch.from_numpy(W).cuda(), torch.from_numpy(idx).cuda(), ds,
                   mask=torch.from_numpy(mask).cuda())
  ref = O.glm_potential(W, X, y, idx, N, O.LINEAR_GAUSSIAN, 0.5, 3.0, 1.0,
                        mask=mask)
  check(r, ref)


@pytest.mark.parametrize("case", json.loads((GOLDEN / "potential_kat.json").read_text()))
def test_linear_potential_closed_form(lib, case):
  """tests/test_potential.py:66-92 on the GPU: U = -6 * obs exactly."""
  import torch
  from gbsgmc import data, likelihoods as L, potential
  obs, dim = case["obs"], case["dim"]
  X = np.tile(np.arange(4.0), (dim, 1)).astype(np.float32)
  loader = data.NumpyDataLoader(x=X)
  pot = potential.minibatch_potential(L.FlatPrior(), L.Linear())
  batch = data.IndexedBatch(loader.device_dataset(),
                            torch.arange(dim, dtype=torch.int32, device="cuda"))
  info = data.MiniBatchInformation(observation_count=obs, batch_size=dim,
                                   mask=None)
  for strategy in ("map", "vmap"):
    pot.strategy = strategy
    U, _ = pot(np.ones(4, np.float32), (batch, info))
    assert float(U) == case["U_flat_prior"]


@pytest.mark.parametrize("obs,dim", list(itertools.product([7, 11], [3, 5])))
def test_zero_potential_and_gradient(lib, obs, dim):
  """tests/test_potential.py:95-122 and 221-263: zero likelihood."""
  import torch
  from gbsgmc import data, likelihoods as L, potential
  rng = np.random.default_rng(0)
  X = rng.exponential(size=(obs, dim)).astype(np.float32)
  loader = data.NumpyDataLoader(x=X)
  pot = potential.minibatch_potential(L.FlatPrior(), L.Linear())
  batch = data.IndexedBatch(loader.device_dataset(),
                            torch.arange(obs, dtype=torch.int32, device="cuda"))
  info = data.MiniBatchInformation(observation_count=obs, batch_size=obs, mask=None)
  (U, _), g = pot.value_and_grad(np.zeros(dim, np.float32), (batch, info))
  assert float(U) == 0.0
  np.testing.assert_allclose(g.cpu().numpy(), -X.sum(0), rtol=1e-6)


def test_full_potential_equals_minibatch_over_all(lib):
  """tests/test_potential.py:299-333."""
  import torch
  from gbsgmc import data, likelihoods as L, potential
  N, d = 70_000, 16
  X, y = make_data(N, d, O.LINEAR_GAUSSIAN)
  loader = data.NumpyDataLoader(x=X, y=y)
  full = potential.full_potential(L.GaussianPrior(2.0), L.LinearGaussian(sigma=0.5))
  fmap = data.full_reference_data(loader, 2, 3)
  w = np.random.default_rng(0).normal(size=d).astype(np.float32) * 0.1
  U, _ = full(w, fmap[0](), fmap[1])
  U_ref, _ = O.full_potential(w, X, y, O.LINEAR_GAUSSIAN, 0.5, 2.0)
  assert float(U) == pytest.approx(U_ref, rel=2e-6)


def test_torch_autograd_twin_and_finite_differences(lib):
  import torch
  from gbsgmc import data, likelihoods as L, potential
  N, d = 500, 6
  X, y = make_data(N, d, O.LOGISTIC)
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), L.Logistic())
  batch = data.IndexedBatch(loader.device_dataset(),
                            torch.arange(0, N, 5, dtype=torch.int32, device="cuda"))
  info = data.MiniBatchInformation(observation_count=N, batch_size=100, mask=None)
  f = pot.torch_function((batch, info))
  w = torch.full((d,), 0.1, dtype=torch.float32, device="cuda", requires_grad=True)
  U = f(w)
  U.backward()
  wd = w.detach().double().cpu().numpy()
  idx = np.arange(0, N, 5)[None]
  eps = 1e-5
  for j in range(d):
    wp, wm = wd.copy(), wd.copy()
    wp[j] += eps
    wm[j] -= eps
    fd = (O.glm_potential(wp, X, y, idx, N, O.LOGISTIC, 1, 1.0).U[0]
          - O.glm_potential(wm, X, y, idx, N, O.LOGISTIC, 1, 1.0).U[0]) / (2 * eps)
    assert float(w.grad[j]) == pytest.approx(fd, rel=1e-3, abs=1e-3)


def test_out_of_range_index_sets_status(lib):
  import torch
  from gbsgmc import _lib
  N, d = 100, 8
  X, y = make_data(N, d, O.LOGISTIC)
  ds = dataset(X, y)
  pot = potential_for(O.LOGISTIC)
  W = torch.zeros((1, d), dtype=torch.float32, device="cuda")
  idx = torch.tensor([[0, 5, N + 3, 7]], dtype=torch.int32, device="cuda")
  pot.evaluate(W, idx, ds)
  with pytest.raises(_lib.GbsgmcError) as e:
    pot.check_status()
  assert e.value.code == _lib.ERR_INDEX
  # The status word was cleared and the context is still usable.
  idx = torch.tensor([[0, 5, 9, 7]], dtype=torch.int32, device="cuda")
  pot.evaluate(W, idx, ds)
  pot.check_status()




@pytest.mark.parametrize("d,ld,inline", [(6, 6, 0), (8, 8, 0), (5, 6, 1), (7, 12, 1),
                                         (256, 256, 0)])
def test_row_layouts_through_the_abi(lib, d, ld, inline):
  """Targets in a separate array or inline at column d; row strides that do
  (bulk copies) or do not (plain loads) allow 16-byte aligned rows."""
  import torch
  from gbsgmc import _lib
  N, C, n = 3000, 3, 200
  X, y = make_data(N, d, O.LOGISTIC, seed=d + ld)
  Xd = torch.zeros((N, ld), dtype=torch.float32, device="cuda")
  Xd[:, :d] = torch.from_numpy(X).cuda()
  yd = torch.from_numpy(y).cuda()
  if inline:
    Xd[:, d] = yd
  m = _lib.Glm(_lib.GLM_LOGISTIC, d, N, ld, Xd.data_ptr(),
               None if inline else yd.data_ptr(), 1.0, 2.0, 1.0, inline, N)
  rng = np.random.default_rng(d)
  W = (rng.normal(size=(C, d)) / np.sqrt(d)).astype(np.float32)
  idx = rng.integers(0, N, (C, n)).astype(np.int32)
  Wd, idxd = torch.from_numpy(W).cuda(), torch.from_numpy(idx).cuda()
  U = torch.zeros(C, dtype=torch.float64, device="cuda")
  G = torch.zeros((C, d), dtype=torch.float32, device="cuda")
  var = torch.zeros(C, dtype=torch.float64, device="cuda")
  ws = torch.zeros(int(lib.gbsgmc_glm_workspace_bytes(C, n, d)), dtype=torch.uint8,
                   device="cuda")
  _lib.call("gbsgmc_glm_value_and_grad", m, C, n, _lib.ptr(idxd), n, None,
            _lib.ptr(Wd), _lib.ptr(U), _lib.ptr(G), None, _lib.ptr(var),
            _lib.ptr(ws), ws.numel(), None, None)
  ref = O.glm_potential(W, X, y, idx, N, O.LOGISTIC, 1.0, 2.0, 1.0)
  from types import SimpleNamespace
  check(SimpleNamespace(U=U, grad=G, lk_var=var), ref)


@pytest.mark.parametrize("family", ["logistic", "lingauss"])
@pytest.mark.parametrize("n", [4096, 16384])
def test_potential_sum_is_compensated(lib, family, n):
  """U sums the minibatch's fp32 likelihoods with a compensated (Neumaier)
  sum per lane and fp64 across lanes, so U differs from the exact sum of the
  kernel's own per-row likelihoods by summation error alone: at most 1e-10
  relative here, where uncompensated fp32 lane sums left about 5e-9.  The
  remaining distance to the FP64 oracle (under 3e-8 relative) is the fp32
  rounding of the per-row likelihoods themselves."""
  import torch
  from gbsgmc import data, likelihoods as L, potential
  rng = np.random.default_rng(n)
  N, d, C = 50_000, 64, 16
  X = rng.normal(size=(N, d)).astype(np.float32)
  w = rng.normal(size=d)
  if family == "logistic":
    y = (rng.random(N) < 1 / (1 + np.exp(-X @ w / 4))).astype(np.float32)
    lik, fam = L.Logistic(), O.LOGISTIC
  else:
    y = (X @ w + 3.0 + 0.5 * rng.normal(size=N)).astype(np.float32)
    lik, fam = L.LinearGaussian(sigma=0.5), O.LINEAR_GAUSSIAN
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), lik)
  W = (rng.normal(size=(C, d)) * 0.2).astype(np.float32)
  idx = rng.integers(0, N, (C, n)).astype(np.int32)
  r = pot.evaluate(torch.from_numpy(W).cuda(), torch.from_numpy(idx).cuda(),
                   data.NumpyDataLoader(x=X, y=y).device_dataset(), lk=True)
  pot.check_status()
  U = r.U.cpu().numpy()
  lp, _ = O.log_prior(W, 1.0)
  U_lk = -(N / n) * r.lk.cpu().numpy().astype(np.float64).sum(1) - lp
  assert np.max(np.abs(U - U_lk) / np.abs(U_lk)) <= 1e-10
  ref = O.glm_potential(W, X, y, idx, N, fam, 0.5, 1.0)
  assert np.max(np.abs(U - ref.U) / np.abs(ref.U)) <= 3e-8
