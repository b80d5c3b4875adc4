"""Replica exchange on the tanh network: ragged (per-replica) minibatches,
the adjacent-pair exchange against the oracle, and the reSGLD plan against
the same steps issued one C-ABI call at a time.

Tolerances: the ragged potential uses the BF16 bounds of test_gpu_mlp.py;
the exchange (FP64 decisions, row swaps), the SA update and the plan
against its per-step twin are exact.
"""

import numpy as np
import pytest

from oracle import sgmc_oracle as O

import test_gpu_mlp as M

pytestmark = pytest.mark.gpu


def test_ragged_minibatches_match_oracle(lib):
  import torch
  lik, X, y, W, idx, ds, pot, Wd, idxd = M.setup(64, 256, 256, 1500, 4, 384, 21)
  rows = np.array([100, 128, 257, 384], np.int32)
  r = pot.evaluate(Wd, idxd, ds, grad=True, lk=True, observation_count=1500,
                   rows=torch.from_numpy(rows))
  pot.check_status()
  for c in range(4):
    sub = idx[c:c + 1, :rows[c]]
    ref = O.mlp_potential(W[c:c + 1], X, y, sub, 1500, 64, 256, 256, M.SIGMA,
                          prior_scale=1.0)

    class One:
      U = r.U[c:c + 1]
      grad = r.grad[c:c + 1]
      lk = r.lk[c:c + 1, :rows[c]]
      lk_var = r.lk_var[c:c + 1]
    M.check(lik, One, ref, W[c:c + 1], X, y, sub, 1500)
    assert np.all(r.lk[c, rows[c]:].cpu().numpy() == 0)


def test_ragged_with_full_rows_equals_uniform_call(lib):
  import torch
  lik, X, y, W, idx, ds, pot, Wd, idxd = M.setup(64, 256, 512, 900, 3, 256, 22)
  a = pot.evaluate(Wd, idxd, ds, grad=True, lk=True)
  b = pot.evaluate(Wd, idxd, ds, grad=True, lk=True,
                   rows=torch.full((3,), 256, dtype=torch.int32))
  pot.check_status()
  assert torch.equal(a.U, b.U) and torch.equal(a.grad, b.grad)
  assert torch.equal(a.lk, b.lk) and torch.equal(a.lk_var, b.lk_var)


@pytest.mark.parametrize("round_,given_u", [(3, True), (4, True), (5, False), (8, False)])
def test_adjacent_exchange_matches_oracle(lib, round_, given_u):
  import torch
  from gbsgmc import _lib
  rng = np.random.default_rng(round_)
  R, P, every, seed, F = 7, 1000, 50, 0xABCDEF0123, 1.3
  U = rng.normal(1000.0, 3.0, R)
  var = rng.uniform(0.5, 2.0, R)
  ssq = rng.uniform(0.5, 2.0, R - 1)
  ladder = (100.0 ** (np.arange(R) / (R - 1))).astype(np.float32)
  x = rng.normal(size=(R, P)).astype(np.float32)
  v = rng.normal(size=(R, P)).astype(np.float32)
  u = rng.uniform(size=R - 1)
  step = round_ * every - 1
  dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
  Ud, vard, ssqd, lad, xd, vd, ud = map(dev, (U, var, ssq, ladder, x, v, u))
  flags = torch.zeros(R - 1, dtype=torch.int32, device="cuda")
  counts = torch.zeros(R - 1, dtype=torch.int32, device="cuda")
  log_s = torch.zeros(R - 1, dtype=torch.float64, device="cuda")
  sch = _lib.sched(step_size=1e-3, temperature=1.0, offset=step,
                   chain_temperature_dev=lad)
  _lib.call("gbsgmc_resgld_exchange_adjacent", R, P, _lib.ptr(xd), _lib.ptr(vd),
            _lib.ptr(Ud), _lib.ptr(vard), sch, every, _lib.ptr(ssqd), F, seed,
            _lib.ptr(ud) if given_u else None, _lib.ptr(flags), _lib.ptr(counts),
            _lib.ptr(log_s), _lib.stream_handle())
  torch.cuda.synchronize()
  uu = u if given_u else [O.swap_uniform(seed, r, round_) for r in range(R - 1)]
  f_ref, U_ref, var_ref, ls_ref = O.resgld_exchange_adjacent(
      U, var, ssq, ladder.astype(np.float64), F, round_, uu)
  np.testing.assert_array_equal(flags.cpu().numpy(), f_ref)
  np.testing.assert_array_equal(counts.cpu().numpy(), f_ref)
  np.testing.assert_allclose(log_s.cpu().numpy(), ls_ref, rtol=1e-12, atol=1e-12)
  np.testing.assert_array_equal(Ud.cpu().numpy(), U_ref)
  np.testing.assert_array_equal(vard.cpu().numpy(), var_ref)
  perm = np.arange(R)
  for r in np.nonzero(f_ref)[0]:
    perm[[r, r + 1]] = perm[[r + 1, r]]
  np.testing.assert_array_equal(xd.cpu().numpy(), x[perm])
  np.testing.assert_array_equal(vd.cpu().numpy(), v[perm])
  assert all(f_ref[r] == 0 for r in range(1 - round_ % 2, R - 1, 2))


def test_sa_update_matches_oracle(lib):
  import torch
  from gbsgmc import _lib
  rng = np.random.default_rng(3)
  var, ssq = rng.uniform(size=9), rng.uniform(size=8)
  vd, sd = torch.from_numpy(var).cuda(), torch.from_numpy(ssq).cuda()
  kd = torch.tensor([4], dtype=torch.int64, device="cuda")
  for _ in range(3):
    _lib.call("gbsgmc_resgld_sa_update", 9, _lib.ptr(vd), _lib.ptr(sd), _lib.ptr(kd),
              _lib.stream_handle())
  k = 4
  for _ in range(3):
    ssq, k = O.resgld_sa_update(var, ssq, k)
  np.testing.assert_allclose(sd.cpu().numpy(), ssq, rtol=1e-15)
  assert int(kd.item()) == k == 7


def pcg_states(R):
  import torch
  words = []
  for c in range(R):
    st = O.loader_rng(c).bit_generator.state
    s, inc = st["state"]["state"], st["state"]["inc"]
    m = (1 << 64) - 1
    words.append([(s >> 64) & m, s & m, (inc >> 64) & m, inc & m, 0])
  return torch.from_numpy(np.array(words, np.uint64).view(np.int64).copy()).cuda()


def test_resgld_plan_equals_per_step_calls(lib):
  import torch
  from gbsgmc import _lib, engine, likelihoods as L, potential
  from gbsgmc.data import NumpyDataLoader
  R, N, n_max, steps, every = 4, 2000, 256, 8, 2
  lik = L.MLPGaussian(d_in=64, h1=256, h2=256, sigma=0.1)
  rng = np.random.default_rng(31)
  X = rng.normal(size=(N, 64)).astype(np.float32)
  y = (np.tanh(X[:, 1]) + 0.1 * rng.normal(size=N)).astype(np.float32)
  ds = NumpyDataLoader(x=X, y=y).device_dataset()
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), lik)
  W0 = np.stack([lik.init(np.random.default_rng(50 + r)) for r in range(R)])
  rows = np.array([64, 200, 256, 130], np.int32)
  ladder = np.array([1.0, 3.0, 9.0, 27.0], np.float32)
  h = torch.full((steps,), 2e-6, dtype=torch.float32, device="cuda")
  t = torch.ones(steps, dtype=torch.float32, device="cuda")

  Xp = torch.from_numpy(W0).cuda()
  Vp = torch.ones_like(Xp)
  plan = engine.ResgldPlan(pot, ds, Xp, Vp, rows, n_max, ladder, h, t,
                           engine.IndexSource(pcg=pcg_states(R)), noise_seed=9,
                           swap_seed=77, every=every, block_steps=4)
  plan.run(0, steps)
  plan.check_status()

  # The same steps one C-ABI call at a time.
  Xs = torch.from_numpy(W0).cuda()
  Vs = torch.ones_like(Xs)
  pcg = pcg_states(R)
  rows_d = torch.from_numpy(rows).cuda()
  lad = torch.from_numpy(ladder).cuda()
  U = torch.zeros(R, dtype=torch.float64, device="cuda")
  var = torch.zeros(R, dtype=torch.float64, device="cuda")
  ssq = torch.zeros(R - 1, dtype=torch.float64, device="cuda")
  k = torch.zeros(1, dtype=torch.int64, device="cuda")
  flags = torch.zeros(R - 1, dtype=torch.int32, device="cuda")
  counts = torch.zeros(R - 1, dtype=torch.int32, device="cuda")
  idx = torch.zeros((R, n_max), dtype=torch.int32, device="cuda")
  status = torch.zeros(1, dtype=torch.int32, device="cuda")
  noise = _lib.noise(9, 0)
  for s in range(steps):
    _lib.call("gbsgmc_index_draw_pcg64", _lib.ptr(pcg), R, N, n_max, n_max,
              _lib.ptr(idx), n_max, R * n_max, _lib.ptr(status), _lib.stream_handle())
    r = pot.evaluate(Xs, idx, ds, grad=True, rows=rows_d)
    U.copy_(r.U)
    var.copy_(r.lk_var)
    sch = _lib.sched(step_size=2e-6, temperature=1.0, offset=s, chain_temperature_dev=lad)
    _lib.call("gbsgmc_sgld_update", R, Xs.shape[1], _lib.ptr(Xs), _lib.ptr(r.grad),
              _lib.ptr(Vs), 0.9, 1e-5, sch, noise, None, _lib.stream_handle())
    _lib.call("gbsgmc_resgld_sa_update", R, _lib.ptr(var), _lib.ptr(ssq), _lib.ptr(k),
              _lib.stream_handle())
    if (s + 1) % every == 0:
      _lib.call("gbsgmc_resgld_exchange_adjacent", R, Xs.shape[1], _lib.ptr(Xs),
                _lib.ptr(Vs), _lib.ptr(U), _lib.ptr(var), sch, every, _lib.ptr(ssq), 1.0,
                77, None, _lib.ptr(flags), _lib.ptr(counts), None, _lib.stream_handle())
  torch.cuda.synchronize()
  pot.check_status()
  assert torch.isfinite(Xp).all()
  assert torch.equal(Xp, Xs) and torch.equal(Vp, Vs)
  assert torch.equal(plan.U, U) and torch.equal(plan.ssq, ssq)
  assert torch.equal(plan.counts, counts)
  assert int(plan.k.item()) == steps
