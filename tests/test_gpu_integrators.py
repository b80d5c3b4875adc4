"""Integrator kernels, the fused SGLD step and plans vs the oracle.

Elementwise updates agree with the fp32 oracle to 1e-5 relative (+1e-6
absolute); K-step trajectories (gradients accumulated in fp32 on the GPU,
fp64 in the oracle) to 1e-4 relative (+1e-5 absolute); kinetic energies and
FP64 swap quantities to 1e-6 / 1e-12 relative.
"""

import numpy as np
import pytest

from oracle import sgmc_oracle as O

pytestmark = pytest.mark.gpu


def cuda(a, dtype=None):
  import torch
  t = torch.from_numpy(np.ascontiguousarray(a))
  if dtype is not None:
    t = t.to(dtype)
  return t.cuda()


def test_sgld_update_rmsprop_and_plain(lib):
  import torch
  from gbsgmc import _lib
  rng = np.random.default_rng(0)
  C, P = 3, 1003
  x = rng.normal(size=(C, P)).astype(np.float32)
  g = (rng.normal(size=(C, P)) * 30).astype(np.float32)
  v = rng.random((C, P)).astype(np.float32) + 0.5
  xi = rng.normal(size=(C, P)).astype(np.float32)
  for rms in (True, False):
    xd, gd, vd, nd = cuda(x), cuda(g), cuda(v), cuda(xi)
    samples = torch.zeros((2, C, P), dtype=torch.float32, device="cuda")
    keep = cuda(np.array([-1, -1, 1], np.int32))
    h_tab = cuda(np.array([0, 0, 1e-3], np.float32))
    t_tab = cuda(np.array([1, 1, 0.7], np.float32))
    sch = _lib.sched(step_size=0, temperature=0, step_size_dev=h_tab,
                     temperature_dev=t_tab, keep_slot_dev=keep, offset=2)
    _lib.call("gbsgmc_sgld_update", C, P, _lib.ptr(xd), _lib.ptr(gd),
              _lib.ptr(vd) if rms else None, 0.9, 1e-5, sch,
              _lib.noise(noise_dev=nd, noise_stride=P), _lib.ptr(samples), None)
    xr, vr = O.sgld_step(x, g, v, xi, 1e-3, 0.7, 0.9, 1e-5, rms)
    np.testing.assert_allclose(xd.cpu().numpy(), xr, rtol=1e-5, atol=1e-6)
    if rms:
      np.testing.assert_allclose(vd.cpu().numpy(), vr, rtol=1e-5, atol=1e-6)
    np.testing.assert_array_equal(samples[1].cpu().numpy(), xd.cpu().numpy())


def test_obabo_halves(lib):
  import torch
  from gbsgmc import _lib
  rng = np.random.default_rng(1)
  C, P = 2, 517
  x, p, g1, g2, xi1, xi2 = (rng.normal(size=(C, P)).astype(np.float32) for _ in range(6))
  mass = (rng.random(P) + 0.5).astype(np.float32)
  xd, pd = cuda(x), cuda(p)
  g1d, g2d, md, x1d, x2d = cuda(g1), cuda(g2), cuda(mass), cuda(xi1), cuda(xi2)
  ke0 = torch.zeros(C, dtype=torch.float64, device="cuda")
  ke1 = torch.zeros(C, dtype=torch.float64, device="cuda")
  sch = _lib.sched(step_size=0.01, temperature=0.8, offset=3)
  _lib.call("gbsgmc_obabo_first", C, P, _lib.ptr(xd), _lib.ptr(pd), _lib.ptr(g1d),
            _lib.ptr(md), 0.7, _lib.ptr(ke0), sch,
            _lib.noise(noise_dev=x1d, noise_stride=P), None)
  _lib.call("gbsgmc_obabo_second", C, P, _lib.ptr(pd), _lib.ptr(g2d),
            _lib.ptr(md), 0.7, _lib.ptr(ke1), sch,
            _lib.noise(noise_dev=x2d, noise_stride=P), None)
  xr, pr, ker0 = O.obabo_first(x, p, g1, xi1, 0.01, 0.8, 0.7, mass)
  pr, ker1 = O.obabo_second(pr, g2, xi2, 0.01, 0.8, 0.7, mass)
  np.testing.assert_allclose(xd.cpu().numpy(), xr, rtol=1e-5, atol=1e-6)
  np.testing.assert_allclose(pd.cpu().numpy(), pr, rtol=1e-5, atol=1e-6)
  np.testing.assert_allclose(ke0.cpu().numpy(), ker0, rtol=1e-6)
  np.testing.assert_allclose(ke1.cpu().numpy(), ker1, rtol=1e-6)


def test_sghmc_pieces(lib):
  from gbsgmc import _lib
  rng = np.random.default_rng(2)
  C, P = 2, 301
  x, g, xi0, xi1 = (rng.normal(size=(C, P)).astype(np.float32) for _ in range(4))
  fric = (rng.random(P) + 0.1).astype(np.float32)
  mass = (rng.random(P) + 0.5).astype(np.float32)
  xd = cuda(x)
  pd = cuda(np.zeros((C, P), np.float32))
  md, fd, gd, x0d, x1d = cuda(mass), cuda(fric), cuda(g), cuda(xi0), cuda(xi1)
  sch = _lib.sched(step_size=0.02, temperature=1.0, offset=0)
  _lib.call("gbsgmc_sghmc_resample", C, P, _lib.ptr(pd), _lib.ptr(md), sch,
            _lib.noise(noise_dev=x0d, noise_stride=P), None)
  _lib.call("gbsgmc_sghmc_position", C, P, _lib.ptr(xd), _lib.ptr(pd),
            _lib.ptr(md), _lib.ptr(fd), 0.0, sch, None)
  _lib.call("gbsgmc_sghmc_momentum", C, P, _lib.ptr(pd), _lib.ptr(gd),
            _lib.ptr(fd), 0.0, sch,
            _lib.noise(noise_dev=x1d, noise_stride=P), None)
  p = O.sghmc_resample(xi0, mass)
  xr, p = O.sghmc_position(x, p, 0.02, fric, mass)
  p = O.sghmc_momentum(p, g, xi1, 0.02, fric)
  np.testing.assert_allclose(xd.cpu().numpy(), xr, rtol=1e-5, atol=1e-6)
  np.testing.assert_allclose(pd.cpu().numpy(), p, rtol=1e-5, atol=1e-6)


def test_resgld_swap_kernel(lib):
  import torch
  from gbsgmc import _lib
  rng = np.random.default_rng(3)
  pairs = 64
  Un, Uh = rng.normal(size=pairs) * 5, rng.normal(size=pairs) * 5
  var = rng.random(pairs) * 2
  Tn, Th = np.ones(pairs), np.full(pairs, 10.0)
  ssq = rng.random(pairs)
  k = rng.integers(0, 20, pairs).astype(np.int64)
  u = rng.random(pairs)
  d = lambda a: cuda(np.asarray(a, np.float64))
  ssq_d, k_d = d(ssq), cuda(k)
  Un_d, Uh_d, var_d, Tn_d, Th_d, u_d = d(Un), d(Uh), d(var), d(Tn), d(Th), d(u)
  perm = torch.zeros(pairs, dtype=torch.int32, device="cuda")
  log_s = torch.zeros(pairs, dtype=torch.float64, device="cuda")
  _lib.call("gbsgmc_resgld_swap_f64", pairs, _lib.ptr(Un_d), _lib.ptr(Uh_d),
            _lib.ptr(var_d), _lib.ptr(Tn_d), _lib.ptr(Th_d), 1.5,
            _lib.ptr(ssq_d), _lib.ptr(k_d), _lib.ptr(u_d), 0, 0,
            _lib.ptr(log_s), _lib.ptr(perm), None)
  for i in range(pairs):
    sw, s2, kk, ls = O.resgld_swap(Un[i], Uh[i], var[i], Tn[i], Th[i], ssq[i],
                                   int(k[i]), u[i], 1.5)
    assert int(perm[i]) == int(sw)
    assert float(ssq_d[i]) == pytest.approx(s2, rel=1e-12)
    assert int(k_d[i]) == kk
    assert float(log_s[i]) == pytest.approx(ls, rel=1e-12, abs=1e-12)
  a = cuda(rng.normal(size=(pairs, 9)).astype(np.float32))
  b = cuda(rng.normal(size=(pairs, 9)).astype(np.float32))
  a0, b0 = a.clone(), b.clone()
  _lib.call("gbsgmc_swap_rows", pairs, 9, _lib.ptr(a), _lib.ptr(b), _lib.ptr(perm), None)
  sw = perm.bool()[:, None]
  assert torch.equal(a, torch.where(sw, b0, a0)) and torch.equal(b, torch.where(sw, a0, b0))


def _glm_problem(N, d, family, seed=0):
  rng = np.random.default_rng(seed)
  X = rng.normal(size=(N, d)).astype(np.float32)
  if family == O.LOGISTIC:
    y = (rng.random(N) < 1 / (1 + np.exp(-(X @ (rng.normal(size=d) / np.sqrt(d)))))
         ).astype(np.float32)
  else:
    y = (X @ rng.normal(size=d) + 0.5 * rng.normal(size=N)).astype(np.float32)
  return X, y


@pytest.mark.parametrize("family,rms", [(O.LOGISTIC, True), (O.LINEAR_GAUSSIAN, True),
                                        (O.LOGISTIC, False)])
def test_fused_step_matches_oracle_with_injected_noise(lib, family, rms):
  import torch
  from gbsgmc import _lib, data, likelihoods as L, potential
  N, d, C, n = 5000, 64, 9, 300
  X, y = _glm_problem(N, d, family)
  loader = data.NumpyDataLoader(x=X, y=y)
  lik = L.Logistic() if family == O.LOGISTIC else L.LinearGaussian(sigma=0.5)
  pot = potential.minibatch_potential(L.GaussianPrior(2.0), lik, temperature=1.3)
  m, keep = pot.model(loader.device_dataset())
  rng = np.random.default_rng(5)
  W = (rng.normal(size=(C, d)) * 0.1).astype(np.float32)
  V = np.ones((C, d), np.float32)
  idx = rng.integers(0, N, (C, n)).astype(np.int32)
  xi = rng.normal(size=(C, d)).astype(np.float32)
  Wd, Vd = cuda(W), cuda(V)
  U = torch.zeros(C, dtype=torch.float64, device="cuda")
  var = torch.zeros(C, dtype=torch.float64, device="cuda")
  samples = torch.zeros((1, C, d), dtype=torch.float32, device="cuda")
  slik = torch.zeros((1, C), dtype=torch.float64, device="cuda")
  ws = pot.workspace(C, n, d)
  status = torch.zeros(1, dtype=torch.int32, device="cuda")
  keep_d, idx_d, xi_d = cuda(np.array([0], np.int32)), cuda(idx), cuda(xi)
  sch = _lib.sched(step_size=2e-4, temperature=0.9, keep_slot_dev=keep_d,
                   offset=0)
  _lib.call("gbsgmc_sgld_glm_step", m, C, n, _lib.ptr(idx_d), n, _lib.ptr(Wd),
            _lib.ptr(Vd) if rms else None, 0.9, 1e-5, sch,
            _lib.noise(noise_dev=xi_d, noise_stride=d), _lib.ptr(U),
            _lib.ptr(var), _lib.ptr(samples), _lib.ptr(slik), _lib.ptr(ws),
            ws.numel(), _lib.ptr(status), None)
  ref = O.glm_potential(W, X, y, idx, N, family, 0.5, 2.0, 1.3)
  Wr, Vr = O.sgld_step(W, ref.grad.astype(np.float32), V, xi, 2e-4, 0.9, 0.9,
                       1e-5, rms)
  np.testing.assert_allclose(U.cpu().numpy(), ref.U, rtol=1e-5, atol=1e-3)
  np.testing.assert_allclose(var.cpu().numpy(), ref.var, rtol=1e-4, atol=1e-4)
  np.testing.assert_allclose(Wd.cpu().numpy(), Wr, rtol=1e-4, atol=1e-5)
  if rms:
    np.testing.assert_allclose(Vd.cpu().numpy(), Vr, rtol=1e-3, atol=1e-3)
  np.testing.assert_array_equal(samples[0].cpu().numpy(), Wd.cpu().numpy())
  np.testing.assert_allclose(slik[0].cpu().numpy(), -ref.U, rtol=1e-5, atol=1e-3)
  assert int(status.item()) == 0


def _pcg_words(rng):
  st = rng.bit_generator.state
  s, inc = st["state"]["state"], st["state"]["inc"]
  m = (1 << 64) - 1
  return np.array([(s >> 64) & m, s & m, (inc >> 64) & m, inc & m,
                   (int(st["uinteger"]) << 32) | int(st["has_uint32"])],
                  np.uint64).view(np.int64)


def _run_plan(pot, loader, W, V, n, K, h, T, keep, n_kept, seeds, block,
              noise_seed=11):
  import torch
  from gbsgmc import engine
  pcg = cuda(np.stack([_pcg_words(O.loader_rng(s)) for s in seeds]))
  Wd = cuda(W)
  Vd = cuda(V) if V is not None else None
  return engine.run_sgld_glm(pot, loader.device_dataset(), Wd, Vd, n, K, h, T,
                             keep, n_kept, engine.IndexSource(pcg=pcg),
                             noise_seed=noise_seed, block_steps=block), pcg


@pytest.mark.parametrize("family", [O.LOGISTIC, O.LINEAR_GAUSSIAN])
def test_plan_trajectory_matches_oracle(lib, family):
  """K steps with the reference loader's index stream (numpy PCG64, seeds =
  chain ids) and Philox noise, against the oracle driven by the same
  indices and normals."""
  from gbsgmc import likelihoods as L, potential, data
  N, d, C, n, K = 4000, 32, 4, 128, 60
  X, y = _glm_problem(N, d, family, seed=7)
  loader = data.NumpyDataLoader(x=X, y=y)
  lik = L.Logistic() if family == O.LOGISTIC else L.LinearGaussian(sigma=0.5)
  pot = potential.minibatch_potential(L.GaussianPrior(10.0), lik)
  W0 = np.zeros((C, d), np.float32)
  V0 = np.ones((C, d), np.float32)
  h = O.polynomial_first_last(1e-3, 1e-5, 0.33, K).astype(np.float32) * 0.1
  T = np.ones(K, np.float32)
  keep = np.full(K, -1, np.int32)
  keep[::7] = np.arange(len(keep[::7]))
  run, _ = _run_plan(pot, loader, W0, V0, n, K, h, T, keep,
                     int((keep >= 0).sum()), range(C), block=16)
  idx = np.stack([O.loader_draws(O.loader_rng(c), N, n, K) for c in range(C)], 1)
  xi = np.stack([[O.philox_normals(11, c, k, 0, d) for c in range(C)]
                 for k in range(K)]).astype(np.float32)
  Ws, Us, Vs = O.sgld_glm_trajectory(X, y, W0, idx, xi, h, T, family, 0.5, 10.0)
  np.testing.assert_allclose(run.w.cpu().numpy(), Ws[-1], rtol=1e-4, atol=1e-5)
  np.testing.assert_allclose(run.U.cpu().numpy(), Us[-1], rtol=1e-5, atol=1e-3)
  kept = np.nonzero(keep >= 0)[0]
  np.testing.assert_allclose(run.samples.cpu().numpy(), Ws[kept + 1], rtol=1e-4,
                             atol=1e-5)
  np.testing.assert_allclose(run.sample_lik.cpu().numpy(), -Us[kept], rtol=1e-5,
                             atol=1e-3)


def test_plan_is_deterministic_and_block_invariant(lib):
  """Graph replay, block size and the slice count do not change results."""
  import torch
  from gbsgmc import likelihoods as L, potential, data
  N, d, C, n, K = 20_000, 256, 16, 1024, 23
  X, y = _glm_problem(N, d, O.LOGISTIC, seed=9)
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), L.Logistic())
  W0 = np.zeros((C, d), np.float32)
  V0 = np.ones((C, d), np.float32)
  h = np.full(K, 1e-4, np.float32)
  T = np.ones(K, np.float32)
  keep = np.full(K, -1, np.int32)
  outs = []
  for block in (1, 5, 23, 50):
    run, pcg = _run_plan(pot, loader, W0, V0, n, K, h, T, keep, 0,
                         range(C), block)
    outs.append((run.w.cpu(), run.U.cpu(), pcg.cpu()))
  for w, U, pcg in outs[1:]:
    assert torch.equal(w, outs[0][0]) and torch.equal(U, outs[0][1])
    assert torch.equal(pcg, outs[0][2])
  # The device streams advanced exactly like numpy's.
  for c in range(C):
    rng = O.loader_rng(c)
    O.loader_draws(rng, N, n, K)
    np.testing.assert_array_equal(outs[0][2][c].numpy(), _pcg_words(rng))


def test_plain_step_matches_fused(lib):
  import torch
  from gbsgmc import _lib, data, likelihoods as L, potential
  N, d, n = 3000, 48, 256
  X, y = _glm_problem(N, d, O.LOGISTIC, seed=4)
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), L.Logistic())
  m, keep = pot.model(loader.device_dataset())
  rng = np.random.default_rng(0)
  W = (rng.normal(size=(1, d)) * 0.1).astype(np.float32)
  idx = cuda(rng.integers(0, N, (1, n)).astype(np.int32))
  Wa, Va, Wb, Vb = cuda(W), cuda(np.ones_like(W)), cuda(W), cuda(np.ones_like(W))
  Ua = torch.zeros(1, dtype=torch.float64, device="cuda")
  Ub = torch.zeros(1, dtype=torch.float64, device="cuda")
  sch = _lib.sched(step_size=1e-3, temperature=1.0, offset=5)
  nz = _lib.noise(seed=3)
  ws = pot.workspace(1, n, d)
  _lib.call("gbsgmc_sgld_glm_step", m, 1, n, _lib.ptr(idx), n, _lib.ptr(Wa),
            _lib.ptr(Va), 0.9, 1e-5, sch, nz, _lib.ptr(Ua), None, None, None,
            _lib.ptr(ws), ws.numel(), None, None)
  buf = torch.zeros(int(lib.gbsgmc_plain_buffer_bytes(n, d)), dtype=torch.uint8,
                    device="cuda")
  _lib.call("gbsgmc_plain_sgld_glm_step", m, n, _lib.ptr(idx), _lib.ptr(Wb),
            _lib.ptr(Vb), 0.9, 1e-5, sch, nz, _lib.ptr(Ub), _lib.ptr(buf), None,
            None)
  np.testing.assert_allclose(Wb.cpu().numpy(), Wa.cpu().numpy(), rtol=1e-5, atol=1e-6)
  np.testing.assert_allclose(Ub.cpu().numpy(), Ua.cpu().numpy(), rtol=1e-6)
