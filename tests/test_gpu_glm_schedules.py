"""Launch schedules of the fused GLM step through the C ABI: the
dynamically scheduled kernel (warps claim row items of any chain) and
multi-step launches (one CTA per chain runs a block of steps).

GBSGMC_GLM_DYN=1 selects the dynamic kernel for shapes no plan has autotuned
in this process; GBSGMC_GLM_SLICES sets the CTAs or items per chain,
GBSGMC_GLM_RW the rows a warp holds and GBSGMC_GLM_MULTISTEP a plan's launch
per block.  Against the FP64 oracle the tolerances are those of the static
kernel's tests: U within 1e-5 relative (+1e-3 absolute), gradients within
3e-4 of max|grad| per chain, trajectories 1e-4 relative (+1e-5 absolute).
Results must not depend on which warp finishes a chain or on how steps are
grouped into launches, so those comparisons are bit for bit.
"""

import numpy as np
import pytest

from oracle import sgmc_oracle as O

pytestmark = pytest.mark.gpu


def cuda(a):
  import torch
  return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _problem(N, d, family, seed):
  rng = np.random.default_rng(seed)
  X = rng.normal(size=(N, d)).astype(np.float32)
  if family == O.LOGISTIC:
    w = rng.normal(size=d) / np.sqrt(d)
    y = (rng.random(N) < 1 / (1 + np.exp(-(X @ w)))).astype(np.float32)
  else:
    y = (X @ rng.normal(size=d) + 0.5 * rng.normal(size=N)).astype(np.float32)
  return X, y


def _pot(family, prior=3.0, temperature=1.0):
  from gbsgmc import likelihoods as L, potential
  lik = L.Logistic() if family == O.LOGISTIC else L.LinearGaussian(sigma=0.5)
  return potential.minibatch_potential(L.GaussianPrior(prior), lik,
                                       temperature=temperature)


@pytest.fixture
def dynamic(monkeypatch):
  def set_shape(items, rw):
    monkeypatch.setenv("GBSGMC_GLM_DYN", "1")
    monkeypatch.setenv("GBSGMC_GLM_SLICES", str(items))
    monkeypatch.setenv("GBSGMC_GLM_RW", str(rw))
  return set_shape


# (chains, n, d, items per chain, rows per warp, family, masked)
CASES = [
    (37, 1000, 256, 16, 8, O.LOGISTIC, False),
    (37, 1000, 256, 4, 4, O.LOGISTIC, True),
    (5, 333, 64, 8, 2, O.LINEAR_GAUSSIAN, False),
    (3, 4096, 7, 16, 8, O.LINEAR_GAUSSIAN, True),
    (1, 65, 128, 3, 4, O.LOGISTIC, False),
    (301, 33, 8, 1, 8, O.LOGISTIC, False),
    (9, 2048, 201, 16, 4, O.LOGISTIC, True),
]


@pytest.mark.parametrize("C,n,d,items,rw,family,masked", CASES)
def test_value_and_grad_matches_oracle(lib, dynamic, C, n, d, items, rw, family,
                                       masked):
  import torch
  from gbsgmc.data import NumpyDataLoader
  dynamic(items, rw)
  N = 6000
  X, y = _problem(N, d, family, seed=d + n)
  ds = NumpyDataLoader(x=X, y=y).device_dataset()
  pot = _pot(family, temperature=1.3)
  rng = np.random.default_rng(C)
  W = (rng.normal(size=(C, d)) / np.sqrt(d)).astype(np.float32)
  idx = rng.integers(0, N, (C, n)).astype(np.int32)
  mask = (rng.random((C, n)) < 0.7).astype(np.float32) if masked else None
  r = pot.evaluate(cuda(W), cuda(idx), ds, lk=True,
                   mask=cuda(mask) if masked else None)
  ref = O.glm_potential(W, X, y, idx, N, family, 0.5, 3.0, 1.3, mask=mask)
  np.testing.assert_allclose(r.U.cpu().numpy(), ref.U, rtol=1e-5, atol=1e-3)
  g = r.grad.cpu().numpy()
  scale = np.abs(ref.grad).max(axis=1, keepdims=True) + 1e-6
  assert np.all(np.abs(g - ref.grad) <= 3e-4 * scale), np.abs(g - ref.grad).max()
  np.testing.assert_allclose(r.lk_var.cpu().numpy(), ref.var, rtol=1e-4, atol=1e-4)
  np.testing.assert_allclose(r.lk.cpu().numpy(), ref.lk, rtol=1e-4, atol=1e-4)
  pot.check_status()
  # The chain's partials are added in item order whichever warp ends last.
  for _ in range(3):
    r2 = pot.evaluate(cuda(W), cuda(idx), ds, lk=True,
                      mask=cuda(mask) if masked else None)
    assert torch.equal(r.U, r2.U) and torch.equal(r.grad, r2.grad)
    assert torch.equal(r.lk_var, r2.lk_var)


@pytest.mark.parametrize("rms", [True, False])
def test_fused_step_matches_oracle_with_injected_noise(lib, dynamic, rms):
  import torch
  from gbsgmc import _lib, data
  dynamic(8, 8)
  N, d, C, n = 5000, 96, 11, 700
  X, y = _problem(N, d, O.LOGISTIC, seed=12)
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = _pot(O.LOGISTIC, prior=2.0, temperature=1.3)
  m, keep = pot.model(loader.device_dataset())
  rng = np.random.default_rng(6)
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
  ref = O.glm_potential(W, X, y, idx, N, O.LOGISTIC, 0.5, 2.0, 1.3)
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
  # Tickets, claim and exit counters are back at zero after the launch.
  C2 = C + 2
  tail = ws.view(torch.uint8)[-256 * ((4 * C2 + 255) // 256):]
  assert int(tail.view(torch.int32)[:C2].abs().sum().item()) == 0


def test_plan_trajectory_matches_oracle(lib, dynamic, monkeypatch):
  """Many launches in a row: each one must find the claim counter reset by
  the previous one."""
  from gbsgmc import data, engine
  dynamic(16, 4)
  monkeypatch.setenv("GBSGMC_AUTOTUNE", "0")
  N, d, C, n, K = 4000, 40, 6, 512, 40
  X, y = _problem(N, d, O.LOGISTIC, seed=8)
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = _pot(O.LOGISTIC, prior=10.0)
  W0 = np.zeros((C, d), np.float32)
  V0 = np.ones((C, d), np.float32)
  h = np.full(K, 1e-4, np.float32)
  T = np.ones(K, np.float32)
  keep = np.full(K, -1, np.int32)
  keep[::5] = np.arange(len(keep[::5]))

  def words(c):
    st = O.loader_rng(c).bit_generator.state
    s, inc = st["state"]["state"], st["state"]["inc"]
    mk = (1 << 64) - 1
    return np.array([(s >> 64) & mk, s & mk, (inc >> 64) & mk, inc & mk, 0],
                    np.uint64).view(np.int64)

  pcg = cuda(np.stack([words(c) for c in range(C)]))
  run = engine.run_sgld_glm(pot, loader.device_dataset(), cuda(W0), cuda(V0), n,
                            K, h, T, keep, int((keep >= 0).sum()),
                            engine.IndexSource(pcg=pcg), noise_seed=11,
                            block_steps=8)
  idx = np.stack([O.loader_draws(O.loader_rng(c), N, n, K) for c in range(C)], 1)
  xi = np.stack([[O.philox_normals(11, c, k, 0, d) for c in range(C)]
                 for k in range(K)]).astype(np.float32)
  Ws, Us, _ = O.sgld_glm_trajectory(X, y, W0, idx, xi, h, T, O.LOGISTIC, 0.5, 10.0)
  np.testing.assert_allclose(run.w.cpu().numpy(), Ws[-1], rtol=1e-4, atol=1e-5)
  np.testing.assert_allclose(run.U.cpu().numpy(), Us[-1], rtol=1e-5, atol=1e-3)
  kept = np.nonzero(keep >= 0)[0]
  np.testing.assert_allclose(run.samples.cpu().numpy(), Ws[kept + 1], rtol=1e-4,
                             atol=1e-5)


@pytest.mark.parametrize("slices,dyn", [(1, False), (3, False), (8, True)])
def test_multi_step_launch_equals_single_steps(lib, monkeypatch, slices, dyn):
  """gbsgmc_sgld_glm_steps over K steps (one launch with one CTA per chain,
  else a launch per step) equals K gbsgmc_sgld_glm_step calls bit for bit,
  with step-size, temperature and keep-slot tables."""
  import torch
  from gbsgmc import _lib, data
  monkeypatch.setenv("GBSGMC_GLM_SLICES", str(slices))
  monkeypatch.setenv("GBSGMC_GLM_RW", "8")
  monkeypatch.setenv("GBSGMC_GLM_DYN", "1" if dyn else "0")
  N, d, C, n, K = 7000, 128, 19, 640, 7
  X, y = _problem(N, d, O.LOGISTIC, seed=21)
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = _pot(O.LOGISTIC, prior=1.0)
  m, _ = pot.model(loader.device_dataset())
  rng = np.random.default_rng(3)
  W0 = (rng.normal(size=(C, d)) * 0.1).astype(np.float32)
  idx = cuda(rng.integers(0, N, (K, C, n)).astype(np.int32))
  h = cuda((1e-3 * 0.8 ** np.arange(K)).astype(np.float32))
  T = cuda(np.linspace(1.0, 0.5, K).astype(np.float32))
  keep = cuda(np.array([-1, 0, -1, 1, 2, -1, 3], np.int32))
  sch = _lib.sched(step_size_dev=h, temperature_dev=T, keep_slot_dev=keep)
  nz = _lib.noise(seed=17)
  outs = []
  for multi in (True, False):
    W, V = cuda(W0), cuda(np.ones_like(W0))
    U = torch.zeros(C, dtype=torch.float64, device="cuda")
    var = torch.zeros(C, dtype=torch.float64, device="cuda")
    smp = torch.zeros((4, C, d), dtype=torch.float32, device="cuda")
    slk = torch.zeros((4, C), dtype=torch.float64, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    ws = pot.workspace(C, n, d)
    if multi:
      _lib.call("gbsgmc_sgld_glm_steps", m, C, n, _lib.ptr(idx), n, C * n, K,
                _lib.ptr(W), _lib.ptr(V), 0.9, 1e-5, sch, nz, _lib.ptr(U),
                _lib.ptr(var), _lib.ptr(smp), _lib.ptr(slk), _lib.ptr(ws),
                ws.numel(), _lib.ptr(st), None)
    else:
      for j in range(K):
        sj = _lib.sched(step_size_dev=h, temperature_dev=T, keep_slot_dev=keep,
                        offset=j)
        _lib.call("gbsgmc_sgld_glm_step", m, C, n, _lib.ptr(idx[j]), n,
                  _lib.ptr(W), _lib.ptr(V), 0.9, 1e-5, sj, nz, _lib.ptr(U),
                  _lib.ptr(var), _lib.ptr(smp), _lib.ptr(slk), _lib.ptr(ws),
                  ws.numel(), _lib.ptr(st), None)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    outs.append((W, V, U, var, smp, slk))
  for a, b in zip(*outs):
    assert torch.equal(a, b)
  assert bool(torch.isfinite(outs[0][0]).all())


def test_multi_step_plan_matches_per_step_plan_and_oracle(lib, monkeypatch):
  """A plan whose blocks run in one launch (with the next block's index
  draws overlapped, or not) against the same plan with one launch per step
  -- bit for bit, including the PCG64 stream states left behind -- and
  against the oracle trajectory."""
  import torch
  from gbsgmc import data, engine
  monkeypatch.setenv("GBSGMC_AUTOTUNE", "0")
  monkeypatch.setenv("GBSGMC_GLM_SLICES", "1")
  monkeypatch.setenv("GBSGMC_GLM_RW", "8")
  N, d, C, n, K = 4000, 64, 5, 384, 45
  X, y = _problem(N, d, O.LOGISTIC, seed=31)
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = _pot(O.LOGISTIC, prior=10.0)
  W0 = np.zeros((C, d), np.float32)
  V0 = np.ones((C, d), np.float32)
  h = np.full(K, 1e-4, np.float32)
  T = np.ones(K, np.float32)
  keep = np.full(K, -1, np.int32)
  keep[3::6] = np.arange(len(keep[3::6]))

  def words(c):
    st = O.loader_rng(c).bit_generator.state
    s, inc = st["state"]["state"], st["state"]["inc"]
    mk = (1 << 64) - 1
    return np.array([(s >> 64) & mk, s & mk, (inc >> 64) & mk, inc & mk, 0],
                    np.uint64).view(np.int64)

  runs, streams = [], []
  for multi, pipe, block in (("1", "1", 10), ("1", "0", 10), ("1", "1", 45),
                             ("1", "1", 20), ("0", "1", 10)):
    monkeypatch.setenv("GBSGMC_GLM_MULTISTEP", multi)
    monkeypatch.setenv("GBSGMC_PLAN_PIPELINE", pipe)
    pcg = cuda(np.stack([words(c) for c in range(C)]))
    runs.append(engine.run_sgld_glm(pot, loader.device_dataset(), cuda(W0),
                                    cuda(V0), n, K, h, T, keep,
                                    int((keep >= 0).sum()),
                                    engine.IndexSource(pcg=pcg), noise_seed=11,
                                    block_steps=block))
    streams.append(pcg)
  for r, pcg in zip(runs[1:], streams[1:]):
    assert torch.equal(r.w, runs[0].w) and torch.equal(r.U, runs[0].U)
    assert torch.equal(r.samples, runs[0].samples)
    assert torch.equal(pcg, streams[0])
  # The streams advanced by exactly K steps of draws, as numpy's would.
  for c in range(C):
    rng = O.loader_rng(c)
    O.loader_draws(rng, N, n, K)
    st = rng.bit_generator.state
    mk = (1 << 64) - 1
    got = streams[0][c].cpu().numpy().view(np.uint64)
    assert (int(got[0]) << 64) | int(got[1]) == st["state"]["state"]
  idx = np.stack([O.loader_draws(O.loader_rng(c), N, n, K) for c in range(C)], 1)
  xi = np.stack([[O.philox_normals(11, c, k, 0, d) for c in range(C)]
                 for k in range(K)]).astype(np.float32)
  Ws, Us, _ = O.sgld_glm_trajectory(X, y, W0, idx, xi, h, T, O.LOGISTIC, 0.5, 10.0)
  np.testing.assert_allclose(runs[0].w.cpu().numpy(), Ws[-1], rtol=1e-4, atol=1e-5)
  np.testing.assert_allclose(runs[0].U.cpu().numpy(), Us[-1], rtol=1e-5, atol=1e-3)
  kept = np.nonzero(keep >= 0)[0]
  np.testing.assert_allclose(runs[0].samples.cpu().numpy(), Ws[kept + 1],
                             rtol=1e-4, atol=1e-5)


@pytest.mark.parametrize("kind", ["obabo", "sghmc"])
def test_glm_obabo_sghmc_plan_equals_per_chain_steps(lib, monkeypatch, kind):
  """OBABO and SGHMC chains on the logistic potential through one plan
  (gbsgmc_glm_plan_create) against the per-chain step path.  With one CTA
  per chain the GLM kernel's arithmetic for a chain does not depend on the
  other chains, and both paths draw the same PCG64 indices and Philox
  noise, so the samples agree bit for bit."""
  from gbsgmc import alias, data, engine, likelihoods as L, potential
  monkeypatch.setenv("GBSGMC_GLM_SLICES", "1")
  monkeypatch.setenv("GBSGMC_GLM_RW", "4")
  N, d, n, C = 3000, 24, 96, 3
  X, y = _problem(N, d, O.LOGISTIC, seed=41)
  pot = potential.minibatch_potential(L.GaussianPrior(2.0), L.Logistic())
  common = dict(cache_size=32, batch_size=n, first_step_size=1e-3,
                last_step_size=1e-4, burn_in=0, accepted_samples=4)
  rng = np.random.default_rng(5)
  inits = [{"w": (0.1 * rng.normal(size=d)).astype(np.float32)} for _ in range(C)]
  made = []
  real_init = engine.NetPlan.__init__

  def spy(self, *args, **kwargs):
    made.append(kind)
    return real_init(self, *args, **kwargs)

  monkeypatch.setattr(engine.NetPlan, "__init__", spy)
  outs = []
  for fused in (True, False):
    # A fresh loader each time: its chains (index seeds, noise keys) are
    # numbered in registration order.
    loader = data.NumpyDataLoader(x=X, y=y)
    if kind == "obabo":
      r = alias.obabo(pot, loader, integration_steps=3, friction=5.0, **common)
    else:
      r = alias.sghmc(pot, loader, integration_steps=2, friction=0.5, **common)
    engine.FUSED_ENABLED = fused
    try:
      outs.append(r(*inits, iterations=8))
    finally:
      engine.FUSED_ENABLED = True
  assert made == [kind]   # the fused run went through one plan
  for ra, rb in zip(*outs):
    assert ra["sample_count"] == rb["sample_count"] == 4
    va = np.asarray(ra["samples"]["variables"]["w"])
    vb = np.asarray(rb["samples"]["variables"]["w"])
    assert np.isfinite(va).all() and not np.array_equal(va[0], va[-1])
    np.testing.assert_array_equal(va, vb)


def test_sharded_plans_equal_one_plan(lib, monkeypatch):
  """Replicas on one GPU: two plans over chain ids [0, C) and [C, 2C) --
  bench.py's shard_chains, index streams seeded and noise keyed by the chain
  id -- equal one plan over all 2C chains bit for bit (one CTA per chain,
  so a chain's arithmetic does not depend on the others)."""
  import torch
  from gbsgmc import data, engine
  from gbsgmc.data.numpy_loader import pcg64_words
  monkeypatch.setenv("GBSGMC_AUTOTUNE", "0")
  monkeypatch.setenv("GBSGMC_GLM_SLICES", "1")
  monkeypatch.setenv("GBSGMC_GLM_RW", "8")
  monkeypatch.setenv("GBSGMC_GLM_MULTISTEP", "1")
  N, d, C, n, K = 4000, 64, 4, 256, 30
  X, y = _problem(N, d, O.LOGISTIC, seed=51)
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = _pot(O.LOGISTIC, prior=5.0)
  h = np.full(K, 1e-4, np.float32)
  T = np.ones(K, np.float32)
  keep = np.full(K, -1, np.int32)
  keep[::6] = np.arange(len(keep[::6]))
  words = np.array([pcg64_words(c) for c in range(2 * C)], np.uint64).view(np.int64)

  def run(lo, hi):
    pcg = cuda(words[lo:hi])
    r = engine.run_sgld_glm(pot, loader.device_dataset(),
                            cuda(np.zeros((hi - lo, d), np.float32)),
                            cuda(np.ones((hi - lo, d), np.float32)), n, K, h, T,
                            keep, int((keep >= 0).sum()),
                            engine.IndexSource(pcg=pcg, chain_base=lo),
                            noise_seed=11, chain_base=lo, block_steps=10)
    return r, pcg

  whole, pw = run(0, 2 * C)
  a, pa = run(0, C)
  b, pb = run(C, 2 * C)
  assert torch.equal(whole.w, torch.cat([a.w, b.w]))
  assert torch.equal(whole.U, torch.cat([a.U, b.U]))
  assert torch.equal(whole.samples, torch.cat([a.samples, b.samples], 1))
  assert torch.equal(pw, torch.cat([pa, pb]))
