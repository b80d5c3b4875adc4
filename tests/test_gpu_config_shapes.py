"""Parity at the workloads' own shapes, where the oracle can follow a few
chains of the full-size run.

* Logistic regression (N = 10^6, d = 256, 256 chains, minibatch 1024): ten
  steps of the fused, graph-captured SGLD plan with the reference loader's
  PCG64 streams, against the oracle's trajectory of six of the chains driven
  by the same indices and Philox normals (1e-4 relative, as the smaller
  trajectory tests); every chain's stream ends in numpy's own state.
* Tanh network 64-1024-1024-1 (64 chains, minibatch 2048): one value and
  gradient of all chains; three chains against the FP64 oracle with the
  BF16 bounds of test_gpu_mlp.py.
* The replica-exchange ladder (32 replicas, minibatches 96..4000 of that
  network): one ragged value and gradient; the replicas with 96, 2001 and
  4000 rows against the oracle, then one exchange round at T_r =
  100^(r/31) on those potentials against the oracle's rule (exact).
"""

import numpy as np
import pytest

from oracle import sgmc_oracle as O

import test_gpu_mlp as M

pytestmark = pytest.mark.gpu


def test_logistic_full_size_plan_matches_oracle_on_sampled_chains(lib):
  import torch
  import bench
  from gbsgmc import data, engine, likelihoods as L, potential
  from gbsgmc.data.numpy_loader import pcg64_words_many
  X, y = bench.make_data()
  N, d, C, n, K = bench.N_OBS, bench.D, bench.CHAINS, bench.MB, 10
  loader = data.NumpyDataLoader(copy=False, x=X, y=y)
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), L.Logistic(),
                                      strategy="vmap")
  h = O.polynomial_first_last(bench.FIRST, bench.LAST, bench.GAMMA,
                              bench.K_CONFIG)[:K].astype(np.float32)
  T = np.ones(K, np.float32)
  keep = np.arange(K, dtype=np.int32)
  pcg = torch.from_numpy(pcg64_words_many(range(C)).view(np.int64)).cuda()
  W = torch.zeros((C, d), dtype=torch.float32, device="cuda")
  V = torch.ones((C, d), dtype=torch.float32, device="cuda")
  run = engine.run_sgld_glm(pot, loader.device_dataset(), W, V, n, K, h, T, keep,
                            K, engine.IndexSource(pcg=pcg), noise_seed=0,
                            block_steps=5)
  sub = [0, 1, 77, 128, 201, 255]
  idx = np.stack([O.loader_draws(O.loader_rng(c), N, n, K) for c in sub], 1)
  rows, inv = np.unique(idx, return_inverse=True)
  xi = np.stack([[O.philox_normals(0, c, k, 0, d) for c in sub]
                 for k in range(K)]).astype(np.float32)
  Ws, Us, _ = O.sgld_glm_trajectory(X[rows], y[rows], np.zeros((len(sub), d), np.float32),
                                    inv.reshape(idx.shape), xi, h, T, O.LOGISTIC,
                                    1.0, 1.0, n_obs=N)
  got = run.samples.cpu().numpy()[:, sub]
  np.testing.assert_allclose(got, Ws[1:], rtol=1e-4, atol=1e-5)
  np.testing.assert_allclose(run.U.cpu().numpy()[sub], Us[-1], rtol=1e-5)
  np.testing.assert_allclose(run.sample_lik.cpu().numpy()[:, sub], -Us, rtol=1e-5)
  # Every chain's device stream ends where numpy's generator ends.
  want = np.empty((C, 5), np.uint64)
  for c in range(C):
    rng = O.loader_rng(c)
    rng.choice(np.arange(N), size=K * n, replace=True)
    st = rng.bit_generator.state
    s, inc = st["state"]["state"], st["state"]["inc"]
    m = (1 << 64) - 1
    want[c] = [(s >> 64) & m, s & m, (inc >> 64) & m, inc & m,
               (int(st["uinteger"]) << 32) | int(st["has_uint32"])]
  np.testing.assert_array_equal(pcg.cpu().numpy().view(np.uint64), want)


def _network(N, C, n, seed):
  import torch
  from gbsgmc import likelihoods as L, potential
  from gbsgmc.data import NumpyDataLoader
  lik = L.MLPGaussian(d_in=64, h1=1024, h2=1024, sigma=M.SIGMA)
  X, y, w_star, rng = M.teacher_data(lik, N, seed)
  W = M.chains_near(w_star, C, rng)
  idx = rng.integers(0, N, size=(C, n)).astype(np.int32)
  ds = NumpyDataLoader(x=X, y=y).device_dataset()
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), lik)
  return lik, X, y, W, idx, ds, pot, torch.from_numpy(W).cuda(), \
      torch.from_numpy(idx).cuda()


class _One:
  def __init__(self, r, c, rows=None):
    self.U = r.U[c:c + 1]
    self.grad = r.grad[c:c + 1]
    self.lk = r.lk[c:c + 1] if rows is None else r.lk[c:c + 1, :rows]
    self.lk_var = r.lk_var[c:c + 1]


def test_mlp_64_chains_at_minibatch_2048_match_oracle(lib):
  N, C, n = 100_000, 64, 2048
  lik, X, y, W, idx, ds, pot, Wd, idxd = _network(N, C, n, 31)
  r = pot.evaluate(Wd, idxd, ds, grad=True, lk=True, observation_count=N)
  pot.check_status()
  assert np.isfinite(r.grad.cpu().numpy()).all()
  for c in (0, 31, 63):
    ref = O.mlp_potential(W[c:c + 1], X, y, idx[c:c + 1], N, 64, 1024, 1024,
                          M.SIGMA, prior_scale=1.0)
    M.check(lik, _One(r, c), ref, W[c:c + 1], X, y, idx[c:c + 1], N)


def test_resgld_ladder_ragged_gradient_and_exchange_match_oracle(lib):
  import torch
  import bench
  from gbsgmc import _lib
  sizes = bench.resgld_sizes().astype(np.int32)
  R, n_max, N = sizes.size, 4096, 100_000
  lik, X, y, W, idx, ds, pot, Wd, idxd = _network(N, R, n_max, 32)
  r = pot.evaluate(Wd, idxd, ds, grad=True, lk=True, observation_count=N,
                   rows=torch.from_numpy(sizes))
  pot.check_status()
  for target in (96, 2001, 4000):
    c = int(np.nonzero(sizes == target)[0][0])
    sub = idx[c:c + 1, :sizes[c]]
    ref = O.mlp_potential(W[c:c + 1], X, y, sub, N, 64, 1024, 1024, M.SIGMA,
                          prior_scale=1.0)
    M.check(lik, _One(r, c, sizes[c]), ref, W[c:c + 1], X, y, sub, N)
  # One exchange round of the ladder on these potentials.
  ladder = (100.0 ** (np.arange(R) / (R - 1))).astype(np.float32)
  U = r.U.clone()
  var = r.lk_var.clone()
  U_np, var_np = U.cpu().numpy(), var.cpu().numpy()
  ssq_np = np.random.default_rng(5).uniform(0.5, 2.0, R - 1)
  x = Wd.clone()
  v = torch.ones_like(x)
  ssq = torch.from_numpy(ssq_np).cuda()
  flags = torch.zeros(R - 1, dtype=torch.int32, device="cuda")
  counts = torch.zeros(R - 1, dtype=torch.int32, device="cuda")
  log_s = torch.zeros(R - 1, dtype=torch.float64, device="cuda")
  every, seed, round_ = bench.RE_EVERY, 0x5EED, 3
  sch = _lib.sched(step_size=1e-4, temperature=1.0, offset=round_ * every - 1,
                   chain_temperature_dev=torch.from_numpy(ladder).cuda())
  _lib.call("gbsgmc_resgld_exchange_adjacent", R, W.shape[1], _lib.ptr(x),
            _lib.ptr(v), _lib.ptr(U), _lib.ptr(var), sch, every, _lib.ptr(ssq),
            1.0, seed, None, _lib.ptr(flags), _lib.ptr(counts), _lib.ptr(log_s),
            _lib.stream_handle())
  torch.cuda.synchronize()
  u = [O.swap_uniform(seed, k, round_) for k in range(R - 1)]
  f_ref, U_ref, var_ref, ls_ref = O.resgld_exchange_adjacent(
      U_np, var_np, ssq_np, ladder.astype(np.float64), 1.0, round_, u)
  np.testing.assert_array_equal(flags.cpu().numpy(), f_ref)
  np.testing.assert_allclose(log_s.cpu().numpy(), ls_ref, rtol=1e-12, atol=1e-12)
  np.testing.assert_array_equal(U.cpu().numpy(), U_ref)
  perm = np.arange(R)
  for k in np.nonzero(f_ref)[0]:
    perm[[k, k + 1]] = perm[[k + 1, k]]
  np.testing.assert_array_equal(x.cpu().numpy(), W[perm])
