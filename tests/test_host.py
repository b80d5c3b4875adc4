"""Host-side logic and the C ABI library on the CPU (no GPU needed)."""

import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
  text = (ROOT / "include" / "gbsgmc.h").read_text()
  text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
  return sorted(set(re.findall(r"\b(gbsgmc_[a-z0-9_]+)\s*\(", text)))


def test_library_builds_loads_and_exports_every_declared_symbol():
  from gbsgmc import _build, _lib
  _build.build()
  lib = _lib.load()
  names = declared_functions()
  assert len(names) >= 20
  for name in names:
    assert hasattr(lib, name), name
    assert name in _lib.SIGNATURES, f"{name} has no ctypes signature"
  assert lib.gbsgmc_version() == 100


def test_argument_validation_without_a_gpu():
  from gbsgmc import _lib
  lib = _lib.load()
  assert lib.gbsgmc_index_draw_pcg64(None, 1, 10, 4, 4, None, 4, 4, None,
                                     None) == _lib.ERR_ARG
  assert b"null" in lib.gbsgmc_last_error()
  assert lib.gbsgmc_glm_value_and_grad(None, 1, 1, None, 1, None, None, None,
                                       None, None, None, None, 0, None,
                                       None) == _lib.ERR_ARG
  assert lib.gbsgmc_resgld_swap_f64(-1, None, None, None, None, None, 1.0,
                                    None, None, None, 0, 0, None, None,
                                    None) == _lib.ERR_ARG
  assert lib.gbsgmc_glm_workspace_bytes(0, 1, 1) == 0
  assert lib.gbsgmc_glm_workspace_bytes(256, 1024, 256) > 256 * 1024


def test_multi_step_abi_validation_without_a_gpu():
  """gbsgmc_sgld_glm_steps rejects a step count below one, a negative
  index step stride and injected noise over several steps before touching
  the device (the pointers below are never dereferenced)."""
  import ctypes as C
  from gbsgmc import _lib
  lib = _lib.load()
  fake = C.c_void_p(4096)
  m = _lib.Glm(family=1, d=8, n_obs=100, ld=9, X=4096, y=None, sigma=1.0,
               prior_scale=1.0, temperature=1.0, y_inline=1, n_rows=100)
  sch = _lib.sched(step_size=1e-3)
  gen = _lib.noise(seed=1)
  injected = _lib.Noise(4096, 8, 0, 0, 0)

  def call(steps, stride, nz):
    return lib.gbsgmc_sgld_glm_steps(C.byref(m), 2, 16, fake, 16, stride, steps,
                                     fake, None, 0.9, 1e-5, C.byref(sch),
                                     C.byref(nz), None, None, None, None, fake,
                                     1 << 20, None, None)

  assert call(0, 32, gen) == _lib.ERR_ARG
  assert call(3, -1, gen) == _lib.ERR_ARG
  assert call(3, 32, injected) == _lib.ERR_ARG
  assert b"injected noise" in lib.gbsgmc_last_error()


def test_mlp_abi_shapes_and_validation_without_a_gpu():
  import ctypes as C
  from gbsgmc import _lib, likelihoods as L
  lib = _lib.load()
  m = _lib.Mlp(64, 1024, 1024, 1, 500_000, 500_000, 72, 16, None, 0.1, 1.0,
               1.0, 0)
  assert lib.gbsgmc_mlp_param_count(C.byref(m)) == 1_117_185
  assert L.MLPGaussian().param_count == 1_117_185
  ws = lib.gbsgmc_mlp_workspace_bytes(C.byref(m), 64, 2048)
  assert 64 * 10 * 2**20 < ws < 64 * 12 * 2**20
  assert lib.gbsgmc_mlp_workspace_bytes(C.byref(m), 64, 2000) == 0
  args = lambda n, mm=m: (C.byref(mm), 2, n, 16, n, None, 16, 16, None, None,
                          None, 256, 1 << 40, 16, None)
  assert lib.gbsgmc_mlp_value_and_grad(*args(200)) == _lib.ERR_SHAPE
  bad = _lib.Mlp(64, 1000, 1024, 1, 10, 10, 72, 16, None, 0.1, 1.0, 1.0, 0)
  assert lib.gbsgmc_mlp_value_and_grad(*args(256, bad)) == _lib.ERR_SHAPE
  neg = _lib.Mlp(64, 1024, 1024, 1, 10, 10, 72, 16, None, -0.1, 1.0, 1.0, 0)
  assert lib.gbsgmc_mlp_value_and_grad(*args(256, neg)) == _lib.ERR_ARG
  short = _lib.Mlp(64, 1024, 1024, 1, 10, 10, 64, 16, None, 0.1, 1.0, 1.0, 0)
  assert lib.gbsgmc_mlp_value_and_grad(*args(256, short)) == _lib.ERR_ARG
  # Too small a workspace is caught before anything is launched.
  small = (C.byref(m), 2, 256, 16, 256, None, 16, 16, None, None, None, 256,
           1024, 16, None)
  assert lib.gbsgmc_mlp_value_and_grad(*small) == _lib.ERR_ARG
  assert b"workspace" in lib.gbsgmc_last_error()
  with pytest.raises(ValueError):
    L.MLPGaussian(d_in=60)


def test_cnn_and_plan_abi_validation_without_a_gpu():
  import ctypes as C
  from gbsgmc import _lib, likelihoods as L
  lib = _lib.load()
  assert lib.gbsgmc_cnn_param_count() == 113_738 == L.CNNSoftmax().param_count
  assert lib.gbsgmc_cnn_workspace_bytes(8, 255) == 0
  assert lib.gbsgmc_cnn_workspace_bytes(8, 256) > 8 * 256 * 1024 * 64 * 2
  m = _lib.Cnn(1000, 1000, 3080, 16, 16 + 4 * 3072, 3080, 1.0, 1.0)
  assert lib.gbsgmc_cnn_value_and_grad(C.byref(m), 2, 7, 16, 7, None, 16, 16,
                                       None, None, None, 256, 1 << 40, 16,
                                       None) == _lib.ERR_SHAPE
  short = _lib.Cnn(1000, 1000, 1000, 16, 16, 3080, 1.0, 1.0)
  assert lib.gbsgmc_cnn_value_and_grad(C.byref(short), 2, 8, 16, 8, None, 16,
                                       16, None, None, None, 256, 1 << 40, 16,
                                       None) == _lib.ERR_ARG
  # Plans reject inconsistent integrator settings before touching the GPU.
  mlp = _lib.Mlp(64, 256, 256, 1, 100, 100, 72, 16, None, 0.1, 1.0, 1.0, 0)
  h = C.c_void_p()
  bad = _lib.Integrator(_lib.INTEGRATOR_SGHMC, 3, 0.5, 0.9, 1e-5, 0, None)
  rc = lib.gbsgmc_mlp_plan_create(C.byref(h), C.byref(mlp), 2, 128, C.byref(bad),
                                  16, 16, _lib.sched(), _lib.noise(),
                                  _lib.IndexSrc(None, 0, 0, 0), 16, None, None,
                                  50, 16)
  assert rc == _lib.ERR_ARG and b"leapfrog" in lib.gbsgmc_last_error()
  nomom = _lib.Integrator(_lib.INTEGRATOR_OBABO, 1, 0.5, 0.9, 1e-5, 0, None)
  rc = lib.gbsgmc_mlp_plan_create(C.byref(h), C.byref(mlp), 2, 128, C.byref(nomom),
                                  16, None, _lib.sched(), _lib.noise(),
                                  _lib.IndexSrc(None, 0, 0, 0), 16, None, None,
                                  50, 16)
  assert rc == _lib.ERR_ARG
  tp = _lib.Tempering(50, 0, 1.0, 7, 16, 16, 16, 16)
  rc = lib.gbsgmc_mlp_resgld_plan_create(C.byref(h), C.byref(mlp), 4, 128, 16,
                                         16, None, 0.9, 1e-5, _lib.sched(),
                                         _lib.noise(), _lib.IndexSrc(None, 0, 0, 0),
                                         C.byref(tp), 16, None, 60, 16)
  assert rc == _lib.ERR_ARG  # 60 steps per block is not a multiple of 50
  assert lib.gbsgmc_resgld_exchange_adjacent(1, 10, 16, None, 16, None,
                                             _lib.sched(), 50, 16, 1.0, 0, None,
                                             16, None, None, None) == _lib.ERR_ARG


def test_cnn_unravel_follows_sorted_keys():
  from gbsgmc import likelihoods as L, util
  lik = L.CNNSoftmax()
  flat = lik.init(np.random.default_rng(0))
  tree = lik.unravel(flat)
  again, _ = util.ravel(tree)
  np.testing.assert_array_equal(again, flat)
  assert tree["conv2"]["w"].shape == (3, 3, 32, 64)
  assert tree["linear"]["w"].shape == (2048, 10)


def test_mlp_unravel_follows_sorted_keys():
  from gbsgmc import likelihoods as L, util
  lik = L.MLPGaussian(d_in=64, h1=256, h2=512)
  flat = lik.init(np.random.default_rng(0))
  tree = lik.unravel(flat)
  assert list(tree) == sorted(tree)
  again, _ = util.ravel(tree)
  np.testing.assert_array_equal(again, flat)
  assert tree["W3"].shape == (512, 1) and tree["b3"].shape == (1,)


def test_ravel_matches_ravel_pytree_order():
  from gbsgmc import util
  tree = {"b": np.arange(6.0).reshape(2, 3), "a": np.float32(7.0),
          "c": [np.ones(2), (np.zeros(1),)]}
  flat, tdef = util.ravel(tree)
  np.testing.assert_array_equal(flat, [7, 0, 1, 2, 3, 4, 5, 1, 1, 0])
  back = util.unravel(tdef, flat)
  np.testing.assert_array_equal(back["b"], tree["b"])
  assert back["c"][1][0].shape == (1,)
  batched = util.unravel(tdef, np.stack([flat, flat + 1]))
  assert batched["b"].shape == (2, 2, 3)


class TestScheduler:
  """Ports of tests/test_scheduler.py to the host scheduler."""

  @pytest.mark.parametrize("first,last,gamma,its",
                           [(1.0, 0.01, 0.33, 100), (0.05, 0.0009, 0.55, 14723),
                            (1.0, 0.0009, 0.33, 14723), (0.05, 0.01, 0.55, 100)])
  def test_first_last(self, first, last, gamma, its):
    from gbsgmc import scheduler
    sched = scheduler.polynomial_step_size_first_last(first, last, gamma)
    state = sched.init(its)
    assert sched.get(state, 0) == pytest.approx(first, rel=1e-5)
    assert sched.get(state, its - 1) == pytest.approx(last, rel=1e-5)

  @pytest.mark.parametrize("n", [123, 243])
  def test_initial_burn_in(self, n):
    from gbsgmc import scheduler
    burn_in = scheduler.initial_burn_in(n=n)
    state, _ = burn_in.init(1000)
    for idx in range(n):
      assert burn_in.get(state, idx) == 0.0
      state = burn_in.update(state, idx)
    assert burn_in.get(state, n + 1) == 1.0

  def test_tables_keep_slots(self):
    from gbsgmc import scheduler
    ss = scheduler.polynomial_step_size_first_last(0.05, 0.001)
    bi = scheduler.initial_burn_in(30)
    th = scheduler.random_thinning(ss, bi, selections=20)
    sched = scheduler.init_scheduler(step_size=ss, burn_in=bi, thinning=th)
    h, t, keep, n_kept, static = scheduler.tables(sched, 100)
    assert n_kept == 20 == static.samples_collected
    assert np.all(keep[:30] == -1)
    assert sorted(keep[keep >= 0]) == list(range(20))
    assert h[0] == pytest.approx(0.05, rel=1e-5)
    assert np.all(t == 1.0)

  def test_random_thinning_respects_burn_in(self):
    from gbsgmc import scheduler
    accepted = np.random.default_rng(0).random(100) < 0.3
    burn_in = scheduler.specific_scheduler(lambda *a: (None, int(accepted.sum())),
                                           lambda *a, **k: None,
                                           lambda _, it, **k: float(accepted[it]))
    step = scheduler.polynomial_step_size(a=1.0, b=1.0, gamma=1.0)
    sel = int(0.5 * accepted.sum())
    thin = scheduler.random_thinning(step, burn_in, selections=sel)
    state, _ = thin.init(100)
    picked = [i for i in range(100) if thin.get(state, i)]
    assert len(picked) == sel and all(accepted[i] for i in picked)


class TestNumpyLoader:
  """Host semantics of NumpyDataLoader (tests/test_data.py)."""

  def loader(self):
    from gbsgmc.data import NumpyDataLoader
    return NumpyDataLoader(ordered_indices=np.arange(50), x=np.ones((50, 3)))

  def test_invalid_arguments_raise(self):
    from gbsgmc import data
    loader = self.loader()
    with pytest.raises(ValueError):
      loader.register_random_pipeline(cache_size=2, mb_size=51)
    with pytest.raises(ValueError):
      loader.register_random_pipeline(cache_size=2, mb_size=3, in_epochs=True)
    with pytest.raises(ValueError):
      data.random_reference_data(loader, 1, 51)
    with pytest.raises(ValueError):
      data.random_reference_data(loader, 0, 5)
    with pytest.raises(ValueError):
      data.NumpyDataLoader(a=np.zeros(3), b=np.zeros(4))

  def test_seeding(self):
    loader = self.loader()
    a1 = loader.register_random_pipeline(1, 1, seed=1)
    a2 = loader.register_random_pipeline(1, 1, seed=1)
    b = loader.register_random_pipeline(1, 1, seed=2)
    ga, gb, gc = (loader.get_batches(c)[0]["ordered_indices"] for c in (a1, a2, b))
    assert ga == gb and gc != gb

  @pytest.mark.parametrize("shuffle,in_epochs", [(False, False), (True, False), (True, True)])
  def test_cache_size_order(self, shuffle, in_epochs):
    loader = self.loader()
    small = loader.register_random_pipeline(3, 2, seed=0, shuffle=shuffle,
                                            in_epochs=in_epochs)
    big = loader.register_random_pipeline(5, 2, seed=0, shuffle=shuffle,
                                          in_epochs=in_epochs)
    sb, _ = loader.get_batches(small)
    bb, _ = loader.get_batches(big)
    np.testing.assert_array_equal(sb["ordered_indices"], bb["ordered_indices"][:3])

  @pytest.mark.parametrize("shuffle,in_epochs", [(False, False), (True, False), (True, True)])
  def test_checkpoint(self, shuffle, in_epochs):
    loader = self.loader()
    a = loader.register_random_pipeline(3, 2, shuffle=shuffle, in_epochs=in_epochs)
    for _ in range(8):
      loader.get_batches(a)
    ck = loader.save_state(a)
    want = loader.get_batches(a)
    b = loader.register_random_pipeline(3, 2, shuffle=shuffle, in_epochs=in_epochs)
    loader.load_state(b, ck)
    got = loader.get_batches(b)
    np.testing.assert_array_equal(want[0]["ordered_indices"], got[0]["ordered_indices"])
    np.testing.assert_array_equal(want[1], got[1])


def test_potential_rejects_arbitrary_callables():
  from gbsgmc import likelihoods as L, potential
  with pytest.raises(TypeError):
    potential.minibatch_potential(lambda w: 0.0, L.Logistic())
  with pytest.raises(TypeError):
    potential.minibatch_potential(L.FlatPrior(), lambda w, x: 0.0)
  with pytest.raises(NotImplementedError):
    potential.minibatch_potential(L.FlatPrior(), L.Logistic(), strategy="smap")
  with pytest.raises(ValueError):
    L.LinearGaussian(sigma=0.0)


def test_unported_presets_raise():
  from gbsgmc import adaption, integrator
  with pytest.raises(AssertionError):        # needs the potential
    adaption.fisher_information()
  # The dense noise model exists (d <= 128, on the generalised-linear families).
  adaption.fisher_information(minibatch_potential=object(), diagonal=False)
  # The dense mass exists too (up to 128 parameters).
  assert adaption.mass_matrix(diagonal=False).kind == "mass_matrix"
  with pytest.raises(NotImplementedError):   # langevin adapts with rms_prop only
    integrator.langevin_diffusion(None, (None, None, None),
                                  adaption=adaption.mass_matrix())
  with pytest.raises(NotImplementedError):   # per-parameter friction
    integrator.reversible_leapfrog(None, (None, None, None), friction=[0.1, 0.2])


def test_moments_saving_and_mass_adaption_strategy_shapes():
  from gbsgmc import adaption, io
  assert io.moments().kind == "moments"
  strat = adaption.mass_matrix(burn_in=7)
  assert strat.kind == "mass_matrix" and len(tuple(strat)[:3]) == 3


@pytest.mark.parametrize("N,mb,cache,counts", [
    (1000, 100, 3, [1, 2, 7, 15, 3, 40]),
    (1037, 64, 5, [5, 33, 1, 70]),
    (500, 500, 1, [1, 1, 3, 2]),
    (10, 3, 2, [1, 4, 9, 2]),
])
def test_take_shuffled_equals_the_per_batch_ring(N, mb, cache, counts):
  """NumpyDataLoader.take_shuffled (the bulk draw the fused plans read
  shuffled streams from) hands out the batches of
  numpy_loader.py:391-431 one call at a time would, and leaves the chain's
  generator, ring and counters where those calls would."""
  from gbsgmc import data
  from gbsgmc.data.numpy_loader import chain_rng
  from oracle import sgmc_oracle as O
  X = np.zeros((N, 2), np.float32)
  bulk, single = data.NumpyDataLoader(x=X), data.NumpyDataLoader(x=X)
  cb = bulk.register_random_pipeline(cache, mb_size=mb, shuffle=True)
  cs = single.register_random_pipeline(cache, mb_size=mb, shuffle=True)
  oracle = O.ShuffledBatches(chain_rng(cb), N, mb)
  for count in counts:
    got = bulk.take_shuffled(cb, count)
    want = np.stack([oracle.next() for _ in range(count)])
    np.testing.assert_array_equal(got, want)
    per = np.stack([single._shuffle_indices(single._chains[cs])[0]
                    for _ in range(count)])
    np.testing.assert_array_equal(got, per)
    a, b = bulk._chains[cb], single._chains[cs]
    assert (a["draws"], a["remaining_samples"]) == (b["draws"], b["remaining_samples"])
    np.testing.assert_array_equal(a["random_indices"], b["random_indices"])
    assert a["rng"].bit_generator.state == b["rng"].bit_generator.state
  # Every permutation is one: each index appears once per N entries.
  stream = O.ShuffledBatches(chain_rng(0), N, mb)
  first = np.concatenate([stream.next() for _ in range(N // mb)])
  assert len(np.unique(first)) == len(first)


def test_take_shuffled_rejects_other_pipelines():
  from gbsgmc import data
  loader = data.NumpyDataLoader(x=np.zeros((20, 1), np.float32))
  c = loader.register_random_pipeline(2, mb_size=4)
  with pytest.raises(ValueError):
    loader.take_shuffled(c, 1)
  e = loader.register_random_pipeline(2, mb_size=4, shuffle=True, in_epochs=True)
  with pytest.raises(ValueError):
    loader.take_shuffled(e, 1)


@pytest.mark.parametrize("in_epochs", [False, True])
@pytest.mark.parametrize("k", [1, 2])
def test_shuffled_feed_hands_out_each_chains_batches_in_order(k, in_epochs):
  """ShuffledFeed (the host side of a plan's external index source): per
  step and chain, the next k batches the chain's own batch function would
  use -- its cached batches, then cache-sized refills -- whatever the block
  sizes asked for."""
  import torch
  from gbsgmc import data
  from gbsgmc.data.core import CacheState, ShuffledFeed
  N, mb, C, cache = 1000, 16, 3, 5
  X = np.zeros((N, 1), np.float32)
  fed, ref = data.NumpyDataLoader(x=X), data.NumpyDataLoader(x=X)
  states, ref_states = [], []
  for _ in range(C):
    for loader, out in ((fed, states), (ref, ref_states)):
      cid = loader.register_random_pipeline(cache, mb_size=mb, shuffle=True,
                                            in_epochs=in_epochs)
      idx, _ = loader._get_indices(cid)
      out.append(CacheState(cached_batches=torch.from_numpy(idx.astype(np.int32)),
                            cached_batches_count=cache, current_line=0,
                            chain_id=cid))
  assert ShuffledFeed.qualifies(fed, states)
  feed = ShuffledFeed(fed, states, k)
  try:
    got = np.concatenate([feed.next(s).copy() for s in (3, 7, 1, 12)])
  finally:
    feed.close()
  for c in range(C):
    batches = list(ref_states[c].cached_batches.numpy())
    while len(batches) < got.shape[0] * k:
      idx, _ = ref._get_indices(ref_states[c].chain_id)
      batches += list(idx)
    want = np.array(batches[:got.shape[0] * k]).reshape(got.shape[0], k * mb)
    np.testing.assert_array_equal(got[:, c, :], want)


@pytest.mark.parametrize("N,mb,counts", [(1000, 64, [1, 5, 16, 40, 3]),
                                         (96, 32, [2, 3, 7]), (50, 50, [1, 4])])
def test_take_in_epochs_equals_the_per_batch_epochs(N, mb, counts):
  """NumpyDataLoader.take_in_epochs hands out what _shuffle_in_epochs
  (numpy_loader.py:433-460) does one call at a time -- a permutation per
  epoch of ceil(N / mb) batches, the last batch ending with ring entries
  past N -- and leaves the same chain state."""
  from gbsgmc import data
  X = np.zeros((N, 1), np.float32)
  bulk, single = data.NumpyDataLoader(x=X), data.NumpyDataLoader(x=X)
  cb = bulk.register_random_pipeline(2, mb_size=mb, shuffle=True, in_epochs=True)
  cs = single.register_random_pipeline(2, mb_size=mb, shuffle=True, in_epochs=True)
  for count in counts:
    got = bulk.take_in_epochs(cb, count)
    want = np.stack([single._shuffle_in_epochs(single._chains[cs])[0]
                     for _ in range(count)])
    np.testing.assert_array_equal(got, want)
    a, b = bulk._chains[cb], single._chains[cs]
    assert a["draws"] == b["draws"]
    np.testing.assert_array_equal(a["random_indices"], b["random_indices"])
    assert a["rng"].bit_generator.state == b["rng"].bit_generator.state
  with pytest.raises(ValueError):
    bulk.take_in_epochs(bulk.register_random_pipeline(2, mb_size=mb, shuffle=True), 1)


def test_statistics_fisher_and_external_index_abi_validation_without_a_gpu():
  """The sample-statistics, Fisher and external-index entry points reject
  bad arguments on the host, before any device work."""
  import ctypes as C
  from gbsgmc import _lib
  lib = _lib.load()
  # Moments: negative chains, a chain stride below P, n < 1.
  assert lib.gbsgmc_moments_accumulate(-1, 10, 1, 16, 10, 10, 0, 16, 16, 16,
                                       None) == _lib.ERR_ARG
  assert lib.gbsgmc_moments_accumulate(2, 10, 1, 16, 20, 5, 0, 16, 16, 16,
                                       None) == _lib.ERR_ARG
  assert lib.gbsgmc_moments_accumulate(2, 10, 0, None, 0, 0, 0, None, None, None,
                                       None) == _lib.OK   # nothing to add
  assert lib.gbsgmc_moments_finalize(2, 10, 0, 16, 16, 16, 16, 16, None) == _lib.ERR_ARG
  # Mass adaption counts updates from 1.
  assert lib.gbsgmc_mass_adapt(10, 0, 5, 16, 16, 16, 16, 16, None, None) == _lib.ERR_ARG
  # Fisher noise: null model, a minibatch of one row, an unknown family.
  assert lib.gbsgmc_glm_fisher_noise(None, 1, 8, 16, 8, 16, 16, None, 1.0, 0.1, 16,
                                     None, 16, None) == _lib.ERR_ARG
  glm = _lib.Glm()
  glm.family, glm.d, glm.n_obs, glm.ld, glm.X, glm.y = _lib.GLM_LOGISTIC, 4, 100, 4, 16, 16
  assert lib.gbsgmc_glm_fisher_noise(C.byref(glm), 1, 1, 16, 1, 16, 16, None, 1.0,
                                     0.1, 16, None, 16, None) == _lib.ERR_SHAPE
  glm.family = 9
  assert lib.gbsgmc_glm_fisher_noise(C.byref(glm), 1, 8, 16, 8, 16, 16, None, 1.0,
                                     0.1, 16, None, 16, None) == _lib.ERR_ARG
  assert lib.gbsgmc_sghmc_momentum_noise_model(1, 10, None, 16, 16, _lib.sched(),
                                               _lib.noise(), None) == _lib.ERR_ARG
  # External indices need a plan created with an external source.
  assert lib.gbsgmc_plan_set_indices(None, 16, 1, None) == _lib.ERR_ARG
  # A replica-exchange plan does not take an external source.
  mlp = _lib.Mlp(64, 256, 256, 1, 100, 100, 72, 16, None, 0.1, 1.0, 1.0, 0)
  tp = _lib.Tempering(50, 0, 1.0, 7, 16, 16, 16, 16)
  h = C.c_void_p()
  rc = lib.gbsgmc_mlp_resgld_plan_create(C.byref(h), C.byref(mlp), 4, 128, 16,
                                         16, None, 0.9, 1e-5, _lib.sched(),
                                         _lib.noise(), _lib.IndexSrc(None, 0, 0, 1),
                                         C.byref(tp), 16, None, 50, 16)
  assert rc == _lib.ERR_UNSUPPORTED


def test_bulk_pcg64_seeding_equals_numpy():
  """pcg64_words_many restates SeedSequence(seed).spawn(1)[0] -> PCG64 for
  many seeds at once; it must give numpy's own states bit for bit."""
  from gbsgmc.data.numpy_loader import pcg64_words, pcg64_words_many
  seeds = list(range(600)) + [2**31 - 1, 2**32 - 1, 2**32, 2**40 + 7,
                              2**63 + 11, 2**64 + 3, 2**100 + 12345,
                              2**128 - 1, 2**128, 2**130 + 5]
  got = pcg64_words_many(seeds)
  want = np.array([pcg64_words(s) for s in seeds], np.uint64)
  np.testing.assert_array_equal(got, want)
  assert pcg64_words_many([]).shape == (0, 5)


def test_bulk_pipeline_registration_equals_one_by_one():
  from gbsgmc import data
  X = np.random.default_rng(0).normal(size=(500, 3)).astype(np.float32)
  a = data.NumpyDataLoader(x=X)
  b = data.NumpyDataLoader(x=X)
  a.register_random_pipeline(4, mb_size=7)          # chains before the bulk
  b.register_random_pipeline(4, mb_size=7)
  ids = [a.register_random_pipeline(4, mb_size=7) for _ in range(5)]
  got_ids, words = b.register_random_pipelines(5, 4, mb_size=7)
  assert list(got_ids) == ids
  for c in ids:
    st = a._chains[c]["rng"].bit_generator.state
    s, inc = st["state"]["state"], st["state"]["inc"]
    w = words[c - 1]
    assert (int(w[0]) << 64 | int(w[1])) == s and (int(w[2]) << 64 | int(w[3])) == inc
    # The lazily built generator and the checkpoint are the one-by-one ones.
    assert a.save_state(c) == b.save_state(c)
    np.testing.assert_array_equal(a.get_batches(c)[0]["x"], b.get_batches(c)[0]["x"])
  with pytest.raises(ValueError):
    b.register_random_pipelines(2, 4, mb_size=7, shuffle=True)
  with pytest.raises(ValueError):
    b.register_random_pipelines(2, 4, mb_size=501)


def test_ravel_many_and_unraveler_match_ravel_and_unravel():
  from gbsgmc import util
  rng = np.random.default_rng(1)
  trees = [{"w": rng.normal(size=(3, 2)), "b": rng.normal(size=4).astype(np.float32)}
           for _ in range(6)]
  flat, tdef = util.ravel_many(trees)
  assert flat.dtype == np.float32 and flat.shape == (6, 10)
  for c, t in enumerate(trees):
    one, d = util.ravel(t)
    np.testing.assert_array_equal(flat[c], one)
  f = util.unraveler(tdef)
  stacked = np.stack([flat, 2 * flat])          # leading axes as in [S, P]
  for k, v in util.unravel(tdef, stacked).items():
    np.testing.assert_array_equal(f(stacked)[k], v)
  nested = [{"a": [np.ones(2), np.zeros(1)]} for _ in range(3)]
  flat2, _ = util.ravel_many(nested)
  np.testing.assert_array_equal(flat2, np.tile([1, 1, 0], (3, 1)))
  with pytest.raises(ValueError):
    util.ravel_many([{"w": np.ones(2)}, {"v": np.ones(2)}])
  with pytest.raises(ValueError):
    util.ravel_many([{"w": np.ones(2)}, {"w": np.ones(3)}])


def test_pcg64_seed_in_c_matches_numpy():
  """gbsgmc_pcg64_seed (the library's host restatement of SeedSequence
  mixing and PCG64 seeding) gives the words of numpy's own fresh
  generators, for seeds below 2**32, below 2**64 and up to 2**128."""
  import numpy as np
  from gbsgmc.data import numpy_loader as nl
  rng = np.random.default_rng(4)
  seeds = list(range(0, 300)) + [2**32 - 1, 2**32, 2**40 + 7, 2**63 + 5, 2**64 - 1, 2**64,
                                 2**100 + 3, 2**128 - 1]
  seeds += [int(x) for x in rng.integers(0, 2**63, size=50)]
  fast = nl.pcg64_words_fast(seeds)
  np.testing.assert_array_equal(fast, nl.pcg64_words_many(seeds))
  for s in seeds[::7] + seeds[-12:]:
    np.testing.assert_array_equal(fast[seeds.index(s)], np.array(nl.pcg64_words(s), np.uint64))


def test_seeding_and_bf16_gemm_validation_without_a_gpu():
  """gbsgmc_pcg64_seed rejects a negative count and missing buffers (a zero
  count is a no-op), and gbsgmc_gemm_bf16_c16 rejects a C it cannot write
  with TMA store boxes -- a row stride that is not a multiple of 8 elements,
  a C that is not 16-byte aligned -- before touching the device (the
  pointers are never dereferenced)."""
  from gbsgmc import _lib
  lib = _lib.load()
  assert lib.gbsgmc_pcg64_seed(None, None, -1, None) == _lib.ERR_ARG
  assert lib.gbsgmc_pcg64_seed(None, None, 3, None) == _lib.ERR_ARG
  assert b"null" in lib.gbsgmc_last_error()
  assert lib.gbsgmc_pcg64_seed(None, None, 0, None) == 0

  def gemm(C_ptr, ldc):
    return lib.gbsgmc_gemm_bf16_c16(0, 0, 4096, 128, 128 * 128, 4096, 128,
                                    128 * 128, C_ptr, ldc, 128 * ldc, 2, 128,
                                    128, 128, 4096, None)

  assert gemm(8192, 100) == _lib.ERR_ARG
  assert b"multiples of 8" in lib.gbsgmc_last_error()
  assert gemm(8192 + 8, 128) == _lib.ERR_SHAPE
  assert b"16-byte" in lib.gbsgmc_last_error()


def test_postprocess_chains_shared_layout_equals_per_chain_unravel():
  """The result dicts built from per-leaf views of the host buffer (all
  chains share one tree definition) equal those of the general path, which
  unravels each chain with its own definition (forced here by equal but
  distinct definition objects), for host saving and for no saving."""
  import torch
  from gbsgmc import io, util
  rng = np.random.default_rng(5)
  tree = {"w": np.zeros((3, 4), np.float32), "b": np.zeros(5, np.float32),
          "s": np.zeros((), np.float32)}
  flat, td = util.ravel(tree)
  count, C, P = 6, 4, flat.size
  variables = torch.from_numpy(rng.normal(size=(count, C, P)).astype(np.float32))
  extras = {"likelihood": torch.from_numpy(rng.normal(size=(count, C)))}
  states = [None] * C
  distinct = [util.ravel(tree)[1] for _ in range(C)]
  for make_saving in (lambda: io.save(io.MemoryCollector()), io.no_save):
    fast = io.postprocess_chains(make_saving(), count, variables, [td] * C, extras, states)
    slow = io.postprocess_chains(make_saving(), count, variables, distinct, extras, states)
    assert len(fast) == len(slow) == C
    for a, b in zip(fast, slow):
      assert a["sample_count"] == b["sample_count"] == count
      va, vb = a["samples"]["variables"], b["samples"]["variables"]
      assert sorted(va) == sorted(vb) == ["b", "s", "w"]
      for k in va:
        assert va[k].shape == vb[k].shape
        np.testing.assert_array_equal(va[k], vb[k])
      np.testing.assert_array_equal(a["samples"]["likelihood"], b["samples"]["likelihood"])
    # chain 1's first sample is row (0, 1) of the buffer in ravel order
    v = fast[1]["samples"]["variables"]
    again, _ = util.ravel({k: v[k][0] for k in v})
    np.testing.assert_array_equal(again, variables[0, 1].numpy())


def test_pcg64_seed_above_2_128_takes_the_numpy_restatement():
  """Seeds of 2**128 and above (more than four entropy words) are outside
  the C function's range; pcg64_words_fast then gives the numpy
  restatement's words, which equal numpy's own generators."""
  from gbsgmc.data import numpy_loader as nl
  seeds = [2**128, 2**200 + 5, 3]
  fast = nl.pcg64_words_fast(seeds)
  np.testing.assert_array_equal(fast, nl.pcg64_words_many(seeds))
  for i, s in enumerate(seeds):
    np.testing.assert_array_equal(fast[i], np.array(nl.pcg64_words(s), np.uint64))
