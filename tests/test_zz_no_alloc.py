"""gbsgmc_sgld_glm_step_noalloc: the fused SGLD step for callers that cannot
allocate device memory (code inside another runtime's memory pool, host code
that receives device pointers but owns no allocator).  It must give what
gbsgmc_sgld_glm_step gives with a caller-allocated workspace, call after
call, although its scratch is one array inside the library that every call
reuses.

The step is forced to three CTAs per chain (GBSGMC_GLM_SLICES, read by the
library at each launch), so the partial gradients and sums really pass
through the scratch.  A larger shape runs before a smaller one, so the
smaller call starts from the tickets and partials the larger one left behind.

This file sorts last so that a run stopping at the first failure has
already run every other test.  Tolerance: the 1e-5 relative (+1e-6 absolute)
used for fp32 updates elsewhere; both paths run the same kernel, so in
practice the results are identical.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(N=20_000, d=256, C=64, n=1024, seed=11):
  rng = np.random.default_rng(seed)
  X = rng.normal(size=(N, d)).astype(np.float32)
  w = rng.normal(size=d) / np.sqrt(d)
  y = (rng.random(N) < 1 / (1 + np.exp(-(X @ w)))).astype(np.float32)
  idx = rng.integers(0, N, (2, C, n)).astype(np.int32)
  W0 = (rng.normal(size=(C, d)) * 0.05).astype(np.float32)
  return X, y, idx, W0


def _compare_two_calls(lib, shapes):
  """Runs, for each (C, n) in `shapes` in turn, two SGLD steps through the
  workspace entry point and two through the allocation-free one, and checks
  that they agree after each call."""
  import torch
  from gbsgmc import _lib, data, likelihoods as L, potential
  X, y, idx_np, W0 = _problem(C=max(c for c, _ in shapes),
                              n=max(m for _, m in shapes))
  d = X.shape[1]
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), L.Logistic())
  model, keep_alive = pot.model(loader.device_dataset())
  noise = _lib.noise(seed=7)
  stream = _lib.stream_handle()
  for C, n in shapes:
    need = lib.gbsgmc_glm_workspace_bytes(C, n, d)
    assert 0 < need <= _lib.STATIC_SCRATCH_BYTES
    idx = torch.from_numpy(np.ascontiguousarray(idx_np[:, :C, :n])).cuda()
    ws = torch.zeros(int(need), dtype=torch.uint8, device="cuda")

    def buffers():
      return dict(W=torch.from_numpy(W0[:C].copy()).cuda(),
                  V=torch.ones((C, d), dtype=torch.float32, device="cuda"),
                  U=torch.zeros(C, dtype=torch.float64, device="cuda"),
                  var=torch.zeros(C, dtype=torch.float64, device="cuda"),
                  status=torch.zeros(1, dtype=torch.int32, device="cuda"))

    a, b = buffers(), buffers()
    for call in range(2):
      sched = _lib.sched(step_size=1e-4, temperature=1.0, offset=call)
      _lib.call("gbsgmc_sgld_glm_step", model, C, n, _lib.ptr(idx[call]), n,
                _lib.ptr(a["W"]), _lib.ptr(a["V"]), 0.9, 1e-5, sched, noise,
                _lib.ptr(a["U"]), _lib.ptr(a["var"]), None, None, _lib.ptr(ws),
                ws.numel(), _lib.ptr(a["status"]), stream)
      _lib.call("gbsgmc_sgld_glm_step_noalloc", model, C, n,
                _lib.ptr(idx[call]), n, _lib.ptr(b["W"]), _lib.ptr(b["V"]),
                0.9, 1e-5, sched, noise, _lib.ptr(b["U"]), _lib.ptr(b["var"]),
                None, None, _lib.ptr(b["status"]), stream)
      torch.cuda.synchronize()
      for key in ("W", "V", "U", "var"):
        np.testing.assert_allclose(b[key].cpu().numpy(), a[key].cpu().numpy(),
                                   rtol=1e-5, atol=1e-6,
                                   err_msg=f"{key}, shape {(C, n)}, call {call}")
      assert int(a["status"].item()) == 0 and int(b["status"].item()) == 0


def test_noalloc_step_matches_workspace_step_twice(lib, monkeypatch):
  monkeypatch.setenv("GBSGMC_GLM_SLICES", "3")
  _compare_two_calls(lib, [(64, 1024)])


def test_noalloc_after_a_larger_shape(lib, monkeypatch):
  monkeypatch.setenv("GBSGMC_GLM_SLICES", "3")
  _compare_two_calls(lib, [(96, 1536), (40, 640)])


def test_noalloc_rejects_shapes_beyond_the_static_scratch(lib):
  from gbsgmc import _lib
  m = _lib.Glm(_lib.GLM_LOGISTIC, 1024, 10**6, 1024, 16, 16, 1.0, 1.0, 1.0, 0,
               10**6)
  # ABI order: model, chains, n, idx, idx_stride, w, v, alpha, lmbd, sched,
  # noise, U, lk_var, samples, sample_lik, status, stream.  Every pointer is
  # NULL, so only the scratch-size check can produce ERR_SHAPE.
  rc = lib.gbsgmc_sgld_glm_step_noalloc(m, 4096, 4096, None, 4096, None, None,
                                        0.9, 1e-5, _lib.sched(), _lib.noise(),
                                        None, None, None, None, None, None)
  assert rc == _lib.ERR_SHAPE
  assert b"static scratch" in lib.gbsgmc_last_error()
