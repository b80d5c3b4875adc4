"""Index and noise streams on the GPU vs the golden fixtures and the oracle.

Bit-exact: PCG64 index draws and stream states (numpy's own stream),
Philox index draws.  Tolerance 2e-6 (relative, plus 2e-6 absolute) for
Philox normals, whose Box-Muller runs in fp32 with CUDA's logf/sincospif.
"""

import ctypes
from pathlib import Path

import numpy as np
import pytest

from oracle import sgmc_oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def state_words(state):
  st, inc = state["state"]["state"], state["state"]["inc"]
  m = (1 << 64) - 1
  w = np.array([(st >> 64) & m, st & m, (inc >> 64) & m, inc & m,
                (int(state["uinteger"]) << 32) | int(state["has_uint32"])],
               dtype=np.uint64)
  return w.view(np.int64)


def to_state(words):
  w = np.asarray(words).view(np.uint64)
  return {"state": {"state": (int(w[0]) << 64) | int(w[1]),
                    "inc": (int(w[2]) << 64) | int(w[3])},
          "has_uint32": int(w[4]) & 0xFFFFFFFF, "uinteger": int(w[4]) >> 32}


def draw(lib, states_np, n_obs, draws, per_step, chain_stride=None,
         step_stride=None, out_shape=None):
  import torch
  from gbsgmc import _lib
  C = states_np.shape[0]
  st = torch.from_numpy(states_np.copy()).cuda()
  chain_stride = draws if chain_stride is None else chain_stride
  step_stride = per_step if step_stride is None else step_stride
  size = out_shape if out_shape is not None else (C * draws,)
  out = torch.full(size, -7, dtype=torch.int32, device="cuda")
  _lib.call("gbsgmc_index_draw_pcg64", _lib.ptr(st), C, n_obs, draws,
            per_step, _lib.ptr(out), chain_stride, step_stride, None, None)
  torch.cuda.synchronize()
  return out.cpu().numpy(), st.cpu().numpy()


def test_pcg64_draws_match_golden(lib):
  g = np.load(GOLDEN / "index_streams.npz")
  for seed in range(8):
    for N in (10_000, 1_000_000):
      for n in (128, 1024):
        key = f"s{seed}_N{N}_n{n}"
        b = g[key + "_before"].astype(np.uint64)
        words = np.array([b[0], b[1], b[2], b[3], (b[5] << np.uint64(32)) | b[4]],
                         dtype=np.uint64).view(np.int64)
        idx, st = draw(lib, words[None], N, 3 * n, n)
        np.testing.assert_array_equal(idx.reshape(3, n), g[key + "_idx"], err_msg=key)
        a = g[key + "_after"].astype(np.uint64)
        want = np.array([a[0], a[1], a[2], a[3], (a[5] << np.uint64(32)) | a[4]],
                        dtype=np.uint64).view(np.int64)
        np.testing.assert_array_equal(st[0], want, err_msg=key)


# Draw counts around the kernel's rounds of 2048 halves; N = 1,431,655,766
# rejects a third of all 32-bit values (2^32 mod N = 1,431,655,764).
@pytest.mark.parametrize("N", [1, 2, 3, 7, 1000, 999_983, 1_431_655_766, 2**31 - 1])
@pytest.mark.parametrize("draws", [1, 2, 3, 511, 512, 513, 2047, 2048, 2049, 5000,
                                   20_000])
def test_pcg64_many_chains_edge_sizes(lib, N, draws):
  C = 5
  rngs = [O.loader_rng(100 + c) for c in range(C)]
  # Chain 3 starts with a buffered half: consume one 32-bit draw first.
  rngs[3].integers(0, 10, 1, dtype=np.int64)
  states = np.stack([state_words(r.bit_generator.state) for r in rngs])
  idx, st = draw(lib, states, N, draws, draws)
  for c in range(C):
    want = rngs[c].integers(0, N, draws, dtype=np.int64)
    np.testing.assert_array_equal(idx[c * draws:(c + 1) * draws], want)
    got = to_state(st[c])
    ref = rngs[c].bit_generator.state
    assert got["state"] == ref["state"]
    assert got["has_uint32"] == ref["has_uint32"]
    if ref["has_uint32"]:
      assert got["uinteger"] == ref["uinteger"]


def test_pcg64_step_major_layout_and_continuation(lib):
  """Blocks of steps laid out [step, chain, n]; two calls == one call."""
  C, n, steps, N = 3, 64, 4, 10_000
  rngs = [O.loader_rng(c) for c in range(C)]
  states = np.stack([state_words(r.bit_generator.state) for r in rngs])
  out1, st1 = draw(lib, states, N, 2 * n, n, chain_stride=n, step_stride=C * n,
                   out_shape=(2 * C * n,))
  out2, _ = draw(lib, st1, N, 2 * n, n, chain_stride=n, step_stride=C * n,
                 out_shape=(2 * C * n,))
  got = np.concatenate([out1.reshape(2, C, n), out2.reshape(2, C, n)])
  for c in range(C):
    want = O.loader_draws(rngs[c], N, n, steps)
    np.testing.assert_array_equal(got[:, c, :], want)


def test_philox_indices_match_oracle(lib):
  import torch
  from gbsgmc import _lib
  C, steps, n, N, seed = 3, 2, 101, 999_983, 0xDEADBEEF12345
  out = torch.empty(C * steps * n, dtype=torch.int32, device="cuda")
  _lib.call("gbsgmc_index_draw_philox", seed, 5, C, 40, steps, n, N,
            _lib.ptr(out), steps * n, n, None)
  got = out.cpu().numpy().reshape(C, steps, n)
  for c in range(C):
    for s in range(steps):
      want = O.philox_indices(seed, 5 + c, 40 + s, n, N)
      np.testing.assert_array_equal(got[c, s], want)


def test_philox_normals_match_oracle(lib):
  import torch
  from gbsgmc import _lib
  C, P, seed, step, tag = 4, 1001, 77, 12345, 2
  out = torch.empty((C, P + 3), dtype=torch.float32, device="cuda")
  _lib.call("gbsgmc_philox_normal", seed, 9, C, step, tag, P, _lib.ptr(out),
            P + 3, None)
  got = out.cpu().numpy()[:, :P]
  for c in range(C):
    want = O.philox_normals(seed, 9 + c, step, tag, P)
    np.testing.assert_allclose(got[c], want, rtol=2e-6, atol=2e-6)


def test_bad_arguments_are_rejected(lib):
  from gbsgmc import _lib
  rc = lib.gbsgmc_index_draw_pcg64(None, 1, 10, 4, 4, None, 4, 4, None, None)
  assert rc == _lib.ERR_ARG
  assert b"null" in lib.gbsgmc_last_error()
  import torch
  st = torch.zeros(5, dtype=torch.int64, device="cuda")
  out = torch.zeros(4, dtype=torch.int32, device="cuda")
  rc = lib.gbsgmc_index_draw_pcg64(st.data_ptr(), 1, 0, 4, 4, out.data_ptr(),
                                   4, 4, None, None)
  assert rc == _lib.ERR_SHAPE
