"""The N > 1 path on the CPU: two `gloo` ranks (world size 2) each run their
shard of chains -- bench.py's `shard_chains` -- with no data-path
collective, and rank 0 gathers the samples and takes the slowest rank's
time (`max_over_ranks`).  Each chain is the oracle's SGLD(+RMSprop)
trajectory with the product's per-chain streams (PCG64 index draws seeded
with the chain id, Philox noise keyed by it), so the gathered shards must
equal one process running every chain, bit for bit.
"""

import os
import socket
from pathlib import Path

import numpy as np
import pytest

from oracle import sgmc_oracle as O

ROOT = Path(__file__).resolve().parents[1]
PER_RANK, N, D, MB, K = 3, 500, 8, 32, 5


def _problem():
  rng = np.random.default_rng(17)
  X = rng.normal(size=(N, D)).astype(np.float32)
  y = (rng.random(N) < 1 / (1 + np.exp(-X @ rng.normal(size=D)))).astype(np.float32)
  return X, y


def _chains(ids):
  """Final w of the chains `ids`, each stepped K times."""
  from gbsgmc.data.numpy_loader import chain_rng
  X, y = _problem()
  h = np.full(K, 1e-3, np.float32)
  T = np.ones(K, np.float32)
  out = []
  for c in ids:
    idx = O.loader_draws(chain_rng(c), N, MB, K)[:, None, :]
    xi = np.stack([O.philox_normals(11, c, k, 0, D) for k in range(K)])[:, None, :]
    Ws, _, _ = O.sgld_glm_trajectory(X, y, np.zeros((1, D), np.float32), idx,
                                     xi.astype(np.float32), h, T, O.LOGISTIC,
                                     1.0, 2.0)
    out.append(Ws[-1][0])
  return np.stack(out)


def _rank(rank, world, port, out_dir):
  import sys
  for p in (ROOT / "jax-sgmc_gb300", ROOT):
    sys.path.insert(0, str(p))
  import torch
  import torch.distributed as dist
  import bench
  os.environ["MASTER_ADDR"] = "127.0.0.1"
  os.environ["MASTER_PORT"] = str(port)
  dist.init_process_group("gloo", rank=rank, world_size=world)
  try:
    base, ids = bench.shard_chains(rank, PER_RANK)
    assert base == rank * PER_RANK and len(ids) == PER_RANK
    mine = torch.from_numpy(_chains(ids))
    parts = [torch.empty_like(mine) for _ in range(world)]
    dist.all_gather(parts, mine)
    slowest = bench.max_over_ranks(10.0 * (rank + 1), world, "cpu")
    if rank == 0:
      np.save(Path(out_dir) / "w.npy", torch.cat(parts).numpy())
      np.save(Path(out_dir) / "ms.npy", np.array([slowest]))
  finally:
    dist.destroy_process_group()


def _free_port():
  with socket.socket() as s:
    s.bind(("127.0.0.1", 0))
    return s.getsockname()[1]


def test_two_gloo_ranks_equal_one_process(tmp_path):
  mp = pytest.importorskip("torch.multiprocessing")
  world = 2
  mp.start_processes(_rank, args=(world, _free_port(), str(tmp_path)),
                     nprocs=world, join=True, start_method="spawn")
  got = np.load(tmp_path / "w.npy")
  want = _chains(range(world * PER_RANK))
  np.testing.assert_array_equal(got, want)
  assert np.load(tmp_path / "ms.npy")[0] == 20.0
  # Distinct chains stay distinct across the shard boundary.
  assert not np.array_equal(got[PER_RANK - 1], got[PER_RANK])
