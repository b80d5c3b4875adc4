"""Numpy data loaders (mirrors jax_sgmc/data/numpy_loader.py).

``NumpyDataLoader`` keeps the reference's host semantics -- one numpy
``Generator(PCG64)`` per registered chain, seeded with
``SeedSequence(seed).spawn(1)[0]`` and ``seed`` defaulting to the chain id
(numpy_loader.py:231-282), checkpointable through ``save_state`` /
``load_state`` -- and additionally exposes its arrays resident in HBM.  The
GPU draws of :mod:`gbsgmc.data.core` continue each chain's PCG64 stream
bit for bit, so host ``get_batches`` and device draws see the same indices.

``DeviceNumpyDataLoader`` draws indices with Philox4x32-10 on the device
(the reference uses ``jax.random.randint``, numpy_loader.py:128-141, whose
threefry stream is not reproduced).
"""

from __future__ import annotations

import itertools
import math
from copy import deepcopy
from typing import Any, Dict, List, Tuple

import numpy as onp

from .core import (DeviceDataLoader, HostDataLoader, DataLoader,
                   MiniBatchInformation)

PyTree = Any


def chain_rng(seed: int) -> onp.random.Generator:
  """The index stream of a chain registered with ``seed``: numpy's PCG64
  seeded with ``SeedSequence(seed).spawn(1)[0]`` (numpy_loader.py:261-265)."""
  return onp.random.default_rng(onp.random.SeedSequence(seed).spawn(1)[0])


def pcg64_words(seed: int) -> List[int]:
  """The five 64-bit words of ``gbsgmc_pcg64`` (state high/low, increment
  high/low, buffered half) of :func:`chain_rng`'s fresh generator."""
  st = chain_rng(seed).bit_generator.state
  s, inc = st["state"]["state"], st["state"]["inc"]
  m = (1 << 64) - 1
  return [(s >> 64) & m, s & m, (inc >> 64) & m, inc & m,
          (int(st["uinteger"]) << 32) | int(st["has_uint32"])]


class NumpyBase(DataLoader):

  def __init__(self, on_device: bool = True, copy=True, **reference_data):
    super().__init__()
    observation_counts = []
    self._reference_data = {}
    for name, array in reference_data.items():
      observation_counts.append(len(array))
      self._reference_data[name] = onp.array(array, copy=copy)
    if observation_counts:
      if onp.any(onp.array(observation_counts) != observation_counts[0]):
        raise ValueError("All reference_data arrays must have the same length "
                         "in the first dimension.")
      self._observation_count = observation_counts[0]
    else:
      self._observation_count = 0

  @property
  def reference_data(self):
    """Returns the reference data as a dictionary."""
    return self._reference_data

  @property
  def _format(self):
    return {name: (tuple(int(s) for s in a.shape[1:]), a.dtype)
            for name, a in self._reference_data.items()}

  @property
  def static_information(self):
    return {"observation_count": self._observation_count}


class DeviceNumpyDataLoader(NumpyBase, DeviceDataLoader):
  """Whole dataset in HBM; random draws by Philox on the device."""

  def __init__(self, copy=True, **reference_data):
    super().__init__(on_device=True, copy=copy, **reference_data)

  def init_random_data(self, *args, **kwargs) -> PyTree:
    del args
    key = kwargs.get("key", 0)
    key = onp.asarray(key, dtype=onp.uint64).ravel()
    seed = 0
    for k in key:
      seed = ((seed << 32) | (int(k) & 0xFFFFFFFF)) & ((1 << 64) - 1)
    return seed

  def get_random_data(self, state, batch_size):
    raise NotImplementedError("use data.random_reference_data: draws happen "
                              "on the device inside the batch function")

  def get_full_data(self) -> Dict:
    return self._reference_data


def _ring_read(ring, start, length):
  """ring[(start + arange(length)) % len(ring)] as at most two slices."""
  R = len(ring)
  start %= R
  first = min(length, R - start)
  if first == length:
    return ring[start:start + length].copy()
  return onp.concatenate([ring[start:], ring[:length - first]])


def _ring_write(ring, start, values):
  """ring[(start + arange(len(values))) % len(ring)] = values, as slices
  (values no longer than the ring)."""
  R = len(ring)
  start %= R
  first = min(len(values), R - start)
  ring[start:start + first] = values[:first]
  ring[:len(values) - first] = values[first:]


class NumpyDataLoader(NumpyBase, HostDataLoader):
  """Load complete dataset into memory from multiple numpy arrays."""

  def __init__(self, copy=True, **reference_data):
    super().__init__(on_device=False, copy=copy, **reference_data)
    self._chains: List = []

  def save_state(self, chain_id: int) -> PyTree:
    chain_data = self._chains[chain_id]
    if chain_data['type'] == 'random':
      data = {key: deepcopy(value)
              for key, value in chain_data.items() if key != 'rng'}
      return {'random': (chain_data['rng'].bit_generator.state, data)}
    elif chain_data['type'] == 'ordered':
      return {'ordered': chain_data['idx_offset']}
    raise ValueError(f"Chain type {chain_data['type']} is unknown.")

  def load_state(self, chain_id: int, data) -> None:
    kind, value = data.popitem()
    if kind == 'random':
      rng_state, chain_data = value
      self._chains[chain_id]['rng'].bit_generator.state = rng_state
      for key, val in chain_data.items():
        self._chains[chain_id][key] = val
    elif kind == 'ordered':
      self._chains[chain_id]['idx_offset'] = value
    else:
      raise ValueError(f"Chain type {kind} is unknown.")

  def register_random_pipeline(self, cache_size: int = 1, mb_size: int = None,
                               in_epochs: bool = False, shuffle: bool = False,
                               **kwargs: Any) -> int:
    """Registers a random chain (numpy_loader.py:231-282)."""
    if mb_size > self._observation_count:
      raise ValueError(f"The batch size cannot be bigger than the observation "
                       f"count. Provided {mb_size} and "
                       f"{self._observation_count}")
    if not shuffle and in_epochs:
      raise ValueError("in_epochs = True can only be used for shuffle = True.")
    chain_id = len(self._chains)
    seed = kwargs.get("seed", chain_id)
    rng = chain_rng(seed)
    self._chains.append({'type': 'random', 'rng': rng, 'idx_offset': None,
                         'in_epochs': in_epochs, 'shuffle': shuffle,
                         'remaining_samples': 0,
                         'draws': math.ceil(self._observation_count / mb_size),
                         'random_indices': None, 'mb_size': mb_size,
                         'cache_size': cache_size})
    return chain_id

  def register_ordered_pipeline(self, cache_size: int = 1, mb_size: int = None,
                                **kwargs) -> int:
    assert mb_size <= self._observation_count, \
      (f"The batch size cannot be bigger than the observation count. Provided "
       f"{mb_size} and {self._observation_count}")
    chain_id = len(self._chains)
    self._chains.append({'type': 'ordered', 'rng': None, 'idx_offset': 0,
                         'mb_size': mb_size, 'cache_size': cache_size})
    return chain_id

  def get_batches(self, chain_id: int):
    """Host gather of ``cache_size`` batches (numpy_loader.py:314-340)."""
    selections_idx, selections_mask = self._get_indices(chain_id)
    selected = {}
    for key, data in self._reference_data.items():
      selected[key] = data[selections_idx]
    return selected, onp.array(selections_mask, dtype=onp.bool_)

  def _get_indices(self, chain_id: int):
    chain = self._chains[chain_id]
    if chain['type'] == 'ordered':
      index_fn = self._ordered_indices
    elif chain['in_epochs']:
      index_fn = self._shuffle_in_epochs
    elif chain['shuffle']:
      index_fn = self._shuffle_indices
    else:
      index_fn = self._draw_indices
    indices, masks = list(zip(*[index_fn(chain)
                                for _ in range(chain['cache_size'])]))
    return onp.array(indices), onp.array(masks, dtype=onp.bool_)

  def _ordered_indices(self, chain):
    idcs = onp.arange(chain['mb_size']) + chain['idx_offset']
    mask = idcs < self._observation_count
    if chain['idx_offset'] + chain['mb_size'] >= self._observation_count:
      chain['idx_offset'] = 0
    else:
      chain['idx_offset'] += chain['mb_size']
    return onp.mod(idcs, self._observation_count), mask

  def _draw_indices(self, chain):
    selections = chain['rng'].choice(onp.arange(0, self._observation_count),
                                     size=chain['mb_size'], replace=True)
    return selections, onp.ones(chain['mb_size'], dtype=onp.bool_)

  def _shuffle_indices(self, chain):
    floor_draws = math.floor(self._observation_count / chain['mb_size'])
    ceil_draws = floor_draws + 2
    if chain['remaining_samples'] < chain['mb_size']:
      new_indices = chain['rng'].choice(onp.arange(0, self._observation_count),
                                        size=self._observation_count,
                                        replace=False)
      if chain['random_indices'] is None:
        chain['draws'] = 0
        chain['random_indices'] = onp.zeros(ceil_draws * chain['mb_size'],
                                            dtype=onp.int_)
      update_idxs = onp.mod(onp.arange(self._observation_count)
                            + chain['draws'] * chain['mb_size']
                            + chain['remaining_samples'],
                            ceil_draws * chain['mb_size'])
      chain['random_indices'][update_idxs] = new_indices
      chain['remaining_samples'] += self._observation_count
    mask = onp.ones(chain['mb_size'], dtype=onp.bool_)
    selections_idxs = onp.mod(onp.arange(chain['mb_size'])
                              + chain['draws'] * chain['mb_size'],
                              chain['mb_size'] * ceil_draws)
    selections = onp.copy(chain['random_indices'][selections_idxs])
    chain['draws'] = (chain['draws'] + 1) % ceil_draws
    chain['remaining_samples'] -= chain['mb_size']
    return selections, mask

  def take_in_epochs(self, chain_id: int, count: int) -> onp.ndarray:
    """``count`` consecutive minibatches ``[count, mb_size]`` of an in-epoch
    pipeline (shuffle=True, in_epochs=True), leaving the chain's state as
    ``count`` calls of ``_shuffle_in_epochs`` (numpy_loader.py:433-460)
    would: a new permutation at the start of each epoch of ceil(N / mb)
    batches, the batches read in order from the ring (whose entries past N
    are never written, so the last batch of an epoch ends with them)."""
    chain = self._chains[chain_id]
    if not chain['in_epochs'] or chain['type'] != 'random':
      raise ValueError("take_in_epochs needs an in_epochs=True pipeline")
    N, mb = self._observation_count, chain['mb_size']
    epoch = math.ceil(N / mb)
    out = onp.empty((int(count), mb), dtype=onp.int_)
    done = 0
    while done < count:
      if chain['draws'] == epoch:
        perm = chain['rng'].choice(onp.arange(0, N), size=N, replace=False)
        if chain['random_indices'] is None:
          chain['random_indices'] = onp.zeros(epoch * mb, dtype=onp.int_)
        chain['random_indices'][0:N] = perm
        chain['draws'] = 0
      d = chain['draws']
      m = min(count - done, epoch - d)
      out[done:done + m] = chain['random_indices'][mb * d:mb * (d + m)].reshape(m, mb)
      chain['draws'] = d + m
      done += m
    return out

  def take_shuffled(self, chain_id: int, count: int) -> onp.ndarray:
    """``count`` consecutive minibatches ``[count, mb_size]`` of a shuffled
    pipeline (shuffle=True, in_epochs=False), leaving the chain's state --
    generator, ring, draws, remaining -- exactly as ``count`` calls of
    ``_shuffle_indices`` would.

    Those calls hand out the concatenation of successive permutations
    ``rng.choice(arange(N), N, replace=False)`` in pieces of mb: the ring of
    (floor(N/mb) + 2) mb >= N + mb entries never overwrites an unread entry,
    a permutation is appended at the write head whenever fewer than mb
    entries are unread, and after `count` calls ceil((count mb - r0) / N)
    permutations have been appended (r0 the unread entries before).  So the
    batches are the unread entries followed by those permutations, cut into
    pieces of mb, and the ring receives each permutation at the position
    the per-call code would write it to."""
    chain = self._chains[chain_id]
    if not chain['shuffle'] or chain['in_epochs'] or chain['type'] != 'random':
      raise ValueError("take_shuffled needs a shuffle=True, in_epochs=False "
                       "random pipeline")
    N, mb = self._observation_count, chain['mb_size']
    ceil_draws = N // mb + 2
    R = ceil_draws * mb
    count = int(count)
    if count <= 0:
      return onp.empty((0, mb), dtype=onp.int_)
    r0 = chain['remaining_samples']
    ring = chain['random_indices']
    d0 = chain['draws'] if ring is not None else 0
    need = count * mb
    k = max(0, -((r0 - need) // N))   # ceil((need - r0) / N), at least 0
    if ring is None:
      ring = onp.zeros(R, dtype=onp.int_)
      chain['random_indices'] = ring
    parts = [_ring_read(ring, d0 * mb, r0)]
    head = d0 * mb + r0
    for t in range(k):
      perm = chain['rng'].choice(onp.arange(0, N), size=N, replace=False)
      _ring_write(ring, head + t * N, perm)
      parts.append(perm)
    stream = onp.concatenate(parts)[:need]
    chain['draws'] = (d0 + count) % ceil_draws
    chain['remaining_samples'] = r0 + k * N - need
    return stream.reshape(count, mb)

  def _shuffle_in_epochs(self, chain):
    ceil_draws = math.ceil(self._observation_count / chain['mb_size'])
    if chain['draws'] == ceil_draws:
      new_indices = chain['rng'].choice(onp.arange(0, self._observation_count),
                                        size=self._observation_count,
                                        replace=False)
      if chain['random_indices'] is None:
        chain['draws'] = 0
        chain['random_indices'] = onp.zeros(ceil_draws * chain['mb_size'],
                                            dtype=onp.int_)
      chain['random_indices'][0:self._observation_count] = new_indices
      chain['draws'] = 0
    start_idx = chain['mb_size'] * chain['draws']
    end_idx = chain['mb_size'] * (chain['draws'] + 1)
    mask = onp.arange(start_idx, end_idx) < self._observation_count
    selections = onp.copy(chain['random_indices'][start_idx:end_idx])
    chain['draws'] += 1
    return selections, mask
