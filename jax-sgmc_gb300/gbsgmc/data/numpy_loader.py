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


# numpy's SeedSequence is M. O'Neill's seed_seq_fe entropy mixer ("Developing
# a seed_seq Alternative", 2015) over a pool of four 32-bit words; these are
# its published hash and mix constants.
_SS_INIT_A, _SS_MULT_A = 0x43B0D7E5, 0x931E8875
_SS_INIT_B, _SS_MULT_B = 0x8B51F9DD, 0x58F38DED
_SS_MIX_L, _SS_MIX_R = 0xCA01F9DD, 0x4973F715
_PCG64_MULT = 0x2360ED051FC65DA44385DF649FCCF645   # PCG's 128-bit LCG multiplier
_M32, _M64, _M128 = (1 << 32) - 1, (1 << 64) - 1, (1 << 128) - 1


def pcg64_words_fast(seeds) -> onp.ndarray:
  """:func:`pcg64_words_many` through the library's host function
  ``gbsgmc_pcg64_seed`` (the same mixing in C, about a microsecond for a few
  hundred chains); :func:`pcg64_words_many` itself when the library is not
  loaded or a seed is negative or of 2**128 and above."""
  seeds = [int(s) for s in seeds]
  if not seeds or any(s < 0 or s >> 128 for s in seeds):
    return pcg64_words_many(seeds)
  try:
    from .. import _lib
    lib = _lib.load()
  except Exception:   # no library in this process: the numpy restatement
    return pcg64_words_many(seeds)
  lo = onp.array([s & _M64 for s in seeds], onp.uint64)
  hi = onp.array([s >> 64 for s in seeds], onp.uint64)
  out = onp.empty((len(seeds), 5), onp.uint64)
  rc = lib.gbsgmc_pcg64_seed(lo.ctypes.data, hi.ctypes.data, len(seeds), out.ctypes.data)
  if rc != 0:
    raise _lib.GbsgmcError(rc, "gbsgmc_pcg64_seed")
  return out


def pcg64_words_many(seeds) -> onp.ndarray:
  """:func:`pcg64_words` of many chains at once, ``[C, 5]`` uint64.

  The seed hashing runs vectorised over the chains: each chain's assembled
  entropy is its seed as four little-endian 32-bit words followed by the
  spawn key word 0 (``SeedSequence(seed).spawn(1)[0]``); the pool is mixed
  as seed_seq_fe does and four 64-bit words are generated from it, which
  seed PCG64 as numpy does (state = 0, inc = 2 initseq + 1, one step,
  state += initstate, one step).  Seeds of 2**128 and above (more entropy
  words than the pool) fall back to numpy per chain."""
  seeds = [int(s) for s in seeds]
  C = len(seeds)
  if C == 0:
    return onp.zeros((0, 5), onp.uint64)
  if any(s < 0 or s >> 128 for s in seeds):
    return onp.array([pcg64_words(s) for s in seeds], dtype=onp.uint64)
  u32 = onp.uint32
  if all(s >> 32 == 0 for s in seeds):
    ent = [onp.array(seeds, u32)] + [onp.zeros(C, u32) for _ in range(3)]
  else:
    ent = [onp.array([(s >> (32 * k)) & _M32 for s in seeds], u32)
           for k in range(4)]
  ent.append(onp.zeros(C, u32))                      # the spawn key (0,)
  with onp.errstate(over="ignore"):
    h = [_SS_INIT_A]

    def hashmix(v):
      v = v ^ u32(h[0])
      h[0] = (h[0] * _SS_MULT_A) & _M32
      v = v * u32(h[0])
      return v ^ (v >> u32(16))

    def mix(x, y):
      r = u32(_SS_MIX_L) * x - u32(_SS_MIX_R) * y
      return r ^ (r >> u32(16))

    pool = [hashmix(ent[i]) for i in range(4)]
    for i_src in range(4):
      for i_dst in range(4):
        if i_src != i_dst:
          pool[i_dst] = mix(pool[i_dst], hashmix(pool[i_src]))
    for i_dst in range(4):
      pool[i_dst] = mix(pool[i_dst], hashmix(ent[4]))
    hb = _SS_INIT_B
    words = []
    for i in range(8):
      v = pool[i % 4] ^ u32(hb)
      hb = (hb * _SS_MULT_B) & _M32
      v = v * u32(hb)
      words.append((v ^ (v >> u32(16))).astype(onp.uint64))
    # generate_state(4, uint64) pairs the words little-endian: 64-bit word k
    # is words[2k] | words[2k+1] << 32; initstate = w0 << 64 | w1 and
    # initseq = w2 << 64 | w3.  As 32-bit limbs, least significant first:
    init = [words[2], words[3], words[0], words[1]]
    seq = [words[6], words[7], words[4], words[5]]
    m32 = onp.uint64(_M32)
    one, s31, s32 = onp.uint64(1), onp.uint64(31), onp.uint64(32)
    # inc = 2 initseq + 1 (mod 2**128)
    inc = [((seq[0] << one) | one) & m32]
    inc += [((seq[k] << one) | (seq[k - 1] >> s31)) & m32 for k in range(1, 4)]
    # state = (inc + initstate) * MULT + inc (mod 2**128), limb by limb.
    a, carry = [], onp.zeros(C, onp.uint64)
    for k in range(4):
      t = inc[k] + init[k] + carry
      a.append(t & m32)
      carry = t >> s32
    mult = [onp.uint64((_PCG64_MULT >> (32 * k)) & _M32) for k in range(4)]
    acc = [onp.zeros(C, onp.uint64) for _ in range(4)]
    for i in range(4):
      for j in range(4 - i):
        prod = a[i] * mult[j]                 # < 2**64
        acc[i + j] += prod & m32
        if i + j + 1 < 4:
          acc[i + j + 1] += prod >> s32       # each limb sums < 2**35
    state, carry = [], onp.zeros(C, onp.uint64)
    for k in range(4):
      t = acc[k] + inc[k] + carry
      state.append(t & m32)
      carry = t >> s32
  out = onp.zeros((C, 5), onp.uint64)
  out[:, 0] = (state[3] << s32) | state[2]
  out[:, 1] = (state[1] << s32) | state[0]
  out[:, 2] = (inc[3] << s32) | inc[2]
  out[:, 3] = (inc[1] << s32) | inc[0]
  return out


class _RandomChain(dict):
  """A random chain's record whose numpy Generator (``'rng'``) is built
  from its seed on first use.  Chains registered in bulk start with their
  PCG64 words alone; the record's items are those of a chain registered
  one by one."""

  __slots__ = ("seed",)

  def __missing__(self, key):
    if key == "rng":
      rng = chain_rng(self.seed)
      self["rng"] = rng
      return rng
    raise KeyError(key)


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

  def register_random_pipelines(self, count: int, cache_size: int = 1,
                                mb_size: int = None, **kwargs: Any):
    """Registers ``count`` random chains at once, as ``count`` calls of
    :meth:`register_random_pipeline` with the same arguments would (the same
    chain ids and seeds, so the same streams).  The chains' numpy Generators
    are built only when first used; their fresh PCG64 states come back as
    ``[count, 5]`` uint64 ``gbsgmc_pcg64`` words, computed for all chains at
    once (:func:`pcg64_words_many`).  Returns ``(chain ids, words)``.
    Shuffled pipelines register one by one."""
    if kwargs.get("shuffle") or kwargs.get("in_epochs"):
      raise ValueError("shuffled pipelines are registered one by one")
    if mb_size > self._observation_count:
      raise ValueError(f"The batch size cannot be bigger than the observation "
                       f"count. Provided {mb_size} and "
                       f"{self._observation_count}")
    first = len(self._chains)
    seeds = [kwargs.get("seed", first + i) for i in range(count)]
    words = pcg64_words_fast(seeds)
    draws = math.ceil(self._observation_count / mb_size)
    for seed in seeds:
      rec = _RandomChain(type='random', idx_offset=None, in_epochs=False,
                         shuffle=False, remaining_samples=0, draws=draws,
                         random_indices=None, mb_size=mb_size,
                         cache_size=cache_size)
      rec.seed = seed
      self._chains.append(rec)
    return range(first, first + count), words

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
