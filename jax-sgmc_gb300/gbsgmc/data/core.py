"""Reference-data access for the GPU hot path.

Mirrors jax_sgmc/data/core.py.  The reference keeps a cache of
``cached_batches_count`` gathered minibatches on the device and refills it
from the host through ``io_callback`` (core.py:664-791).  Here the whole
dataset lives in HBM (uploaded once per loader), and the cache holds only the
*indices* of the next ``cached_batches_count`` minibatches, drawn on the GPU
from the same numpy PCG64 stream the host loader would use (bit-identical,
see ``gbsgmc_index_draw_pcg64``).  The fused kernels gather rows straight
from the resident dataset.

``random_reference_data`` / ``full_reference_data`` keep their signatures and
return the same ``(init_fn, batch_fn, release)`` triplets
(core.py:477-629).  Batches are :class:`IndexedBatch` views: the likelihood
kernels consume them without materialising the rows; indexing a batch by
field name gathers that field on the device for inspection.
"""

from __future__ import annotations

import abc
import itertools
import math
import warnings
from typing import Any, Callable, Dict, NamedTuple, Tuple

import numpy as np

from .. import _lib

PyTree = Any


class MiniBatchInformation(NamedTuple):
  """Bundles all information about the reference data (core.py:49-61).

  Args:
    observation_count: Total number of observations
    mask: Validity of the observations in the batch
    batch_size: Number of observations in the batch
  """
  observation_count: Any
  mask: Any
  batch_size: Any


class CacheState(NamedTuple):
  """State of a random (or ordered) reference-data chain (core.py:240-259).

  ``cached_batches`` holds device int32 indices ``[cached_batches_count,
  mb_size]``; ``state`` holds the chain's device stream state (a numpy PCG64
  state as ``gbsgmc_pcg64`` bytes, or the Philox step counter).
  """
  callback_uuid: Any = None
  cached_batches: Any = None
  cached_batches_count: Any = None
  current_line: Any = None
  chain_id: Any = None
  state: Any = None
  valid: Any = None
  token: Any = None


random_data_state = CacheState


class DataLoader(metaclass=abc.ABCMeta):
  """Common interface of the data loaders (core.py:65-104)."""

  @property
  @abc.abstractmethod
  def static_information(self) -> Dict:
    """Information about the dataset such as the total observation count."""

  @property
  @abc.abstractmethod
  def _format(self):
    """dtype and shape of a single sample."""

  def initializer_batch(self, mb_size: int = None) -> PyTree:
    """Returns a zero-like mini-batch (numpy arrays)."""
    out = {}
    for name, (shape, dtype) in self._format.items():
      shp = tuple(shape) if mb_size is None else (mb_size,) + tuple(shape)
      out[name] = np.zeros(shp, dtype=dtype)
    return out

  def device_dataset(self) -> "DeviceDataset":
    """The loader's arrays resident in HBM (uploaded on first use)."""
    ds = getattr(self, "_gbsgmc_device_dataset", None)
    if ds is None:
      ds = DeviceDataset(self.reference_data)
      self._gbsgmc_device_dataset = ds
    return ds


class DeviceDataLoader(DataLoader, metaclass=abc.ABCMeta):
  """Loader whose random draws happen on the device (core.py:106-128)."""

  @abc.abstractmethod
  def init_random_data(self, *args, **kwargs) -> PyTree:
    """Initializes the state necessary to randomly draw data."""

  @abc.abstractmethod
  def get_random_data(self, state, batch_size):
    """Returns a random batch of the data."""

  @abc.abstractmethod
  def get_full_data(self) -> Dict:
    """Returns the whole dataset as dictionary of arrays."""


class HostDataLoader(DataLoader, metaclass=abc.ABCMeta):
  """Loader whose index streams are defined on the host (core.py:130-230)."""

  def save_state(self, chain_id: int):
    raise NotImplementedError("This method must be overwritten to allow "
                              "checkpointing of the data loader.")

  def load_state(self, chain_id: int, data):
    raise NotImplementedError("This method must be overwritten to allow "
                              "checkpointing of the data loader.")

  @abc.abstractmethod
  def register_random_pipeline(self, cache_size: int = 1, mb_size: int = None,
                               **kwargs) -> int:
    """Register a new chain which assembles batches randomly."""

  @abc.abstractmethod
  def register_ordered_pipeline(self, cache_size: int = 1,
                                mb_size: int = None, **kwargs) -> int:
    """Register a chain which assembles batches in an ordered manner."""

  @abc.abstractmethod
  def get_batches(self, chain_id: int):
    """Return batches from an ordered or random chain (host arrays)."""

  def batch_format(self, cache_size: int, mb_size: int):
    fmt = {name: ((cache_size, mb_size) + tuple(shape), dtype)
           for name, (shape, dtype) in self._format.items()}
    info = MiniBatchInformation(
        observation_count=self.static_information["observation_count"],
        batch_size=mb_size, mask=np.ones(mb_size, dtype=np.bool_))
    return fmt, info


# ---------------------------------------------------------------------------
# Device-resident dataset
# ---------------------------------------------------------------------------

class DeviceDataset:
  """A loader's arrays resident in HBM as fp32, uploaded on first use.

  * ``matrix(name)``: a 2-D field ``[N, d]`` stored row-major with the row
    stride rounded up to a multiple of four floats and zero padding, so that
    every row starts 16-byte aligned and can be fetched with one bulk copy.
  * ``vector(name)``: a width-1 field (targets) as ``[N]``.
  * ``glm_view(x, y)``: the layout the GLM kernels read -- row i holds
    ``[x_i (d floats), y_i, zero padding]`` with a stride that is a multiple
    of eight floats, so every row starts on a 32-byte sector and the target
    arrives in the row's own sectors.
  """

  def __init__(self, arrays: Dict[str, np.ndarray]):
    import torch
    if not torch.cuda.is_available():
      raise RuntimeError("gbsgmc needs a CUDA device: the dataset lives in HBM")
    self._host = {k: np.asarray(v) for k, v in arrays.items()}
    self._fields = {}
    self._views = {}
    self.observation_count = None
    for a in self._host.values():
      self.observation_count = a.shape[0]
      break

  def keys(self):
    return self._host.keys()

  def __contains__(self, name):
    return name in self._host

  def field(self, name: str):
    """(tensor, d, ld) of a field, uploaded on first use."""
    import torch
    got = self._fields.get(name)
    if got is not None:
      return got
    a = self._host[name]
    if a.ndim == 1 or int(np.prod(a.shape[1:])) == 1:
      flat = np.ascontiguousarray(a.reshape(-1), dtype=np.float32)
      got = (torch.from_numpy(flat).cuda(), 1, 1)
    else:
      flat = a.reshape(a.shape[0], -1)
      d = flat.shape[1]
      ld = (d + 3) // 4 * 4
      t = torch.zeros((a.shape[0], ld), dtype=torch.float32, device="cuda")
      t[:, :d].copy_(torch.from_numpy(np.ascontiguousarray(flat, np.float32)))
      got = (t, d, ld)
    self._fields[name] = got
    return got

  @property
  def fields(self):
    return {k: self.field(k) for k in self._host}

  def matrix(self, name: str):
    """(tensor [N, ld], d, ld) of a feature field; 1-D fields give d = 1."""
    t, d, ld = self.field(name)
    if t.dim() == 1:
      return t.view(-1, 1), 1, 1
    return t, d, ld

  def vector(self, name: str):
    t, d, _ = self.field(name)
    if t.dim() != 1:
      raise ValueError(f"field {name!r} is not a vector (width {d})")
    return t

  def feature_dim(self, name: str) -> int:
    a = self._host[name]
    return 1 if a.ndim == 1 else int(np.prod(a.shape[1:]))

  def glm_view(self, x: str, y: str):
    """(tensor [N, ld], d, ld) with y_i stored at column d of row i."""
    import torch
    key = (x, y)
    got = self._views.get(key)
    if got is not None:
      return got
    xa = self._host[x]
    flat = xa.reshape(xa.shape[0], -1)
    d = flat.shape[1]
    ld = (d + 1 + 7) // 8 * 8     # whole 32-byte sectors per row
    t = torch.zeros((xa.shape[0], ld), dtype=torch.float32, device="cuda")
    t[:, :d].copy_(torch.from_numpy(np.ascontiguousarray(flat, np.float32)))
    t[:, d].copy_(torch.from_numpy(
        np.ascontiguousarray(self._host[y].reshape(-1), np.float32)))
    got = (t, d, ld)
    self._views[key] = got
    return got


class IndexedBatch:
  """A minibatch as observation indices into a device-resident dataset.

  ``batch[name]`` gathers that field for inspection; the likelihood kernels
  read ``indices`` directly.
  """

  def __init__(self, dataset: DeviceDataset, indices, loader=None):
    self.dataset = dataset
    self.indices = indices  # device int32 [mb]
    self.loader = loader

  def __getitem__(self, name):
    t, d, _ = self.dataset.field(name)
    rows = t.index_select(0, self.indices.long())
    return rows if t.dim() == 1 else rows[:, :d]

  def keys(self):
    return self.dataset.keys()

  def __len__(self):
    return int(self.indices.numel())


# ---------------------------------------------------------------------------
# Random access
# ---------------------------------------------------------------------------

def _pcg_words(bitgen_state: dict):
  """numpy PCG64 state dict -> host ``gbsgmc_pcg64`` words (int64); the
  first refill moves them to the device."""
  import torch
  st = bitgen_state["state"]["state"]
  inc = bitgen_state["state"]["inc"]
  m64 = (1 << 64) - 1
  words = np.zeros(5, dtype=np.uint64)
  words[0] = (st >> 64) & m64
  words[1] = st & m64
  words[2] = (inc >> 64) & m64
  words[3] = inc & m64
  words[4] = (int(bitgen_state["uinteger"]) << 32) | int(bitgen_state["has_uint32"])
  return torch.from_numpy(words.view(np.int64).copy())


def pcg_from_device(t) -> dict:
  """Device ``gbsgmc_pcg64`` -> numpy PCG64 state dict."""
  words = t.detach().cpu().numpy().view(np.uint64)
  return {"bit_generator": "PCG64",
          "state": {"state": (int(words[0]) << 64) | int(words[1]),
                    "inc": (int(words[2]) << 64) | int(words[3])},
          "has_uint32": int(words[4]) & 0xFFFFFFFF,
          "uinteger": int(words[4]) >> 32}


def draw_indices_pcg64(pcg_dev, n_obs: int, draws: int, per_step: int, out,
                       chains: int = 1, chain_stride: int = None,
                       step_stride: int = None, status=None):
  """Launches ``gbsgmc_index_draw_pcg64`` on torch's current stream."""
  if chain_stride is None:
    chain_stride = draws
  if step_stride is None:
    step_stride = per_step
  _lib.call("gbsgmc_index_draw_pcg64", _lib.ptr(pcg_dev), chains, n_obs,
            draws, per_step, _lib.ptr(out), chain_stride, step_stride,
            _lib.ptr(status), _lib.stream_handle())


def random_reference_data(data_loader: DataLoader, cached_batches_count: int,
                          mb_size: int, verify_calls: bool = False):
  """Random minibatches (core.py:477-520).

  Returns ``(init_fn, batch_fn, release)``.  ``init_fn(**kwargs)`` registers a
  chain (``seed=`` as in the reference) and draws its first index cache on the
  device; ``batch_fn(state, information=False)`` returns the next minibatch
  and refills the index cache after ``cached_batches_count`` calls.
  """
  del verify_calls
  observation_count = data_loader.static_information["observation_count"]
  if observation_count < mb_size:
    raise ValueError(f"Batch size cannot be bigger than the number of total "
                     f"observations. Got {observation_count} and {mb_size}.")
  if cached_batches_count <= 0 or mb_size <= 0:
    raise ValueError(f"Cache size and batch size must be positive, got"
                     f"{cached_batches_count} and {mb_size}.")
  if isinstance(data_loader, HostDataLoader):
    if observation_count < cached_batches_count * mb_size:
      warnings.warn("Cached batches are bigger than the total dataset. "
                    "Consider using a DeviceDataLoader.")
    return _random_reference_data_host(data_loader, cached_batches_count,
                                       mb_size)
  if isinstance(data_loader, DeviceDataLoader):
    if cached_batches_count != 1:
      raise ValueError("No caching on device.")
    return _random_reference_data_device(data_loader, mb_size)
  raise TypeError("The DataLoader must inherit from HostDataLoader or "
                  "DeviceDataLoader")


class RandomBatchFn:
  """Callable batch function that also exposes its loader and sizes, so that
  the fused batched driver can draw the same streams for many chains."""

  def __init__(self, kind, loader, cache, mb_size, fn):
    self.kind = kind            # 'host' | 'device'
    self.loader = loader
    self.cached_batches_count = cache
    self.mb_size = mb_size
    self._fn = fn

  def __call__(self, data_state, information=False, device_count=1):
    return self._fn(data_state, information, device_count)


class _BatchRows:
  """[steps, k * mb] seen as the [steps * k, mb] batch rows it holds, for
  slice assignment (a strided view that reshape cannot give)."""

  def __init__(self, a, mb):
    self.a, self.mb = a, mb
    self.k = a.shape[1] // mb

  def __setitem__(self, sl, value):
    start, stop = sl.start, sl.stop
    for r in range(start, stop):
      s, j = divmod(r, self.k)
      self.a[s, j * self.mb:(j + 1) * self.mb] = value[r - start]


class ShuffledFeed:
  """Minibatch indices of C shuffled host pipelines (shuffle=True, with or
  without in_epochs), step by step, for a plan with an external index
  source.  The integrators use an in-epoch batch's masked tail like any
  other rows (the reference applies a mask only when the caller passes
  one), so the plans need the indices alone.

  Chain c's batches come in the order its own batch function would hand
  them out: the rest of its device cache, then cache-sized chunks from the
  loader (``take_shuffled``: one chunk when the previous one is used up,
  as the batch function refills).  :meth:`next` returns ``[steps, C,
  k * mb]`` int32 (k minibatches per step).  The loader's chain states
  advance exactly as under the per-chain path.  The chains' chunks are
  drawn on a thread pool: numpy releases the GIL while it shuffles."""

  def __init__(self, loader, data_states, per_step=1):
    import concurrent.futures as cf
    import os
    self.loader = loader
    self.states = list(data_states)
    self.k = int(per_step)
    self.cache = int(self.states[0].cached_batches_count)
    self.chunk = [ds.cached_batches.cpu().numpy() for ds in self.states]
    self.pos = [int(ds.current_line) for ds in self.states]
    self.mb = self.chunk[0].shape[1]
    in_epochs = loader._chains[self.states[0].chain_id].get("in_epochs")
    self._draw = loader.take_in_epochs if in_epochs else loader.take_shuffled
    self._pool = cf.ThreadPoolExecutor(max(1, min(len(self.states),
                                                   os.cpu_count() or 1)))

  @staticmethod
  def qualifies(loader, data_states) -> bool:
    chains = getattr(loader, "_chains", None)
    if chains is None or not data_states:
      return False
    for ds in data_states:
      if ds.state is not None or ds.cached_batches is None or ds.chain_id is None:
        return False
      if not chains[ds.chain_id].get("shuffle"):
        return False
    modes = {bool(chains[ds.chain_id].get("in_epochs")) for ds in data_states}
    return len(modes) == 1 and \
        len({int(ds.cached_batches_count) for ds in data_states}) == 1

  def _take(self, c, count, dst):
    """The next ``count`` batches of chain c into dst ([count, mb])."""
    done = 0
    while done < count:
      if self.pos[c] == self.cache:
        self.chunk[c] = self._draw(self.states[c].chain_id, self.cache)
        self.pos[c] = 0
      m = min(count - done, self.cache - self.pos[c])
      dst[done:done + m] = self.chunk[c][self.pos[c]:self.pos[c] + m]
      self.pos[c] += m
      done += m

  def next(self, steps, out=None):
    """Indices of the next ``steps`` steps of every chain, written into
    ``out`` ([>= steps, C, k * mb] int32) when given."""
    C = len(self.states)
    if out is None:
      out = np.empty((steps, C, self.k * self.mb), np.int32)
    view = out[:steps]
    # Chain c's batches are view[:, c, :] read as [steps * k, mb].
    list(self._pool.map(
        lambda c: self._take(c, steps * self.k,
                             view[:, c, :].reshape(steps * self.k, self.mb)
                             if self.k == 1 else _BatchRows(view[:, c, :], self.mb)),
        range(C)))
    return view

  def close(self):
    self._pool.shutdown(wait=True)


class RandomPipelines(NamedTuple):
  """C random pipelines of one host loader registered together: their chain
  ids, their fresh numpy PCG64 stream words as one ``[C, 5]`` int64 host
  tensor (row c is chain c's ``gbsgmc_pcg64``), and the cache size."""
  loader: Any
  chain_ids: Any
  pcg: Any
  cached_batches_count: int

  def state(self, i) -> CacheState:
    """Chain i's :class:`CacheState`, as ``init_fn`` would have returned it
    (its stream words a row view of ``pcg``)."""
    return CacheState(cached_batches=None,
                      cached_batches_count=self.cached_batches_count,
                      current_line=self.cached_batches_count,
                      chain_id=self.chain_ids[i], state=self.pcg[i], valid=None)


def _random_reference_data_host(loader, cache, mb_size):
  import torch
  N = loader.static_information["observation_count"]

  def refill(pcg_dev):
    idx = torch.empty((cache, mb_size), dtype=torch.int32, device="cuda")
    draw_indices_pcg64(pcg_dev, N, cache * mb_size, mb_size, idx)
    return idx

  def init_fn(**kwargs) -> CacheState:
    chain_id = loader.register_random_pipeline(cache, mb_size=mb_size, **kwargs)
    chain = loader._chains[chain_id]
    if chain.get("shuffle") or chain.get("in_epochs"):
      # Shuffled streams are drawn by the host loader (numpy); the indices
      # are uploaded as the cache.
      idx, mask = loader._get_indices(chain_id)
      cached = torch.from_numpy(idx.astype(np.int32)).cuda()
      valid = torch.from_numpy(mask.astype(np.float32)).cuda()
      return CacheState(cached_batches=cached, cached_batches_count=cache,
                        current_line=0, chain_id=chain_id, state=None,
                        valid=valid)
    # The first cache is drawn by the first batch_fn call (the stream order is
    # the reference's: consecutive draws, whatever the cache size).
    pcg = _pcg_words(chain["rng"].bit_generator.state)
    return CacheState(cached_batches=None, cached_batches_count=cache,
                      current_line=cache, chain_id=chain_id, state=pcg,
                      valid=None)

  def init_many(count, **kwargs):
    """``count`` calls of ``init_fn(**kwargs)`` at once, as one
    :class:`RandomPipelines`; None when the chains must register one by one
    (shuffled pipelines, loaders without bulk registration)."""
    if kwargs.get("shuffle") or kwargs.get("in_epochs") or \
        not hasattr(loader, "register_random_pipelines"):
      return None
    ids, words = loader.register_random_pipelines(count, cache,
                                                  mb_size=mb_size, **kwargs)
    return RandomPipelines(loader, ids, torch.from_numpy(words.view(np.int64)),
                           cache)

  init_fn.many = init_many

  def batch_fn(data_state: CacheState, information=False, device_count=1):
    if data_state.current_line == data_state.cached_batches_count:
      if data_state.state is None:
        idx, mask = loader._get_indices(data_state.chain_id)
        cached = torch.from_numpy(idx.astype(np.int32)).cuda()
        valid = torch.from_numpy(mask.astype(np.float32)).cuda()
      else:
        # The draw kernel advances the stream in place on the device.
        if not data_state.state.is_cuda:
          data_state = data_state._replace(state=data_state.state.cuda())
        cached = refill(data_state.state)
        valid = None
      data_state = data_state._replace(cached_batches=cached, valid=valid,
                                       current_line=0)
    line = data_state.current_line % data_state.cached_batches_count
    idx = data_state.cached_batches[line]
    mask = None if data_state.valid is None else data_state.valid[line]
    new_state = data_state._replace(current_line=line + 1)
    batch = IndexedBatch(loader.device_dataset(), idx, loader)
    if information:
      info = MiniBatchInformation(observation_count=N, batch_size=mb_size,
                                  mask=mask)
      return new_state, (batch, info)
    return new_state, batch

  def release():
    pass

  return init_fn, RandomBatchFn("host", loader, cache, mb_size, batch_fn), release


def _random_reference_data_device(loader, mb_size):
  import torch
  N = loader.static_information["observation_count"]

  def init_fn(**kwargs) -> CacheState:
    seed = loader.init_random_data(**kwargs)
    return CacheState(cached_batches_count=1, current_line=0,
                      state=(seed, 0), chain_id=kwargs.get("chain_id", 0))

  def batch_fn(data_state: CacheState, information=False, device_count=1):
    (seed, step) = data_state.state
    idx = torch.empty((mb_size,), dtype=torch.int32, device="cuda")
    _lib.call("gbsgmc_index_draw_philox", seed, int(data_state.chain_id or 0),
              1, step, 1, mb_size, N, _lib.ptr(idx), mb_size, mb_size,
              _lib.stream_handle())
    new_state = data_state._replace(state=(seed, step + 1))
    batch = IndexedBatch(loader.device_dataset(), idx, loader)
    if information:
      info = MiniBatchInformation(observation_count=N, batch_size=mb_size,
                                  mask=None)
      return new_state, (batch, info)
    return new_state, batch

  def release():
    pass

  return init_fn, RandomBatchFn("device", loader, 1, mb_size, batch_fn), release


# ---------------------------------------------------------------------------
# Ordered access over the full dataset
# ---------------------------------------------------------------------------

class FullDataMap:
  """Ordered masked map over all observations (core.py:522-629).

  Calling it as ``batch_scan(fun, data_state, carry, masking, information)``
  maps ``fun(batch, mask, carry)`` over ``ceil(N / mb)`` ordered batches of
  indices exactly like the reference's ``lax.scan``.  ``full_potential``
  reads ``loader`` and ``mb_size`` to evaluate the whole dataset in large
  kernel launches instead.
  """

  def __init__(self, loader, mb_size):
    self.loader = loader
    self.mb_size = mb_size
    self.observation_count = loader.static_information["observation_count"]
    self.num_iterations = int(math.ceil(self.observation_count / mb_size))

  def __call__(self, fun, data_state, carry, masking=False, information=False,
               device_count=1):
    import torch
    ds = self.loader.device_dataset()
    N, mb = self.observation_count, self.mb_size
    results = []
    for it in range(self.num_iterations):
      obs = it * mb + np.arange(mb)
      mask = obs < N
      idx = torch.from_numpy((obs % N).astype(np.int32)).cuda()
      batch = IndexedBatch(ds, idx, self.loader)
      if information:
        batch = (batch, MiniBatchInformation(observation_count=N,
                                             batch_size=mb,
                                             mask=torch.from_numpy(
                                                 mask.astype(np.float32)).cuda()))
      if masking:
        res, carry = fun(batch, torch.from_numpy(mask.astype(np.float32)).cuda(),
                         carry)
      else:
        res, carry = fun(batch, carry)
      results.append(res)
    return data_state, (results, carry)


def full_reference_data(data_loader: DataLoader, cached_batches_count: int = 100,
                        mb_size: int = None):
  """Ordered access to all observations (core.py:522-629)."""
  observation_count = data_loader.static_information["observation_count"]
  if mb_size is None:
    mb_size = observation_count
  if observation_count < mb_size:
    raise ValueError(f"Batch size cannot be bigger than the number of total "
                     f"observations. Got {observation_count} and {mb_size}.")
  fmap = FullDataMap(data_loader, mb_size)

  def init_fn(**kwargs):
    return CacheState(cached_batches_count=cached_batches_count,
                      current_line=0)

  def release():
    pass

  return init_fn, fmap, release


def full_data_mapper(data_loader: DataLoader = None,
                     cached_batches_count: int = 1, mb_size: int = 1):
  """Stateless variant of full_reference_data (core.py:1021-1114)."""
  fmap = FullDataMap(data_loader, mb_size)

  def mapper(fun, carry, masking=False, information=False):
    _, out = fmap(fun, None, carry, masking=masking, information=information)
    return out

  mapper.loader = data_loader
  mapper.mb_size = mb_size

  def release():
    pass

  return mapper, release


def tree_index(pytree, index):
  """Indexes the leaves of the tree in the first dimension (core.py:640-661)."""
  if isinstance(pytree, dict):
    return {k: tree_index(v, index) for k, v in pytree.items()}
  if isinstance(pytree, (list, tuple)):
    return type(pytree)(tree_index(v, index) for v in pytree)
  return pytree[index]
