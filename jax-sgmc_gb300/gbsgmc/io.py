"""Sample collection (mirrors jax_sgmc/io.py).

The reference streams each kept sample to the host with
``host_callback.id_tap`` (io.py:626-771).  Here kept samples are written on
the device by the step kernels into a ``[kept, chains, P]`` buffer (the
``keep_slot`` table says which step goes to which row) and copied to the
host once at the end.  The result format is the reference's
``{'sample_count': S, 'samples': {'variables': pytree of [S, ...], ...}}``
(io.py:768-769).  ``save(MemoryCollector())`` returns numpy arrays (written
to ``save_dir/chain_{i}.npz`` when a directory is given); ``no_save()``
returns device tensors.  ``moments()`` keeps only the FP64 posterior mean
and variance of each chain's samples, taken on the device
(:class:`DeviceMoments`), and copies those to the host instead of the
samples.
"""

from __future__ import annotations

import threading
from pathlib import Path
from typing import Any, NamedTuple

import numpy as np

from . import util


class MemoryCollector:
  """Collects samples in host memory (io.py:502-619)."""

  def __init__(self, save_dir=None):
    self._dir = save_dir
    self._count = 0

  def finalize(self, samples: dict) -> dict:
    chain_id = self._count
    self._count += 1
    if self._dir:
      out = Path(self._dir)
      out.mkdir(exist_ok=True, parents=True)
      flat = {}

      def walk(prefix, t):
        if isinstance(t, dict):
          for k, v in t.items():
            walk(f"{prefix}/{k}" if prefix else str(k), v)
        elif isinstance(t, (list, tuple)):
          for i, v in enumerate(t):
            walk(f"{prefix}/{i}" if prefix else str(i), v)
        elif t is not None:
          flat[prefix] = np.asarray(t)
      walk("", samples)
      np.savez(out / f"chain_{chain_id}.npz", **flat)
    return samples


class Saving(NamedTuple):
  kind: str                 # 'memory' | 'device'
  collector: Any = None


def save(data_collector=None, checkpoint_every: int = 0) -> Saving:
  """Keeps accepted samples and returns them as numpy arrays."""
  del checkpoint_every
  return Saving("memory", data_collector or MemoryCollector())


def no_save() -> Saving:
  """Keeps accepted samples on the device (torch tensors)."""
  return Saving("device", None)


def moments() -> Saving:
  """Returns, per chain, only the FP64 mean and (population) variance of the
  accepted samples: ``{'sample_count': S, 'moments': {'mean': pytree,
  'variance': pytree}, 'samples': {extras of [S]}}`` (numpy float64)."""
  return Saving("moments", None)


class DeviceMoments:
  """Streaming FP64 moments of [chains, P] samples on the device
  (``gbsgmc_moments_accumulate`` / ``gbsgmc_moments_finalize``): shifted
  sums, with each parameter's first sample as the shift.  ``add`` takes
  ``[K, chains, P]`` or ``[chains, P]`` fp32 device tensors whose last axis
  is contiguous."""

  def __init__(self, chains: int, P: int):
    import torch
    self.chains, self.P, self.count = int(chains), int(P), 0
    self.shift = torch.empty((chains, P), dtype=torch.float32, device="cuda")
    self.s1 = torch.zeros((chains, P), dtype=torch.float64, device="cuda")
    self.s2 = torch.zeros((chains, P), dtype=torch.float64, device="cuda")

  def add(self, samples) -> "DeviceMoments":
    from . import _lib
    import torch
    if samples.dim() == 2:
      samples = samples.unsqueeze(0)
    K, C, P = samples.shape
    if (C, P) != (self.chains, self.P):
      raise ValueError(f"samples [{K}, {C}, {P}] do not match moments of "
                       f"[{self.chains}, {self.P}]")
    if samples.dtype != torch.float32 or not samples.is_cuda:
      samples = samples.to(device="cuda", dtype=torch.float32)
    if P > 1 and samples.stride(2) != 1:
      samples = samples.contiguous()
    if K == 0:
      return self
    _lib.call("gbsgmc_moments_accumulate", C, P, K, _lib.ptr(samples),
              samples.stride(0), samples.stride(1), self.count,
              _lib.ptr(self.shift), _lib.ptr(self.s1), _lib.ptr(self.s2),
              _lib.stream_handle())
    self.count += K
    return self

  def finalize(self):
    """(mean, variance): fp64 device tensors [chains, P]."""
    from . import _lib
    import torch
    if self.count == 0:
      raise ValueError("no samples")
    mean = torch.empty_like(self.s1)
    var = torch.empty_like(self.s1)
    _lib.call("gbsgmc_moments_finalize", self.chains, self.P, self.count,
              _lib.ptr(self.shift), _lib.ptr(self.s1), _lib.ptr(self.s2),
              _lib.ptr(mean), _lib.ptr(var), _lib.stream_handle())
    return mean, var


def _moment_results(count, variables, treedefs, extras, model_states,
                    moments=None):
  """Per-chain moment results from a ``[count, C, P]`` device buffer, or
  from the :class:`DeviceMoments` ``moments`` the samples went into."""
  if moments is not None:
    C, P = moments.chains, moments.P
  else:
    C, P = variables.shape[1], variables.shape[2]
  if count == 0:
    mean = var = np.full((C, P), np.nan)
  else:
    if moments is None:
      moments = DeviceMoments(C, P).add(variables[:count])
    mean_d, var_d = moments.finalize()
    mean, var = mean_d.cpu().numpy(), var_d.cpu().numpy()
  out = []
  for c in range(C):
    samples = {k: (v[:, c].detach().cpu().numpy() if hasattr(v, "detach")
                   else np.asarray(v)[:, c]) for k, v in extras.items()}
    samples["model_state"] = model_states[c]
    out.append({"sample_count": count,
                "moments": {"mean": util.unravel(treedefs[c], mean[c]),
                            "variance": util.unravel(treedefs[c], var[c])},
                "samples": samples})
  return out


def postprocess(saving: Saving, count: int, variables, treedef, extras: dict,
                model_state=None) -> dict:
  """Builds one chain's result dict from its device sample buffers."""
  if saving is not None and saving.kind == "moments":
    import torch
    v = variables if hasattr(variables, "is_cuda") else torch.from_numpy(
        np.ascontiguousarray(variables))
    ext = {k: (x.reshape(-1, 1) if hasattr(x, "reshape") else
               np.asarray(x).reshape(-1, 1)) for k, x in extras.items()}
    return _moment_results(count, v[:, None, :], [treedef], ext,
                           [model_state])[0]
  if saving is None or saving.kind == "device":
    # Device results: one torch view per leaf of the [count, P] buffer.
    leaves, o = [], 0
    for shape in util.leaf_shapes(treedef):
      n = int(np.prod(shape, dtype=np.int64))
      leaves.append(variables[:, o:o + n].reshape((count,) + tuple(shape)))
      o += n
    var_tree = util.tree_unflatten(treedef, leaves)
    samples = {"variables": var_tree, **extras, "model_state": model_state}
    return {"sample_count": count, "samples": samples}
  host = variables if isinstance(variables, np.ndarray) else \
      variables.detach().cpu().numpy()
  samples = {"variables": util.unravel(treedef, host)}
  for k, v in extras.items():
    samples[k] = v.detach().cpu().numpy() if hasattr(v, "detach") else v
  samples["model_state"] = model_state
  samples = saving.collector.finalize(samples)
  return {"sample_count": count, "samples": samples}


class HostBuffers:
  """Host arrays whose pages a background thread touches while the GPU
  runs, so that the final device-to-host copy does not pay the page faults
  of fresh memory (most of its cost for a few hundred MB)."""

  # Below this total the arrays are made in the caller's thread (starting
  # a thread would cost more than the page faults it hides).
  SMALL_BYTES = 32 << 20

  def __init__(self, specs):
    self._specs = list(specs)
    self._arrays = None
    self._thread = None
    total = sum(int(np.prod(shape, dtype=np.int64)) * np.dtype(dt).itemsize
                for shape, dt in self._specs)
    if total < self.SMALL_BYTES:
      self._arrays = [np.empty(shape, dt) for shape, dt in self._specs]
      return
    self._thread = threading.Thread(target=self._fill, daemon=True)
    self._thread.start()

  def _fill(self):
    out = []
    for shape, dtype in self._specs:
      a = np.empty(shape, dtype)
      if a.size:
        a.reshape(-1).view(np.uint8)[::4096] = 0
      out.append(a)
    self._arrays = out

  def get(self):
    if self._thread is not None:
      self._thread.join()
    return self._arrays


class SampleDrain:
  """Copies kept samples to host arrays while later steps run: after each
  block of steps the caller reports the slots the block filled
  (:meth:`filled`), and a thread waits for that block on the device and
  copies those rows of every buffer ([slots, ...] device tensors) into the
  matching host arrays on its own stream.  ``host`` is a list of arrays or a
  :class:`HostBuffers`, fetched by the thread (it may still be faulting in
  its pages).  With ``ring`` the device buffers hold only ``ring`` rows and
  slot s lives in row s % ring; :meth:`wait_copied` tells the caller when a
  row may be written again."""

  def __init__(self, buffers, host, ring=None):
    import queue
    import torch
    self._buffers = list(buffers)
    self._host = host
    self._ring = ring
    self._arrays = None
    self._queue = queue.Queue()
    self._device = self._buffers[0].device
    self._stream = torch.cuda.Stream(device=self._device)
    self._error = None
    self._done = 0                   # slots [0, done) are on the host
    self._cond = threading.Condition()
    self._thread = threading.Thread(target=self._work, daemon=True)
    self._thread.start()

  def wait_copied(self, slot: int):
    """Blocks until slot ``slot`` has reached the host."""
    with self._cond:
      self._cond.wait_for(lambda: self._done > slot or self._error is not None)

  def filled(self, s0: int, s1: int):
    import torch
    if s1 <= s0:
      return
    ev = torch.cuda.Event()
    ev.record()
    self._queue.put((ev, int(s0), int(s1)))

  def _work(self):
    import torch
    try:
      arrays = self._host.get() if hasattr(self._host, "get") else self._host
      self._arrays = arrays
      with torch.cuda.device(self._device), torch.cuda.stream(self._stream):
        while True:
          item = self._queue.get()
          if item is None:
            break
          ev, s0, s1 = item
          self._stream.wait_event(ev)
          for buf, arr in zip(self._buffers, arrays):
            if self._ring is None:
              torch.from_numpy(arr[s0:s1]).copy_(buf[s0:s1])
            else:
              for slot in range(s0, s1):
                torch.from_numpy(arr[slot]).copy_(buf[slot % self._ring])
          # Copies into pageable memory have completed when copy_ returns.
          with self._cond:
            self._done = s1
            self._cond.notify_all()
        self._stream.synchronize()
    except Exception as e:  # reported by finish()
      with self._cond:
        self._error = e
        self._cond.notify_all()
      while self._queue.get() is not None:
        pass

  def finish(self) -> list:
    """Waits for every copy; returns the host arrays."""
    self._queue.put(None)
    self._thread.join()
    if self._error is not None:
      raise self._error
    return self._arrays


def moment_results(count, moments, treedefs, extras, model_states) -> list:
  """Result dicts of ``io.moments()`` saving from samples that were streamed
  into ``moments`` (a :class:`DeviceMoments`) during the run."""
  return _moment_results(count, None, treedefs, extras, model_states, moments)


def postprocess_chains(saving: Saving, count: int, variables, treedefs,
                       extras: dict, model_states, host=None,
                       host_filled=False) -> list:
  """Result dicts of C chains from a contiguous ``[count, C, P]`` device
  buffer (extras ``[count, C]``).  With host saving, the buffers of all
  chains are copied to the host at once (one plain device-to-host copy each,
  no kernel), and each chain's arrays are strided views of that copy.
  ``host`` optionally gives the destination arrays (``[count, C, P]``, then
  one ``[count, C]`` per extra, e.g. from :class:`HostBuffers`);
  ``host_filled`` says they already hold the data (a :class:`SampleDrain`
  copied it during the run)."""
  import torch
  C = variables.shape[1]
  if saving is not None and saving.kind == "moments":
    return _moment_results(count, variables, treedefs, extras, model_states)
  if saving is None or saving.kind == "device":
    return [postprocess(saving, count, variables[:, c], treedefs[c],
                        {k: v[:, c] for k, v in extras.items()},
                        model_states[c]) for c in range(C)]
  if host is None:
    host = [np.empty(tuple(variables.shape), np.float32)]
    host += [np.empty(tuple(v.shape), np.float64) for v in extras.values()]
  if not host_filled:
    torch.from_numpy(host[0]).copy_(variables.contiguous())
  hext = {}
  for (k, v), h in zip(extras.items(), host[1:]):
    if not host_filled:
      torch.from_numpy(h).copy_(v.contiguous())
    hext[k] = h
  host = host[0]
  td0 = treedefs[0] if C else None
  if C and td0.kind == "dict" and td0.children and \
      all(ch.kind == "leaf" for ch in td0.children) and \
      all(td is td0 for td in treedefs):
    # One tree definition of array leaves for all chains: each leaf is one
    # [count, C, *shape] view of the host buffer, and chain c's arrays are
    # its views [:, c] -- the arrays unravel() would give, without
    # re-deriving the layout per chain.
    views, o = [], 0
    for k, ch in zip(td0.keys, td0.children):
      n = int(np.prod(ch.shape, dtype=np.int64))
      views.append((k, host[:, :, o:o + n].reshape((count, C) + tuple(ch.shape))))
      o += n
    fin = saving.collector.finalize
    ext = list(hext.items())
    out = []
    for c in range(C):
      samples = {"variables": {k: v[:, c] for k, v in views}}
      for k, v in ext:
        samples[k] = v[:, c]
      samples["model_state"] = model_states[c]
      out.append({"sample_count": count, "samples": fin(samples)})
    return out
  # What postprocess() does for host saving, with each tree definition's
  # leaf layout worked out once for all chains that share it.
  unravelers = {}
  out = []
  for c in range(C):
    td = treedefs[c]
    f = unravelers.get(id(td))
    if f is None:
      f = unravelers[id(td)] = util.unraveler(td)
    samples = {"variables": f(host[:, c])}
    for k, v in hext.items():
      samples[k] = v[:, c]
    samples["model_state"] = model_states[c]
    out.append({"sample_count": count,
                "samples": saving.collector.finalize(samples)})
  return out
