"""Sample collection (mirrors jax_sgmc/io.py).

The reference streams each kept sample to the host with
``host_callback.id_tap`` (io.py:626-771).  Here kept samples are written on
the device by the step kernels into a ``[kept, chains, P]`` buffer (the
``keep_slot`` table says which step goes to which row) and copied to the
host once at the end.  The result format is the reference's
``{'sample_count': S, 'samples': {'variables': pytree of [S, ...], ...}}``
(io.py:768-769).  ``save(MemoryCollector())`` returns numpy arrays (written
to ``save_dir/chain_{i}.npz`` when a directory is given); ``no_save()``
returns device tensors.
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


def postprocess(saving: Saving, count: int, variables, treedef, extras: dict,
                model_state=None) -> dict:
  """Builds one chain's result dict from its device sample buffers."""
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

  def __init__(self, specs):
    self._specs = list(specs)
    self._arrays = None
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
    self._thread.join()
    return self._arrays


def postprocess_chains(saving: Saving, count: int, variables, treedefs,
                       extras: dict, model_states, host=None) -> list:
  """Result dicts of C chains from a contiguous ``[count, C, P]`` device
  buffer (extras ``[count, C]``).  With host saving, the buffers of all
  chains are copied to the host at once (one plain device-to-host copy each,
  no kernel), and each chain's arrays are strided views of that copy.
  ``host`` optionally gives the destination arrays (``[count, C, P]``, then
  one ``[count, C]`` per extra, e.g. from :class:`HostBuffers`)."""
  import torch
  C = variables.shape[1]
  if saving is None or saving.kind == "device":
    return [postprocess(saving, count, variables[:, c], treedefs[c],
                        {k: v[:, c] for k, v in extras.items()},
                        model_states[c]) for c in range(C)]
  if host is None:
    host = [np.empty(tuple(variables.shape), np.float32)]
    host += [np.empty(tuple(v.shape), np.float64) for v in extras.values()]
  torch.from_numpy(host[0]).copy_(variables.contiguous())
  hext = {}
  for (k, v), h in zip(extras.items(), host[1:]):
    torch.from_numpy(h).copy_(v.contiguous())
    hext[k] = h
  host = host[0]
  return [postprocess(saving, count, host[:, c], treedefs[c],
                      {k: v[:, c] for k, v in hext.items()}, model_states[c])
          for c in range(C)]
