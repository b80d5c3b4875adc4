"""Pytree helpers: flatten a sample pytree into one fp32 vector and back.

The order of leaves follows ``jax.flatten_util.ravel_pytree``: dict entries in
sorted key order, lists and tuples in order, each leaf raveled in C order
(jax_sgmc/adaption.py:107-118 uses ravel_pytree for the same purpose).
Leaves may be numpy arrays, torch tensors or Python scalars.
"""

from __future__ import annotations

from typing import Any, List, NamedTuple, Tuple

import numpy as np

PyTree = Any


class TreeDef(NamedTuple):
  kind: str            # 'dict' | 'list' | 'tuple' | 'leaf'
  keys: Tuple          # dict keys (sorted) or child count
  children: Tuple      # TreeDefs of the children
  shape: Tuple = ()    # leaf shape
  dtype: Any = None    # leaf numpy dtype


def _is_leaf(x) -> bool:
  return not isinstance(x, (dict, list, tuple))


def _to_numpy(x) -> np.ndarray:
  try:
    import torch
    if isinstance(x, torch.Tensor):
      return x.detach().cpu().numpy()
  except ImportError:  # pragma: no cover
    pass
  return np.asarray(x)


def tree_flatten(tree: PyTree) -> Tuple[List[np.ndarray], TreeDef]:
  if isinstance(tree, dict):
    keys = tuple(sorted(tree.keys()))
    leaves, defs = [], []
    for k in keys:
      l, d = tree_flatten(tree[k])
      leaves += l
      defs.append(d)
    return leaves, TreeDef("dict", keys, tuple(defs))
  if isinstance(tree, (list, tuple)):
    leaves, defs = [], []
    for v in tree:
      l, d = tree_flatten(v)
      leaves += l
      defs.append(d)
    kind = "list" if isinstance(tree, list) else "tuple"
    return leaves, TreeDef(kind, (len(tree),), tuple(defs))
  a = _to_numpy(tree)
  return [a], TreeDef("leaf", (), (), tuple(a.shape), a.dtype)


def tree_unflatten(tdef: TreeDef, leaves: List[Any]) -> PyTree:
  it = iter(leaves)

  def build(d: TreeDef):
    if d.kind == "leaf":
      return next(it)
    if d.kind == "dict":
      return {k: build(c) for k, c in zip(d.keys, d.children)}
    out = [build(c) for c in d.children]
    return out if d.kind == "list" else tuple(out)

  return build(tdef)


def leaf_sizes(tdef: TreeDef) -> List[int]:
  if tdef.kind == "leaf":
    return [int(np.prod(tdef.shape, dtype=np.int64))]
  out = []
  for c in tdef.children:
    out += leaf_sizes(c)
  return out


def leaf_shapes(tdef: TreeDef) -> List[Tuple]:
  if tdef.kind == "leaf":
    return [tdef.shape]
  out = []
  for c in tdef.children:
    out += leaf_shapes(c)
  return out


def ravel(tree: PyTree) -> Tuple[np.ndarray, TreeDef]:
  """Flattens a sample pytree into a float32 vector."""
  leaves, tdef = tree_flatten(tree)
  if not leaves:
    return np.zeros(0, np.float32), tdef
  flat = np.concatenate([np.ravel(l).astype(np.float32) for l in leaves])
  return flat, tdef


def ravel_many(trees) -> Tuple[np.ndarray, TreeDef]:
  """:func:`ravel` of each tree of one structure, as the rows of one
  ``[len(trees), P]`` float32 array, with the first tree's definition.
  Dicts of array leaves are stacked key by key; other trees are raveled one
  by one.  Raises ValueError when the trees differ in structure."""
  trees = list(trees)
  if not trees:
    raise ValueError("no trees")
  _, tdef = tree_flatten(trees[0])
  C = len(trees)
  if tdef.kind == "dict" and tdef.children and \
      all(c.kind == "leaf" for c in tdef.children) and \
      all(type(t) is dict and len(t) == len(tdef.keys) for t in trees):
    try:
      cols = []
      for k, child in zip(tdef.keys, tdef.children):
        a = np.stack([np.asarray(t[k]) for t in trees])
        if a.shape[1:] != tuple(child.shape):
          raise ValueError("leaf shapes differ")
        cols.append(a.reshape(C, -1).astype(np.float32, copy=False))
      flat = cols[0] if len(cols) == 1 else np.concatenate(cols, axis=1)
      return np.ascontiguousarray(flat, np.float32), tdef
    except (KeyError, TypeError, ValueError, RuntimeError):
      pass
  rows = []
  for t in trees:
    flat, d = ravel(t)
    if d.kind != tdef.kind or d.keys != tdef.keys or \
        leaf_shapes(d) != leaf_shapes(tdef):
      raise ValueError("the samples differ in structure")
    rows.append(flat)
  return np.stack(rows).astype(np.float32, copy=False), tdef


def unraveler(tdef: TreeDef):
  """:func:`unravel` for one tree definition, with its leaf layout worked
  out once: returns ``f(flat) -> tree`` for numpy or torch ``flat``."""
  if tdef.kind == "dict" and all(c.kind == "leaf" for c in tdef.children):
    spec, o = [], 0
    for k, c in zip(tdef.keys, tdef.children):
      n = int(np.prod(c.shape, dtype=np.int64))
      spec.append((k, o, o + n, tuple(c.shape)))
      o += n

    def f(flat):
      flat = _to_numpy(flat)
      lead = flat.shape[:-1]
      return {k: flat[..., a:b].reshape(lead + shape) for k, a, b, shape in spec}

    return f
  return lambda flat: unravel(tdef, flat)


def unravel(tdef: TreeDef, flat) -> PyTree:
  """Inverse of :func:`ravel`; ``flat`` may carry leading batch axes."""
  flat = _to_numpy(flat)
  lead = flat.shape[:-1]
  leaves, o = [], 0
  for shape in leaf_shapes(tdef):
    n = int(np.prod(shape, dtype=np.int64))
    leaves.append(flat[..., o:o + n].reshape(lead + tuple(shape)))
    o += n
  return tree_unflatten(tdef, leaves)
