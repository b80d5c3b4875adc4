"""Kernel-backed likelihood and prior families.

In jax_sgmc the likelihood and prior passed to ``minibatch_potential`` are
arbitrary Python callables that JAX traces (jax_sgmc/potential.py:94-99).
Here they are descriptions of the models the CUDA kernels implement; any
other callable is rejected with a TypeError (there is no CPU fallback).

Families (per observation i, z_i = x_i . w):

* :class:`LinearGaussian` -- ``lk_i = log N(y_i | z_i, sigma^2)``, i.e.
  ``jax.scipy.stats.norm.logpdf(y - x.w, scale=sigma)`` as written in the
  reference's regression tests (tests/test_alias.py:96-105).
* :class:`Logistic` -- Bernoulli-logit ``lk_i = y_i z_i - softplus(z_i)``
  (``y log sigmoid(z) + (1-y) log(1-sigmoid(z))``).
* :class:`Linear` -- ``lk_i = z_i`` (the linear likelihood
  ``jnp.sum(sample * reference_data)`` of tests/test_potential.py:26-31).

Dense network (per observation, the parameters a pytree of matrices):

* :class:`MLPGaussian` -- ``out = tanh(tanh(x W1 + b1) W2 + b2) W3 + b3``,
  ``lk = log N(y | out, sigma^2)``; BF16 tensor-core GEMMs with fp32
  accumulation.
* :class:`CNNSoftmax` -- three conv3x3/ReLU/max-pool stages and a dense
  layer, ``lk = log softmax(logits)[label]``; convolutions as BF16 GEMMs.

Priors: :class:`GaussianPrior` (``sum norm.logpdf(w, 0, scale)``, constants
included) and :class:`FlatPrior` (``log p = 0``).
"""

from __future__ import annotations

import math
from dataclasses import dataclass

from . import _lib


@dataclass(frozen=True)
class GaussianPrior:
  """Isotropic Gaussian prior N(0, scale^2 I) on the flat parameter vector."""
  scale: float = 1.0

  def __post_init__(self):
    if not self.scale > 0:
      raise ValueError(f"GaussianPrior scale must be positive, got {self.scale}")

  def log_prob_scalar_const(self, d: int) -> float:
    return -d * (math.log(self.scale) + 0.5 * math.log(2 * math.pi))


@dataclass(frozen=True)
class FlatPrior:
  """Improper flat prior: log p(w) = 0 (the reference tests' ``lambda _: 0.``)."""

  @property
  def scale(self) -> float:
    return 0.0


@dataclass(frozen=True)
class GLMLikelihood:
  """Base of the generalised-linear families: z = x . w over one leaf ``w``."""
  x: str = "x"
  y: str = "y"

  family: int = -1

  def check_data(self, data: dict) -> None:
    for k in (self.x, self.y):
      if k not in data:
        raise KeyError(f"reference data has no field {k!r} "
                       f"(fields: {sorted(data)})")


@dataclass(frozen=True)
class LinearGaussian(GLMLikelihood):
  """lk = log N(y | x.w, sigma^2) with a known noise scale ``sigma``."""
  sigma: float = 1.0
  family: int = _lib.GLM_LINEAR_GAUSSIAN

  def __post_init__(self):
    if not self.sigma > 0:
      raise ValueError(f"sigma must be positive, got {self.sigma}")


@dataclass(frozen=True)
class Logistic(GLMLikelihood):
  """Bernoulli-logit likelihood with labels y in {0, 1}."""
  sigma: float = 1.0
  family: int = _lib.GLM_LOGISTIC


@dataclass(frozen=True)
class Linear(GLMLikelihood):
  """lk = x . w (no target; ``y`` is ignored and may be absent)."""
  y: str = None
  sigma: float = 1.0
  family: int = _lib.GLM_LINEAR

  def check_data(self, data: dict) -> None:
    if self.x not in data:
      raise KeyError(f"reference data has no field {self.x!r}")


@dataclass(frozen=True)
class MLPGaussian:
  """Two-hidden-layer tanh network with a Gaussian likelihood.

  The sample is the pytree ``{"W1": [d_in, h1], "W2": [h1, h2], "W3": [h2, 1],
  "b1": [h1], "b2": [h2], "b3": [1]}`` (or its ravel in that sorted key
  order, as jax.flatten_util.ravel_pytree produces it).  The kernels need
  d_in % 64 == 0, h1 % 256 == 0, h2 % 256 == 0 and minibatches of a multiple
  of 128 observations.
  """
  d_in: int = 64
  h1: int = 1024
  h2: int = 1024
  sigma: float = 0.1
  x: str = "x"
  y: str = "y"

  def __post_init__(self):
    if not self.sigma > 0:
      raise ValueError(f"sigma must be positive, got {self.sigma}")
    if self.d_in % 64 or self.h1 % 256 or self.h2 % 256:
      raise ValueError("MLPGaussian needs d_in % 64 == 0, h1 % 256 == 0 and "
                       f"h2 % 256 == 0 (got {self.d_in}, {self.h1}, {self.h2})")

  def shapes(self):
    return {"W1": (self.d_in, self.h1), "W2": (self.h1, self.h2),
            "W3": (self.h2, 1), "b1": (self.h1,), "b2": (self.h2,),
            "b3": (1,)}

  @property
  def param_count(self) -> int:
    return sum(math.prod(v) for v in self.shapes().values())

  def init(self, rng, scale: float = 1.0):
    """Random parameters (N(0, scale^2 / fan_in) weights, zero biases) as the
    flat float32 vector."""
    import numpy as np
    parts = []
    for name, shp in self.shapes().items():
      if name.startswith("W"):
        parts.append(rng.normal(0.0, scale / math.sqrt(shp[0]), size=shp))
      else:
        parts.append(np.zeros(shp))
    return np.concatenate([p.reshape(-1) for p in parts]).astype(np.float32)

  def unravel(self, flat):
    """Flat vector -> dict of leaves (views for numpy and torch inputs)."""
    out, o = {}, 0
    for name, shp in self.shapes().items():
      k = math.prod(shp)
      out[name] = flat[..., o:o + k].reshape(tuple(flat.shape[:-1]) + shp)
      o += k
    return out

  def check_data(self, data: dict) -> None:
    for k in (self.x, self.y):
      if k not in data:
        raise KeyError(f"reference data has no field {k!r} "
                       f"(fields: {sorted(data)})")


@dataclass(frozen=True)
class CNNSoftmax:
  """Convolutional classifier with the softmax (negative cross-entropy)
  likelihood of the reference's classifier example (examples/cifar.md:
  203-210): 32x32x3 images, conv3x3 32/64/128 each with ReLU and 2x2
  max-pool (SAME padding), dense 10.

  The sample is ``{"conv1": {"b", "w"}, "conv2": ..., "conv3": ...,
  "linear": {"b", "w"}}`` (HWIO conv weights, [2048, 10] dense weights) or
  its sorted-key ravel, P = 113,738.  Labels are class indices 0..9.
  Minibatch sizes must be even.
  """
  image: str = "image"
  label: str = "label"

  CHANNELS = (3, 32, 64, 128)

  def shapes(self):
    c = self.CHANNELS
    return {"conv1": {"b": (c[1],), "w": (3, 3, c[0], c[1])},
            "conv2": {"b": (c[2],), "w": (3, 3, c[1], c[2])},
            "conv3": {"b": (c[3],), "w": (3, 3, c[2], c[3])},
            "linear": {"b": (10,), "w": (4 * 4 * c[3], 10)}}

  @property
  def param_count(self) -> int:
    return sum(math.prod(s) for d in self.shapes().values() for s in d.values())

  def init(self, rng):
    """He-normal weights, zero biases, as the flat float32 vector."""
    import numpy as np
    parts = []
    for layer in self.shapes().values():
      for name, shp in layer.items():
        if name == "w":
          fan_in = math.prod(shp[:-1])
          parts.append(rng.normal(0.0, math.sqrt(2.0 / fan_in), size=shp))
        else:
          parts.append(np.zeros(shp))
    return np.concatenate([p.reshape(-1) for p in parts]).astype(np.float32)

  def unravel(self, flat):
    out, o = {}, 0
    for lname, layer in self.shapes().items():
      out[lname] = {}
      for name, shp in layer.items():
        k = math.prod(shp)
        out[lname][name] = flat[..., o:o + k].reshape(tuple(flat.shape[:-1]) + shp)
        o += k
    return out

  def check_data(self, data: dict) -> None:
    for k in (self.image, self.label):
      if k not in data:
        raise KeyError(f"reference data has no field {k!r} "
                       f"(fields: {sorted(data)})")


def is_prior(p) -> bool:
  return isinstance(p, (GaussianPrior, FlatPrior))


def is_likelihood(l) -> bool:
  return (isinstance(l, GLMLikelihood) and l.family >= 0) or \
      isinstance(l, (MLPGaussian, CNNSoftmax))


def is_cnn(l) -> bool:
  return isinstance(l, CNNSoftmax)


def is_mlp(l) -> bool:
  return isinstance(l, MLPGaussian)
