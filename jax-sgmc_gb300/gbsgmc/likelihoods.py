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


def is_prior(p) -> bool:
  return isinstance(p, (GaussianPrior, FlatPrior))


def is_likelihood(l) -> bool:
  return isinstance(l, GLMLikelihood) and l.family >= 0
