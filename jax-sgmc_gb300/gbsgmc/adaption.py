"""Manifold adaption (mirrors jax_sgmc/adaption.py, RMSprop only).

``rms_prop()`` returns the reference's ``(init, update, get)`` triplet on a
flat fp32 device vector (the reference ravels the pytree every call,
adaption.py:120-222; here parameters are flat already):

    init:   v = 1                                      (adaption.py:238-252)
    update: v <- alpha v + (1 - alpha) g^2             (adaption.py:254-272)
    get:    G = 1 / (lmbd + sqrt v), sqrt(G), Gamma = 0 (adaption.py:274-291)

The integrators do not call update/get separately: the SGLD kernels fuse
them into the parameter update (``gbsgmc_sgld_update``,
``gbsgmc_sgld_glm_step``).  ``mass_matrix`` and ``fisher_information`` are
not provided.
"""

from __future__ import annotations

from typing import Any, NamedTuple


class Manifold(NamedTuple):
  g_inv: Any
  sqrt_g_inv: Any
  gamma: Any


class MassMatrix(NamedTuple):
  inv: Any
  sqrt: Any


class RmsPropState(NamedTuple):
  v: Any        # fp32 [P], on the device once the chain has stepped
  alpha: float
  lmbd: float


class AdaptionStrategy(NamedTuple):
  init: Any
  update: Any
  get: Any
  kind: str = "rms_prop"


def rms_prop() -> AdaptionStrategy:
  """RMSprop adaption [https://arxiv.org/abs/1512.07666]."""

  def init(sample, alpha=0.9, lmbd=1e-5):
    import torch
    n = sample.numel() if hasattr(sample, "numel") else len(sample)
    dev = sample.device if hasattr(sample, "device") else "cuda"
    return RmsPropState(torch.ones(n, dtype=torch.float32, device=dev),
                        float(alpha), float(lmbd))

  def update(state: RmsPropState, sample, sample_grad, *args, **kwargs):
    v = state.alpha * state.v + (1 - state.alpha) * sample_grad * sample_grad
    return RmsPropState(v, state.alpha, state.lmbd)

  def get(state: RmsPropState, sample, sample_grad, *args, **kwargs):
    g = 1.0 / (state.lmbd + state.v.sqrt())
    return Manifold(g, g.sqrt(), g * 0.0)

  return AdaptionStrategy(init, update, get, "rms_prop")


def mass_matrix(diagonal=True, burn_in=1000):
  raise NotImplementedError("mass_matrix adaption is not part of the GPU "
                            "hot path")


def fisher_information(minibatch_potential=None, diagonal=True):
  raise NotImplementedError("fisher_information is not part of the GPU "
                            "hot path")
