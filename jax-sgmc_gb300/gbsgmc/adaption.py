"""Manifold adaption (mirrors jax_sgmc/adaption.py, RMSprop only).

``rms_prop()`` returns the reference's ``(init, update, get)`` triplet on a
flat fp32 device vector (the reference ravels the pytree every call,
adaption.py:120-222; here parameters are flat already):

    init:   v = 1                                      (adaption.py:238-252)
    update: v <- alpha v + (1 - alpha) g^2             (adaption.py:254-272)
    get:    G = 1 / (lmbd + sqrt v), sqrt(G), Gamma = 0 (adaption.py:274-291)

The integrators do not call update/get separately: the SGLD kernels fuse
them into the parameter update (``gbsgmc_sgld_update``,
``gbsgmc_sgld_glm_step``).

``mass_matrix(diagonal=True)`` adapts the diagonal mass of the MH samplers
(AMAGOLD, SGGMC) on the device with ``gbsgmc_mass_adapt``
(adaption.py:296-368).  ``fisher_information(diagonal=True)`` is SGHMC's
empirical-Fisher noise model (adaption.py:371-457) on the generalised-linear
likelihoods (``gbsgmc_glm_fisher_noise``) and the MLP
(``gbsgmc_mlp_fisher_noise``), and with ``diagonal=False`` its dense form
for up to 128 parameters of a generalised-linear likelihood
(``gbsgmc_glm_fisher_noise_dense``);
``mass_matrix(diagonal=False)`` the dense mass for up to 128 parameters
(``gbsgmc_mass_adapt_dense``, the dense integrator kernels).
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


class NoiseModel(NamedTuple):
  """SGHMC noise model (adaption.py:79-90): sqrt(friction - B) and sqrt(B)."""
  cb_diff_sqrt: Any
  b_sqrt: Any


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

  def init_many(samples, alpha=0.9, lmbd=1e-5):
    """``init`` of the rows of ``samples`` ([C, P]) at once: returns
    ``(v, alpha, lmbd)`` with ``v`` one [C, P] tensor of ones, whose row c
    is chain c's state."""
    import torch
    V = torch.ones(tuple(samples.shape), dtype=torch.float32,
                   device=samples.device)
    return V, float(alpha), float(lmbd)

  init.many = init_many

  def update(state: RmsPropState, sample, sample_grad, *args, **kwargs):
    v = state.alpha * state.v + (1 - state.alpha) * sample_grad * sample_grad
    return RmsPropState(v, state.alpha, state.lmbd)

  def get(state: RmsPropState, sample, sample_grad, *args, **kwargs):
    g = 1.0 / (state.lmbd + state.v.sqrt())
    return Manifold(g, g.sqrt(), g * 0.0)

  return AdaptionStrategy(init, update, get, "rms_prop")


class MassState(NamedTuple):
  """Diagonal mass adaption state (adaption.py:321-340), fp32 device [P]
  vectors.  ``mass`` is the mass the integrator kernels take (they use 1/M
  and sqrt(M)); the adaption writes it with ``inv`` and ``sqrt``."""
  iteration: int
  mean: Any
  ssq: Any
  inv: Any
  sqrt: Any
  mass: Any
  burn_in: int


def _flat_device(tree):
  import torch
  if hasattr(tree, "is_cuda"):
    t = tree.reshape(-1).to(torch.float32)
    return t if t.is_cuda else t.cuda()
  from . import util
  flat, _ = util.ravel(tree)
  return torch.from_numpy(flat).cuda()


class DenseMassState(NamedTuple):
  """Dense mass adaption state (adaption.py:321-340): fp32 device mean [P],
  ssq [P, P], inverse mass inv [P, P] and root sqrt [P, P], with the
  eigendecomposition buffers of the final update."""
  iteration: int
  mean: Any
  ssq: Any
  inv: Any
  sqrt: Any
  eig_w: Any
  eig_v: Any
  burn_in: int


def _dense_mass_matrix(burn_in):
  def init(sample, init_cov=None) -> DenseMassState:
    import torch
    x = _flat_device(sample)
    P = x.numel()
    if P > 128:
      raise NotImplementedError("the dense mass is adapted for up to 128 "
                                f"parameters (got {P})")
    cov = torch.ones_like(x) if init_cov is None else _flat_device(init_cov)
    if cov.numel() != P:
      raise ValueError(f"init_cov has {cov.numel()} entries, the sample {P}")
    # The reference's initial dense mass: inv = diag(init_cov),
    # sqrt = diag(1 / sqrt(init_cov)) (adaption.py:333-335).
    return DenseMassState(
        iteration=0, mean=torch.zeros_like(x),
        ssq=torch.zeros((P, P), dtype=torch.float32, device="cuda"),
        inv=torch.diag(cov).contiguous(),
        sqrt=torch.diag(1.0 / cov.sqrt()).contiguous(),
        eig_w=torch.zeros(P, dtype=torch.float32, device="cuda"),
        eig_v=torch.zeros((P, P), dtype=torch.float32, device="cuda"),
        burn_in=int(burn_in))

  def update(state: DenseMassState, sample, *args, **kwargs) -> DenseMassState:
    from . import _lib
    del args, kwargs
    x = _flat_device(sample)
    it = state.iteration + 1
    _lib.call("gbsgmc_mass_adapt_dense", x.numel(), it, state.burn_in,
              _lib.ptr(x), _lib.ptr(state.mean), _lib.ptr(state.ssq),
              _lib.ptr(state.inv), _lib.ptr(state.sqrt), _lib.ptr(state.eig_w),
              _lib.ptr(state.eig_v), _lib.stream_handle())
    return state._replace(iteration=it)

  def get(state: DenseMassState) -> MassMatrix:
    return MassMatrix(inv=state.inv, sqrt=state.sqrt)

  return AdaptionStrategy(init, update, get, "mass_matrix")


def mass_matrix(diagonal=True, burn_in=1000) -> AdaptionStrategy:
  """Adapts the mass for the MH samplers from the accepted samples during
  the first ``burn_in`` updates (adaption.py:296-368): a running mean and
  sum of squared deviations, and at update ``burn_in`` the inverse mass
  ssq / burn_in (the sample variance) and sqrt(burn_in / ssq).  Before then
  the mass is the initial one: inverse ``init_cov`` (ones by default).
  With ``diagonal=False`` (up to 128 parameters) ssq is the P x P sum of
  outer products, the inverse mass ssq / burn_in and the root the product
  V^T diag(sqrt(w)) V of its eigendecomposition, as adaption.py:314-317
  writes it; the integrators then multiply by these matrices."""
  if not diagonal:
    return _dense_mass_matrix(burn_in)

  def init(sample, init_cov=None) -> MassState:
    import torch
    x = _flat_device(sample)
    cov = torch.ones_like(x) if init_cov is None else _flat_device(init_cov)
    if cov.numel() != x.numel():
      raise ValueError(f"init_cov has {cov.numel()} entries, the sample "
                       f"{x.numel()}")
    return MassState(iteration=0, mean=torch.zeros_like(x),
                     ssq=torch.zeros_like(x), inv=cov.clone(),
                     sqrt=1.0 / cov.sqrt(), mass=1.0 / cov,
                     burn_in=int(burn_in))

  def update(state: MassState, sample, *args, **kwargs) -> MassState:
    from . import _lib
    del args, kwargs
    x = _flat_device(sample)
    it = state.iteration + 1
    _lib.call("gbsgmc_mass_adapt", x.numel(), it, state.burn_in, _lib.ptr(x),
              _lib.ptr(state.mean), _lib.ptr(state.ssq), _lib.ptr(state.inv),
              _lib.ptr(state.sqrt), _lib.ptr(state.mass), _lib.stream_handle())
    return state._replace(iteration=it)

  def get(state: MassState) -> MassMatrix:
    return MassMatrix(inv=state.inv, sqrt=state.sqrt)

  return AdaptionStrategy(init, update, get, "mass_matrix")


def fisher_information(minibatch_potential=None, diagonal=True) -> AdaptionStrategy:
  """Empirical Fisher information of the minibatch as SGHMC's noise model
  (adaption.py:371-457, after https://arxiv.org/abs/1206.6380).  Stateless:
  ``get(state, sample, sample_grad, friction, mini_batch=..., step_size=...)``
  returns the :class:`NoiseModel` of the current minibatch, computed on the
  device from the per-observation likelihood gradients: for the
  generalised-linear families elementwise (``diagonal=True``) or from the
  d x d matrices (``diagonal=False``, d <= 128) through their
  eigendecompositions (``gbsgmc_glm_fisher_noise_dense``); for the MLP
  elementwise, the sums of the gradients and of their squares from GEMMs
  on the tensor cores (``gbsgmc_mlp_fisher_noise``)."""
  assert minibatch_potential, "Fisher information requires potential function."
  if getattr(minibatch_potential, "is_cnn", False):
    raise NotImplementedError("per-observation gradients are provided for the "
                              "generalised-linear and MLP likelihoods")
  if getattr(minibatch_potential, "is_mlp", False) and not diagonal:
    raise NotImplementedError("the dense Fisher noise model is built for the "
                              "generalised-linear likelihoods (d <= 128)")
  pot = minibatch_potential

  def init(*args, **kwargs):
    del args, kwargs

  def update(*args, **kwargs):
    del args, kwargs

  def get(state, sample, sample_grad, friction, *args, mini_batch=None,
          step_size=1.0, **kwargs) -> NoiseModel:
    import numpy as np
    import torch
    from . import _lib
    del state, args, kwargs
    assert mini_batch, "Adaption strategy requires mini-batch"
    batch, info = mini_batch
    ds = batch.dataset
    n_obs = info.observation_count if info is not None else ds.observation_count
    m, keep = pot.model(ds, n_obs)
    x = _flat_device(sample)
    P = x.numel()
    g = _flat_device(sample_grad)
    idx = batch.indices.reshape(-1).to(device="cuda", dtype=torch.int32).contiguous()
    if np.isscalar(friction):
      fric, f = None, float(friction)
    else:
      fric, f = _flat_device(friction), 0.0
    cb = torch.empty(P, dtype=torch.float32, device="cuda")
    bs = torch.empty(P, dtype=torch.float32, device="cuda")
    if pot.is_mlp:
      n = idx.numel()
      ws = pot.fisher_workspace(1, n, m)
      _lib.call("gbsgmc_mlp_fisher_noise", m, 1, n, _lib.ptr(idx), n,
                _lib.ptr(x), _lib.ptr(g), _lib.ptr(fric), f, float(step_size),
                _lib.ptr(cb), _lib.ptr(bs), _lib.ptr(ws), ws.numel(),
                _lib.ptr(pot.status()), _lib.stream_handle())
      del keep
      return NoiseModel(cb_diff_sqrt=cb, b_sqrt=bs)
    _lib.call("gbsgmc_glm_fisher_noise" if diagonal else "gbsgmc_glm_fisher_noise_dense",
              m, 1, idx.numel(), _lib.ptr(idx),
              idx.numel(), _lib.ptr(x), _lib.ptr(g), _lib.ptr(fric), f,
              float(step_size), _lib.ptr(cb), _lib.ptr(bs),
              _lib.ptr(pot.status()), _lib.stream_handle())
    del keep
    return NoiseModel(cb_diff_sqrt=cb, b_sqrt=bs)

  return AdaptionStrategy(init, update, get, "fisher_information")
