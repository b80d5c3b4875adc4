"""Stochastic and full potentials evaluated by the GLM kernels.

Mirrors jax_sgmc/potential.py.  ``minibatch_potential(prior, likelihood,
strategy, has_state, is_batched, temperature)`` returns a callable with the
reference signature ``(sample, reference_data, state=None, mask=None,
likelihoods=False)`` computing (potential.py:159-214)

    U = (-N/n * sum_i lk_i - log p(sample)) / temperature     (mask is None)
    U = (-N/n * sum_i mask_i lk_i - log p(sample)) / temperature

on the GPU through ``gbsgmc_glm_value_and_grad``.  Gradients come from the
hand-written adjoint in the same launch (the reference differentiates with
``jax.value_and_grad``, integrator.py:166,593,792): use
:meth:`StochasticPotential.value_and_grad`, or :meth:`torch_function` for a
``torch.autograd.Function`` twin.  ``prior`` and ``likelihood`` must be the
kernel-backed families of :mod:`gbsgmc.likelihoods`.
"""

from __future__ import annotations

from typing import Any, NamedTuple

import numpy as np

from . import _lib, likelihoods as lkmod, util
from .data.core import IndexedBatch, MiniBatchInformation

PyTree = Any


class GlmEval(NamedTuple):
  U: Any        # float64 [C]
  grad: Any     # float32 [C, d] or None
  lk: Any       # float32 [C, n] or None
  lk_var: Any   # float64 [C]


def _flat_device(sample, d):
  import torch
  if isinstance(sample, torch.Tensor) and sample.is_cuda:
    w = sample.detach().reshape(-1).to(torch.float32).contiguous()
  else:
    flat, _ = util.ravel(sample)
    w = torch.from_numpy(flat).cuda()
  if w.numel() != d:
    raise ValueError(f"sample has {w.numel()} parameters, the model needs {d}")
  return w


class StochasticPotential:
  """Minibatch potential backed by the GLM kernels (potential.py:94-216)."""

  def __init__(self, prior, likelihood, strategy="map", has_state=False,
               is_batched=False, temperature=1.0):
    if strategy not in ("map", "vmap", "pmap"):
      raise NotImplementedError(f"Strategy {strategy} is unknown")
    if not lkmod.is_prior(prior):
      raise TypeError("prior must be a gbsgmc.likelihoods prior "
                      "(GaussianPrior, FlatPrior): arbitrary callables have "
                      "no kernel")
    if not lkmod.is_likelihood(likelihood):
      raise TypeError("likelihood must be a gbsgmc.likelihoods family "
                      "(LinearGaussian, Logistic, Linear, MLPGaussian): "
                      "arbitrary callables have no kernel")
    if not temperature > 0:
      raise ValueError("temperature must be positive")
    self.prior = prior
    self.likelihood = likelihood
    self.strategy = strategy
    self.has_state = has_state
    self.is_batched = is_batched
    self.temperature = float(temperature)
    self._ws = {}
    self._status = None

  # -- model description ---------------------------------------------------
  @property
  def is_mlp(self) -> bool:
    return lkmod.is_mlp(self.likelihood)

  @property
  def is_cnn(self) -> bool:
    return lkmod.is_cnn(self.likelihood)

  @property
  def is_network(self) -> bool:
    return self.is_mlp or self.is_cnn

  def model(self, dataset, observation_count=None):
    """``gbsgmc_glm`` (or ``gbsgmc_mlp`` / ``gbsgmc_cnn``) for a device
    dataset.  The GLM families read feature rows padded to 16 bytes and the
    targets from their own vector (4 bytes per observation, small enough to
    stay in L2 while the rows stream past); the networks read targets stored
    inline in the feature rows (DeviceDataset.glm_view)."""
    n_obs = dataset.observation_count if observation_count is None \
        else observation_count
    if self.is_cnn:
      lik = self.likelihood
      X, d, ld = dataset.glm_view(lik.image, lik.label)
      if d != 32 * 32 * 3:
        raise ValueError(f"field {lik.image!r} holds {d} values per "
                         "observation, the network takes 32x32x3 images")
      return _lib.Cnn(int(n_obs), int(dataset.observation_count), ld,
                      X.data_ptr(), X.data_ptr() + 4 * d, ld,
                      float(self.prior.scale), float(self.temperature)), (X,)
    if self.is_mlp:
      lik = self.likelihood
      X, d, ld = dataset.glm_view(lik.x, lik.y)
      if d != lik.d_in:
        raise ValueError(f"field {lik.x!r} has {d} features, the network "
                         f"takes {lik.d_in}")
      return _lib.Mlp(lik.d_in, lik.h1, lik.h2, 1, int(n_obs),
                      int(dataset.observation_count), ld, X.data_ptr(), None,
                      float(lik.sigma), float(self.prior.scale),
                      float(self.temperature), 0), (X,)
    X, d, ld = dataset.matrix(self.likelihood.x)
    y = None if self.likelihood.y is None else dataset.vector(self.likelihood.y)
    return _lib.Glm(self.likelihood.family, d, int(n_obs), ld, X.data_ptr(),
                    None if y is None else y.data_ptr(),
                    float(self.likelihood.sigma), float(self.prior.scale),
                    float(self.temperature), 0,
                    int(dataset.observation_count)), (X, y)

  def dim(self, dataset) -> int:
    if self.is_network:
      return self.likelihood.param_count
    return dataset.feature_dim(self.likelihood.x)

  def status(self):
    import torch
    if self._status is None:
      self._status = torch.zeros(1, dtype=torch.int32, device="cuda")
    return self._status

  def check_status(self):
    """Raises if a kernel reported an error on this potential's status word."""
    if self._status is not None:
      code = int(self._status.item())
      if code != 0:
        self._status.zero_()
        raise _lib.GbsgmcError(code, "device status")

  def workspace(self, chains, n, d, model=None):
    import torch
    key = (chains, n, d)
    ws = self._ws.get(key)
    if ws is None:
      if self.is_cnn:
        nbytes = int(_lib.load().gbsgmc_cnn_workspace_bytes(chains, n))
        if nbytes == 0:
          raise _lib.GbsgmcError(_lib.ERR_SHAPE,
                                 f"CNN minibatch of {n} images: needs an even "
                                 "positive size")
      elif self.is_mlp:
        nbytes = int(_lib.load().gbsgmc_mlp_workspace_bytes(model, chains, n))
        if nbytes == 0:
          raise _lib.GbsgmcError(_lib.ERR_SHAPE,
                                 f"MLP minibatch of {n} rows: needs a "
                                 "positive multiple of 128")
      else:
        nbytes = int(_lib.load().gbsgmc_glm_workspace_bytes(chains, n, d))
      ws = torch.zeros(max(nbytes, 16), dtype=torch.uint8, device="cuda")
      self._ws[key] = ws
    return ws

  def fisher_workspace(self, chains, n, model):
    """Device workspace of gbsgmc_mlp_fisher_noise, cached per shape."""
    import torch
    key = ("fisher", chains, n)
    ws = self._ws.get(key)
    if ws is None:
      nbytes = int(_lib.load().gbsgmc_mlp_fisher_workspace_bytes(model, chains, n))
      if nbytes == 0:
        raise _lib.GbsgmcError(_lib.ERR_SHAPE,
                               f"MLP minibatch of {n} rows: needs a positive "
                               "multiple of 128")
      ws = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
      self._ws[key] = ws
    return ws

  # -- batched evaluation --------------------------------------------------
  def evaluate(self, W, idx, dataset, mask=None, grad=True, lk=False,
               observation_count=None, model=None, rows=None):
    """U, grad, lk, var for ``C`` chains: W [C, d], idx [C, n] int32.
    ``rows`` (network likelihoods only): int32 device [C], chain c uses the
    first rows[c] indices of its row of ``idx``."""
    import torch
    C, d = W.shape
    n = idx.shape[-1]
    if model is None:
      m, keep = self.model(dataset, observation_count)
    else:
      m, keep = model
    if self.is_network:
      if d != self.likelihood.param_count:
        raise ValueError(f"parameters per chain {d} != network parameters "
                         f"{self.likelihood.param_count}")
    elif m.d != d:
      raise ValueError(f"parameters per chain {d} != features {m.d}")
    U = torch.empty(C, dtype=torch.float64, device="cuda")
    var = torch.empty(C, dtype=torch.float64, device="cuda")
    g = torch.empty((C, d), dtype=torch.float32, device="cuda") if grad else None
    lko = torch.empty((C, n), dtype=torch.float32, device="cuda") if lk else None
    ws = self.workspace(C, n, d, m)
    W = W.to(torch.float32).contiguous()
    idx = idx.to(torch.int32).contiguous()
    if mask is not None:
      mask = mask.to(device="cuda", dtype=torch.float32).reshape(C, n).contiguous()
    if rows is not None:
      if not self.is_mlp:
        raise NotImplementedError("per-chain minibatch sizes are implemented "
                                  "for the network likelihoods")
      rows = rows.to(device="cuda", dtype=torch.int32).contiguous()
      _lib.call("gbsgmc_mlp_value_and_grad_ragged", m, C, n, _lib.ptr(rows),
                _lib.ptr(idx), idx.stride(0) if idx.dim() == 2 else n,
                _lib.ptr(mask), _lib.ptr(W), _lib.ptr(U), _lib.ptr(g),
                _lib.ptr(lko), _lib.ptr(var), _lib.ptr(ws), ws.numel(),
                _lib.ptr(self.status()), _lib.stream_handle())
      return GlmEval(U, g, lko, var)
    fn = "gbsgmc_cnn_value_and_grad" if self.is_cnn else \
        "gbsgmc_mlp_value_and_grad" if self.is_mlp else \
        "gbsgmc_glm_value_and_grad"
    _lib.call(fn, m, C, n, _lib.ptr(idx),
              idx.stride(0) if idx.dim() == 2 else n, _lib.ptr(mask),
              _lib.ptr(W), _lib.ptr(U), _lib.ptr(g),
              _lib.ptr(lko), _lib.ptr(var), _lib.ptr(ws), ws.numel(),
              _lib.ptr(self.status()), _lib.stream_handle())
    return GlmEval(U, g, lko, var)

  # -- reference-style interface ---------------------------------------------
  def _unpack(self, reference_data):
    if isinstance(reference_data, tuple) and len(reference_data) >= 2:
      batch, info = reference_data[0], reference_data[1]
    else:
      batch, info = reference_data, None
    if not isinstance(batch, IndexedBatch):
      raise TypeError("reference_data must come from gbsgmc.data "
                      "(an IndexedBatch and its MiniBatchInformation)")
    return batch, info

  def _eval_sample(self, sample, reference_data, mask, grad, lk):
    batch, info = self._unpack(reference_data)
    ds = batch.dataset
    self.likelihood.check_data(ds)
    d = self.dim(ds)
    w = _flat_device(sample, d).view(1, d)
    idx = batch.indices.reshape(1, -1)
    n_obs = info.observation_count if info is not None else ds.observation_count
    if mask is None and info is not None and info.mask is not None:
      mask = None  # the reference applies the mask only when passed explicitly
    return self.evaluate(w, idx, ds, mask=mask, grad=grad, lk=lk,
                         observation_count=n_obs)

  def __call__(self, sample, reference_data, state=None, mask=None,
               likelihoods=False):
    r = self._eval_sample(sample, reference_data, mask, grad=False,
                          lk=likelihoods)
    U = r.U[0]
    if likelihoods:
      return U, (r.lk[0], state)
    return U, state

  def value_and_grad(self, sample, reference_data, state=None, mask=None,
                     likelihoods=False):
    """``jax.value_and_grad(potential_fn, has_aux=True)`` equivalent:
    returns ``((U, aux), grad)`` with grad a flat fp32 device vector."""
    r = self._eval_sample(sample, reference_data, mask, grad=True,
                          lk=likelihoods)
    aux = (r.lk[0], state) if likelihoods else state
    return (r.U[0], aux), r.grad[0]

  def variance(self, sample, reference_data):
    r = self._eval_sample(sample, reference_data, None, grad=False, lk=False)
    return r.lk_var[0]

  def torch_function(self, reference_data):
    """A differentiable ``w -> U`` (torch.autograd.Function twin)."""
    import torch
    pot = self

    class _Potential(torch.autograd.Function):

      @staticmethod
      def forward(ctx, w):
        (U, _), g = pot.value_and_grad(w, reference_data)
        ctx.save_for_backward(g.view_as(w))
        return U.to(w.dtype)

      @staticmethod
      def backward(ctx, gU):
        (g,) = ctx.saved_tensors
        return gU * g

    return _Potential.apply


def minibatch_potential(prior, likelihood, strategy="map", has_state=False,
                        is_batched=False, temperature=1.0):
  """Initializes the potential function for a minibatch of data."""
  return StochasticPotential(prior, likelihood, strategy=strategy,
                             has_state=has_state, is_batched=is_batched,
                             temperature=temperature)


class FullPotential:
  """Potential over the complete dataset (potential.py:219-293):
  ``U = (-sum_{all i} lk_i - log p(sample)) / temperature``, evaluated in
  ordered chunks of observations with the GLM kernel."""

  CHUNK = 65536

  def __init__(self, prior, likelihood, strategy="map", has_state=False,
               is_batched=False, temperature=1.0):
    assert strategy != 'pmap', "Pmap is currently not supported"
    self.prior = prior
    self.likelihood = likelihood
    self.temperature = float(temperature)
    self._unit = StochasticPotential(prior, likelihood, strategy, has_state,
                                     is_batched, 1.0)
    self._flat = StochasticPotential(lkmod.FlatPrior(), likelihood, strategy,
                                     has_state, is_batched, 1.0)

  def value_and_grad_all(self, W, dataset):
    """U [C] and grad [C, d] over all observations for C chains."""
    import torch
    C, d = W.shape
    N = dataset.observation_count
    U = torch.zeros(C, dtype=torch.float64, device="cuda")
    g = torch.zeros((C, d), dtype=torch.float32, device="cuda")
    for start in range(0, N, self.CHUNK):
      n = min(self.CHUNK, N - start)
      idx = torch.arange(start, start + n, dtype=torch.int32, device="cuda")
      mask = None
      if self._unit.is_mlp and n % 128:
        # The network kernels take whole 128-row tiles: pad with row 0 at
        # mask weight 0.
        pad = 128 - n % 128
        idx = torch.cat([idx, torch.zeros(pad, dtype=torch.int32,
                                          device="cuda")])
        mask = torch.cat([torch.ones(n, device="cuda"),
                          torch.zeros(pad, device="cuda")]).expand(C, -1)
        n += pad
      idx = idx.expand(C, n)
      pot = self._unit if start == 0 else self._flat
      # n_obs = n makes the N/n scale 1: the chunk contributes -sum lk.
      r = pot.evaluate(W, idx, dataset, mask=mask, grad=True,
                       observation_count=n)
      U += r.U
      g += r.grad
    return U / self.temperature, g / self.temperature

  def __call__(self, sample, data_state, full_data_map_fn, state=None):
    loader = getattr(full_data_map_fn, "loader", None)
    if loader is None:
      raise TypeError("full_data_map_fn must come from "
                      "gbsgmc.data.full_reference_data / full_data_mapper")
    ds = loader.device_dataset()
    d = self._unit.dim(ds)
    w = _flat_device(sample, d).view(1, d)
    U, _ = self.value_and_grad_all(w, ds)
    return U[0], (data_state, state)


def full_potential(prior, likelihood, strategy="map", has_state=False,
                   is_batched=False, temperature=1.0):
  """Transforms a pdf to compute the full potential over all reference data."""
  return FullPotential(prior, likelihood, strategy=strategy,
                       has_state=has_state, is_batched=is_batched,
                       temperature=temperature)
