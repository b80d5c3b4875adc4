"""CPU restatement of jax_sgmc's sampling hot path -- TEST INFRASTRUCTURE ONLY.

The CUDA path is checked against it by tests/, __graft_entry__.smoke() and
bench.py's CPU baseline; the product path never calls it.  numpy only.  Each function cites the
reference (jax_sgmc 0.1.5) file:line it follows; float32 variants follow the
reference's operation order so that results agree with the fp32 kernels to
rounding, float64 variants serve as the accuracy oracle.
"""

from __future__ import annotations

import math
from typing import NamedTuple

import numpy as np

# ---------------------------------------------------------------------------
# Index streams
# ---------------------------------------------------------------------------


def loader_rng(seed: int) -> np.random.Generator:
  """The per-chain generator of NumpyDataLoader.register_random_pipeline
  (jax_sgmc/data/numpy_loader.py:261-265)."""
  return np.random.default_rng(np.random.SeedSequence(seed).spawn(1)[0])


def loader_draws(rng: np.random.Generator, n_obs: int, mb_size: int,
                 batches: int) -> np.ndarray:
  """``batches`` consecutive minibatches of NumpyDataLoader._draw_indices
  (jax_sgmc/data/numpy_loader.py:382-389), shape [batches, mb_size]."""
  return np.stack([rng.choice(np.arange(0, n_obs), size=mb_size, replace=True)
                   for _ in range(batches)])


_M128 = (1 << 128) - 1
_PCG_MULT = 0x2360ED051FC65DA44385DF649FCCF645


def _pcg_out(s: int) -> int:
  hi, lo = s >> 64, s & ((1 << 64) - 1)
  x, rot = hi ^ lo, s >> 122
  return ((x >> rot) | (x << ((64 - rot) & 63))) & ((1 << 64) - 1)


def pcg64_bounded(state: dict, n_obs: int, count: int):
  """Restatement of numpy's bounded int64 draws on PCG64 (pure Python ints).

  PCG64 = 128-bit LCG with XSL-RR output (O'Neill 2014); next_uint32 returns
  the low half of a fresh output and buffers the high half
  (has_uint32/uinteger); Generator.integers(0, N) for N < 2^32 uses Lemire's
  bounded method on those 32-bit values (Lemire 2019).  Returns
  (indices, new_state) with new_state shaped like numpy's state dict.
  """
  s = state["state"]["state"]
  inc = state["state"]["inc"]
  has = state["has_uint32"]
  u = state["uinteger"]
  out = np.empty(count, np.int64)
  if n_obs == 1:
    out[:] = 0
    return out, dict(state)
  thr = (1 << 32) % n_obs
  for i in range(count):
    while True:
      if has:
        has, x = 0, u
      else:
        s = (s * _PCG_MULT + inc) & _M128
        o = _pcg_out(s)
        has, u, x = 1, o >> 32, o & 0xFFFFFFFF
      m = x * n_obs
      if (m & 0xFFFFFFFF) >= thr:
        break
    out[i] = m >> 32
  new = {"bit_generator": "PCG64", "state": {"state": s, "inc": inc},
         "has_uint32": has, "uinteger": u}
  return out, new


# ---------------------------------------------------------------------------
# Philox4x32-10 (Salmon et al., SC'11) and the production noise mapping
# ---------------------------------------------------------------------------

_M0, _M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
_W0, _W1 = 0x9E3779B9, 0xBB67AE85


def philox4x32_10(ctr, key):
  """Vectorised Philox4x32-10.  ctr: uint32 [..., 4]; key: (k0, k1)."""
  c = np.asarray(ctr, dtype=np.uint64) & np.uint64(0xFFFFFFFF)
  c0, c1, c2, c3 = (c[..., i].copy() for i in range(4))
  k0, k1 = int(key[0]) & 0xFFFFFFFF, int(key[1]) & 0xFFFFFFFF
  mask = np.uint64(0xFFFFFFFF)
  for r in range(10):
    if r:
      k0 = (k0 + _W0) & 0xFFFFFFFF
      k1 = (k1 + _W1) & 0xFFFFFFFF
    p0 = _M0 * c0
    p1 = _M1 * c2
    n0 = ((p1 >> np.uint64(32)) ^ c1 ^ np.uint64(k0)) & mask
    n1 = p1 & mask
    n2 = ((p0 >> np.uint64(32)) ^ c3 ^ np.uint64(k1)) & mask
    n3 = p0 & mask
    c0, c1, c2, c3 = n0, n1, n2, n3
  return np.stack([c0, c1, c2, c3], axis=-1).astype(np.uint32)


def _open01(v):
  return ((v.astype(np.uint64) >> np.uint64(9)).astype(np.float64) + 0.5) / 8388608.0


def philox_normals(seed: int, chain: int, step: int, tag: int, count: int):
  """Normals of one chain/step/tag: group g of 4 parameters uses
  Philox(counter=(g, step, chain, tag), key=seed) and Box-Muller on the pairs
  (u0,u1), (u2,u3) with u = (top 23 bits + 0.5) / 2^23 (float64)."""
  groups = (count + 3) // 4
  ctr = np.zeros((groups, 4), np.uint64)
  ctr[:, 0] = np.arange(groups)
  ctr[:, 1] = step & 0xFFFFFFFF
  ctr[:, 2] = chain & 0xFFFFFFFF
  ctr[:, 3] = tag
  r = philox4x32_10(ctr, (seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF))
  out = np.empty((groups, 4), np.float64)
  for a, b, i in ((0, 1, 0), (2, 3, 2)):
    u1, u2 = _open01(r[:, a]), _open01(r[:, b])
    rad = np.sqrt(-2.0 * np.log(u1))
    out[:, i] = rad * np.cos(2 * np.pi * u2)
    out[:, i + 1] = rad * np.sin(2 * np.pi * u2)
  return out.reshape(-1)[:count]


def philox_indices(seed: int, chain: int, step: int, per_step: int, n_obs: int):
  """Counter-based index draws: pair p uses Philox(counter=(p, step, chain,
  6), key=seed); draw 2p = floor(((r1<<32)|r0) * N / 2^64), 2p+1 from
  (r3, r2)."""
  pairs = (per_step + 1) // 2
  ctr = np.zeros((pairs, 4), np.uint64)
  ctr[:, 0] = np.arange(pairs)
  ctr[:, 1] = step & 0xFFFFFFFF
  ctr[:, 2] = chain & 0xFFFFFFFF
  ctr[:, 3] = 6
  r = philox4x32_10(ctr, (seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF))
  out = np.empty(2 * pairs, np.int64)
  for j, (lo, hi) in enumerate(((0, 1), (2, 3))):
    u = (r[:, hi].astype(object) << 32) | r[:, lo].astype(object)
    out[j::2] = np.array([(int(x) * n_obs) >> 64 for x in u], dtype=np.int64)
  return out[:per_step]


# ---------------------------------------------------------------------------
# Likelihood families and the stochastic potential
# ---------------------------------------------------------------------------

LINEAR_GAUSSIAN, LOGISTIC, LINEAR = 0, 1, 2


def glm_lk(family, z, y, sigma=1.0):
  """Per-observation log-likelihood and dlk/dz (float64)."""
  z = np.asarray(z, np.float64)
  y = np.asarray(y, np.float64)
  if family == LOGISTIC:
    sp = np.maximum(z, 0.0) + np.log1p(np.exp(-np.abs(z)))
    return y * z - sp, y - 1.0 / (1.0 + np.exp(-z))
  if family == LINEAR:
    return z.copy(), np.ones_like(z)
  r = y - z
  return (-0.5 * r * r / sigma ** 2 - math.log(sigma) - 0.5 * math.log(2 * math.pi),
          r / sigma ** 2)


def log_prior(w, prior_scale):
  """sum_j norm.logpdf(w_j, 0, prior_scale); 0 for prior_scale <= 0."""
  w = np.asarray(w, np.float64)
  if prior_scale is None or prior_scale <= 0:
    return np.zeros(w.shape[:-1]), np.zeros_like(w)
  s2 = prior_scale ** 2
  d = w.shape[-1]
  lp = -0.5 * np.sum(w * w, -1) / s2 - d * (math.log(prior_scale)
                                           + 0.5 * math.log(2 * math.pi))
  return lp, -w / s2


class Potential(NamedTuple):
  U: np.ndarray
  grad: np.ndarray
  lk: np.ndarray
  var: np.ndarray


def glm_potential(W, X, y, idx, n_obs, family, sigma=1.0, prior_scale=0.0,
                  temperature=1.0, mask=None) -> Potential:
  """Minibatch potential and gradient for C chains, float64.

  U = (-N * mean_i lk_i - log p(w)) / T, or with a mask
  U = (-N/n * sum_i mask_i lk_i - log p(w)) / T
  (jax_sgmc/potential.py:159-214); var = jnp.var(lk) (integrator.py:880).
  W [C, d], idx [C, n].
  """
  W = np.atleast_2d(np.asarray(W, np.float64))
  idx = np.atleast_2d(np.asarray(idx))
  Xb = np.asarray(X, np.float64)[idx]              # [C, n, d]
  yb = np.asarray(y, np.float64)[idx]              # [C, n]
  z = np.einsum("cnd,cd->cn", Xb, W)
  lk, dz = glm_lk(family, z, yb, sigma)
  n = idx.shape[-1]
  m = np.ones_like(lk) if mask is None else np.asarray(mask, np.float64).reshape(lk.shape)
  lp, dlp = log_prior(W, prior_scale)
  U = (-(n_obs / n) * np.sum(m * lk, -1) - lp) / temperature
  grad = (-(n_obs / n) * np.einsum("cn,cnd->cd", m * dz, Xb) - dlp) / temperature
  return Potential(U, grad, lk, np.var(lk, axis=-1))


def full_potential(w, X, y, family, sigma=1.0, prior_scale=0.0,
                   temperature=1.0):
  """Full-data potential (-sum_i lk_i - log p) / T (potential.py:219-293)."""
  w = np.asarray(w, np.float64)
  z = np.asarray(X, np.float64) @ w
  lk, dz = glm_lk(family, z, y, sigma)
  lp, dlp = log_prior(w[None], prior_scale)
  U = (-np.sum(lk) - lp[0]) / temperature
  g = (-(dz @ np.asarray(X, np.float64)) - dlp[0]) / temperature
  return U, g


def fisher_variance(w, X, y, idx, grad, n_obs, family, sigma):
  """v = ssq / (n - 1) of fisher_information's get (jax_sgmc/adaption.py
  403-437), float64, one chain: the per-observation gradients of the
  likelihoods lk_i (not the potential) against grad / N."""
  w = np.asarray(w, np.float64)
  Xb = np.asarray(X, np.float64)[np.asarray(idx)]
  yb = np.asarray(y, np.float64)[np.asarray(idx)]
  _, dz = glm_lk(family, Xb @ w, yb, sigma)
  gbar = np.asarray(grad, np.float64) / n_obs
  ssq = np.sum((dz[:, None] * Xb - gbar) ** 2, axis=0)
  return 1.0 / (len(idx) - 1) * ssq


def fisher_noise_from_ssq(ssq, n, friction, step_size):
  """The diagonal branch of fisher_information's get (jax_sgmc/adaption.py
  432-445) from ssq [P] of one chain: v = ssq / (n - 1), b = 0.5 h v,
  corr = friction - b with corr <= 0 replaced by the smallest positive corr;
  returns (sqrt(corr), sqrt(friction - corr))."""
  b = 0.5 * step_size * (np.asarray(ssq, np.float64) / (n - 1))
  f = np.broadcast_to(np.asarray(friction, np.float64), b.shape)
  corr = f - b
  smallest = np.min(np.where(corr <= 0, np.inf, corr))
  pc = np.where(corr <= 0, smallest, corr)
  return np.sqrt(pc), np.sqrt(f - pc)


def fisher_noise(w, X, y, idx, grad, n_obs, family, sigma, friction, step_size):
  """fisher_information(diagonal=True).get (jax_sgmc/adaption.py:403-455),
  float64, one chain: :func:`fisher_noise_from_ssq` of the ssq of
  :func:`fisher_variance`."""
  n = len(idx)
  v = fisher_variance(w, X, y, idx, grad, n_obs, family, sigma)
  return fisher_noise_from_ssq(v * (n - 1), n, friction, step_size)


def sym_eig(A):
  """Symmetric eigendecomposition with the library's conventions (float64,
  numpy.linalg.eigh): eigenvalues ascending, each eigenvector's
  largest-magnitude component (the first of equal ones) positive."""
  w, V = np.linalg.eigh(0.5 * (np.asarray(A, np.float64) + np.asarray(A, np.float64).T))
  k = np.argmax(np.abs(V), axis=0)
  return w, V * np.where(V[k, np.arange(V.shape[1])] < 0, -1.0, 1.0)


def fisher_noise_dense(w, X, y, idx, grad, n_obs, family, sigma, friction,
                       step_size):
  """fisher_information(diagonal=False).get (jax_sgmc/adaption.py:403-452),
  float64, one chain: b = 0.5 h / (n - 1) sum_i d_i d_i^T with d_i the
  per-observation likelihood gradient minus grad / N;
  cb_diff_sqrt = u sqrt(s) of svd(diag(friction) - b), b_sqrt = u sqrt(s)
  of svd(b).  For these symmetric matrices the SVD is taken from
  :func:`sym_eig` (s = |eigenvalue|, u = the eigenvectors), the sign
  convention the library uses where LAPACK's is unspecified."""
  w = np.asarray(w, np.float64)
  Xb = np.asarray(X, np.float64)[np.asarray(idx)]
  yb = np.asarray(y, np.float64)[np.asarray(idx)]
  _, dz = glm_lk(family, Xb @ w, yb, sigma)
  D = dz[:, None] * Xb - np.asarray(grad, np.float64) / n_obs
  b = 0.5 * step_size / (len(idx) - 1) * (D.T @ D)
  f = np.broadcast_to(np.asarray(friction, np.float64), (b.shape[0],))

  def root(M):
    lam, U = sym_eig(M)
    return U @ np.sqrt(np.abs(lam))

  return root(np.diag(f) - b), root(b)


# ---------------------------------------------------------------------------
# Dense tanh network with a Gaussian likelihood
# ---------------------------------------------------------------------------
# The reference leaves the likelihood to user code (minibatch_potential's
# ``likelihood`` argument, jax_sgmc/potential.py:94-99) and differentiates the
# potential with jax.value_and_grad (integrator.py:166,593,792).  The network
# below is the one of the MLP regression workload: parameters are the pytree
# {W1 [D,H1], W2 [H1,H2], W3 [H2,1], b1 [H1], b2 [H2], b3 [1]}, raveled in
# sorted key order as jax.flatten_util.ravel_pytree does.  The adjoint is the
# chain rule written out; tests pin it to torch autograd and to central
# finite differences.


def mlp_offsets(d_in, h1, h2):
  """Offsets of W1, W2, W3, b1, b2, b3 in the flat vector, and P."""
  sizes = [d_in * h1, h1 * h2, h2, h1, h2, 1]
  off = np.concatenate([[0], np.cumsum(sizes)])
  return [int(v) for v in off[:-1]], int(off[-1])


def mlp_unravel(w, d_in, h1, h2):
  """Leaves of the flat vector (numpy arrays, or views of a torch tensor)."""
  if not hasattr(w, "reshape"):
    w = np.asarray(w)
  (o1, o2, o3, ob1, ob2, ob3), _ = mlp_offsets(d_in, h1, h2)
  return (w[..., o1:o2].reshape(w.shape[:-1] + (d_in, h1)),
          w[..., o2:o3].reshape(w.shape[:-1] + (h1, h2)),
          w[..., o3:ob1], w[..., ob1:ob2], w[..., ob2:ob3], w[..., ob3])


def mlp_forward(W, Xb, d_in, h1, h2):
  """out [C, n] and the hidden activations Z1, Z2 for rows Xb [C, n, D]."""
  W1, W2, W3, b1, b2, b3 = mlp_unravel(W, d_in, h1, h2)
  Z1 = np.tanh(Xb @ W1 + b1[:, None, :])
  Z2 = np.tanh(Z1 @ W2 + b2[:, None, :])
  out = (Z2 @ W3[..., None])[..., 0] + b3[:, None]
  return out, Z1, Z2


def mlp_potential(W, X, y, idx, n_obs, d_in, h1, h2, sigma, prior_scale=0.0,
                  temperature=1.0, mask=None) -> Potential:
  """Minibatch potential of the tanh network for C chains, float64.

  out = tanh(tanh(x W1 + b1) W2 + b2) W3 + b3, lk = log N(y | out, sigma^2),
  U = (-N/n sum_i m_i lk_i - log p(w)) / T (potential.py:159-214), var =
  jnp.var(lk) (integrator.py:880).  W [C, P], idx [C, n].
  """
  W = np.atleast_2d(np.asarray(W, np.float64))
  idx = np.atleast_2d(np.asarray(idx))
  C, P = W.shape
  W1, W2, W3, b1, b2, b3 = mlp_unravel(W, d_in, h1, h2)
  Xb = np.asarray(X, np.float64)[idx][..., :d_in]   # [C, n, D]
  yb = np.asarray(y, np.float64)[idx]                # [C, n]
  n = idx.shape[-1]
  out, Z1, Z2 = mlp_forward(W, Xb, d_in, h1, h2)
  r = yb - out
  lk = -0.5 * (r / sigma) ** 2 - math.log(sigma) - 0.5 * math.log(2 * math.pi)
  m = np.ones_like(lk) if mask is None else np.asarray(mask, np.float64).reshape(lk.shape)
  lp, dlp = log_prior(W, prior_scale)
  U = (-(n_obs / n) * np.sum(m * lk, -1) - lp) / temperature
  g = -(n_obs / n) * m * r / sigma ** 2 / temperature          # dU/dout
  G2 = g[..., None] * W3[:, None, :] * (1.0 - Z2 ** 2)
  G1 = (G2 @ W2.transpose(0, 2, 1)) * (1.0 - Z1 ** 2)
  grad = np.concatenate([
      (Xb.transpose(0, 2, 1) @ G1).reshape(C, -1),
      (Z1.transpose(0, 2, 1) @ G2).reshape(C, -1),
      (g[:, None, :] @ Z2)[:, 0, :],
      G1.sum(1), G2.sum(1), g.sum(1, keepdims=True)], axis=1)
  grad = grad - dlp / temperature
  return Potential(U, grad, lk, np.var(lk, axis=-1))


def mlp_fisher_sums(W, X, y, idx, d_in, h1, h2, sigma):
  """Sums over the minibatch of the per-observation likelihood gradients
  d_i = d lk_i / d w and of their squares (S1, S2 [C, P]), float64: the
  adjoint of mlp_potential seeded with d lk_i / d out = (y_i - out_i) /
  sigma^2, and d_i^2 summed leaf by leaf (for W2: (Z1^2)^T (G2^2))."""
  W = np.atleast_2d(np.asarray(W, np.float64))
  idx = np.atleast_2d(np.asarray(idx))
  C = W.shape[0]
  _, W2, W3, _, _, _ = mlp_unravel(W, d_in, h1, h2)
  Xb = np.asarray(X, np.float64)[idx][..., :d_in]
  yb = np.asarray(y, np.float64)[idx]
  out, Z1, Z2 = mlp_forward(W, Xb, d_in, h1, h2)
  g = (yb - out) / sigma ** 2
  G2 = g[..., None] * W3[:, None, :] * (1.0 - Z2 ** 2)
  G1 = (G2 @ W2.transpose(0, 2, 1)) * (1.0 - Z1 ** 2)
  tr = lambda a: a.transpose(0, 2, 1)
  S1 = np.concatenate([(tr(Xb) @ G1).reshape(C, -1), (tr(Z1) @ G2).reshape(C, -1),
                       (g[:, None, :] @ Z2)[:, 0, :], G1.sum(1), G2.sum(1),
                       g.sum(1, keepdims=True)], axis=1)
  S2 = np.concatenate([(tr(Xb ** 2) @ G1 ** 2).reshape(C, -1),
                       (tr(Z1 ** 2) @ G2 ** 2).reshape(C, -1),
                       ((g ** 2)[:, None, :] @ Z2 ** 2)[:, 0, :], (G1 ** 2).sum(1),
                       (G2 ** 2).sum(1), (g ** 2).sum(1, keepdims=True)], axis=1)
  return S1, S2


def mlp_fisher_noise(W, X, y, idx, grad, n_obs, d_in, h1, h2, sigma, friction,
                     step_size):
  """fisher_information(diagonal=True).get (jax_sgmc/adaption.py:403-455) on
  the tanh network, float64, C chains: ssq = sum_i (d_i - grad / N)^2 from
  :func:`mlp_fisher_sums` as S2 - 2 gbar S1 + n gbar^2 (exact algebra; fp64
  holds it without cancellation here), then the correction of
  :func:`fisher_noise`.  Returns (cb_diff_sqrt, b_sqrt) [C, P]."""
  S1, S2 = mlp_fisher_sums(W, X, y, idx, d_in, h1, h2, sigma)
  n = np.atleast_2d(idx).shape[-1]
  gbar = np.atleast_2d(np.asarray(grad, np.float64)) / n_obs
  ssq = np.maximum(S2 - 2.0 * gbar * S1 + n * gbar ** 2, 0.0)
  b = 0.5 * step_size * ssq / (n - 1)
  f = np.broadcast_to(np.asarray(friction, np.float64), (b.shape[-1],))
  corr = f - b
  cb, bs = np.empty_like(b), np.empty_like(b)
  for c in range(b.shape[0]):
    pos = corr[c] > 0
    smallest = np.min(corr[c][pos]) if pos.any() else np.inf
    pc = np.where(corr[c] <= 0, smallest, corr[c])
    cb[c], bs[c] = np.sqrt(pc), np.sqrt(f - pc)
  return cb, bs


# ---------------------------------------------------------------------------
# Convolutional classifier (softmax likelihood)
# ---------------------------------------------------------------------------
# conv3x3(32) ReLU maxpool2 -> conv3x3(64) ReLU maxpool2 -> conv3x3(128)
# ReLU maxpool2 -> dense(10), NHWC, SAME padding; lk = -softmax cross entropy
# (examples/cifar.md:203-210).  Parameters: the sorted ravel of
# {conv1: {b, w}, conv2: {b, w}, conv3: {b, w}, linear: {b, w}}, HWIO weights.

CNN_CHANNELS = (3, 32, 64, 128)
CNN_CLASSES = 10


def cnn_offsets():
  sizes, names = [], []
  for l in range(3):
    ci, co = CNN_CHANNELS[l], CNN_CHANNELS[l + 1]
    names += [f"b{l + 1}", f"W{l + 1}"]
    sizes += [co, 9 * ci * co]
  names += ["bd", "Wd"]
  sizes += [CNN_CLASSES, 4 * 4 * 128 * CNN_CLASSES]
  off = np.concatenate([[0], np.cumsum(sizes)]).astype(int)
  return dict(zip(names, zip(off[:-1], off[1:]))), int(off[-1])


def _im2col(x):
  """x [n, H, W, C] -> [n*H*W, 9C] with columns (kh, kw, ci), SAME padding."""
  n, H, W, C = x.shape
  xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
  cols = [xp[:, kh:kh + H, kw:kw + W, :] for kh in range(3) for kw in range(3)]
  return np.concatenate(cols, axis=-1).reshape(n * H * W, 9 * C)


def _col2im(dcols, shape):
  n, H, W, C = shape
  d = dcols.reshape(n, H, W, 9, C)
  out = np.zeros((n, H + 2, W + 2, C))
  for t in range(9):
    kh, kw = divmod(t, 3)
    out[:, kh:kh + H, kw:kw + W, :] += d[:, :, :, t, :]
  return out[:, 1:H + 1, 1:W + 1, :]


def _pool(a):
  """2x2 max-pool with the argmax (first maximum, row-major in the window)."""
  n, H, W, C = a.shape
  win = a.reshape(n, H // 2, 2, W // 2, 2, C).transpose(0, 1, 3, 2, 4, 5)
  win = win.reshape(n, H // 2, W // 2, 4, C)
  return win.max(axis=3), win.argmax(axis=3)


def _unpool(dp, arg, shape):
  n, H, W, C = shape
  d = np.zeros((n, H // 2, W // 2, 4, C))
  np.put_along_axis(d, arg[:, :, :, None, :], dp[:, :, :, None, :], axis=3)
  d = d.reshape(n, H // 2, W // 2, 2, 2, C).transpose(0, 1, 3, 2, 4, 5)
  return d.reshape(n, H, W, C)


def round_bf16(x):
  """Round-to-nearest-even to bfloat16 (the top 16 bits of float32), as
  float64.  Used to give the oracle the activation precision of a BF16
  pipeline."""
  a = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
  r = ((a + 0x7FFF + ((a >> 16) & 1)) >> 16) << 16
  return r.astype(np.uint32).view(np.float32).astype(np.float64)


def cnn_potential(w, images, labels, idx, n_obs, prior_scale=0.0,
                  temperature=1.0, mask=None, activations=None,
                  bf16_operands=False) -> Potential:
  """Minibatch potential of the classifier for ONE chain, float64:
  U = (-N/n sum_i m_i lk_i - log p(w)) / T, lk_i = log softmax(logits_i)[y_i].

  ``activations`` (e.g. round_bf16) is applied to each ReLU output before
  pooling: a 2x2 max over BF16-rounded values can pick a different window
  element than the exact maximum, and that changes where the gradient flows.
  ``bf16_operands`` rounds, to BF16, exactly the values a BF16 GEMM pipeline
  feeds its tensor cores -- the images, the conv weights, the pooled maps and
  the conv output gradients dY -- and keeps everything else (accumulation,
  ReLU outputs, the dense layer, the input gradients dY W^T summed over the
  taps, which the kernels compute as one transposed convolution into fp32)
  in float64: the arithmetic of the GPU kernels up to summation order.
  """
  off, P = cnn_offsets()
  w = np.asarray(w, np.float64)
  rnd = round_bf16 if bf16_operands else (lambda v: v)
  get = lambda k: w[off[k][0]:off[k][1]]
  x = rnd(np.asarray(images, np.float64)[idx].reshape(-1, 32, 32, 3))
  y = np.asarray(labels)[idx].astype(int)
  n = x.shape[0]
  acts = []
  h = x
  for l in range(3):
    ci, co = CNN_CHANNELS[l], CNN_CHANNELS[l + 1]
    cols = _im2col(h)
    wl = rnd(get(f"W{l + 1}")).reshape(9 * ci, co)
    z = cols @ wl + get(f"b{l + 1}")
    a = np.maximum(z, 0).reshape(h.shape[0], h.shape[1], h.shape[2], co)
    if activations is not None:
      a = activations(a)
    p, arg = _pool(a)
    acts.append((h.shape, cols, a, arg, wl))
    h = rnd(p)
  flat = h.reshape(n, -1)
  logits = flat @ get("Wd").reshape(-1, CNN_CLASSES) + get("bd")
  mx = logits.max(1, keepdims=True)
  lse = (mx + np.log(np.exp(logits - mx).sum(1, keepdims=True)))[:, 0]
  lk = logits[np.arange(n), y] - lse
  m = np.ones(n) if mask is None else np.asarray(mask, np.float64).reshape(n)
  lp, dlp = log_prior(w[None], prior_scale)
  U = (-(n_obs / n) * np.sum(m * lk) - lp[0]) / temperature
  soft = np.exp(logits - lse[:, None])
  onehot = np.zeros_like(soft)
  onehot[np.arange(n), y] = 1
  g = -(n_obs / n) * m[:, None] * (onehot - soft) / temperature
  grad = np.zeros(P)
  grad[off["Wd"][0]:off["Wd"][1]] = (flat.T @ g).reshape(-1)
  grad[off["bd"][0]:off["bd"][1]] = g.sum(0)
  dh = (g @ get("Wd").reshape(-1, CNN_CLASSES).T).reshape(h.shape)
  for l in (2, 1, 0):
    shape_in, cols, a, arg, wl = acts[l]
    co = CNN_CHANNELS[l + 1]
    da = rnd(_unpool(dh, arg, a.shape) * (a > 0))
    dz = da.reshape(-1, co)
    grad[off[f"W{l + 1}"][0]:off[f"W{l + 1}"][1]] = (cols.T @ dz).reshape(-1)
    grad[off[f"b{l + 1}"][0]:off[f"b{l + 1}"][1]] = dz.sum(0)
    if l > 0:
      dh = _col2im(dz @ wl.T, shape_in)
  grad = grad - dlp[0] / temperature
  return Potential(np.array([U]), grad[None], lk[None], np.array([np.var(lk)]))


def linear_posterior(X, y, sigma, prior_scale):
  """Closed-form posterior of Bayesian linear regression with known noise:
  Sigma = (X^T X / s^2 + I / p^2)^-1, mu = Sigma X^T y / s^2."""
  X = np.asarray(X, np.float64)
  d = X.shape[1]
  prec = X.T @ X / sigma ** 2 + np.eye(d) / prior_scale ** 2
  cov = np.linalg.inv(prec)
  mu = cov @ (X.T @ np.asarray(y, np.float64)) / sigma ** 2
  return mu, cov


# ---------------------------------------------------------------------------
# Integrator steps (float32, reference operation order)
# ---------------------------------------------------------------------------

f32 = np.float32


def sgld_step(x, g, v, xi, h, T, alpha=0.9, lmbd=1e-5, rms_prop=True):
  """langevin_diffusion.update_fn (jax_sgmc/integrator.py:882-912) with
  rms_prop update-then-get (jax_sgmc/adaption.py:254-291).  Returns (x', v')."""
  x, g, xi = (np.asarray(a, f32) for a in (x, g, xi))
  h, T = f32(h), f32(T)
  scaled_gradient = (-h) * g
  scaled_noise = np.sqrt(f32(2.0) * T * h, dtype=f32) * xi
  if not rms_prop:
    return (x + (scaled_gradient + scaled_noise)).astype(f32), v
  a = f32(alpha)
  v = (a * np.asarray(v, f32) + (f32(1.0) - a) * (g * g)).astype(f32)
  G = (f32(1.0) / (f32(lmbd) + np.sqrt(v, dtype=f32))).astype(f32)
  upd = (f32(0.0) + G * scaled_gradient) + np.sqrt(G, dtype=f32) * scaled_noise
  return (x + upd).astype(f32), v


def obabo_first(x, p, g1, xi1, h, T, friction, mass=None):
  """O, KE_start, B, A of obabo._leapfrog_steps (integrator.py:192-241)."""
  x, p, g1, xi1 = (np.asarray(a, f32) for a in (x, p, g1, xi1))
  h, T, f = f32(h), f32(T), f32(friction)
  mi = f32(1.0) if mass is None else (f32(1.0) / np.asarray(mass, f32))
  ms = f32(1.0) if mass is None else np.sqrt(np.asarray(mass, f32))
  perm = np.exp(-f * h, dtype=f32)
  p = np.sqrt(perm, dtype=f32) * p + np.sqrt((f32(1) - perm) * T, dtype=f32) * (ms * xi1)
  ke = 0.5 * np.sum(p.astype(np.float64) * (mi * p).astype(np.float64), -1)
  p = (-(f32(0.5) * h)) * g1 + p
  x = x + h * (mi * p)
  return x.astype(f32), p.astype(f32), ke


def obabo_second(p, g2, xi2, h, T, friction, mass=None):
  """B, KE_end, O of obabo._leapfrog_steps (integrator.py:243-273)."""
  p, g2, xi2 = (np.asarray(a, f32) for a in (p, g2, xi2))
  h, T, f = f32(h), f32(T), f32(friction)
  mi = f32(1.0) if mass is None else (f32(1.0) / np.asarray(mass, f32))
  ms = f32(1.0) if mass is None else np.sqrt(np.asarray(mass, f32))
  p = (-(f32(0.5) * h)) * g2 + p
  ke = 0.5 * np.sum(p.astype(np.float64) * (mi * p).astype(np.float64), -1)
  perm = np.exp(-f * h, dtype=f32)
  p = np.sqrt(perm, dtype=f32) * p + np.sqrt((f32(1) - perm) * T, dtype=f32) * (ms * xi2)
  return p.astype(f32), ke


def sghmc_resample(xi, mass=None):
  """p = sqrt(M) xi (integrator.py:735-738)."""
  ms = f32(1.0) if mass is None else np.sqrt(np.asarray(mass, f32))
  return (ms * np.asarray(xi, f32)).astype(f32)


def sghmc_position(x, p, h, friction, mass=None):
  """x += h M^-1 p; p += (-h f) M^-1 p (integrator.py:608-619)."""
  x, p = np.asarray(x, f32), np.asarray(p, f32)
  h = f32(h)
  f = np.asarray(friction, f32)
  mi = f32(1.0) if mass is None else (f32(1.0) / np.asarray(mass, f32))
  sm = mi * p
  return (x + h * sm).astype(f32), (p + ((-h) * f) * sm).astype(f32)


def sghmc_momentum(p, g, xi, h, friction):
  """p += -h g; p += f sqrt(2h) xi (integrator.py:621-655, no noise model)."""
  p, g, xi = (np.asarray(a, f32) for a in (p, g, xi))
  h = f32(h)
  f = np.asarray(friction, f32)
  p = p + (-h) * g
  return (p + f * (np.sqrt(f32(2.0) * h, dtype=f32) * xi)).astype(f32)


def leapfrog_position(x, p, h, scale, mass=None):
  """x + (scale h) M^-1 p: the half / full position steps of
  reversible_leapfrog (integrator.py:383-388), fp32."""
  x, p = np.asarray(x, f32), np.asarray(p, f32)
  mi = f32(1.0) if mass is None else (f32(1.0) / np.asarray(mass, f32))
  s = f32(scale) * f32(h)
  return (x + s * (mi * p)).astype(f32)


def amagold_momentum(p, g, xi, h, friction, mass=None):
  """One momentum step of reversible_leapfrog (integrator.py:402-458):
  p' = ((1 - h f) p - h g + sqrt(4 f h) sqrt(M) xi) / (1 + h f), and the
  energy 0.5 h (p + p') . M^-1 g (fp64 sum of fp32 products).  Returns
  (p', energy)."""
  p, g, xi = (np.asarray(a, f32) for a in (p, g, xi))
  h, f = f32(h), f32(friction)
  mi = f32(1.0) if mass is None else (f32(1.0) / np.asarray(mass, f32))
  ms = f32(1.0) if mass is None else np.sqrt(np.asarray(mass, f32))
  decay = f32(1.0) - h * f
  inv = f32(1.0) / (f32(1.0) + h * f)
  ns = np.sqrt(f32(4.0) * f * h, dtype=f32)
  pn = (inv * ((decay * p + (-h) * g) + ns * (ms * xi))).astype(f32)
  energy = 0.5 * float(h) * float(np.sum((p + pn).astype(np.float64) *
                                         (mi * g).astype(np.float64)))
  return pn, energy


def reversible_leapfrog(x, p, grad_fn, xis, h, friction, mass=None):
  """integrate of reversible_leapfrog (integrator.py:510-553): half position
  step, len(xis) momentum steps (a full position step before each but the
  first; grad_fn(x, j) gives the stochastic gradient of step j), half
  position step.  Returns (x, p, accumulated energy)."""
  x = leapfrog_position(x, p, h, 0.5, mass)
  energy = 0.0
  for j, xi in enumerate(xis):
    if j > 0:
      x = leapfrog_position(x, p, h, 1.0, mass)
    p, e = amagold_momentum(p, grad_fn(x, j), xi, h, friction, mass)
    energy += e
  x = leapfrog_position(x, p, h, 0.5, mass)
  return x, p, energy


def dense_leapfrog_position(x, p, h, scale, minv):
  """x + (scale h) M^-1 p with a dense inverse mass (integrator.py:383-388
  with tensor_matmul of an ndim-2 Tensor, util/tree_util.py:38-56); float64,
  rows [C, P] of chains."""
  x, p = np.asarray(x, np.float64), np.asarray(p, np.float64)
  return x + float(scale) * float(h) * (p @ np.asarray(minv, np.float64).T)


def dense_amagold_momentum(p, g, xi, h, friction, minv, msqrt):
  """amagold_momentum with dense matrices (integrator.py:390-458): p' = ((1 -
  h f) p - h g + sqrt(4 f h) M^1/2 xi) / (1 + h f), energy 0.5 h (p + p') .
  M^-1 g per chain; float64.  Returns (p', energy [C])."""
  p, g, xi = (np.asarray(a, np.float64) for a in (p, g, xi))
  mi, ms = np.asarray(minv, np.float64), np.asarray(msqrt, np.float64)
  h, f = float(h), float(friction)
  pn = ((1 - h * f) * p - h * g + math.sqrt(4 * f * h) * (xi @ ms.T)) / (1 + h * f)
  return pn, 0.5 * h * np.sum((p + pn) * (g @ mi.T), -1)


def dense_obabo_first(x, p, g1, xi1, h, T, friction, minv, msqrt):
  """obabo_first with dense matrices (integrator.py:177-241): O with
  M^1/2 xi1, the kinetic energy 0.5 p . M^-1 p, B, A with M^-1 p; float64.
  Returns (x', p', ke_start [C])."""
  x, p, g1, xi1 = (np.asarray(a, np.float64) for a in (x, p, g1, xi1))
  mi, ms = np.asarray(minv, np.float64), np.asarray(msqrt, np.float64)
  h, T, f = float(h), float(T), float(friction)
  perm = math.exp(-f * h)
  p = math.sqrt(perm) * p + math.sqrt((1 - perm) * T) * (xi1 @ ms.T)
  ke = 0.5 * np.sum(p * (p @ mi.T), -1)
  p = p - 0.5 * h * g1
  return x + h * (p @ mi.T), p, ke


def dense_obabo_second(p, g2, xi2, h, T, friction, minv, msqrt):
  """obabo_second with dense matrices (integrator.py:243-273): B, the
  kinetic energy, O with M^1/2 xi2; float64.  Returns (p', ke_end [C])."""
  p, g2, xi2 = (np.asarray(a, np.float64) for a in (p, g2, xi2))
  mi, ms = np.asarray(minv, np.float64), np.asarray(msqrt, np.float64)
  h, T, f = float(h), float(T), float(friction)
  p = p - 0.5 * h * g2
  ke = 0.5 * np.sum(p * (p @ mi.T), -1)
  perm = math.exp(-f * h)
  return math.sqrt(perm) * p + math.sqrt((1 - perm) * T) * (xi2 @ ms.T), ke


def mh_log_alpha(kind, U_old, U_new, energy=0.0, ke_start=0.0, ke_end=0.0,
                 T=1.0):
  """The capped log acceptance of solver.amagold (kind 'amagold',
  solver.py:381-383: U_old - U_new + E, NaN kept) or solver.sggmc (kind
  'sggmc', solver.py:518-524: -(U_new - U_old + KE_end - KE_start) / T, NaN
  capped to 0), FP64."""
  if kind == "amagold":
    la = U_old - U_new + energy
    return 0.0 if la > 0.0 else la
  la = -1.0 / T * (U_new - U_old + ke_end - ke_start)
  return la if la <= 0.0 else 0.0


def mh_uniform(seed: int, chain: int, step: int) -> float:
  """The MH uniform: Philox(counter=(chain, step, 0, 9), key=seed), 53 bits
  as in swap_uniform."""
  r = philox4x32_10(np.array([[chain & 0xFFFFFFFF, step & 0xFFFFFFFF, 0, 9]],
                             np.uint64),
                    (seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF))[0]
  bits = ((int(r[0]) >> 5) << 26) | (int(r[1]) >> 6)
  return (bits + 0.5) / 9007199254740992.0


def resgld_swap(U_n, U_h, var_n, T_n, T_h, ssq, k, u, F=1.0):
  """solver.parallel_tempering.update exchange step (solver.py:273-291), FP64.
  Returns (swapped, ssq', k', log_s); swapped is True when NOT log u < log s
  (lax.cond keeps the pair in its true branch)."""
  k = k + 1
  sa = 1.0 / k
  ssq = (1 - sa) * ssq + sa * var_n
  dbeta = 1.0 / T_n - 1.0 / T_h
  log_s = dbeta * (U_n - U_h - dbeta * ssq / F)
  swapped = not (math.log(u) < log_s)
  return swapped, ssq, k, log_s


def swap_uniform(seed: int, pair: int, step: int) -> float:
  """The exchange uniform: Philox(counter=(pair, step, 0, 5), key=seed), 53
  bits ((r0 >> 5) << 26 | r1 >> 6) + 0.5 over 2^53."""
  r = philox4x32_10(np.array([[pair, step & 0xFFFFFFFF, 0, 5]], np.uint64),
                    (seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF))[0]
  bits = ((int(r[0]) >> 5) << 26) | (int(r[1]) >> 6)
  return (bits + 0.5) / 9007199254740992.0


def resgld_sa_update(var, ssq, k):
  """Every step: k += 1, ssq[r] = (1 - 1/k) ssq[r] + (1/k) var[r] for the
  adjacent pairs (r, r+1) -- solver.py:273-276 applied per pair, fed by the
  colder replica's variance as the reference feeds the normal chain's."""
  k = k + 1
  sa = 1.0 / k
  return (1 - sa) * np.asarray(ssq, np.float64) + sa * np.asarray(var, np.float64)[:-1], k


def resgld_exchange_adjacent(U, var, ssq, T, F, round_, u):
  """One exchange round over a temperature ladder T [R] (coldest first):
  pairs r with r % 2 == round % 2 evaluate the rule of solver.py:278-291
  (log_s = dbeta (U_r - U_{r+1} - dbeta ssq_r / F); exchange unless
  log u_r < log_s).  Returns (flags [R-1], U', var', log_s)."""
  U = np.array(U, np.float64)
  var = np.array(var, np.float64)
  R = U.size
  flags = np.zeros(R - 1, np.int32)
  log_s = np.zeros(R - 1)
  for r in range(round_ % 2, R - 1, 2):
    dbeta = 1.0 / T[r] - 1.0 / T[r + 1]
    log_s[r] = dbeta * (U[r] - U[r + 1] - dbeta * ssq[r] / F)
    flags[r] = 0 if math.log(u[r]) < log_s[r] else 1
  for r in np.nonzero(flags)[0]:
    U[[r, r + 1]] = U[[r + 1, r]]
    var[[r, r + 1]] = var[[r + 1, r]]
  return flags, U, var, log_s


class ShuffledBatches:
  """Minibatches of a shuffled random pipeline, one call at a time, as
  NumpyDataLoader._shuffle_indices hands them out
  (jax_sgmc/data/numpy_loader.py:391-431): a ring of (floor(N/mb) + 2) mb
  entries; when fewer than mb are unread, a permutation
  rng.choice(arange(N), N, replace=False) is written after the unread ones;
  each call reads the next mb entries."""

  def __init__(self, rng: np.random.Generator, n_obs: int, mb: int):
    self.rng, self.N, self.mb = rng, n_obs, mb
    self.R = (n_obs // mb + 2) * mb
    self.ring = np.zeros(self.R, dtype=np.int64)
    self.read = 0       # next ring position to read (mod R)
    self.unread = 0

  def next(self) -> np.ndarray:
    if self.unread < self.mb:
      perm = self.rng.choice(np.arange(self.N), size=self.N, replace=False)
      write = (self.read + self.unread + np.arange(self.N)) % self.R
      self.ring[write] = perm
      self.unread += self.N
    out = self.ring[(self.read + np.arange(self.mb)) % self.R].copy()
    self.read = (self.read + self.mb) % self.R
    self.unread -= self.mb
    return out


# ---------------------------------------------------------------------------
# Sample statistics
# ---------------------------------------------------------------------------


class MassAdaption(NamedTuple):
  iteration: int
  mean: np.ndarray
  ssq: np.ndarray
  inv: np.ndarray
  sqrt: np.ndarray


def mass_adapt_init(sample, init_cov=None) -> MassAdaption:
  """mass_matrix(diagonal=True) init (jax_sgmc/adaption.py:321-340), fp32."""
  x = np.asarray(sample, np.float32)
  cov = np.ones_like(x) if init_cov is None else np.asarray(init_cov, np.float32)
  return MassAdaption(0, np.zeros_like(x), np.zeros_like(x), cov.copy(),
                      (np.float32(1) / np.sqrt(cov)).astype(np.float32))


def mass_adapt_update(state: MassAdaption, sample, burn_in) -> MassAdaption:
  """One update (jax_sgmc/adaption.py:342-362) with the matrix computed at
  iteration == burn_in (:309-319), fp32 in the reference's operation order:
  the int32 iteration divides as float32 ((i - 1) / i, 1 / i), products and
  sums unfused."""
  x = np.asarray(sample, np.float32)
  it = state.iteration + 1
  fi = np.float32(it)
  a = np.float32(it - 1) / fi
  b = np.float32(1) / fi
  mean = (a * state.mean + b * x).astype(np.float32)
  ssq = (state.ssq + (x - state.mean) * (x - mean)).astype(np.float32)
  inv, sq = state.inv, state.sqrt
  if it == burn_in:
    inv = (ssq / fi).astype(np.float32)
    sq = np.sqrt(fi / ssq).astype(np.float32)
  return MassAdaption(it, mean, ssq, inv, sq)


def dense_mass_adapt_init(sample, init_cov=None) -> MassAdaption:
  """mass_matrix(diagonal=False) init (jax_sgmc/adaption.py:321-340): ssq
  [P, P] zeros, inv = diag(init_cov), sqrt = diag(1 / sqrt(init_cov))."""
  x = np.asarray(sample, np.float32).reshape(-1)
  cov = np.ones_like(x) if init_cov is None else np.asarray(init_cov, np.float32)
  return MassAdaption(0, np.zeros_like(x), np.zeros((x.size, x.size), np.float32),
                      np.diag(cov), np.diag(np.float32(1) / np.sqrt(cov)))


def dense_mass_adapt_update(state: MassAdaption, sample, burn_in) -> MassAdaption:
  """One dense update (jax_sgmc/adaption.py:342-362): the mean as in
  :func:`mass_adapt_update`, ssq += outer(x - mean, x - mean') (fp32), and
  at iteration == burn_in (:309-317) inv = ssq / i and
  sqrt = V^T diag(sqrt(w)) V with (w, V) = :func:`sym_eig` (inv) (float64,
  the eigenvectors as V's columns; negative rounding of w counts as 0)."""
  x = np.asarray(sample, np.float32).reshape(-1)
  it = state.iteration + 1
  fi = np.float32(it)
  a = np.float32(it - 1) / fi
  b = np.float32(1) / fi
  mean = (a * state.mean + b * x).astype(np.float32)
  ssq = (state.ssq + np.outer(x - state.mean, x - mean)).astype(np.float32)
  inv, sq = state.inv, state.sqrt
  if it == burn_in:
    inv = (ssq / fi).astype(np.float32)
    w, V = sym_eig(inv)
    sq = V.T @ np.diag(np.sqrt(np.maximum(w, 0.0))) @ V
  return MassAdaption(it, mean, ssq, inv, sq)


def sample_moments(samples):
  """FP64 mean and population variance over the first axis (the posterior
  moments of kept samples)."""
  a = np.asarray(samples, np.float64)
  return a.mean(axis=0), a.var(axis=0)


# ---------------------------------------------------------------------------
# Scheduler
# ---------------------------------------------------------------------------

def polynomial_first_last(first, last, gamma, iterations):
  """polynomial_step_size_first_last (scheduler.py:494-542), float64."""
  ginv = 1.0 / gamma
  apow = (last ** -ginv - first ** -ginv) / (iterations - 1)
  a = apow ** -gamma
  b = (first / a) ** -ginv
  return a * (b + np.arange(iterations)) ** -gamma


# ---------------------------------------------------------------------------
# Trajectories
# ---------------------------------------------------------------------------

def sgld_glm_trajectory(X, y, w0, idx, xi, h, T, family, sigma=1.0,
                        prior_scale=0.0, temperature=1.0, rms_prop=True,
                        alpha=0.9, lmbd=1e-5, n_obs=None):
  """K SGLD steps of C chains with given minibatch indices idx [K, C, n] and
  injected normals xi [K, C, d]; gradients in float64, updates in float32.
  ``n_obs`` (default: the rows of X) is the N of the N/n scaling, so that X
  may hold only the rows the indices reach.
  Returns (W [K+1, C, d], U [K, C], var [K, C])."""
  W = np.atleast_2d(np.asarray(w0, f32)).copy()
  V = np.ones_like(W)
  K = idx.shape[0]
  Ws, Us, Vs = [W.copy()], [], []
  n_obs = X.shape[0] if n_obs is None else n_obs
  for k in range(K):
    pot = glm_potential(W, X, y, idx[k], n_obs, family, sigma, prior_scale,
                        temperature)
    W, V = sgld_step(W, pot.grad.astype(f32), V, xi[k], h[k], T[k], alpha,
                     lmbd, rms_prop)
    Ws.append(W.copy())
    Us.append(pot.U)
    Vs.append(pot.var)
  return np.stack(Ws), np.stack(Us), np.stack(Vs)


def sgld_glm_cpu_steps(X, y, W, V, rngs, steps, h, T, family, sigma=1.0,
                       prior_scale=0.0, temperature=1.0, alpha=0.9,
                       lmbd=1e-5, noise_rng=None, threads=1):
  """The reference's SGLD(+RMSprop) hot loop on the CPU in float32 for C
  chains: per chain and step the loader's index draw (numpy_loader.py:
  382-389), the host gather (numpy_loader.py:330-340), the per-observation
  likelihoods, the potential U and var(lk) that update_fn stores every step
  (integrator.py:875-880), the gradient, RMSprop and the update.  Used as
  the timed CPU baseline.  Chains are split over ``threads`` worker threads.
  Returns (W, V, U [C], var [C]) after the last step."""
  import concurrent.futures as cf
  C, d = W.shape
  n_obs = X.shape[0]
  noise_rng = noise_rng or np.random.default_rng(0)
  Xf = np.asarray(X, f32)
  yf = np.asarray(y, f32)
  inv_p2 = f32(0.0) if not prior_scale else f32(1.0 / prior_scale ** 2)
  lp_const = 0.0 if not prior_scale else \
      d * (math.log(prior_scale) + 0.5 * math.log(2 * math.pi))
  U = np.zeros(C)
  var = np.zeros(C)

  def chain_block(cs, k, xi):
    for c in cs:
      idx = rngs[c].choice(np.arange(0, n_obs), size=steps_n, replace=True)
      xb, yb = Xf[idx], yf[idx]
      z = xb @ W[c]
      if family == LOGISTIC:
        lk = yb * z - (np.maximum(z, f32(0.0)) + np.log1p(np.exp(-np.abs(z))))
        dz = yb - f32(1.0) / (f32(1.0) + np.exp(-z))
      else:
        r = yb - z
        lk = (f32(-0.5 / sigma ** 2) * (r * r)
              - f32(math.log(sigma) + 0.5 * math.log(2 * math.pi)))
        dz = r / f32(sigma ** 2)
      lp = -0.5 * float(inv_p2) * float(W[c] @ W[c]) - lp_const
      U[c] = (-(n_obs / steps_n) * float(lk.sum(dtype=np.float64)) - lp) / temperature
      var[c] = float(np.var(lk, dtype=np.float64))
      g = (-(f32(n_obs / steps_n)) * (dz @ xb) + W[c] * inv_p2) / f32(temperature)
      W[c], V[c] = sgld_step(W[c], g, V[c], xi[c], h[k], T[k], alpha, lmbd, True)

  steps_n = steps[1]
  K = steps[0]
  blocks = np.array_split(np.arange(C), max(1, threads))
  with cf.ThreadPoolExecutor(max_workers=max(1, threads)) as ex:
    for k in range(K):
      xi = noise_rng.standard_normal((C, d), dtype=f32)
      list(ex.map(lambda cs: chain_block(cs, k, xi), blocks))
  return W, V, U, var


def alias_chains_1d(kind, curvature, h, C, rng, x0=0.0, **kw):
  """C independent chains of one of the reference's alias samplers on the
  1-D potential U(w) = curvature w^2 / 2 with exact gradients (a batch that
  every draw makes the same), vectorised over chains with numpy normals.
  Returns the position after each iteration, [len(h), C] (what
  solver.mcmc keeps, solver.py:95-121, after update).

  kind:
    'sgld_rms'  alias.sgld(rms_prop=True): langevin_diffusion with rms_prop
                (integrator.py:860-922, adaption.py:254-291), one step per
                iteration;
    're_sgld'   alias.re_sgld: a normal (T = 1) and a hot (T = kw['T_hot'])
                plain SGLD chain, then solver.parallel_tempering's exchange
                (solver.py:264-293) on the potentials at the pre-update
                positions with var(lk) = 0 (one observation per batch), F = 1;
                the normal chain is kept;
    'obabo'     alias.obabo: obabo._leapfrog_steps kw['steps'] times per
                iteration (integrator.py:192-273), momentum from zero and
                kept across iterations, friction kw['friction'];
    'sghmc'     alias.sghmc: momentum resampled, then kw['steps'] friction
                leapfrog steps (integrator.py:603-666, 735-738), friction
                kw['friction'].
  """
  A = f32(curvature)
  x = np.full(C, x0, f32)
  out = np.empty((len(h), C), f32)
  if kind == "sgld_rms":
    v = np.ones(C, f32)
    for k, hk in enumerate(h):
      x, v = sgld_step(x, A * x, v, rng.normal(size=C), hk, 1.0)
      out[k] = x
  elif kind == "re_sgld":
    xh = x.copy()
    T_h = float(kw["T_hot"])
    ssq, it = np.zeros(C), 0
    for k, hk in enumerate(h):
      Un = 0.5 * float(A) * x.astype(np.float64) ** 2
      Uh = 0.5 * float(A) * xh.astype(np.float64) ** 2
      x, _ = sgld_step(x, A * x, None, rng.normal(size=C), hk, 1.0, rms_prop=False)
      xh, _ = sgld_step(xh, A * xh, None, rng.normal(size=C), hk, T_h,
                        rms_prop=False)
      it += 1
      ssq = (1 - 1.0 / it) * ssq          # + (1/k) var(lk), var(lk) = 0
      dbeta = 1.0 - 1.0 / T_h
      log_s = dbeta * (Un - Uh - dbeta * ssq)
      swap = ~(np.log(rng.random(C)) < log_s)
      x, xh = np.where(swap, xh, x), np.where(swap, x, xh)
      out[k] = x
  elif kind == "obabo":
    p = np.zeros((C, 1), f32)
    xc = x[:, None]
    for k, hk in enumerate(h):
      for _ in range(int(kw["steps"])):
        xc, p, _ = obabo_first(xc, p, A * xc, rng.normal(size=(C, 1)), hk, 1.0,
                               kw["friction"])
        p, _ = obabo_second(p, A * xc, rng.normal(size=(C, 1)), hk, 1.0,
                            kw["friction"])
      out[k] = xc[:, 0]
  elif kind == "sghmc":
    for k, hk in enumerate(h):
      p = sghmc_resample(rng.normal(size=C))
      for _ in range(int(kw["steps"])):
        x, p = sghmc_position(x, p, hk, kw["friction"])
        p = sghmc_momentum(p, A * x, rng.normal(size=C), hk, kw["friction"])
      out[k] = x
  else:
    raise ValueError(kind)
  return out
