"""ctypes binding of the libgbsgmc C ABI (``include/gbsgmc.h``).

Every call goes through the C ABI with raw device pointers taken from torch
tensors and the handle of torch's current CUDA stream.  There is no fallback:
if the library is missing or no GPU is present, the call raises.
"""

from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from . import _build

_lock = threading.Lock()
_lib = None

OK = 0
ERR_ARG, ERR_SHAPE, ERR_INDEX, ERR_NONFINITE, ERR_TIMEOUT, ERR_CUDA, \
  ERR_UNSUPPORTED = range(1, 8)
STATUS_NAMES = {0: "ok", 1: "bad argument", 2: "unsupported shape",
                3: "observation index out of range",
                4: "non-finite potential or gradient",
                5: "device wait timed out", 6: "CUDA error",
                7: "unsupported"}

GLM_LINEAR_GAUSSIAN = 0
GLM_LOGISTIC = 1
GLM_LINEAR = 2
STATIC_SCRATCH_BYTES = 8 << 20

TAG_SGLD, TAG_OBABO_1, TAG_OBABO_2, TAG_SGHMC_RESAMPLE, TAG_SGHMC_STEP, \
  TAG_SWAP, TAG_INDEX, TAG_AMAGOLD, TAG_AMAGOLD_INIT, TAG_MH = range(10)
MH_AMAGOLD, MH_SGGMC = 0, 1


class GbsgmcError(RuntimeError):
  """A non-zero status from the C ABI or from a device status word."""

  def __init__(self, code: int, message: str):
    super().__init__(f"[{STATUS_NAMES.get(code, code)}] {message}")
    self.code = code


class Pcg64(C.Structure):
  _fields_ = [("state_hi", C.c_uint64), ("state_lo", C.c_uint64),
              ("inc_hi", C.c_uint64), ("inc_lo", C.c_uint64),
              ("has_uint32", C.c_uint32), ("uinteger", C.c_uint32)]


class Glm(C.Structure):
  _fields_ = [("family", C.c_int), ("d", C.c_int), ("n_obs", C.c_int64),
              ("ld", C.c_int64), ("X", C.c_void_p), ("y", C.c_void_p),
              ("sigma", C.c_float), ("prior_scale", C.c_float),
              ("temperature", C.c_float), ("y_inline", C.c_int),
              ("n_rows", C.c_int64)]


class Mlp(C.Structure):
  _fields_ = [("d_in", C.c_int), ("h1", C.c_int), ("h2", C.c_int),
              ("y_inline", C.c_int), ("n_obs", C.c_int64),
              ("n_rows", C.c_int64), ("ld", C.c_int64), ("X", C.c_void_p),
              ("y", C.c_void_p), ("sigma", C.c_float),
              ("prior_scale", C.c_float), ("temperature", C.c_float),
              ("_reserved", C.c_int)]


class Cnn(C.Structure):
  _fields_ = [("n_obs", C.c_int64), ("n_rows", C.c_int64), ("ld", C.c_int64),
              ("X", C.c_void_p), ("labels", C.c_void_p),
              ("label_ld", C.c_int64), ("prior_scale", C.c_float),
              ("temperature", C.c_float)]


class Integrator(C.Structure):
  _fields_ = [("kind", C.c_int), ("leapfrog_steps", C.c_int),
              ("friction", C.c_float), ("alpha", C.c_float),
              ("lmbd", C.c_float), ("_pad", C.c_int),
              ("mass_dev", C.c_void_p)]


INTEGRATOR_SGLD, INTEGRATOR_OBABO, INTEGRATOR_SGHMC = 0, 1, 2


class Tempering(C.Structure):
  _fields_ = [("every", C.c_int), ("_pad", C.c_int), ("F", C.c_double),
              ("seed", C.c_uint64), ("ssq_dev", C.c_void_p),
              ("k_dev", C.c_void_p), ("counts_dev", C.c_void_p),
              ("flags_dev", C.c_void_p)]


class Sched(C.Structure):
  _fields_ = [("step_size_dev", C.c_void_p), ("temperature_dev", C.c_void_p),
              ("base_dev", C.c_void_p), ("keep_slot_dev", C.c_void_p),
              ("offset", C.c_int64), ("step_size", C.c_float),
              ("temperature", C.c_float),
              ("chain_temperature_dev", C.c_void_p)]


class Noise(C.Structure):
  _fields_ = [("noise_dev", C.c_void_p), ("noise_stride", C.c_int64),
              ("seed", C.c_uint64), ("chain_base", C.c_int),
              ("_pad", C.c_int)]


class IndexSrc(C.Structure):
  _fields_ = [("pcg_dev", C.c_void_p), ("index_seed", C.c_uint64),
              ("chain_base", C.c_int), ("external", C.c_int)]


_vp, _i, _i64, _u64, _f, _d, _sz = (C.c_void_p, C.c_int, C.c_int64,
                                    C.c_uint64, C.c_float, C.c_double,
                                    C.c_size_t)
_P = C.POINTER

# name -> (restype, argtypes)
SIGNATURES = {
    "gbsgmc_last_error": (C.c_char_p, []),
    "gbsgmc_version": (_i, []),
    "gbsgmc_index_draw_pcg64": (_i, [_vp, _i, _i64, _i64, _i, _vp, _i64, _i64,
                                     _vp, _vp]),
    "gbsgmc_index_draw_philox": (_i, [_u64, _i, _i, _i64, _i, _i, _i64, _vp,
                                      _i64, _i64, _vp]),
    "gbsgmc_philox_normal": (_i, [_u64, _i, _i, _i64, C.c_uint32, _i64, _vp,
                                  _i64, _vp]),
    "gbsgmc_glm_workspace_bytes": (_sz, [_i, _i, _i]),
    "gbsgmc_glm_value_and_grad": (_i, [_P(Glm), _i, _i, _vp, _i64, _vp, _vp,
                                       _vp, _vp, _vp, _vp, _vp, _sz, _vp,
                                       _vp]),
    "gbsgmc_mlp_param_count": (_i64, [_P(Mlp)]),
    "gbsgmc_mlp_workspace_bytes": (_sz, [_P(Mlp), _i, _i]),
    "gbsgmc_mlp_value_and_grad": (_i, [_P(Mlp), _i, _i, _vp, _i64, _vp, _vp,
                                       _vp, _vp, _vp, _vp, _vp, _sz, _vp,
                                       _vp]),
    "gbsgmc_mlp_value_and_grad_ragged": (_i, [_P(Mlp), _i, _i, _vp, _vp, _i64,
                                              _vp, _vp, _vp, _vp, _vp, _vp,
                                              _vp, _sz, _vp, _vp]),
    "gbsgmc_pcg64_seed": (_i, [_vp, _vp, _i, _vp]),
    "gbsgmc_mlp_fisher_workspace_bytes": (_sz, [_P(Mlp), _i, _i]),
    "gbsgmc_mlp_fisher_noise": (_i, [_P(Mlp), _i, _i, _vp, _i64, _vp, _vp, _vp,
                                     _f, _f, _vp, _vp, _vp, _sz, _vp, _vp]),
    "gbsgmc_cnn_param_count": (_i64, []),
    "gbsgmc_cnn_workspace_bytes": (_sz, [_i, _i]),
    "gbsgmc_cnn_value_and_grad": (_i, [_P(Cnn), _i, _i, _vp, _i64, _vp, _vp,
                                       _vp, _vp, _vp, _vp, _vp, _sz, _vp,
                                       _vp]),
    "gbsgmc_sgld_update": (_i, [_i, _i64, _vp, _vp, _vp, _f, _f, _P(Sched),
                                _P(Noise), _vp, _vp]),
    "gbsgmc_obabo_first": (_i, [_i, _i64, _vp, _vp, _vp, _vp, _f, _vp,
                                _P(Sched), _P(Noise), _vp]),
    "gbsgmc_obabo_second": (_i, [_i, _i64, _vp, _vp, _vp, _f, _vp, _P(Sched),
                                 _P(Noise), _vp]),
    "gbsgmc_sghmc_resample": (_i, [_i, _i64, _vp, _vp, _P(Sched), _P(Noise),
                                   _vp]),
    "gbsgmc_sghmc_position": (_i, [_i, _i64, _vp, _vp, _vp, _vp, _f,
                                   _P(Sched), _vp]),
    "gbsgmc_sghmc_momentum": (_i, [_i, _i64, _vp, _vp, _vp, _f, _P(Sched),
                                   _P(Noise), _vp]),
    "gbsgmc_leapfrog_position": (_i, [_i, _i64, _vp, _vp, _vp, _f, _P(Sched),
                                      _vp]),
    "gbsgmc_amagold_momentum": (_i, [_i, _i64, _vp, _vp, _vp, _f, _vp,
                                     _P(Sched), _P(Noise), _vp]),
    "gbsgmc_mh_accept": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp, _P(Sched), _vp,
                              _u64, _i, _vp, _vp, _vp, _vp]),
    "gbsgmc_mh_select": (_i, [_i, _i64, _vp, _vp, _vp, _vp, _vp, _f, _vp]),
    "gbsgmc_moments_accumulate": (_i, [_i, _i64, _i, _vp, _i64, _i64, _i64, _vp,
                                       _vp, _vp, _vp]),
    "gbsgmc_moments_finalize": (_i, [_i, _i64, _i64, _vp, _vp, _vp, _vp, _vp,
                                     _vp]),
    "gbsgmc_mass_adapt": (_i, [_i64, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gbsgmc_glm_fisher_noise": (_i, [_P(Glm), _i, _i, _vp, _i64, _vp, _vp, _vp,
                                     _f, _f, _vp, _vp, _vp, _vp]),
    "gbsgmc_glm_fisher_noise_dense": (_i, [_P(Glm), _i, _i, _vp, _i64, _vp, _vp,
                                           _vp, _f, _f, _vp, _vp, _vp, _vp]),
    "gbsgmc_sym_eig": (_i, [_i, _i, _vp, _vp, _vp, _vp]),
    "gbsgmc_leapfrog_position_dense": (_i, [_i, _i64, _vp, _vp, _vp, _f,
                                            _P(Sched), _vp]),
    "gbsgmc_amagold_momentum_dense": (_i, [_i, _i64, _vp, _vp, _vp, _vp, _f,
                                           _vp, _P(Sched), _P(Noise), _vp]),
    "gbsgmc_obabo_first_dense": (_i, [_i, _i64, _vp, _vp, _vp, _vp, _vp, _f,
                                      _vp, _P(Sched), _P(Noise), _vp]),
    "gbsgmc_obabo_second_dense": (_i, [_i, _i64, _vp, _vp, _vp, _vp, _f, _vp,
                                       _P(Sched), _P(Noise), _vp]),
    "gbsgmc_dense_matvec": (_i, [_i, _i64, _vp, _vp, _vp, _vp]),
    "gbsgmc_mass_adapt_dense": (_i, [_i64, _i, _i, _vp, _vp, _vp, _vp, _vp,
                                     _vp, _vp, _vp]),
    "gbsgmc_sghmc_momentum_noise_model": (_i, [_i, _i64, _vp, _vp, _vp, _P(Sched),
                                               _P(Noise), _vp]),
    "gbsgmc_resgld_swap_f64": (_i, [_i, _vp, _vp, _vp, _vp, _vp, _d, _vp, _vp,
                                    _vp, _u64, _i64, _vp, _vp, _vp]),
    "gbsgmc_swap_rows": (_i, [_i, _i64, _vp, _vp, _vp, _vp]),
    "gbsgmc_sgld_glm_step": (_i, [_P(Glm), _i, _i, _vp, _i64, _vp, _vp, _f, _f,
                                  _P(Sched), _P(Noise), _vp, _vp, _vp, _vp,
                                  _vp, _sz, _vp, _vp]),
    "gbsgmc_sgld_glm_steps": (_i, [_P(Glm), _i, _i, _vp, _i64, _i64, _i, _vp, _vp,
                                   _f, _f, _P(Sched), _P(Noise), _vp, _vp, _vp,
                                   _vp, _vp, _sz, _vp, _vp]),
    "gbsgmc_sgld_glm_step_noalloc": (_i, [_P(Glm), _i, _i, _vp, _i64, _vp, _vp,
                                          _f, _f, _P(Sched), _P(Noise), _vp,
                                          _vp, _vp, _vp, _vp, _vp]),
    "gbsgmc_sgld_glm_plan_create": (_i, [_P(_vp), _P(Glm), _i, _i, _vp, _vp,
                                         _f, _f, _P(Sched), _P(Noise),
                                         _P(IndexSrc), _vp, _vp, _vp, _vp, _i,
                                         _vp]),
    "gbsgmc_mlp_plan_create": (_i, [_P(_vp), _P(Mlp), _i, _i, _P(Integrator),
                                    _vp, _vp, _P(Sched), _P(Noise),
                                    _P(IndexSrc), _vp, _vp, _vp, _i, _vp]),
    "gbsgmc_cnn_plan_create": (_i, [_P(_vp), _P(Cnn), _i, _i, _P(Integrator),
                                    _vp, _vp, _P(Sched), _P(Noise),
                                    _P(IndexSrc), _vp, _vp, _vp, _i, _vp]),
    "gbsgmc_glm_plan_create": (_i, [_P(_vp), _P(Glm), _i, _i, _P(Integrator),
                                    _vp, _vp, _P(Sched), _P(Noise),
                                    _P(IndexSrc), _vp, _vp, _vp, _i, _vp]),
    "gbsgmc_resgld_sa_update": (_i, [_i, _vp, _vp, _vp, _vp]),
    "gbsgmc_resgld_exchange_adjacent": (_i, [_i, _i64, _vp, _vp, _vp, _vp,
                                             _P(Sched), _i, _vp, _d, _u64,
                                             _vp, _vp, _vp, _vp, _vp]),
    "gbsgmc_mlp_resgld_plan_create": (_i, [_P(_vp), _P(Mlp), _i, _i, _vp, _vp,
                                           _vp, _f, _f, _P(Sched), _P(Noise),
                                           _P(IndexSrc), _P(Tempering), _vp,
                                           _vp, _i, _vp]),
    "gbsgmc_mlp_resgld_plan_create_keep": (_i, [_P(_vp), _P(Mlp), _i, _i, _vp, _vp,
                                                _vp, _f, _f, _P(Sched), _P(Noise),
                                                _P(IndexSrc), _P(Tempering), _vp,
                                                _vp, _vp, _vp, _i, _vp]),
    "gbsgmc_mlp_resgld_pairs_plan_create": (_i, [_P(_vp), _P(Mlp), _i, _i, _vp, _vp,
                                                 _f, _f, _P(Sched), _P(Noise),
                                                 _P(IndexSrc), _P(Tempering), _vp, _vp,
                                                 _vp, _vp, _vp, _vp, _i, _vp]),
    "gbsgmc_glm_resgld_plan_create": (_i, [_P(_vp), _P(Glm), _i, _i, _vp, _vp,
                                           _f, _f, _P(Sched), _P(Noise),
                                           _P(IndexSrc), _P(Tempering), _vp, _vp,
                                           _vp, _vp, _vp, _vp, _i, _vp]),
    "gbsgmc_plan_run": (_i, [_vp, _i64, _i64, _vp]),
    "gbsgmc_plan_launches": (_i64, [_vp, _i64]),
    "gbsgmc_plan_set_indices": (_i, [_vp, _vp, _i, _vp]),
    "gbsgmc_plan_launch_shape": (_i, [_vp, _P(_i), _P(_i), _P(_i), _P(_i), _P(_i),
                                      _P(_i)]),
    "gbsgmc_plan_destroy": (_i, [_vp]),
    "gbsgmc_gemm_bf16": (_i, [_i, _i, _vp, _i64, _i64, _vp, _i64, _i64, _vp,
                              _i64, _i64, _i, _i, _i, _i, _vp, _vp]),
    "gbsgmc_gemm_bf16_c16": (_i, [_i, _i, _vp, _i64, _i64, _vp, _i64, _i64, _vp,
                              _i64, _i64, _i, _i, _i, _i, _vp, _vp]),
    "gbsgmc_gemm_bf16_wait_limit": (_i, [_i, _i, _vp, _i64, _i64, _vp, _i64, _i64,
                                         _vp, _i64, _i64, _i, _i, _i, _i,
                                         C.c_uint64, _vp, _vp]),
    "gbsgmc_gemm_bf16_nt": (_i, [_vp, _i64, _i64, _vp, _i64, _i64, _vp, _i64,
                                 _i64, _i, _i, _i, _i, _vp, _vp]),
    "gbsgmc_plain_buffer_bytes": (_sz, [_i, _i]),
    "gbsgmc_plain_sgld_glm_step": (_i, [_P(Glm), _i, _vp, _vp, _vp, _f, _f,
                                        _P(Sched), _P(Noise), _vp, _vp, _vp,
                                        _vp]),
}


def lib_path() -> Path:
  return _build.LIB_PATH


def load(build_if_missing: bool = True):
  """Loads (and if needed builds) libgbsgmc.so and declares its signatures."""
  global _lib
  with _lock:
    if _lib is not None:
      return _lib
    path = _build.LIB_PATH
    if not path.exists():
      if not build_if_missing:
        raise RuntimeError(f"libgbsgmc is not built ({path} missing)")
      _build.build()
    lib = C.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
      fn = getattr(lib, name)
      fn.restype = res
      fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int, what: str = "") -> None:
  if rc != OK:
    msg = load().gbsgmc_last_error().decode(errors="replace")
    raise GbsgmcError(rc, f"{what}: {msg}" if what else msg)


def call(name: str, *args) -> None:
  """Calls an int-returning entry point and raises on a non-zero status."""
  check(getattr(load(), name)(*args), name)


def ptr(t) -> int | None:
  """Device pointer of a torch tensor (None for None)."""
  if t is None:
    return None
  return t.data_ptr()


def stream_handle(stream=None) -> int | None:
  import torch
  s = stream if stream is not None else torch.cuda.current_stream()
  return s.cuda_stream or None


def sched(step_size=0.0, temperature=1.0, step_size_dev=None,
          temperature_dev=None, base_dev=None, keep_slot_dev=None,
          offset=0, chain_temperature_dev=None) -> Sched:
  return Sched(ptr(step_size_dev), ptr(temperature_dev), ptr(base_dev),
               ptr(keep_slot_dev), int(offset), float(step_size),
               float(temperature), ptr(chain_temperature_dev))


def noise(seed=0, chain_base=0, noise_dev=None, noise_stride=0) -> Noise:
  return Noise(ptr(noise_dev), int(noise_stride), int(seed) & (2**64 - 1),
               int(chain_base), 0)
