"""The tcgen05 BF16 GEMM (C = A B^T, fp32 accumulation) against torch.

Inputs are BF16, so products are exact in fp32; the tolerance covers fp32
summation order over K: |C - C_ref| <= 1e-3 * (|A| |B|^T) elementwise bound.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("batch,M,N,K", [(1, 128, 128, 64), (1, 128, 256, 64),
                                         (2, 256, 256, 128), (3, 384, 512, 1024),
                                         (1, 2048, 1024, 1024), (2, 128, 384, 320)])
def test_gemm_matches_torch(lib, batch, M, N, K):
  import torch
  from gbsgmc import _lib
  g = torch.Generator(device="cuda").manual_seed(M + N + K)
  A = torch.randn((batch, M, K), generator=g, device="cuda").to(torch.bfloat16)
  B = torch.randn((batch, N, K), generator=g, device="cuda").to(torch.bfloat16)
  C = torch.full((batch, M, N), float("nan"), device="cuda")
  status = torch.zeros(1, dtype=torch.int32, device="cuda")
  _lib.call("gbsgmc_gemm_bf16_nt", A.data_ptr(), K, M * K, B.data_ptr(), K, N * K,
            C.data_ptr(), N, M * N, batch, M, N, K, status.data_ptr(),
            _lib.stream_handle())
  torch.cuda.synchronize()
  assert int(status.item()) == 0
  ref = torch.bmm(A.float(), B.float().transpose(1, 2))
  bound = torch.bmm(A.float().abs(), B.float().abs().transpose(1, 2))
  err = (C - ref).abs()
  assert torch.isfinite(C).all()
  assert bool((err <= 1e-3 * bound + 1e-4).all()), float((err / (bound + 1e-6)).max())


@pytest.mark.parametrize("a_mn,b_mn", [(0, 1), (1, 0), (1, 1), (0, 0)])
@pytest.mark.parametrize("batch,M,N,K", [(1, 128, 128, 64), (2, 256, 256, 128),
                                         (3, 384, 512, 1024), (2, 128, 384, 320),
                                         (1, 1024, 1024, 2048)])
def test_gemm_operand_layouts(lib, a_mn, b_mn, batch, M, N, K):
  """MN-major ("transposed") operands: A stored K x M, B stored K x N."""
  import torch
  from gbsgmc import _lib
  g = torch.Generator(device="cuda").manual_seed(7 * M + N + K + 2 * a_mn + b_mn)
  A = torch.randn((batch, M, K), generator=g, device="cuda").to(torch.bfloat16)
  B = torch.randn((batch, N, K), generator=g, device="cuda").to(torch.bfloat16)
  As = A.transpose(1, 2).contiguous() if a_mn else A
  Bs = B.transpose(1, 2).contiguous() if b_mn else B
  C = torch.full((batch, M, N), float("nan"), device="cuda")
  status = torch.zeros(1, dtype=torch.int32, device="cuda")
  _lib.call("gbsgmc_gemm_bf16", a_mn, b_mn, As.data_ptr(), M if a_mn else K,
            M * K, Bs.data_ptr(), N if b_mn else K, N * K, C.data_ptr(), N,
            M * N, batch, M, N, K, status.data_ptr(), _lib.stream_handle())
  torch.cuda.synchronize()
  assert int(status.item()) == 0
  ref = torch.bmm(A.float(), B.float().transpose(1, 2))
  bound = torch.bmm(A.float().abs(), B.float().abs().transpose(1, 2))
  err = (C - ref).abs()
  assert torch.isfinite(C).all()
  assert bool((err <= 1e-3 * bound + 1e-4).all()), float((err / (bound + 1e-6)).max())


def test_gemm_rejects_unsupported_shapes(lib):
  from gbsgmc import _lib
  rc = lib.gbsgmc_gemm_bf16_nt(16, 64, 0, 16, 64, 0, 16, 100, 0, 1, 100, 128, 64,
                               16, None)
  assert rc == _lib.ERR_SHAPE
  rc = lib.gbsgmc_gemm_bf16(1, 0, 16, 64, 0, 16, 64, 0, 16, 128, 0, 1, 128, 128,
                            64, None, None)
  assert rc == _lib.ERR_ARG


def test_gemm_progress_wait_bound_runs_out_cleanly(lib):
  """The bounded waits are the GEMM's failure detection.  With a 1 us bound
  on the waits for pipeline progress, the epilogue warps (whose first
  accumulator needs 32 K slices of MMAs, several microseconds) give up:
  each CTA records GBSGMC_ERR_TIMEOUT, stops issuing copies and MMAs, waits
  for those in flight, frees its TMEM and returns.  The device stays usable:
  the same GEMM with the default bound then completes and is correct, twice
  in a row."""
  import torch
  from gbsgmc import _lib
  batch, M, N, K = 2, 1024, 1024, 2048
  g = torch.Generator(device="cuda").manual_seed(99)
  A = torch.randn((batch, M, K), generator=g, device="cuda").to(torch.bfloat16)
  B = torch.randn((batch, N, K), generator=g, device="cuda").to(torch.bfloat16)
  ref = torch.bmm(A.float(), B.float().transpose(1, 2))
  bound = torch.bmm(A.float().abs(), B.float().abs().transpose(1, 2))
  for _ in range(2):
    C = torch.zeros((batch, M, N), device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.call("gbsgmc_gemm_bf16_wait_limit", 0, 0, A.data_ptr(), K, M * K,
              B.data_ptr(), K, N * K, C.data_ptr(), N, M * N, batch, M, N, K,
              1000, status.data_ptr(), _lib.stream_handle())
    torch.cuda.synchronize()
    assert int(status.item()) == _lib.ERR_TIMEOUT
    status.zero_()
    C.fill_(float("nan"))
    _lib.call("gbsgmc_gemm_bf16", 0, 0, A.data_ptr(), K, M * K, B.data_ptr(), K,
              N * K, C.data_ptr(), N, M * N, batch, M, N, K, status.data_ptr(),
              _lib.stream_handle())
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert bool(((C - ref).abs() <= 1e-3 * bound + 1e-4).all())


@pytest.mark.parametrize("a_mn,b_mn", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_pair_and_single_cta_gemms_agree(lib, monkeypatch, a_mn, b_mn):
  """The CTA-pair kernel (256 x 256 tiles on two SMs, tcgen05 cta_group::2,
  used where M % 256 == 0 and N % 256 == 0) and the single-CTA kernel
  (GBSGMC_GEMM_PAIR=0) both meet the fp32-summation bound against torch, in
  every operand layout, and agree with each other to that bound."""
  import torch
  from gbsgmc import _lib
  batch, M, N, K = 3, 512, 768, 576
  g = torch.Generator(device="cuda").manual_seed(31 + 2 * a_mn + b_mn)
  A = torch.randn((batch, M, K), generator=g, device="cuda").to(torch.bfloat16)
  B = torch.randn((batch, N, K), generator=g, device="cuda").to(torch.bfloat16)
  As = A.transpose(1, 2).contiguous() if a_mn else A
  Bs = B.transpose(1, 2).contiguous() if b_mn else B
  ref = torch.bmm(A.float(), B.float().transpose(1, 2))
  bound = torch.bmm(A.float().abs(), B.float().abs().transpose(1, 2))
  out = []
  for pair in ("1", "0"):
    monkeypatch.setenv("GBSGMC_GEMM_PAIR", pair)
    C = torch.full((batch, M, N), float("nan"), device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.call("gbsgmc_gemm_bf16", a_mn, b_mn, As.data_ptr(), M if a_mn else K,
              M * K, Bs.data_ptr(), N if b_mn else K, N * K, C.data_ptr(), N,
              M * N, batch, M, N, K, status.data_ptr(), _lib.stream_handle())
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert torch.isfinite(C).all()
    assert bool(((C - ref).abs() <= 1e-3 * bound + 1e-4).all())
    out.append(C)
  assert bool(((out[0] - out[1]).abs() <= 1e-3 * bound + 1e-4).all())


@pytest.mark.parametrize("pair", ["1", "0"])
def test_gemm_with_bf16_output(lib, monkeypatch, pair):
  """gbsgmc_gemm_bf16_c16: C rounded to BF16 (nearest even) from the same
  accumulators: within the fp32-summation bound plus half a BF16 ulp of
  the result, on the pair kernel and the single-CTA one."""
  import torch
  from gbsgmc import _lib
  monkeypatch.setenv("GBSGMC_GEMM_PAIR", pair)
  batch, M, N, K = 2, 512, 768, 320
  g = torch.Generator(device="cuda").manual_seed(77)
  A = torch.randn((batch, M, K), generator=g, device="cuda").to(torch.bfloat16)
  B = torch.randn((batch, N, K), generator=g, device="cuda").to(torch.bfloat16)
  C = torch.full((batch, M, N), float("nan"), dtype=torch.bfloat16, device="cuda")
  status = torch.zeros(1, dtype=torch.int32, device="cuda")
  _lib.call("gbsgmc_gemm_bf16_c16", 0, 0, A.data_ptr(), K, M * K, B.data_ptr(), K, N * K,
            C.data_ptr(), N, M * N, batch, M, N, K, status.data_ptr(), _lib.stream_handle())
  torch.cuda.synchronize()
  assert int(status.item()) == 0
  ref = torch.bmm(A.float(), B.float().transpose(1, 2))
  bound = torch.bmm(A.float().abs(), B.float().abs().transpose(1, 2))
  err = (C.float() - ref).abs()
  assert torch.isfinite(C.float()).all()
  assert bool((err <= 1e-3 * bound + 2.0 ** -8 * ref.abs() + 1e-4).all())
