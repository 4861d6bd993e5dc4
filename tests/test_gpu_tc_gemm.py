"""tcgen05 BF16 GEMM against a plain PyTorch fp32 reference of the same op (bf16 inputs
widened to fp32).  Tolerance: fp32 results within 1e-4 relative to the largest |C| (the
accumulation order differs); bf16 outputs within one bf16 rounding (2^-8 relative)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def ref(A, B, bias, act):
    import torch
    y = A.float() @ B.float().T
    if bias is not None:
        y = y + bias
    if act == 1:
        y = torch.nn.functional.gelu(y, approximate="tanh")
    return y


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 512, 192), (300, 144, 128), (1000, 128, 512),
                                   (77, 256, 64), (130, 520, 64), (200, 136, 136), (129, 264, 40),
                                   # persistent kernel (at least two tiles per SM): tails in M, N, K
                                   (40037, 512, 192), (39001, 128, 520), (20000, 260, 64), (65536, 512, 512)])
@pytest.mark.parametrize("act", [0, 1])
def test_tc_gemm_matches_torch_fp32(lib, cuda, M, N, K, act):
    import torch
    g = torch.Generator(device="cpu").manual_seed(M * 7 + N + K + act)
    A = (torch.randn(M, K, generator=g) * 0.5).to(torch.bfloat16).to(cuda)
    B = (torch.randn(N, K, generator=g) * 0.5).to(torch.bfloat16).to(cuda)
    bias = (torch.randn(N, generator=g) * 0.1).to(cuda)
    out = torch.full((M, N), float("nan"), dtype=torch.float32, device=cuda)
    pre = torch.empty((M, N), dtype=torch.float32, device=cuda)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    rc = lib.cumf_tc_gemm(A.data_ptr(), B.data_ptr(), M, N, K, bias.data_ptr(), act, out.data_ptr(), 1, N,
                          pre.data_ptr(), status.data_ptr(), None)
    assert rc == 0, lib.cumf_last_error()
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    exp = ref(A, B, bias, act)
    scale = exp.abs().max().item()
    assert torch.isfinite(out).all()
    assert (out - exp).abs().max().item() <= 1e-4 * scale + 1e-6
    assert (pre - ref(A, B, bias, 0)).abs().max().item() <= 1e-4 * scale + 1e-6
    outb = torch.empty((M, N), dtype=torch.bfloat16, device=cuda)
    rc = lib.cumf_tc_gemm(A.data_ptr(), B.data_ptr(), M, N, K, bias.data_ptr(), act, outb.data_ptr(), 0, N,
                          None, None, None)
    assert rc == 0
    torch.cuda.synchronize()
    assert ((outb.float() - exp).abs() <= exp.abs() * 2 ** -8 + 1e-3 * scale).all()


def test_tc_gemm_rejects_bad_k(lib, cuda):
    import torch
    A = torch.zeros(128, 100, dtype=torch.bfloat16, device=cuda)
    out = torch.zeros(128, 128, dtype=torch.float32, device=cuda)
    assert lib.cumf_tc_gemm(A.data_ptr(), A.data_ptr(), 128, 128, 100, None, 0, out.data_ptr(), 1, 128, None,
                            None, None) != 0


@pytest.mark.parametrize("M,N,K", [(128, 512, 16384), (131, 200, 4104), (512, 192, 65536)])
def test_tc_gemm_split_k_matches_torch_fp32(lib, cuda, M, N, K):
    """Plain fp32 products with few output tiles and long K (the weight-gradient shapes) are
    split over K and summed with atomics into the zeroed output."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(M + N + K)
    A = (torch.randn(M, K, generator=g) * 0.5).to(torch.bfloat16).to(cuda)
    B = (torch.randn(N, K, generator=g) * 0.5).to(torch.bfloat16).to(cuda)
    out = torch.full((M, N), float("nan"), dtype=torch.float32, device=cuda)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    for _ in range(2):  # the output is overwritten, not accumulated across calls
        rc = lib.cumf_tc_gemm(A.data_ptr(), B.data_ptr(), M, N, K, None, 0, out.data_ptr(), 1, N, None,
                              status.data_ptr(), None)
        assert rc == 0, lib.cumf_last_error()
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    exp = A.float() @ B.float().T
    scale = exp.abs().max().item()
    assert (out - exp).abs().max().item() <= 1e-4 * scale + 1e-6


def test_wait_timeout_reports_status_and_context_survives(lib, cuda):
    """A product whose operand copies are never issued (a flag nothing sets in normal use):
    its stage wait runs out after about 2 s, the kernel reports CUMF_ERR_TIMEOUT, frees its
    tensor memory and returns; the same context then computes an ordinary product."""
    from cumf_sgd_gb300 import _lib
    status, secs = C.c_int(0), C.c_double(0)
    rc = lib.cumf_selftest_wait_timeout(C.byref(status), C.byref(secs))
    assert rc == 0, lib.cumf_last_error()
    assert status.value == _lib.CUMF_ERR_TIMEOUT
    assert 1.5 <= secs.value <= 12.0
