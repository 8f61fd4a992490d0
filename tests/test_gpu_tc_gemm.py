"""tcgen05 GEMM core against a PyTorch FP32 matmul of the same 16-bit inputs.

Tolerance: inputs are exactly representable in 16 bits and accumulation is FP32, so the
only difference from torch's FP32 matmul is summation order: max |diff| <= 1e-5 * K * max|a||b|.
"""

import ctypes

import pytest
import torch

from cs_afqmc_gb300 import _lib
from cs_afqmc_gb300._engine import stream_ptr

pytestmark = pytest.mark.gpu

SHAPES = [(128, 64, 64, 64), (300, 250, 200, 128), (256, 480, 600, 240), (1000, 700, 136, 256), (200, 300, 72, 48), (130, 600, 2400, 208),
          (64, 16, 8, 64)]


@pytest.mark.parametrize("M,N,K,bn", SHAPES)
@pytest.mark.parametrize("dtype", [torch.bfloat16, torch.float16])
@pytest.mark.parametrize("nterms", [1, 3])
def test_gemm_matches_fp32(M, N, K, bn, dtype, nterms):
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N + K)
    lda = (K + 7) // 8 * 8
    a = torch.randn(nterms, M, lda, device="cuda", generator=g).to(dtype)
    b = torch.randn(nterms, N, lda, device="cuda", generator=g).to(dtype)
    d = torch.full((M, N), float("nan"), device="cuda", dtype=torch.float32)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.call("afq_test_gemm_f16", a.data_ptr(), b.data_ptr(), nterms, M * lda, N * lda,
              d.data_ptr(), M, N, K, lda, lda, int(dtype == torch.bfloat16), bn,
              status.data_ptr(), stream_ptr())
    ref = sum(a[t, :, :K].float() @ b[t, :, :K].float().T for t in range(nterms))
    torch.cuda.synchronize()
    assert status.item() == 0
    err = (d - ref).abs().max().item()
    assert err <= 1e-5 * K * nterms * 16, err
