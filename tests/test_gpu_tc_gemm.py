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
@pytest.mark.parametrize("drain", [0, 1])
def test_gemm_matches_fp32(M, N, K, bn, dtype, nterms, drain):
    if drain and bn > 160:
        pytest.skip("drained accumulation needs 3 bn <= 512 TMEM columns")
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N + K)
    lda = (K + 7) // 8 * 8
    a = torch.randn(nterms, M, lda, device="cuda", generator=g).to(dtype)
    b = torch.randn(nterms, N, lda, device="cuda", generator=g).to(dtype)
    d = torch.full((M, N), float("nan"), device="cuda", dtype=torch.float32)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.call("afq_test_gemm_f16", a.data_ptr(), b.data_ptr(), nterms, M * lda, N * lda,
              d.data_ptr(), M, N, K, lda, lda, int(dtype == torch.bfloat16), bn, drain,
              status.data_ptr(), stream_ptr())
    ref = sum(a[t, :, :K].float() @ b[t, :, :K].float().T for t in range(nterms))
    torch.cuda.synchronize()
    assert status.item() == 0
    err = (d - ref).abs().max().item()
    assert err <= 1e-5 * K * nterms * 16, err


SPLIT_SHAPES = [(128, 256, 64), (300, 700, 600), (2048, 15360, 600), (130, 250, 136), (64, 16, 8),
                (512, 1024, 2400)]


@pytest.fixture(params=["pairs", "single"])
def split_form(request):
    """Run a split-GEMM test with CTA pairs (the default form for M > 128) and with one CTA
    per tile, restoring the library's setting afterwards."""
    lib = _lib.load()
    prev = lib.afq_test_split_pairs(1 if request.param == "pairs" else 0)
    yield request.param
    lib.afq_test_split_pairs(prev)


@pytest.mark.parametrize("M,N,K", SPLIT_SHAPES)
@pytest.mark.parametrize("dtype", [torch.bfloat16, torch.float16])
@pytest.mark.parametrize("terms", ["hi", "hi+alo", "all"])
@pytest.mark.parametrize("drain", [0, 1, 2])
def test_split_gemm_matches_fp32(M, N, K, dtype, terms, drain, split_form):
    """Persistent split GEMM: A_hi B_hi^T (+ A_lo B_hi^T) (+ A_hi B_lo^T) against torch FP32,
    on CTA pairs (odd M tile counts included: 300 rows) and on single CTAs."""
    g = torch.Generator(device="cuda").manual_seed(M + 3 * N + K)
    lda = (K + 7) // 8 * 8
    ah = torch.randn(M, lda, device="cuda", generator=g).to(dtype)
    al = (torch.randn(M, lda, device="cuda", generator=g) * 1e-3).to(dtype)
    bh = torch.randn(N, lda, device="cuda", generator=g).to(dtype)
    bl = (torch.randn(N, lda, device="cuda", generator=g) * 1e-3).to(dtype)
    use_al, use_bl = terms in ("hi+alo", "all"), terms == "all"
    d = torch.full((M, N), float("nan"), device="cuda", dtype=torch.float32)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.call("afq_test_gemm_split", ah.data_ptr(), al.data_ptr() if use_al else None, bh.data_ptr(),
              bl.data_ptr() if use_bl else None, d.data_ptr(), M, N, K, lda, lda,
              int(dtype == torch.bfloat16), drain, status.data_ptr(), stream_ptr())
    A, B = ah[:, :K].float(), bh[:, :K].float()
    ref = A @ B.T
    if use_al:
        ref = ref + al[:, :K].float() @ B.T
    if use_bl:
        ref = ref + A @ bl[:, :K].float().T
    torch.cuda.synchronize()
    assert status.item() == 0
    err = (d - ref).abs().max().item()
    assert err <= 1e-5 * K * 16, err


@pytest.mark.parametrize("drain", [0, 1, 2])
def test_split_accumulation_bias(drain, split_form):
    """Drained runs of the split GEMM remove the tensor core's truncation bias (K = 2400)."""
    M, N, K = 256, 512, 2400
    g = torch.Generator(device="cuda").manual_seed(6)
    a = (torch.rand(M, K, device="cuda", generator=g) * 0.5 + 0.5).half()
    b = (torch.rand(N, K, device="cuda", generator=g) * 0.5 + 0.5).half()
    d = torch.empty(M, N, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.call("afq_test_gemm_split", a.data_ptr(), None, b.data_ptr(), None, d.data_ptr(), M, N, K, K, K,
              0, drain, status.data_ptr(), stream_ptr())
    ref = a.double() @ b.double().T
    bias = ((d.double() - ref) / ref).mean().item()
    assert status.item() == 0
    if drain == 0:
        assert bias < -5e-6
    else:
        assert abs(bias) < 1e-6, bias


@pytest.mark.parametrize("drain", [0, 1, 2])
def test_accumulation_bias(drain):
    """The tensor core truncates when it accumulates: positive sums over K = 2400 come out
    ~1.5e-5 low with one accumulator. Drained accumulation (a fresh accumulator every
    `drain` K tiles, summed with round-to-nearest) must bring the mean bias below 1e-6."""
    M, N, K = 256, 256, 2400
    g = torch.Generator(device="cuda").manual_seed(5)
    a = (torch.rand(1, M, K, device="cuda", generator=g) * 0.5 + 0.5).half()
    b = (torch.rand(1, N, K, device="cuda", generator=g) * 0.5 + 0.5).half()
    d = torch.empty(M, N, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.call("afq_test_gemm_f16", a.data_ptr(), b.data_ptr(), 1, 0, 0, d.data_ptr(), M, N, K, K, K,
              0, 128, drain, status.data_ptr(), stream_ptr())
    ref = a[0].double() @ b[0].double().T
    bias = ((d.double() - ref) / ref).mean().item()
    assert status.item() == 0
    if drain == 0:
        assert bias < -5e-6  # the hardware behaviour this scheme corrects
    else:
        assert abs(bias) < 1e-6, bias
