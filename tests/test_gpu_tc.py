"""GPU: the tensor-core (tcgen05, split-TF32) tall products against FP64
torch: Gram matrices Aᵀ B and block products A Bm, FP32-level accuracy,
including widths beyond one 256-column accumulator (column blocks) and K
beyond 256."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def core():
    from rvgp_gb300 import _core
    _core.require_cuda()
    return _core


@pytest.mark.parametrize("N,p,q,same", [(1000, 228, 228, True), (40000, 228, 228, True), (5000, 100, 60, False),
                                        (333, 256, 256, True), (7, 20, 36, False), (40000, 228, 228, False),
                                        (20001, 129, 129, True), (30000, 564, 564, True), (5000, 300, 257, False),
                                        (2000, 700, 100, False), (777, 257, 600, False)])
def test_tc_gram(core, N, p, q, same):
    g = torch.Generator(device="cuda").manual_seed(N + p)
    A = torch.randn((N, p), device="cuda", generator=g) * torch.logspace(-3, 2, p, device="cuda")
    B = A if same else torch.randn((N, q), device="cuda", generator=g)
    C = core.tc_gram(A, None if same else B)
    ref = A.double().T @ B.double()
    scale = torch.outer(A.double().norm(dim=0), B.double().norm(dim=0))
    err = ((C - ref).abs() / scale).max().item()
    # FP32 accumulation inside a CTA: wide products get fewer row splits per
    # CTA tile (longer FP32 sums), hence the looser bound above 256 columns
    assert err < (3e-6 if max(p, q) <= 256 else 1e-5), err


@pytest.mark.parametrize("N,K,q", [(40000, 228, 228), (1000, 50, 30), (129, 256, 256), (5, 3, 17), (20000, 228, 200),
                                   (30000, 564, 564), (1000, 300, 20), (513, 40, 700)])
def test_tc_gemm(core, N, K, q):
    g = torch.Generator(device="cuda").manual_seed(N + K)
    A = torch.randn((N, K), device="cuda", generator=g)
    Bm = torch.randn((K, q), device="cuda", generator=g) * torch.logspace(-2, 1, q, device="cuda")
    C = core.tc_gemm(A, Bm)
    ref = A.double() @ Bm.double()
    scale = torch.outer(A.double().norm(dim=1), Bm.double().norm(dim=0))
    err = ((C.double() - ref).abs() / scale).max().item()
    assert err < 2e-6, err
