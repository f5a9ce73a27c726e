"""gla_sgemm_3xtf32: the FP32 tensor-core GEMM (tcgen05 kind::tf32 in split
TF32, TMA-fed operands) that the FP32 large-matrix path uses for its
trailing updates and back-transformation, against an FP64 product of the
same FP32 inputs. Tolerance: 4e-6 of sum_k |a_ik||b_kj| per entry (the
scheme's ~2^-21 plus FP32 accumulation)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from glagpu import _lib
    return torch, _lib.load()


def run(torch, L, m, n, k, alpha=1.0, beta=0.0, pad=0, seed=0):
    g = torch.Generator(device="cpu").manual_seed(seed)
    ldat = (k + pad + 3) // 4 * 4
    ldb = (k + pad + 3) // 4 * 4
    At = torch.randn(m, ldat, generator=g)          # column i of At (length ldat) = row i of A
    B = torch.randn(n, ldb, generator=g) * 3.0      # column j of B
    C0 = torch.randn(n, m + 3, generator=g)          # column-major C, ldc = m + 3
    dA, dB, dC = At.cuda(), B.cuda(), C0.clone().cuda()
    p = lambda t: C.c_void_p(t.data_ptr())
    rc = L.gla_sgemm_3xtf32(m, n, k, alpha, p(dA), ldat, p(dB), ldb, beta, p(dC), m + 3, None)
    torch.cuda.synchronize()
    assert rc == 0
    A64 = At[:, :k].double()                 # m x k
    B64 = B[:, :k].double().t()              # k x n
    ref = alpha * (A64 @ B64) + beta * C0[:, :m].double().t()
    bound = 4e-6 * (abs(alpha) * (A64.abs() @ B64.abs()) + abs(beta) * C0[:, :m].double().abs().t()) + 1e-30
    got = dC.cpu().double()[:, :m].t()
    err = ((got - ref).abs() / bound).max().item()
    assert err <= 1.0, err
    # the padding rows of C past m are untouched
    assert torch.equal(dC.cpu()[:, m:], C0[:, m:])


@pytest.mark.parametrize("m,n,k", [(128, 128, 32), (256, 384, 512), (200, 130, 77), (1, 5, 3), (1000, 257, 1000)])
def test_sgemm_3xtf32_matches_fp64(env, m, n, k):
    torch, L = env
    run(torch, L, m, n, k)


def test_sgemm_3xtf32_alpha_beta(env):
    torch, L = env
    run(torch, L, 300, 200, 64, alpha=-1.0, beta=1.0, pad=5, seed=3)
    run(torch, L, 129, 129, 4096, alpha=0.5, beta=-2.0, seed=4)


def test_sgemm_3xtf32_rejects_unaligned(env):
    torch, L = env
    a = torch.zeros(64 * 64, device="cuda")
    p = lambda t, off=0: C.c_void_p(t.data_ptr() + off)
    assert L.gla_sgemm_3xtf32(8, 8, 8, 1.0, p(a), 10, p(a), 8, 0.0, p(a), 8, None) == -6  # ldat % 4
    assert L.gla_sgemm_3xtf32(8, 8, 8, 1.0, p(a, 4), 8, p(a), 8, 0.0, p(a), 8, None) == -5  # At alignment
