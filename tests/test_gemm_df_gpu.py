"""gla_gemm_df: the tcgen05 Ozaki GEMM (double-float accuracy from bf16
slices) against an FP64 product of the same float-pair inputs."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import glagpu._lib as lib
    return lib


def split(x):
    h = x.astype(np.float32)
    return h, (x - h.astype(np.float64)).astype(np.float32)


def run(L, m, n, k, lda=None, ldb=None, ldc=None, alo=True, blo=True, seed=0):
    import torch
    rng = np.random.default_rng(seed)
    lda, ldb, ldc = lda or m, ldb or k, ldc or m
    A = rng.standard_normal((m, k)) * np.exp(rng.uniform(-4, 4, (m, 1)))  # rows of very different scale
    B = rng.standard_normal((k, n)) * np.exp(rng.uniform(-4, 4, (1, n)))
    Ah, Al = split(A)
    Bh, Bl = split(B)
    def dev(x, ld):
        buf = np.zeros((ld, x.shape[1]), np.float32)
        buf[: x.shape[0]] = x
        return torch.tensor(buf.ravel(order="F"), device="cuda")
    dAh, dAl, dBh, dBl = dev(Ah, lda), dev(Al, lda), dev(Bh, ldb), dev(Bl, ldb)
    dCh = torch.zeros(ldc * n, device="cuda")
    dCl = torch.zeros(ldc * n, device="cuda")
    p = lambda t: C.c_void_p(t.data_ptr())
    rc = L.load().gla_gemm_df(m, n, k, p(dAh), p(dAl) if alo else None, lda, p(dBh), p(dBl) if blo else None, ldb,
                              p(dCh), p(dCl), ldc, None)
    torch.cuda.synchronize()
    assert rc == 0
    Cg = (dCh.cpu().numpy().astype(np.float64) + dCl.cpu().numpy()).reshape(n, ldc).T[:m]
    A64 = Ah.astype(np.float64) + (Al if alo else 0)
    B64 = Bh.astype(np.float64) + (Bl if blo else 0)
    den = np.abs(A64) @ np.abs(B64)
    return np.max(np.abs(Cg - A64 @ B64) / den)


@pytest.mark.parametrize("shape", [(128, 64, 32), (100, 70, 50), (257, 129, 300), (640, 520, 1000)])
def test_gemm_df_matches_fp64(L, shape):
    assert run(L, *shape) <= 2e-14


def test_gemm_df_leading_dims_and_null_lo(L):
    assert run(L, 90, 40, 77, lda=96, ldb=80, ldc=100) <= 2e-14
    assert run(L, 90, 40, 77, alo=False, blo=False, seed=3) <= 2e-14


def test_gemm_df_arguments(L):
    lib = L.load()
    assert lib.gla_gemm_df(-1, 1, 1, None, None, 1, None, None, 1, None, None, 1, None) == -1
    assert lib.gla_gemm_df(4, 4, 4, None, None, 4, None, None, 4, None, None, 4, None) == -4
    assert lib.gla_gemm_df(0, 0, 0, None, None, 1, None, None, 1, None, None, 1, None) == 0
