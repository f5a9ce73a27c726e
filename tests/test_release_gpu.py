"""gla_release_workspaces: every single-call entry point that caches a
per-order device workspace runs, the caches are released (device memory is
returned, as cudaMemGetInfo shows), and every entry point runs again with
bit-identical results."""
import numpy as np
import pytest

from helpers import goe

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import glagpu
    return glagpu


def dsyev(torch, L, A):
    import ctypes as C
    n = A.shape[0]
    buf = torch.tensor(A.T.copy(), device="cuda")
    w = torch.empty(n, dtype=torch.float64, device="cuda")
    info = C.c_int(0)
    assert L.gla_dsyev(b"V", b"L", n, C.c_void_p(buf.data_ptr()), n, C.c_void_p(w.data_ptr()), C.byref(info),
                       None) == 0
    return [w, buf]


def gemm_df(torch, L, n):
    import ctypes as C
    g = torch.Generator(device="cpu").manual_seed(9)
    A, B = torch.randn(n, n, generator=g).cuda(), torch.randn(n, n, generator=g).cuda()
    Ch, Cl = torch.empty(n, n, device="cuda"), torch.empty(n, n, device="cuda")
    p = lambda t: C.c_void_p(t.data_ptr())
    assert L.gla_gemm_df(n, n, n, p(A), None, n, p(B), None, n, p(Ch), p(Cl), n, None) == 0
    return [Ch, Cl]


def run_all(G):
    import torch
    from glagpu import _lib
    L = _lib.load()
    rng = np.random.default_rng(12)
    out = dsyev(torch, L, goe(90, 2)) + dsyev(torch, L, goe(260, 2))  # gla_dsyev, small and large orders
    out += gemm_df(torch, L, 256)                                 # gla_gemm_df
    A = torch.tensor(goe(200, 3), device="cuda")
    out += list(G.eigen(A))                                       # gla plan path (large order)
    out += list(G.eigen(torch.tensor(goe(40, 4), device="cuda")))  # batched plan
    d, e = rng.standard_normal(300), rng.standard_normal(299)
    out += list(G.eigen(G.SymTridiagonal(torch.tensor(d, device="cuda"), torch.tensor(e, device="cuda"))))  # gla_dstev
    Z = rng.standard_normal((24, 24)) + 1j * rng.standard_normal((24, 24))
    out += list(G.eigen(torch.tensor(Z + Z.conj().T, device="cuda")))  # gla_zheev
    F = G.symtri(torch.tensor(goe(150, 5), device="cuda"))        # gla_dsytrd
    out.append(F.reflectors.array())                              # gla_dormtr
    return [x.cpu().numpy() if hasattr(x, "cpu") else np.asarray(x) for x in out]


def test_release_then_rerun(G):
    import torch
    first = run_all(G)
    torch.cuda.synchronize()
    before = torch.cuda.mem_get_info()[0]
    G.release_workspaces()
    after = torch.cuda.mem_get_info()[0]
    assert after > before  # the cached workspaces went back to the device
    second = run_all(G)
    assert len(first) == len(second)
    for a, b in zip(first, second):
        assert np.array_equal(a, b)
    G.release_workspaces()  # releasing twice (and with nothing cached) is fine
    G.release_workspaces()
