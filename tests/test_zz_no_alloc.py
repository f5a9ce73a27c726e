"""gla_dsyev_static, the entry point that allocates no device memory (for
callers that cannot call cudaMalloc when they need the decomposition: a
memory pool that already owns the device, a loop where an allocation would
synchronise the device, a fixed memory budget). Its output must match
gla_dsyev's, the allocating entry point, within the tolerances of the other
GPU tests, on consecutive calls that reuse the shared static scratch.

Named to be collected last, so a run that stops at the first failure has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

from helpers import goe, residual, orth, vec_parity

pytestmark = pytest.mark.gpu
EPS64 = 2.0 ** -52


@pytest.fixture(scope="module")
def env():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from glagpu import _lib
    return torch, _lib.load(), _lib


def call(torch, L, fn, A, jobz="V", uplo="L", lda=None):
    n = A.shape[0]
    lda = lda or n
    buf = torch.zeros((n, lda), dtype=torch.float64, device="cuda")  # column-major n x n with leading dim lda
    buf[:, :n] = torch.tensor(A.T, device="cuda")
    w = torch.empty(max(n, 1), dtype=torch.float64, device="cuda")
    info = C.c_int(-7)
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = fn(jobz.encode(), uplo.encode(), n, C.c_void_p(buf.data_ptr()), lda, C.c_void_p(w.data_ptr()),
            C.byref(info), st)
    return rc, info.value, w.cpu().numpy()[:n], buf[:, :n].cpu().numpy().T


def test_static_matches_allocating_entry_point(env):
    torch, L, _ = env
    # two calls in a row (different orders and triangles: the second call runs on
    # the scratch left by the first), each against the allocating gla_dsyev
    for n, uplo, seed in [(128, "L", 1), (37, "U", 2)]:
        A = goe(n, 900 + seed)
        rs, infs, ws, Vs = call(torch, L, L.gla_dsyev_static, A, "V", uplo)
        ra, infa, wa, Va = call(torch, L, L.gla_dsyev, A, "V", uplo)
        assert rs == 0 and infs == 0 and ra == 0 and infa == 0
        nA = np.linalg.norm(A, 2)
        assert np.abs(ws - wa).max() <= 8 * n * EPS64 * nA
        assert residual(A, Vs, ws) <= 1e-13 and orth(Vs) <= 1e-13
        assert vec_parity(A, Vs, Va, wa) <= 1.0


def test_static_values_only_and_lda(env):
    torch, L, _ = env
    A = goe(64, 7)
    rs, infs, ws, _ = call(torch, L, L.gla_dsyev_static, A, "N", "L", lda=70)
    ra, infa, wa, _ = call(torch, L, L.gla_dsyev, A, "N", "L", lda=70)
    assert rs == 0 and infs == 0
    assert np.abs(ws - wa).max() <= 8 * 64 * EPS64 * np.linalg.norm(A, 2)


def test_static_rejects_orders_above_the_limit(env):
    torch, L, lib = env
    w = torch.empty(200, dtype=torch.float64, device="cuda")
    A = torch.zeros(200 * 200, dtype=torch.float64, device="cuda")
    info = C.c_int(0)
    rc = L.gla_dsyev_static(b"V", b"L", lib.GLA_STATIC_MAX_N + 1, C.c_void_p(A.data_ptr()), 200,
                            C.c_void_p(w.data_ptr()), C.byref(info), None)
    assert rc == lib.GLA_ERR_STATIC_TOO_LARGE
    assert b"GLA_STATIC_MAX_N" in L.gla_status_string(rc)


def test_static_call_allocates_no_device_memory(env):
    # cudaMemGetInfo (torch.cuda.mem_get_info) sees every device allocation,
    # raw cudaMalloc included, unlike the caching allocator's statistics
    torch, L, _ = env
    A = goe(96, 31)
    call(torch, L, L.gla_dsyev_static, A, "V", "L")  # warm-up: the per-device set-up
    cases = [(77, b"V"), (77, b"N"), (96, b"V"), (5, b"N")]
    bufs = []
    for n, _ in cases:  # every device buffer exists before the first reading
        b = torch.zeros((96, 96), dtype=torch.float64, device="cuda")
        b[:n, :n] = torch.tensor(goe(n, 40 + n), device="cuda")
        bufs.append(b)
    w = torch.empty(96, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    info = C.c_int(0)
    for (n, jobz), buf in zip(cases, bufs):
        rc = L.gla_dsyev_static(jobz, b"L", n, C.c_void_p(buf.data_ptr()), 96, C.c_void_p(w.data_ptr()),
                                C.byref(info), None)
        assert rc == 0 and info.value == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] >= free0


def test_static_recovers_after_a_failed_call(env):
    # a call stopped early by non-finite input must leave nothing behind that
    # changes the next call's result
    torch, L, _ = env
    n = 50
    A = goe(n, 77)
    Abad = A.copy()
    Abad[7, 3] = Abad[3, 7] = np.nan
    rb, infb, _, _ = call(torch, L, L.gla_dsyev_static, Abad, "V", "L")
    assert rb == 1 and infb != 0
    rs, infs, ws, Vs = call(torch, L, L.gla_dsyev_static, A, "V", "L")
    ra, infa, wa, Va = call(torch, L, L.gla_dsyev, A, "V", "L")
    assert rs == 0 and infs == 0 and ra == 0 and infa == 0
    assert np.abs(ws - wa).max() <= 8 * n * EPS64 * np.linalg.norm(A, 2)
    assert residual(A, Vs, ws) <= 1e-13 and orth(Vs) <= 1e-13
    assert vec_parity(A, Vs, Va, wa) <= 1.0
