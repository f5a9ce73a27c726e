"""Argument checks of the C ABI, which run before any CUDA call (so on the
CPU): a bad argument returns minus its 1-based position, as LAPACK's info
and the reference's LAPACK boundary (src/lapack.jl:40-62) do, and a plan
handle of NULL returns -1 from every plan entry point."""
import ctypes
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "genericlinearalgebra.jl_gb300"))


@pytest.fixture(scope="module")
def lib():
    import importlib.util
    spec = importlib.util.spec_from_file_location("gla_build", os.path.join(ROOT, "genericlinearalgebra.jl_gb300",
                                                                         "build.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    from glagpu import _lib as L
    lib = ctypes.CDLL(m.build())
    for name, (args, ret) in L.SIGNATURES.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = ret
    return lib


def create(lib, prec=0, jobz=b"V", uplo=b"L", ns=(4, 5), tol=0.0, flags=0, out=True, n_null=False):
    h = ctypes.c_void_p()
    n = (ctypes.c_int64 * len(ns))(*ns)
    return lib.gla_plan_create(ctypes.byref(h) if out else None, prec, jobz, uplo, len(ns), None if n_null else n,
                               tol, flags)


def test_plan_create_rejects_each_argument(lib):
    assert create(lib, out=False) == -1
    assert create(lib, prec=7) == -2
    assert create(lib, jobz=b"X") == -3
    assert create(lib, uplo=b"Q") == -4
    h = ctypes.c_void_p()
    assert lib.gla_plan_create(ctypes.byref(h), 0, b"V", b"L", -1, None, 0.0, 0) == -5
    assert create(lib, n_null=True) == -6
    assert create(lib, ns=(4, -1)) == -6
    assert create(lib, ns=(4, 16385)) == -6  # above GLA_MAX_N
    assert create(lib, tol=float("nan")) == -7
    assert create(lib, flags=1 << 20) == -8
    assert create(lib, flags=3) == -8  # algorithm code above GLA_ALG_QR
    # capture-safe plans take orders <= GLA_MAX_SMALL_N only
    assert create(lib, ns=(4, 300), flags=16) == -8


def test_null_plan_handle(lib):
    z = ctypes.c_int(0)
    assert lib.gla_plan_destroy(None) == -1
    assert lib.gla_plan_execute(None, None, None, None, None, None) == -1
    assert lib.gla_plan_execute_host(None, None, None, None, None, None) == -1
    assert lib.gla_plan_execute_eigen2(None, None, None, None, None, None) == -1
    assert lib.gla_plan_host_pipeline(None, ctypes.byref(z), ctypes.byref(z)) == -1
    assert lib.gla_plan_adjoint(None, None, None, None, None, None, 0.0, None) == -1
    size = ctypes.c_size_t(0)
    assert lib.gla_plan_workspace_size(None, ctypes.byref(size)) == -1


def test_single_matrix_drivers_reject_each_argument(lib):
    vp = ctypes.c_void_p
    info = ctypes.c_int(0)
    assert lib.gla_dsyev(b"X", b"L", 4, None, 4, None, ctypes.byref(info), None) == -1
    assert lib.gla_dsyev(b"V", b"X", 4, None, 4, None, ctypes.byref(info), None) == -2
    assert lib.gla_dsyev(b"V", b"L", -1, None, 4, None, ctypes.byref(info), None) == -3
    assert lib.gla_dsyev(b"V", b"L", 4, vp(8), 3, vp(8), ctypes.byref(info), None) == -5  # lda < n
    assert lib.gla_dsyev_static(b"V", b"L", 200, vp(8), 200, vp(8), ctypes.byref(info), None) == -2001
    assert lib.gla_dstev(b"X", 4, None, None, None, 4, 0, ctypes.byref(info), None) == -1


def test_other_entry_points_reject_each_argument(lib):
    p = ctypes.c_void_p(64)
    info = ctypes.c_int(0)
    # complex and quaternion Hermitian (their real embeddings are of order 2n and 4n)
    assert lib.gla_zheev(b"X", b"L", 4, p, 4, p, p, 4, ctypes.byref(info), None) == -1
    assert lib.gla_zheev(b"V", b"X", 4, p, 4, p, p, 4, ctypes.byref(info), None) == -2
    assert lib.gla_zheev(b"V", b"L", -1, p, 4, p, p, 4, ctypes.byref(info), None) == -3
    assert lib.gla_zheev(b"V", b"L", 9000, p, 9000, p, p, 9000, ctypes.byref(info), None) == -3  # 2n > GLA_MAX_N
    assert lib.gla_zheev(b"V", b"L", 4, p, 3, p, p, 4, ctypes.byref(info), None) == -5
    assert lib.gla_zheev(b"V", b"L", 4, p, 4, p, p, 3, ctypes.byref(info), None) == -8
    assert lib.gla_qheev(b"X", b"L", 4, p, 4, p, p, 4, ctypes.byref(info), None) == -1
    assert lib.gla_qheev(b"V", b"L", 5000, p, 5000, p, p, 5000, ctypes.byref(info), None) == -3  # 4n > GLA_MAX_N
    # symtri! and its EigenQ products
    assert lib.gla_dsytrd(b"X", 4, p, 4, p, p, p, None) == -1
    assert lib.gla_dsytrd(b"L", -1, p, 4, p, p, p, None) == -2
    assert lib.gla_dsytrd(b"L", 4, p, 3, p, p, p, None) == -4
    assert lib.gla_dormtr(b"X", b"L", b"N", 4, 4, p, 4, p, p, 4, None) == -1
    assert lib.gla_dormtr(b"L", b"X", b"N", 4, 4, p, 4, p, p, 4, None) == -2
    assert lib.gla_dormtr(b"L", b"L", b"X", 4, 4, p, 4, p, p, 4, None) == -3
    assert lib.gla_dormtr(b"L", b"L", b"N", -1, 4, p, 4, p, p, 4, None) == -4
    # spectrum slicing: an empty index range (iu = il - 1) is a no-op
    assert lib.gla_numnegevals(-1, p, p, 2, p, p, None) == -1
    assert lib.gla_numnegevals(4, p, p, -1, p, p, None) == -4
    assert lib.gla_dstebz(4, p, p, 0, 2, 0.0, p, None) == -4
    assert lib.gla_dstebz(4, p, p, 1, 5, 0.0, p, None) == -5
    assert lib.gla_dstebz(4, p, p, 3, 2, 0.0, p, None) == 0
    # the GEMMs: sizes, and the 16-byte alignment the TMA tensor maps need
    assert lib.gla_sgemm_3xtf32(-1, 4, 4, 1.0, p, 4, p, 4, 0.0, p, 4, None) == -1
    assert lib.gla_sgemm_3xtf32(4, 4, 4, 1.0, ctypes.c_void_p(66), 4, p, 4, 0.0, p, 4, None) == -5
    assert lib.gla_sgemm_3xtf32(4, 4, 4, 1.0, p, 3, p, 4, 0.0, p, 4, None) == -6
    assert lib.gla_gemm_df(-1, 4, 4, p, p, 4, p, p, 4, p, p, 4, None) == -1
