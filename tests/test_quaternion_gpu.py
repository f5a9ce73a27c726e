"""Quaternion Hermitian input (the reference's eigen/eigvals/eigen2 on
Hermitian{Quaternion{Float64}}; test/eigenselfadjoint.jl:54-84) through
gla_qheev. The checker is independent of the device path's real embedding:
quaternion products are written out from the Hamilton product, and the
reference eigenvalues come from LAPACK (scipy eigh, zheevd) on the complex
adjoint matrix chi(A) = [[Z1, Z2], [-conj Z2, conj Z1]] (A = Z1 + Z2 j), whose
eigenvalues are those of A, each twice, and from the oracle's restatement of
the reference's own quaternion path (values, and eigenvectors up to a unit
quaternion factor where the eigenvalue is separated). Norms of quaternion matrices are the
spectral norms of their chi.
Tolerances: eigenvalues within 32 n eps ||A|| (the real embedding has order
4n); residual ||AV - V diag(w)||/||A|| and ||V^H V - I|| <= 1e-13; the
reference's prescribed spectrum at its rtol 1e-13 n."""
import numpy as np
import pytest
import scipy.linalg as sl

from helpers import chi, qeye, qH, qherm_random, qherm_spectrum, qmul, qnorm
from oracle import oracle as O

pytestmark = pytest.mark.gpu

EPS64 = 2.0 ** -52


@pytest.fixture(scope="module")
def G():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import glagpu
    return glagpu


def ref_values(A):
    return sl.eigh(chi(A), eigvals_only=True)[::2]


def check(A, w, V):
    n = A.shape[0]
    nA = max(qnorm(A), 1e-300)
    assert np.all(np.diff(w) >= 0)
    assert np.abs(w - ref_values(A)).max() <= 32 * n * EPS64 * nA
    assert qnorm(qmul(A, V) - V * w[None, :, None]) / nA <= 1e-13
    assert qnorm(qmul(qH(V), V) - qeye(n)) <= 1e-13


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_prescribed_spectrum(G, uplo):
    # test/eigenselfadjoint.jl:54-84, n = 50: lambda = 10 .^ range(-8, 0, n)
    n = 50
    lam = 10.0 ** np.linspace(-8, 0, n)
    A = qherm_spectrum(lam, np.random.default_rng(54))
    junk = np.full((n, n, 4), 9.0)
    keep = np.tril(np.ones((n, n), bool)) if uplo == "L" else np.triu(np.ones((n, n), bool))
    S = np.where(keep[..., None], A, junk)  # the other triangle is never read
    vals, vecs = G.eigen(G.QuaternionMatrix(S), uplo=uplo)
    check(A, vals, vecs)
    assert np.linalg.norm(vals - lam) <= 1e-13 * n * max(np.linalg.norm(vals), np.linalg.norm(lam))
    assert np.abs(G.eigvals(G.QuaternionMatrix(S), uplo=uplo) - vals).max() <= 32 * n * EPS64
    vals2, vecs2 = G.eigen2(G.QuaternionMatrix(S), uplo=uplo)
    assert np.array_equal(vals2, vals)
    assert np.array_equal(vecs2, vecs[[0, n - 1]])
    assert qnorm(qmul(vecs2, qH(vecs2)) - qeye(2)) <= 1e-13


@pytest.mark.parametrize("n", [1, 2, 3, 17, 64, 150])
def test_random(G, n):
    A = qherm_random(n, np.random.default_rng(200 + n))
    vals, vecs = G.eigen(G.QuaternionMatrix(A))
    check(A, vals, vecs)


def test_multiplicities(G):
    # multiplicities 5, 3 and 2: groups of 20, 12 and 8 values of the real embedding
    n = 40
    rng = np.random.default_rng(41)
    lam = np.sort(np.concatenate([[1.0] * 5, [-2.0] * 3, [0.5] * 2, rng.uniform(-3, 3, n - 10)]))
    A = qherm_spectrum(lam, rng)
    vals, vecs = G.eigen(G.QuaternionMatrix(A))
    check(A, vals, vecs)
    assert np.abs(vals - lam).max() <= 32 * n * EPS64 * 3


def test_complex_special_case(G):
    # j and k parts zero: a complex Hermitian matrix, whose values gla_zheev also gives
    n = 33
    rng = np.random.default_rng(5)
    B = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    Z = (B + B.conj().T) / 2
    A = np.zeros((n, n, 4))
    A[..., 0], A[..., 1] = Z.real, Z.imag
    vals, vecs = G.eigen(G.QuaternionMatrix(A))
    check(A, vals, vecs)
    assert np.abs(vals - G.eigvals(Z)).max() <= 32 * n * EPS64 * np.linalg.norm(Z, 2)


def test_device_tensor(G):
    import torch
    A = qherm_random(30, np.random.default_rng(9))
    At = torch.tensor(A, device="cuda")
    vals, vecs = G.eigen(G.QuaternionMatrix(At))
    assert vecs.is_cuda and tuple(vecs.shape) == (30, 30, 4)
    check(A, vals.cpu().numpy(), vecs.cpu().numpy())


def test_host_entry_and_arguments(G):
    import ctypes as C
    from glagpu import _lib
    L = _lib.load()
    n = 20
    A = qherm_random(n, np.random.default_rng(3))
    Ac = np.ascontiguousarray(A.transpose(1, 0, 2))  # column-major, 4 doubles per entry
    w, Vc = np.empty(n), np.empty((n, n, 4))
    info = C.c_int(-7)
    p = lambda a: C.c_void_p(a.ctypes.data)
    assert L.gla_qheev_host(b"V", b"L", n, p(Ac), n, p(w), p(Vc), n, C.byref(info)) == 0 and info.value == 0
    check(A, w, Vc.transpose(1, 0, 2))
    assert L.gla_qheev_host(b"X", b"L", n, p(Ac), n, p(w), p(Vc), n, C.byref(info)) == -1
    assert L.gla_qheev_host(b"V", b"L", n, p(Ac), n - 1, p(w), p(Vc), n, C.byref(info)) == -5
    assert L.gla_qheev_host(b"V", b"L", 4097, p(Ac), 4097, p(w), p(Vc), 4097, C.byref(info)) == -3
    with pytest.raises(Exception):
        G.QuaternionMatrix(np.zeros((3, 3, 3)))


@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("n", [4, 50, 120])
def test_against_oracle_restatement(G, n, uplo):
    A = qherm_random(n, np.random.default_rng(600 + n))
    vals, vecs = G.eigen(G.QuaternionMatrix(A), uplo=uplo)
    wo, Vo, info = O.heev_quaternion(A, "V", uplo)
    assert info == 0
    nA = qnorm(A)
    assert np.abs(vals - wo).max() <= 32 * n * EPS64 * nA
    # v_gpu = v_oracle q with |q| = 1 where the eigenvalue is separated: |v_gpu^H v_oracle| = 1
    gaps = np.full(n, np.inf)
    if n > 1:
        dw = np.diff(wo)
        gaps[:-1] = np.minimum(gaps[:-1], dw)
        gaps[1:] = np.minimum(gaps[1:], dw)
    sep = gaps > 1e-6 * nA
    inner = np.stack([qmul(qH(vecs[:, j:j + 1]), Vo[:, j:j + 1])[0, 0] for j in range(n)])
    overlap = np.sqrt((inner ** 2).sum(axis=1))
    assert sep.sum() >= n // 2
    assert np.all(overlap[sep] >= 1 - 1e-8)
