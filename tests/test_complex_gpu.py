"""Complex Hermitian input (the reference's eigen/eigvals on
Hermitian{<:Complex}; test/eigenselfadjoint.jl:86-91 and :171-176) through
gla_zheev, against LAPACK (scipy eigh, zheevd) and against the oracle's
restatement of the reference's own complex path (values, and eigenvectors
up to their complex phase where the eigenvalue is separated).
Tolerances: eigenvalues within 16 n eps ||A|| (the real embedding has order
2n); residual ||AV - V diag(w)||/||A|| and ||V^H V - I|| <= 1e-13."""
import numpy as np
import pytest
import scipy.linalg as sl

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


def herm(n, seed):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    return (B + B.conj().T) / 2


def check(A, w, V):
    n = A.shape[0]
    nA = max(np.linalg.norm(A, 2), 1e-300)
    assert np.all(np.diff(w) >= 0)
    assert np.abs(w - sl.eigh(A, eigvals_only=True)).max() <= 16 * n * EPS64 * nA
    assert np.linalg.norm(A @ V - V * w, 2) / nA <= 1e-13
    assert np.linalg.norm(V.conj().T @ V - np.eye(n), 2) <= 1e-13


@pytest.mark.parametrize("n", [1, 2, 4, 10, 64, 100, 300])
def test_complex_hermitian_random(G, n):
    A = herm(n, 100 + n)
    r = G.eigen(A)
    check(A, r.values, r.vectors)
    assert np.abs(G.eigvals(A) - r.values).max() <= 16 * n * EPS64 * np.linalg.norm(A, 2)


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_complex_hermitian_uplo(G, uplo):
    A = herm(50, 7)
    junk = np.triu(np.full((50, 50), 5 + 5j), 1) if uplo == "L" else np.tril(np.full((50, 50), 5 + 5j), -1)
    S = (np.tril(A) if uplo == "L" else np.triu(A)) + junk  # the other triangle is never read
    r = G.eigen(S, uplo=uplo)
    check(A, r.values, r.vectors)


def test_complex_hermitian_multiplicities(G):
    # eigenvalues with multiplicity 3 and 2: groups of 6 and 4 real embedding values
    n = 40
    rng = np.random.default_rng(3)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    lam = np.concatenate([[1.0] * 3, [-2.0] * 2, rng.uniform(-3, 3, n - 5)])
    A = (Q * lam) @ Q.conj().T
    A = (A + A.conj().T) / 2
    r = G.eigen(A)
    check(A, r.values, r.vectors)


def test_reference_cases(G):
    # test/eigenselfadjoint.jl:171-176: Hermitian(Tridiagonal(ones(ComplexF64, ...))), n = 3
    M = np.diag(np.ones(3, complex)) + np.diag(np.ones(2, complex), 1) + np.diag(np.ones(2, complex), -1)
    w = G.eigvals(M)
    assert np.abs(w - np.array([1 - np.sqrt(2), 1.0, 1 + np.sqrt(2)])).max() <= 1e-14
    # :86-91: a 4 x 4 complex Hermitian, values against an independent solver
    rng = np.random.default_rng(35)
    B = rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))
    A = np.tril(B) + np.tril(B, -1).conj().T
    A = (A + A.conj().T) / 2
    r = G.eigen(A)
    check(A, r.values, r.vectors)


def test_complex_device_tensor(G):
    import torch
    A = herm(30, 9)
    At = torch.tensor(A, device="cuda")
    r = G.eigen(At)
    assert r.vectors.is_cuda and r.vectors.dtype == torch.complex128
    check(A, r.values.cpu().numpy(), r.vectors.cpu().numpy())


@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("n", [4, 64, 200])
def test_against_oracle_restatement(G, n, uplo):
    A = herm(n, 500 + n)
    r = G.eigen(A, uplo=uplo)
    wo, Vo, info = O.heev(A, "V", uplo)
    assert info == 0
    nA = np.linalg.norm(A, 2)
    assert np.abs(r.values - wo).max() <= 24 * n * EPS64 * nA
    # eigenvectors agree up to a unit complex factor where the eigenvalue is separated
    gaps = np.full(n, np.inf)
    if n > 1:
        dw = np.diff(wo)
        gaps[:-1] = np.minimum(gaps[:-1], dw)
        gaps[1:] = np.minimum(gaps[1:], dw)
    sep = gaps > 1e-6 * nA
    overlap = np.abs(np.sum(r.vectors.conj() * Vo, axis=0))
    assert sep.sum() >= n // 2
    assert np.all(overlap[sep] >= 1 - 1e-8)
