"""The Householder factorisation on its own (gla_dsytrd / gla_dormtr): the
reference's symtri! / SymmetricTridiagonalFactorization and lmul!/rmul! with
its EigenQ (src/eigenSelfAdjoint.jl:6-118, 446-564; tested at
test/eigenselfadjoint.jl:61-68), against the CPU oracle's restatement, in
both the lower (symtriLower!) and upper (symtriUpper!) layouts.
Tolerances: d and e within 1e-12 ||A|| of the oracle's symtri!; tau and
the stored reflectors within 1e-10 (the blocked update order rounds
differently from the reference's unblocked one, and the late reflectors of
small trailing blocks amplify that); the backward checks are tight:
||Q'Q - I||, ||Q' A Q - T||/||A|| and the lmul/rmul identities within 1e-13."""
import numpy as np
import pytest

from helpers import goe
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import glagpu
    return glagpu


def np_(t):
    return t.cpu().numpy()


@pytest.mark.parametrize("n", [1, 2, 3, 17, 64, 200, 333])
def test_symtri_matches_oracle(G, n):
    A = goe(n, 60 + n)
    f = G.symtri(A)
    F_o, tau_o, d_o, e_o = O.symtri(A, "L")
    nA = max(np.linalg.norm(A, 2), 1.0)
    d, e = np_(f.diagonals.dv), np_(f.diagonals.ev)
    assert np.abs(d - d_o).max() <= 1e-12 * nA
    if n > 1:
        assert np.abs(e - e_o).max() <= 1e-12 * nA
        assert np.abs(np_(f.reflectors.tau)[: n - 1] - tau_o).max() <= 1e-10
        F = np_(f.reflectors.factors)
        below = np.tril(np.ones((n, n), bool), -2)
        if below.any():
            assert np.abs(F[below] - F_o[below]).max() <= 1e-10
        # symtriLower!'s layout: d on the diagonal, e below it
        assert np.array_equal(np.diag(F), d) and np.array_equal(np.diag(F, -1), e)


@pytest.mark.parametrize("n", [5, 96, 300])
def test_eigenq_identities(G, n):
    # test/eigenselfadjoint.jl:61-68: Q == lmul!(Q, I), Q ~ rmul!(I, Q), Q'Q ~ QQ' ~ I, Q'AQ ~ T
    import torch
    A = goe(n, 70 + n)
    f = G.symtri(A)
    Q = np_(f.reflectors.array())
    assert np.array_equal(Q, np_(f.reflectors.lmul(torch.eye(n, dtype=torch.float64, device="cuda"))))
    assert np.abs(Q - np_(f.reflectors.rmul(torch.eye(n, dtype=torch.float64, device="cuda")))).max() <= 1e-13
    I = np.eye(n)
    assert np.abs(Q.T @ Q - I).max() <= 1e-13 and np.abs(Q @ Q.T - I).max() <= 1e-13
    d, e = np_(f.diagonals.dv), np_(f.diagonals.ev)
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    assert np.abs(Q.T @ A @ Q - T).max() <= 1e-13 * np.linalg.norm(A, 2)
    # transposed applications and rectangular operands
    rng = np.random.default_rng(n)
    B = rng.standard_normal((n, 7))
    assert np.abs(f.reflectors.lmul(B, trans=True) - Q.T @ B).max() <= 1e-13 * np.abs(B).max() * np.sqrt(n)
    Bt = rng.standard_normal((4, n))
    assert np.abs(f.reflectors.rmul(Bt) - Bt @ Q).max() <= 1e-13 * np.abs(Bt).max() * np.sqrt(n)
    assert np.abs(f.reflectors.rmul(Bt, trans=True) - Bt @ Q.T).max() <= 1e-13 * np.abs(Bt).max() * np.sqrt(n)
    # against the oracle's lmul! with the oracle's own factors
    F_o, tau_o, _, _ = O.symtri(A, "L")
    QB_o, _ = O.eigenq_lmul("L", F_o, tau_o, B)
    assert np.abs(f.reflectors.lmul(B) - QB_o).max() <= 1e-12 * np.abs(B).max() * np.sqrt(n)


@pytest.mark.parametrize("n", [1, 2, 3, 17, 64, 200, 333])
def test_symtri_upper_matches_oracle(G, n):
    # symtriUpper! (:507-564): factors above the diagonal, e on the superdiagonal
    A = goe(n, 80 + n)
    up = np.triu(A) + np.tril(np.full((n, n), 7.0), -1)  # lower part is garbage: only the upper is read
    f = G.symtri(up, uplo="U")
    F_o, tau_o, d_o, e_o = O.symtri(A, "U")
    nA = max(np.linalg.norm(A, 2), 1.0)
    d, e = np_(f.diagonals.dv), np_(f.diagonals.ev)
    assert f.reflectors.uplo == "U"
    assert np.abs(d - d_o).max() <= 1e-12 * nA
    F = np_(f.reflectors.factors)
    assert np.array_equal(np.tril(F, -1), np.tril(up, -1))  # the lower triangle is not touched
    if n > 1:
        assert np.abs(e - e_o).max() <= 1e-12 * nA
        assert np.abs(np_(f.reflectors.tau)[: n - 1] - tau_o).max() <= 1e-10
        above = np.triu(np.ones((n, n), bool), 2)
        if above.any():
            assert np.abs(F[above] - F_o[above]).max() <= 1e-10
        assert np.array_equal(np.diag(F), d) and np.array_equal(np.diag(F, 1), e)


@pytest.mark.parametrize("n", [5, 96, 300])
def test_eigenq_upper_identities(G, n):
    # test/eigenselfadjoint.jl:61-68 with uplo = :U
    import torch
    A = goe(n, 90 + n)
    f = G.symtri(A, uplo="U")
    Q = np_(f.reflectors.array())
    assert np.array_equal(Q, np_(f.reflectors.lmul(torch.eye(n, dtype=torch.float64, device="cuda"))))
    assert np.abs(Q - np_(f.reflectors.rmul(torch.eye(n, dtype=torch.float64, device="cuda")))).max() <= 1e-13
    I = np.eye(n)
    assert np.abs(Q.T @ Q - I).max() <= 1e-13 and np.abs(Q @ Q.T - I).max() <= 1e-13
    d, e = np_(f.diagonals.dv), np_(f.diagonals.ev)
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    assert np.abs(Q.T @ A @ Q - T).max() <= 1e-13 * np.linalg.norm(A, 2)
    rng = np.random.default_rng(n)
    B = rng.standard_normal((n, 7))
    s = 1e-13 * np.sqrt(n)
    assert np.abs(f.reflectors.lmul(B) - Q @ B).max() <= s * np.abs(B).max()
    assert np.abs(f.reflectors.lmul(B, trans=True) - Q.T @ B).max() <= s * np.abs(B).max()
    Bt = rng.standard_normal((4, n))
    assert np.abs(f.reflectors.rmul(Bt) - Bt @ Q).max() <= s * np.abs(Bt).max()
    assert np.abs(f.reflectors.rmul(Bt, trans=True) - Bt @ Q.T).max() <= s * np.abs(Bt).max()
    # against the oracle's 'U' lmul!/rmul! applying the same (device) factors:
    # the application alone, free of the two factorisations' rounding
    # differences (square operands: the reference's 'U' lmul! indexes B's rows
    # by its column count)
    F, tau = np_(f.reflectors.factors), np_(f.reflectors.tau)[: n - 1]
    S = rng.standard_normal((n, n))
    QS_o, _ = O.eigenq_lmul("U", F, tau, S)
    assert np.abs(f.reflectors.lmul(S) - QS_o).max() <= s * np.abs(S).max()
    SQ_o, _ = O.eigenq_rmul("U", F, tau, S)
    assert np.abs(f.reflectors.rmul(S) - SQ_o).max() <= s * np.abs(S).max()


def test_symtri_untouched_triangle(G):
    import torch
    n = 150
    A = goe(n, 5)
    # the unreferenced triangle of the factors' storage is left as given
    X = torch.tensor(A, device="cuda")
    g = G.symtri(X)
    F = np_(g.reflectors.factors)
    assert np.array_equal(np.triu(F, 1), np.triu(A, 1))
    # eigenvalues of T equal those of A
    d, e = np_(g.diagonals.dv), np_(g.diagonals.ev)
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    assert np.abs(np.linalg.eigvalsh(T) - np.linalg.eigvalsh(A)).max() <= 1e-12 * np.linalg.norm(A, 2)


def test_host_buffer_entries(G):
    import ctypes as C
    from glagpu import _lib
    L = _lib.load()
    n = 120
    A = goe(n, 8)
    F = np.asfortranarray(A.copy())
    d, e, tau = np.empty(n), np.empty(n - 1), np.empty(n - 1)
    p = lambda a: C.c_void_p(a.ctypes.data)
    assert L.gla_dsytrd_host(b"L", n, p(F), n, p(d), p(e), p(tau)) == 0
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    Q = np.asfortranarray(np.eye(n))
    assert L.gla_dormtr_host(b"L", b"L", b"N", n, n, p(F), n, p(tau), p(Q), n) == 0
    assert np.abs(Q.T @ A @ Q - T).max() <= 1e-13 * np.linalg.norm(A, 2)
    B = np.asfortranarray(np.random.default_rng(1).standard_normal((3, n)))
    ref = B @ Q
    assert L.gla_dormtr_host(b"R", b"L", b"N", 3, n, p(F), n, p(tau), p(B), 3) == 0
    assert np.abs(B - ref).max() <= 1e-13 * np.sqrt(n) * 4
    assert L.gla_dormtr_host(b"X", b"L", b"N", 3, n, p(F), n, p(tau), p(B), 3) == -1
    assert L.gla_dormtr_host(b"R", b"X", b"N", 3, n, p(F), n, p(tau), p(B), 3) == -2
    assert L.gla_dormtr_host(b"R", b"L", b"X", 3, n, p(F), n, p(tau), p(B), 3) == -3
    # the upper layout through the host entries
    Fu = np.asfortranarray(A.copy())
    assert L.gla_dsytrd_host(b"U", n, p(Fu), n, p(d), p(e), p(tau)) == 0
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    Q = np.asfortranarray(np.eye(n))
    assert L.gla_dormtr_host(b"L", b"U", b"N", n, n, p(Fu), n, p(tau), p(Q), n) == 0
    assert np.abs(Q.T @ A @ Q - T).max() <= 1e-13 * np.linalg.norm(A, 2)
    Qt = np.asfortranarray(np.eye(n))
    assert L.gla_dormtr_host(b"R", b"U", b"T", n, n, p(Fu), n, p(tau), p(Qt), n) == 0
    assert np.abs(Qt - Q.T).max() <= 1e-13 * np.sqrt(n)
