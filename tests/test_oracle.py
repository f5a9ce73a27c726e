"""CPU oracle pinned against the reference's own known answers
(GenericLinearAlgebra.jl test/eigenselfadjoint.jl), LAPACK and the 256-bit
restatement. No GPU."""
import mpmath
import numpy as np
import pytest
import scipy.linalg as sl

from helpers import from_hex, goe, golden, orth, prescribed, residual, signfix, sym_from, vec_parity
from oracle import oracle as O


def test_one_by_one():
    # test/eigenselfadjoint.jl:100-105
    w, _ = O.stev([1.0], [], "N")[:2]
    assert list(w) == [1.0]
    w, V, info = O.stev([1.0], [], "V")
    assert list(w) == [1.0] and V.tolist() == [[1.0]] and info == 0
    w, V, info = O.syev(np.array([[1.0]]))
    assert list(w) == [1.0] and V.tolist() == [[1.0]]


@pytest.mark.parametrize("pos", [0, 2])
def test_issue52_zero_diagonal(pos):
    # test/eigenselfadjoint.jl:108-117: exact equality with LAPACK eigvals
    M = np.zeros((3, 3))
    M[pos, pos] = 0.01
    lap = sl.eigh(M, eigvals_only=True)
    for jobz in "NV":
        w = O.syev(M, jobz)[0]
        assert np.array_equal(w, lap), (jobz, w, lap)


def test_issue139_diagonal():
    # test/eigenselfadjoint.jl:164-170
    A = np.diag([1.0, 2.0])
    assert O.syev(A, "N")[0].tolist() == [1.0, 2.0]
    assert O.syev(A, "V")[0].tolist() == [1.0, 2.0]


def test_issue123_against_256bit():
    # test/eigenselfadjoint.jl:125-133 (matrix read from the test file)
    g = golden()["issue123"]
    M = np.array([[float(v) for v in row] for row in g["A"]])
    w, V, info = O.syev(M)
    assert info == 0
    assert residual(M, V, w) < 1e-14
    w256 = np.array([float(mpmath.mpf(v)) for v in g["w"]])
    assert np.abs(w - w256).max() <= 1e-14 * np.linalg.norm(M, 2)


def test_eig2x2_table():
    # test/eigenselfadjoint.jl:135-149: hypot(c, s) ≈ 1 for every case
    for case in golden()["eig2x2_cases"]:
        d, e, V, c, s = O.eig2x2(case["d"], case["e"])
        assert np.isclose(np.hypot(c, s), 1.0, rtol=np.sqrt(2.2e-16)), case
        assert e[0] == 0.0


def test_generic_givens():
    # test/eigenselfadjoint.jl:93-98
    rng = np.random.default_rng(3)
    for _ in range(20):
        x, y = rng.standard_normal(2)
        for generic in (True, False):
            c, s, r = O.givens(x, y, generic)
            assert np.isclose(c * x + s * y, r, rtol=1e-14)
            assert np.isclose(c * y, s * x, rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_prescribed_spectrum(uplo):
    # test/eigenselfadjoint.jl:54-84 (real version): vals ≈ λ with rtol = 1e-13 n
    n = 50
    lam = 10.0 ** np.linspace(-8, 0, n)
    A = prescribed(lam, 7)
    w, V, info = O.syev(A, "V", uplo)
    assert info == 0
    assert np.linalg.norm(w - lam) <= 1e-13 * n * max(np.linalg.norm(w), np.linalg.norm(lam))
    assert residual(A, V, w) < 1e-13
    assert orth(V) < 1e-13
    wn = O.syev(A, "N", uplo)[0]
    assert np.linalg.norm(wn - w) <= np.sqrt(2.2e-16) * np.linalg.norm(w)


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_symtri_and_eigenq(uplo):
    # test/eigenselfadjoint.jl:61-68: Q == lmul!(Q, I), Q ≈ rmul!(I, Q), Q'Q ≈ I, Q'AQ ≈ T
    n = 12
    A = goe(n, 21)
    F, tau, d, e = O.symtri(A, uplo)
    Q, F1 = O.eigenq_lmul(uplo, F, tau, np.eye(n))
    Q2, _ = O.eigenq_lmul(uplo, F, tau, np.eye(n))
    assert np.array_equal(Q, Q2)
    Q3, _ = O.eigenq_rmul(uplo, F, tau, np.eye(n))
    assert np.allclose(Q, Q3, atol=1e-14)
    assert np.allclose(Q.T @ Q, np.eye(n), atol=1e-14)
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    assert np.allclose(Q.T @ sym_from(A, uplo) @ Q, T, atol=1e-13)


@pytest.mark.parametrize("n,seed", [(3, 11), (5, 12), (8, 13), (16, 14), (24, 15)])
def test_goe_against_256bit(n, seed):
    g = [c for c in golden()["goe"] if c["n"] == n][0]
    A = from_hex(g["A"])
    w256 = np.array([float(mpmath.mpf(v)) for v in g["w"]])
    V256 = np.array(g["V"])
    nA = np.linalg.norm(A, 2)
    for uplo in "LU":
        w, V, info = O.syev(A, "V", uplo)
        assert info == 0
        assert np.abs(w - w256).max() <= 4 * n * 2.2e-16 * nA
        assert vec_parity(A, V, V256, w256) <= 1.0
    # the binary128 run of the same algorithm agrees with the 256-bit one
    whi, wlo, Vhi, Vlo, info = O.syev_quad(A)
    for i in range(n):
        assert abs(mpmath.mpf(whi[i]) + mpmath.mpf(wlo[i]) - mpmath.mpf(g["w"][i])) <= 1e-30 * nA


@pytest.mark.parametrize("n", [64, 128])
def test_goe_large_against_256bit(n):
    # the single-matrix workload (GOE n = 64, seed 1) and a GOE n = 128, at the
    # orders of the reference's own BigFloat testsets (test/eigenselfadjoint.jl:5-52)
    from helpers import golden_large
    A, w256, V256, seed = golden_large(n)
    assert np.array_equal(A, goe(n, seed))  # the fixture holds the seeded input bit for bit
    nA = np.linalg.norm(A, 2)
    for uplo in "LU":
        w, V, info = O.syev(A, "V", uplo)
        assert info == 0
        assert np.abs(w - w256).max() <= 4 * n * 2.2e-16 * nA
        assert vec_parity(A, V, V256, w256) <= 1.0
    # the 256-bit eigenpairs themselves: residual and orthogonality at float64 rounding
    assert residual(A, V256, w256) <= 4 * 2.2e-16 * n and orth(V256) <= 4 * 2.2e-16 * n


def test_against_lapack():
    rng = np.random.default_rng(9)
    for n in [2, 3, 7, 31, 64, 100, 128]:
        A = goe(n, int(rng.integers(1 << 30)))
        ws = sl.eigh(A, eigvals_only=True)
        for use_qr in (False, True):
            w, V, info = O.syev(A, "V", use_qr=use_qr)
            assert info == 0
            assert np.abs(w - ws).max() <= 4 * n * 2.2e-16 * np.linalg.norm(A, 2)
            assert residual(A, V, w) < 1e-13 and orth(V) < 1e-13


def test_symtridiagonal_against_256bit():
    # test/eigenselfadjoint.jl:5-32 (SymTridiagonal, QL default and QR version)
    g = golden()["symtridiagonal"]
    dv = np.array([float.fromhex(v) for v in g["dv"]])
    ev = np.array([float.fromhex(v) for v in g["ev"]])
    T = np.diag(dv) + np.diag(ev, 1) + np.diag(ev, -1)
    w256 = np.array([float(mpmath.mpf(v)) for v in g["w"]])
    nT = np.linalg.norm(T, 2)
    for use_qr in (False, True):
        w, V, info = O.stev(dv, ev, "V", use_qr=use_qr)
        assert info == 0 and np.all(np.diff(w) >= 0)
        assert np.abs(w - w256).max() <= 200 * 2.2e-16 * nT
        assert residual(T, V, w) < 1e-13 and orth(V) < 1e-13
        assert vec_parity(T, V, np.array(g["V"]), w256) <= 1.0
    wp = O.stev(dv, ev, "N")[0]
    wp256 = np.array([float(mpmath.mpf(v)) for v in g["w_pwk"]])
    assert np.abs(wp - wp256).max() <= 200 * 2.2e-16 * nT
    assert np.abs(wp - w).max() <= np.sqrt(2.2e-16) * nT


def test_eigen2_rows_equal_full_vectors():
    # test/eigenselfadjoint.jl:18-24: eigen2 rows == vecs[[1, n], :] exactly
    g = golden()["symtridiagonal"]
    dv = np.array([float.fromhex(v) for v in g["dv"]])
    ev = np.array([float.fromhex(v) for v in g["ev"]])
    n = len(dv)
    d1, _, Vf, _ = O.eigql(dv, ev, np.eye(n))
    V2 = np.zeros((2, n))
    V2[0, 0] = 1
    V2[1, n - 1] = 1
    d2, _, Vp, _ = O.eigql(dv, ev, V2)
    assert np.array_equal(d1, d2)
    assert np.array_equal(Vf[[0, n - 1], :], Vp)


def test_nonfinite_and_cap():
    A = goe(6, 1)
    A[3, 1] = np.nan
    assert O.syev(A)[2] == -1
    A[3, 1] = np.inf
    assert O.syev(A, "N")[2] == -1
    # the reference has no sweep cap; the oracle's cap reports the unconverged count
    B = goe(20, 2)
    w, V, info = O.syev(B, max_sweeps=0)
    assert info > 0


def test_batched_matches_single():
    mats = [goe(n, 100 + n) for n in [1, 2, 5, 17, 64]]
    ws, Vs, info = O.syev_batched(mats)
    for A, w, V in zip(mats, ws, Vs):
        w1, V1, _ = O.syev(A)
        assert np.array_equal(w, w1) and np.array_equal(V, V1)
    assert (info == 0).all()


def test_numnegevals_reference_case():
    # test/tridiag.jl:3-7: numnegevals(T) == count(x -> x < 0, eigvals(T)), n = 20
    for seed in range(5):
        rng = np.random.default_rng(seed)
        d, e = rng.standard_normal(20), rng.standard_normal(19)
        T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
        w = np.linalg.eigvalsh(T)
        assert O.numnegevals(d, e) == int((w < 0).sum())
        # shifted counts match the sorted spectrum away from the eigenvalues
        mids = (w[:-1] + w[1:]) / 2
        assert list(O.numnegevals(d, e, mids)) == list(range(1, 20))


def test_numnegevals_zero_pivot_rule():
    # a zero pivot is replaced by eps (b_k + eps) (src/tridiag.jl:29-32):
    # T = [[0, 1], [1, 0]] at sigma = 0 has delta_1 = 0
    d, e = np.array([0.0, 0.0]), np.array([1.0])
    assert O.numnegevals(d, e, 0.0) == 1  # eigenvalues -1, 1


def herm(n, seed):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    return (B + B.conj().T) / 2


@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("n", [1, 2, 4, 17, 50])
def test_complex_hermitian_against_lapack(n, uplo):
    # the T <: Complex path (n-1 reflectors, :462/:522), pinned as the
    # reference's own test pins it (test/eigenselfadjoint.jl:86-91, against
    # stdlib LAPACK): values within 4 n eps ||A|| of zheevd, and the
    # default testset's properties (residual, orthogonality)
    A = herm(n, 300 + n)
    junk = np.full((n, n), 5 - 5j)
    S = np.where(np.tril(np.ones((n, n), bool)) if uplo == "L" else np.triu(np.ones((n, n), bool)), A, junk)
    w, V, info = O.heev(S, "V", uplo)
    assert info == 0 and np.all(np.diff(w) >= 0)
    nA = max(np.linalg.norm(A, 2), 1e-300)
    eps = 2.0 ** -52
    assert np.abs(w - sl.eigh(A, eigvals_only=True)).max() <= 4 * n * eps * nA
    assert np.linalg.norm(A @ V - V * w, 2) / nA <= 1e-13
    assert np.linalg.norm(V.conj().T @ V - np.eye(n), 2) <= 1e-13
    wn, _, info = O.heev(S, "N", uplo)
    assert info == 0 and np.abs(wn - w).max() <= 4 * n * eps * nA


def test_complex_reference_known_answers():
    # test/eigenselfadjoint.jl:171-176: Hermitian(Tridiagonal(ones(ComplexF64, .)))
    M = np.diag(np.ones(3, complex)) + np.diag(np.ones(2, complex), 1) + np.diag(np.ones(2, complex), -1)
    w, V, info = O.heev(M)
    assert info == 0
    assert np.abs(w - np.array([1 - np.sqrt(2), 1.0, 1 + np.sqrt(2)])).max() <= 4e-16 * 4
    # the complex factorisation leaves a real tridiagonal with Q' A Q = T
    A = herm(30, 9)
    F, tau, d, e = O.symtri_complex(A, "L")
    assert len(tau) == 29  # one more reflector than for real input
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    assert np.abs(np.linalg.eigvalsh(T) - np.linalg.eigvalsh(A)).max() <= 1e-13 * np.linalg.norm(A, 2)


def test_complex_path_on_real_input():
    # a real symmetric matrix through the complex path: the values agree with
    # the real path's to rounding (the real loop stops one reflector earlier)
    A = goe(40, 4)
    wr, _, _ = O.syev(A)
    wz, Vz, info = O.heev(A.astype(complex))
    assert info == 0
    assert np.abs(wz - wr).max() <= 8 * 40 * 2.0 ** -52 * np.linalg.norm(A, 2)
    assert np.linalg.norm(A @ Vz - Vz * wz, 2) / np.linalg.norm(A, 2) <= 1e-13


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_quaternion_hermitian_reference_testset(uplo):
    # test/eigenselfadjoint.jl:54-84, n = 50: Hermitian(V diag(lambda) V', uplo)
    # with V a random unitary quaternion matrix and lambda = 10 .^ range(-8, 0, n)
    from helpers import qeye, qH, qherm_spectrum, qmul, qnorm
    n = 50
    lam = 10.0 ** np.linspace(-8, 0, n)
    A = qherm_spectrum(lam, np.random.default_rng(54))
    vals, vecs, info = O.heev_quaternion(A, "V", uplo)
    assert info == 0 and np.all(np.diff(vals) >= 0)
    # symtri!: Q == lmul!(Q, I), Q'Q ~ QQ' ~ I, Q' A Q ~ T (:61-68)
    F, tau, d, e = O.symtri_quaternion(A, uplo)
    Q = O.eigenq_lmul_quaternion(uplo, F, tau, qeye(n))
    assert qnorm(qmul(qH(Q), Q) - qeye(n)) <= 1e-13 and qnorm(qmul(Q, qH(Q)) - qeye(n)) <= 1e-13
    T = np.zeros((n, n, 4))
    T[..., 0] = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    assert qnorm(qmul(qmul(qH(Q), A), Q) - T) <= 1e-13
    # default: A vecs ~ vecs diag(vals), eigvals(A) ~ vals, vals ~ lambda at rtol 1e-13 n, vecs'vecs ~ I
    assert qnorm(qmul(A, vecs) - vecs * vals[None, :, None]) <= 1e-13
    wn, _, info = O.heev_quaternion(A, "N", uplo)
    assert info == 0 and np.linalg.norm(wn - vals) <= 1e-13 * np.linalg.norm(vals)
    assert np.linalg.norm(vals - lam) <= 1e-13 * n * max(np.linalg.norm(vals), np.linalg.norm(lam))
    assert qnorm(qmul(qH(vecs), vecs) - qeye(n)) <= 1e-13


def test_quaternion_path_on_complex_input():
    # a complex Hermitian matrix as a quaternion one (j, k parts zero): the
    # quaternion path's values equal the complex path's to rounding
    A = herm(30, 12)
    Aq = np.zeros((30, 30, 4))
    Aq[..., 0], Aq[..., 1] = A.real, A.imag
    wq, Vq, info = O.heev_quaternion(Aq)
    wz, _, _ = O.heev(A)
    assert info == 0
    assert np.abs(wq - wz).max() <= 8 * 30 * 2.0 ** -52 * np.linalg.norm(A, 2)
