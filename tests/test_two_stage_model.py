"""The CPU model of the two-stage reduction (tests/two_stage_model.py): the
band and tridiagonal it produces, the eigenvalues they keep (against the
oracle's eigen! of the dense matrix), the back-transform X = Q1 Q2 Z, and
the critical path of its bulge-chasing tasks.

Tolerances (FP64, backward-stable reductions): entries outside the band or
the tridiagonal <= 1e-13 ||A||, eigenvalues within 1e-12 ||A|| of the
oracle, ||AX - X diag(w)|| / ||A|| <= 1e-13 and ||X'X - I|| <= 1e-12."""
import numpy as np
import pytest

from helpers import goe, orth, residual
from oracle import oracle as O
import two_stage_model as M

CASES = [(40, 4), (97, 8), (130, 16), (200, 32), (129, 64)]


def outside(B, w):
    n = B.shape[0]
    i, j = np.indices((n, n))
    return np.abs(B[np.abs(i - j) > w]).max(initial=0.0)


@pytest.mark.parametrize("n,b", CASES)
def test_band_tridiagonal_and_back_transform(n, b):
    A = goe(n, 900 + n)
    nA = np.linalg.norm(A, 2)
    B, panels = M.sy2sb(A, b)
    assert outside(B, b) <= 1e-13 * nA
    assert np.array_equal(B, B.T)
    T, refl = M.sb2st(B, b)
    assert outside(T, 1) <= 1e-13 * nA
    d, e = np.diag(T).copy(), np.diag(T, -1).copy()
    wo = O.syev(A, "N")[0]
    Tt = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    w, Z = np.linalg.eigh(Tt)
    assert np.abs(w - wo).max() <= 1e-12 * nA
    X = M.q1_apply(panels, M.q2_apply(refl, Z))
    assert residual(A, X, w) <= 1e-13
    assert orth(X) <= 1e-12
    # one reflector per task, n^2 / (2 b) of them to first order
    assert len(refl) == sum(1 for _ in M.sb2st_tasks(n, b))


@pytest.mark.parametrize("n,b,nb", [(97, 8, 8), (130, 16, 5), (200, 32, 32), (129, 64, 16)])
def test_blocked_q2_matches_reflector_order(n, b, nb):
    # the compact-WY grouping of the bulge-chase reflectors gives Q2 Z as
    # the reflectors applied one by one in program order (applying a sweep
    # block's groups with t descending instead is off by O(1))
    A = goe(n, 950 + n)
    B, _ = M.sy2sb(A, b)
    _, refl = M.sb2st(B, b)
    Z = np.linalg.qr(np.random.default_rng(n).standard_normal((n, n)))[0]
    X1 = M.q2_apply(refl, Z)
    X2 = M.q2_apply_blocked(refl, Z, b, nb)
    assert np.abs(X1 - X2).max() <= 1e-13


def test_graded_and_already_banded_input():
    # rows scaled over six orders of magnitude, and a matrix that is already
    # tridiagonal (every reflector is the identity: tau = 0)
    A = goe(64, 5)
    D = np.diag(np.logspace(-6, 0, 64))
    for M0 in (D @ A @ D, np.diag(np.arange(1.0, 65.0)) + np.diag(np.ones(63), 1) + np.diag(np.ones(63), -1)):
        nA = np.linalg.norm(M0, 2)
        B, panels = M.sy2sb(M0, 8)
        T, refl = M.sb2st(B, 8)
        w = np.linalg.eigvalsh(np.diag(np.diag(T)) + np.diag(np.diag(T, -1), 1) + np.diag(np.diag(T, -1), -1))
        assert np.abs(w - O.syev(M0, "N")[0]).max() <= 1e-12 * nA


def test_bulge_chase_critical_path():
    # about 3 n unit tasks whatever the band width (2.98 n at n = 4096,
    # b = 32): sweep j + 1 trails sweep j by about three tasks
    for n, b in ((256, 16), (512, 32), (512, 64)):
        tasks, cp, widest = M.critical_path(n, b)
        assert tasks == sum(1 for _ in M.sb2st_tasks(n, b))
        assert 2.6 * n <= cp <= 3.0 * n, (n, b, cp)
        assert widest <= n // b
