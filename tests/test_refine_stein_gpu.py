"""FP32 + refinement, orders <= 128: the FP32 stage's per-eigenvalue solver
(bisection on Sturm counts and one twisted factorisation per eigenvector,
inside the tridiagonalisation kernel) against the CPU oracle, its hand-off
of hard matrices (splits, multiplicities, eigenvalues within 1e-6 ||T|| of
each other) to the QL chase inside the same batch, and agreement with the
QL-chase variant (GLA_FLAG_REFINE_QL).

Tolerance (refined results): eigenvalues within 1e-13 ||A|| of the oracle,
residual ||AV - VW||/||A|| and ||V'V - I|| <= 1e-13."""
import numpy as np
import pytest

from helpers import goe, orth, prescribed, residual
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import glagpu
    return glagpu


def solve(G, mats, **kw):
    plan = G.Plan([m.shape[0] for m in mats], precision="f32_refined", **kw)
    w = np.empty(max(plan.w_elems, 1))
    V = np.empty(max(plan.a_elems, 1))
    info = np.zeros(len(mats), dtype=np.int32)
    plan.execute_host(plan.pack(mats), w, V, info)
    ws, Vs = plan.unpack(w, V)
    st = plan.stats()
    plan.close()
    return ws, Vs, info, st


def check(A, w, V, wo=None):
    # the oracle's eigen! (QL with vectors): its values-only eigvals! (the
    # root-free PWK iteration of the reference) loses ~1e-9 on Wilkinson pairs
    if wo is None:
        wo = O.syev(A, "V")[0]
    nA = max(np.linalg.norm(A, 2), 1e-300)
    assert np.all(np.diff(w) >= 0)
    assert np.abs(w - wo).max() <= 1e-13 * nA
    assert residual(A, V, w) <= 1e-13
    assert orth(V) <= 1e-13


def wilkinson(n):
    m = (n - 1) // 2
    return np.diag(np.abs(np.arange(-m, m + 1)).astype(float)) + np.diag(np.ones(n - 1), 1) + np.diag(np.ones(n - 1), -1)


def hard_matrices():
    rng = np.random.default_rng(41)
    out = [np.eye(7), np.zeros((5, 5)), np.diag([3.0, 1.0, 3.0, 2.0, 1.0, 3.0]), wilkinson(21), wilkinson(101)]
    B = goe(20, 5)
    out.append(np.kron(np.eye(3), B))  # three identical blocks: triple eigenvalues
    lam = np.repeat(rng.standard_normal(16), 4)  # multiplicity 4, dense (no split after reduction)
    out.append(prescribed(lam, 44))
    lam = np.sort(rng.standard_normal(90))
    lam[40:50] = lam[40] + 1e-9 * np.arange(10)  # a tight cluster of ten
    out.append(prescribed(lam, 45))
    return out


def test_goe_batch_solved_without_the_chase(G):
    rng = np.random.default_rng(40)
    sizes = list(rng.integers(1, 129, size=120)) + [1, 2, 3, 31, 32, 33, 64, 127, 128]
    mats = [goe(int(n), 7000 + i) for i, n in enumerate(sizes)]
    ws, Vs, info, st = solve(G, mats)
    assert (info == 0).all()
    for A, w, V in zip(mats, ws, Vs):
        check(A, w, V)
    # GOE spectra have no eigenvalues within 1e-6 ||T|| here: no matrix went
    # to the QL chase, which is what counts rotations
    assert st["rotations"] == 0


def test_hard_matrices_take_the_chase_and_stay_accurate(G):
    hard = hard_matrices()
    easy = [goe(n, 7100 + n) for n in (17, 64, 128)]
    mats = easy[:1] + hard + easy[1:]  # mixed in one plan: the chase works on the hard ones only
    ws, Vs, info, st = solve(G, mats)
    assert (info == 0).all(), info
    for A, w, V in zip(mats, ws, Vs):
        check(A, w, V)
    assert st["rotations"] > 0


def test_matches_the_ql_chase_variant(G):
    rng = np.random.default_rng(42)
    sizes = list(rng.integers(2, 129, size=40))
    mats = [goe(int(n), 7200 + i) for i, n in enumerate(sizes)] + hard_matrices()
    ws1, Vs1, info1, _ = solve(G, mats)
    ws2, Vs2, info2, st2 = solve(G, mats, refine_ql=True)
    assert (info1 == 0).all() and (info2 == 0).all()
    assert st2["rotations"] > 0
    for A, w1, V1, w2, V2 in zip(mats, ws1, Vs1, ws2, Vs2):
        nA = max(np.linalg.norm(A, 2), 1e-300)
        assert np.abs(w1 - w2).max() <= 2e-13 * nA
        check(A, w1, V1)
        check(A, w2, V2)


def test_prescribed_gapped_and_scaled(G):
    # spectra the differentiation workload uses (gaps >= 1e-3, on [-1, 1]),
    # and GOE matrices scaled by 2^+-300 (the FP32 stage sees them rescaled)
    from helpers import gapped_spectrum
    rng = np.random.default_rng(43)
    mats, lams = [], []
    for n in (32, 57, 96):
        lam = gapped_spectrum(n, rng)
        mats.append(prescribed(lam, 50 + n))
        lams.append(np.sort(lam))
    for s in (2.0 ** 300, 2.0 ** -300):
        mats.append(goe(48, 77) * s)
        lams.append(None)
    ws, Vs, info, _ = solve(G, mats)
    assert (info == 0).all()
    for A, lam, w, V in zip(mats, lams, ws, Vs):
        check(A, w, V, wo=lam)


def test_f32_plans_with_the_bisection_flag(G):
    # GLA_FLAG_F32_BISECT on plain FP32 plans (the refined path's internal FP32
    # solves): eigenvalues as accurate as the QL chase's (8 n eps32 ||A||),
    # residual <= 32 n eps32, orthogonality <= 1e-3 (pairs just outside the
    # Gram-Schmidt bound of 1e-3 ||T|| are orthogonal to eps32 ||T|| / gap,
    # about 1e-4; the refinement absorbs it); hard matrices go to the chase
    eps32 = 2.0 ** -23
    rng = np.random.default_rng(44)
    sizes = list(rng.integers(1, 129, size=60))
    mats = [goe(int(n), 7300 + i) for i, n in enumerate(sizes)] + hard_matrices()
    plan = G.Plan([m.shape[0] for m in mats], precision="f32", bisect=True)
    w = np.empty(max(plan.w_elems, 1), np.float32)
    V = np.empty(max(plan.a_elems, 1), np.float32)
    info = np.zeros(len(mats), dtype=np.int32)
    plan.execute_host(plan.pack(mats), w, V, info)
    ws, Vs = plan.unpack(w, V)
    st = plan.stats()
    plan.close()
    assert (info == 0).all()
    assert st["rotations"] > 0  # the hard matrices
    for A, wg, Vg in zip(mats, ws, Vs):
        n = A.shape[0]
        A32 = A.astype(np.float32).astype(np.float64)
        wo = O.syev(A32, "V")[0]
        nA = max(np.linalg.norm(A32, 2), 1e-30)
        wg = wg.astype(np.float64)
        Vg = Vg.astype(np.float64)
        assert np.all(np.diff(wg) >= 0)
        assert np.abs(wg - wo).max() <= 8 * n * eps32 * nA
        assert residual(A32, Vg, wg) <= 32 * n * eps32
        assert orth(Vg) <= 1e-3
