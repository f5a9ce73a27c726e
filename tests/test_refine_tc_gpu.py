"""FP32 + refinement, orders <= 128: the refinement's double-float products
on the tcgen05 tensor cores (the default; seven bf16 slices per operand,
exact integer accumulation in TMEM) against the CPU oracle, and against the
same refinement with its products on the FP32 pipe (GLA_FLAG_REFINE_SIMT),
in the persistent kernel, in the bucketed kernels (GLA_FLAG_REFINE_QL) and
in the hand-off of hard matrices to the QL chase.

Tolerance: eigenvalues within 1e-13 ||A|| of the oracle, residual
||AV - VW||/||A|| and ||V'V - I|| <= 1e-13; the two product paths agree on
eigenvalues within 2e-13 ||A|| and on eigenvectors within
1e-12 ||A|| / gap per column (signs normalised)."""
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
    plan.close()
    return ws, Vs, info


def check(A, w, V):
    wo = O.syev(A, "V")[0]
    nA = max(np.linalg.norm(A, 2), 1e-300)
    assert np.all(np.diff(w) >= 0)
    assert np.abs(w - wo).max() <= 1e-13 * nA
    assert residual(A, V, w) <= 1e-13
    assert orth(V) <= 1e-13


def agree(A, w1, V1, w2, V2):
    nA = max(np.linalg.norm(A, 2), 1e-300)
    n = len(w1)
    assert np.abs(w1 - w2).max() <= 2e-13 * nA
    for j in range(n):
        gap = np.abs(np.delete(w1, j) - w1[j]).min() if n > 1 else np.inf
        if gap <= 1e-6 * nA:
            continue
        a, b = V1[:, j], V2[:, j]
        s = 1.0 if a @ b >= 0 else -1.0
        assert np.abs(a - s * b).max() <= max(1e-12 * nA / gap, 1e-14), (j, gap)


def mixed(seed):
    rng = np.random.default_rng(seed)
    mats = [goe(int(n), seed + i) for i, n in enumerate(rng.integers(1, 129, size=96))]
    mats += [goe(n, seed + 500 + n) for n in (1, 2, 3, 31, 32, 33, 63, 64, 65, 96, 127, 128)]
    lam = np.logspace(-8, 0, 100) * rng.choice([-1.0, 1.0], 100)
    mats.append(prescribed(lam, seed + 7))  # cond 1e8
    mats.append(prescribed(np.repeat([-1.0, 0.5, 2.0], 40), seed + 8))  # multiplicities
    return mats


@pytest.mark.parametrize("refine_ql", [False, True])
def test_tc_products_vs_oracle_and_simt(G, refine_ql):
    # persistent kernel (default) and bucketed kernels (refine_ql), tensor-core
    # products against the oracle and against the FP32-pipe products
    mats = mixed(900 + int(refine_ql))
    w1, V1, i1 = solve(G, mats, refine_ql=refine_ql)
    w2, V2, i2 = solve(G, mats, refine_ql=refine_ql, refine_simt=True)
    assert (i1 == 0).all() and (i2 == 0).all()
    for A, a, b, c, d in zip(mats, w1, V1, w2, V2):
        check(A, a, b)
        agree(A, a, b, c, d)


def test_tc_products_scaled_and_graded(G):
    # power-of-two and non-power-of-two scalings, a graded matrix (row scales
    # spanning 1e-6 .. 1) and a zero row: the slicing scales per row and
    # column of each operand
    rng = np.random.default_rng(77)
    base = goe(48, 77)
    D = np.diag(np.logspace(-3, 0, 48))
    graded = D @ base @ D
    Z = goe(40, 78)
    Z[5, :] = 0.0
    Z[:, 5] = 0.0
    mats = [base * 2.0 ** 40, base * 3.7e-30, graded, Z, rng.standard_normal((1, 1))]
    w, V, info = solve(G, mats)
    assert (info == 0).all()
    for A, a, b in zip(mats, w, V):
        check(A, a, b)


def test_tc_products_repeatable(G):
    # same input, same bits (the MMA accumulation of exact integers is order-free)
    mats = mixed(950)[:40]
    w1, V1, _ = solve(G, mats)
    w2, V2, _ = solve(G, mats)
    for a, b, c, d in zip(w1, V1, w2, V2):
        assert np.array_equal(a, c) and np.array_equal(b, d)
