"""Large-order path (n > 128: blocked tridiagonalisation, divide and conquer,
compact-WY back-transformation) against the CPU oracle (the reference's QL
algorithm restated) and LAPACK (numpy), on GOE, prescribed-spectrum,
clustered (deflation-heavy) and diagonal inputs, in FP64 and FP32."""
import numpy as np
import pytest

from helpers import goe, orth, prescribed, residual, sym_from
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import glagpu
    return glagpu


def solve(G, mats, precision="f64", uplo="L", jobz="V"):
    import torch
    plan = G.Plan([m.shape[0] for m in mats], precision=precision, jobz=jobz, uplo=uplo)
    dt = torch.float32 if precision == "f32" else torch.float64
    A = plan.pack(mats, device="cuda").to(dt)
    w = torch.empty(plan.w_elems, dtype=dt, device="cuda")
    V = torch.empty(plan.a_elems, dtype=dt, device="cuda") if jobz == "V" else None
    info = torch.zeros(len(mats), dtype=torch.int32, device="cuda")
    plan.execute(A, w, V, info)
    torch.cuda.synchronize()
    ws, Vs = plan.unpack(w.cpu().numpy().astype(np.float64), V.cpu().numpy().astype(np.float64) if V is not None else None)
    return ws, Vs, info.cpu().numpy()


@pytest.mark.parametrize("n", [129, 200, 257, 300])
def test_f64_goe_vs_oracle(G, n):
    A = goe(n, 1000 + n)
    ws, Vs, info = solve(G, [A])
    assert info[0] == 0
    wo, Vo, _ = O.syev(A)
    nA = np.linalg.norm(A, 2)
    assert np.max(np.abs(ws[0] - wo)) <= 1e-13 * nA
    assert residual(A, Vs[0], ws[0]) <= 1e-13
    assert orth(Vs[0]) <= 1e-13
    # eigenvectors equal the oracle's up to sign (the spectrum is simple)
    dots = np.abs(np.sum(Vs[0] * Vo, axis=0))
    gaps = np.minimum(np.diff(wo, prepend=-np.inf), np.diff(wo, append=np.inf))
    ok = gaps > 1e-8 * nA
    assert np.all(np.abs(dots[ok] - 1) <= 1e-6)


def test_f64_goe_vs_oracle_n640(G):
    # the oracle (the reference's QL restated) at the largest order it solves
    # in a few seconds
    n = 640
    A = goe(n, 1000 + n)
    ws, Vs, info = solve(G, [A])
    assert info[0] == 0
    wo, _, _ = O.syev(A)
    nA = np.linalg.norm(A, 2)
    assert np.max(np.abs(ws[0] - wo)) <= 1e-13 * nA
    assert residual(A, Vs[0], ws[0]) <= 1e-13
    assert orth(Vs[0]) <= 1e-13


def c3_case(n):
    """The precision workload at order n: A = Q diag(lam) Q', Q Haar (seed 3),
    lam = +-logspace(-6, 0, n) with random signs (cond 1e6)."""
    rng = np.random.default_rng(3)
    lam = np.logspace(-6, 0, n) * rng.choice([-1.0, 1.0], n)
    return prescribed(lam, 3), np.sort(lam)


@pytest.mark.parametrize("precision", ["f64", "f32_refined"])
def test_c3_n2048(G, precision):
    # single n = 2048 of the precision workload, plain FP64 and FP32 + refinement:
    # eigenvalues against the exact spectrum and against LAPACK, residual and
    # orthogonality, all <= 1e-13 (relative to ||A|| = max |lam| = 1)
    n = 2048
    A, lam = c3_case(n)
    ws, Vs, info = solve(G, [A], precision=precision)
    assert info[0] == 0
    w, V = ws[0], Vs[0]
    assert np.max(np.abs(w - lam)) <= 1e-13
    assert np.max(np.abs(w - np.linalg.eigvalsh(A))) <= 1e-13
    assert residual(A, V, w) <= 1e-13
    assert orth(V) <= 1e-13


@pytest.mark.parametrize("n", [513, 1024])
def test_f64_goe_vs_lapack(G, n):
    A = goe(n, 2000 + n)
    ws, Vs, info = solve(G, [A])
    assert info[0] == 0
    wl = np.linalg.eigvalsh(A)
    nA = np.linalg.norm(A, 2)
    assert np.max(np.abs(ws[0] - wl)) <= 1e-13 * nA
    assert residual(A, Vs[0], ws[0]) <= 2e-13
    assert orth(Vs[0]) <= 2e-13


def test_f64_prescribed_cond1e6(G):
    n = 512
    rng = np.random.default_rng(3)
    lam = np.logspace(-6, 0, n) * rng.choice([-1.0, 1.0], n)
    A = prescribed(lam, 7)
    ws, Vs, info = solve(G, [A])
    assert info[0] == 0
    assert np.max(np.abs(ws[0] - np.sort(lam))) <= 1e-13
    assert residual(A, Vs[0], ws[0]) <= 1e-13
    assert orth(Vs[0]) <= 1e-13


def test_f64_clustered_deflation(G):
    # multiplicities and near-multiplicities: exercises both deflation kinds
    n = 300
    rng = np.random.default_rng(5)
    lam = np.concatenate([np.full(100, 1.0), np.full(80, -2.0), 1.0 + 1e-13 * rng.standard_normal(20),
                          rng.uniform(-3, 3, n - 200)])
    A = prescribed(lam, 9)
    ws, Vs, info = solve(G, [A])
    assert info[0] == 0
    assert np.max(np.abs(ws[0] - np.sort(lam))) <= 1e-13 * 3
    assert residual(A, Vs[0], ws[0]) <= 1e-13
    assert orth(Vs[0]) <= 1e-13


def test_f64_diagonal_and_split_tridiagonal(G):
    n = 200
    D = np.diag(np.linspace(-1, 1, n)[np.random.default_rng(1).permutation(n)])
    ws, Vs, info = solve(G, [D])
    assert info[0] == 0
    assert np.array_equal(ws[0], np.sort(np.diag(D)))
    assert residual(D, Vs[0], ws[0]) == 0.0
    assert orth(Vs[0]) <= 1e-15
    # block-diagonal: the tridiagonal has exact zeros inside
    B = np.zeros((260, 260))
    B[:130, :130] = goe(130, 4)
    B[130:, 130:] = goe(130, 5)
    ws, Vs, info = solve(G, [B])
    assert info[0] == 0
    assert np.max(np.abs(ws[0] - np.linalg.eigvalsh(B))) <= 1e-13 * np.linalg.norm(B, 2)
    assert residual(B, Vs[0], ws[0]) <= 1e-13
    assert orth(Vs[0]) <= 1e-13


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_f64_uplo_reads_one_triangle(G, uplo):
    n = 170
    A = goe(n, 77)
    junk = A.copy()
    if uplo == "L":
        junk[np.triu_indices(n, 1)] = np.nan
    else:
        junk[np.tril_indices(n, -1)] = np.nan
    ws, Vs, info = solve(G, [junk], uplo=uplo)
    assert info[0] == 0
    S = sym_from(A, uplo)
    assert np.max(np.abs(ws[0] - np.linalg.eigvalsh(S))) <= 1e-13 * np.linalg.norm(S, 2)
    assert residual(S, Vs[0], ws[0]) <= 1e-13


def test_mixed_small_and_large_plan(G):
    mats = [goe(50, 1), goe(300, 2), goe(7, 3), goe(129, 4), goe(128, 5)]
    ws, Vs, info = solve(G, mats)
    assert (info == 0).all()
    for A, w, V in zip(mats, ws, Vs):
        assert np.max(np.abs(w - np.linalg.eigvalsh(A))) <= 1e-13 * np.linalg.norm(A, 2)
        assert residual(A, V, w) <= 1e-13
        assert orth(V) <= 1e-13


def test_eigvals_only_large(G):
    A = goe(400, 8)
    ws, _, info = solve(G, [A], jobz="N")
    assert info[0] == 0
    assert np.max(np.abs(ws[0] - np.linalg.eigvalsh(A))) <= 1e-13 * np.linalg.norm(A, 2)


@pytest.mark.parametrize("n", [129, 333, 800, 1500])
def test_f32_goe(G, n):
    A = goe(n, 3000 + n)
    ws, Vs, info = solve(G, [A.astype(np.float32)], precision="f32")
    assert info[0] == 0
    A32 = A.astype(np.float32).astype(np.float64)
    nA = np.linalg.norm(A32, 2)
    # FP32 working precision: ~n^0.5 ulps of residual and orthogonality
    assert np.max(np.abs(ws[0] - np.linalg.eigvalsh(A32))) <= 1e-5 * nA
    assert residual(A32, Vs[0], ws[0]) <= 1e-5
    assert orth(Vs[0]) <= 1e-5


def test_large_nonfinite_input(G):
    A = goe(150, 9)
    A[70, 3] = np.inf
    ws, Vs, info = solve(G, [A])
    assert info[0] == -1
    assert np.isnan(ws[0]).all()


@pytest.mark.parametrize("precision,n", [("f64", 260), ("f32", 1100)])
def test_large_deterministic(G, precision, n):
    # bitwise repeatable: every reduction has a fixed order (no atomics), and a
    # cross-CTA race would show up as run-to-run differences
    A = goe(n, 10)
    if precision == "f32":
        A = A.astype(np.float32)
    r1 = solve(G, [A], precision=precision)
    r2 = solve(G, [A], precision=precision)
    assert np.array_equal(r1[0][0], r2[0][0]) and np.array_equal(r1[1][0], r2[1][0])


def test_large_adjoint_vs_analytic(G):
    # orders above the one-CTA bound: three tensor-core GEMMs; mixed with small orders
    import torch
    from helpers import analytic_adjoint
    rng = np.random.default_rng(41)
    ns = [150, 40, 300]
    mats = [goe(n, 4100 + n) for n in ns]
    plan = G.Plan(ns)
    A = plan.pack(mats, device="cuda")
    w = torch.empty(plan.w_elems, dtype=torch.float64, device="cuda")
    V = torch.empty(plan.a_elems, dtype=torch.float64, device="cuda")
    info = torch.zeros(len(ns), dtype=torch.int32, device="cuda")
    plan.execute(A, w, V, info)
    wbar = torch.tensor(rng.standard_normal(plan.w_elems), device="cuda")
    Vbar = torch.tensor(rng.standard_normal(plan.a_elems), device="cuda")
    Abar = torch.empty_like(V)
    plan.adjoint(w, V, wbar, Vbar, Abar)
    ws, Vs = plan.unpack(w.cpu().numpy(), V.cpu().numpy())
    wbs, Vbs = plan.unpack(wbar.cpu().numpy(), Vbar.cpu().numpy())
    _, Abs = plan.unpack(w.cpu().numpy(), Abar.cpu().numpy())
    for wg, Vg, wb, Vb, Ab in zip(ws, Vs, wbs, Vbs, Abs):
        ref = analytic_adjoint(Vg, wg, wb, Vb)
        assert np.linalg.norm(Ab - ref) <= 1e-12 * np.linalg.norm(ref)
        assert np.abs(Ab - Ab.T).max() <= 1e-13 * np.abs(Ab).max()


# ---------------------------------------------------------------- FP32 solve + refinement

def solve_refined(G, mats):
    return solve(G, mats, precision="f32_refined")


@pytest.mark.parametrize("n", [200, 600])
def test_refined_goe_reaches_1e13(G, n):
    A = goe(n, 4000 + n)
    ws, Vs, info = solve_refined(G, [A])
    assert info[0] == 0
    nA = np.linalg.norm(A, 2)
    assert np.max(np.abs(ws[0] - np.linalg.eigvalsh(A))) <= 1e-13 * nA
    assert residual(A, Vs[0], ws[0]) <= 1e-13
    assert orth(Vs[0]) <= 1e-13


def test_refined_prescribed_cond1e6_clusters(G):
    # lam = +-logspace(-6, 0): the FP32 solve cannot separate the small
    # eigenvalues, so the refinement runs nested cluster Rayleigh-Ritz steps
    n = 700
    rng = np.random.default_rng(3)
    lam = np.logspace(-6, 0, n) * rng.choice([-1.0, 1.0], n)
    A = prescribed(lam, 7)
    ws, Vs, info = solve_refined(G, [A])
    assert info[0] == 0
    assert np.max(np.abs(ws[0] - np.sort(lam))) <= 1e-13
    assert residual(A, Vs[0], ws[0]) <= 1e-13
    assert orth(Vs[0]) <= 1e-13


@pytest.mark.parametrize("n", [300, 800])
def test_refined_prescribed_cond1e8(G, n):
    # lam = +-logspace(-8, 0): gaps down to ~1e-10 ||A||; orthogonality must
    # survive the polishing iteration
    rng = np.random.default_rng(n)
    lam = np.logspace(-8, 0, n) * rng.choice([-1.0, 1.0], n)
    A = prescribed(lam, 17 + n)
    ws, Vs, info = solve_refined(G, [A])
    assert info[0] == 0
    assert np.max(np.abs(ws[0] - np.sort(lam))) <= 1e-13
    assert residual(A, Vs[0], ws[0]) <= 1e-13
    assert orth(Vs[0]) <= 1e-13


def test_refined_multiplicities(G):
    n = 260
    rng = np.random.default_rng(11)
    lam = np.concatenate([np.full(60, 0.5), np.full(40, -1.0), rng.uniform(-2, 2, n - 100)])
    A = prescribed(lam, 13)
    ws, Vs, info = solve_refined(G, [A])
    assert info[0] == 0
    assert np.max(np.abs(ws[0] - np.sort(lam))) <= 2e-13
    assert residual(A, Vs[0], ws[0]) <= 1e-13
    assert orth(Vs[0]) <= 1e-13


def test_refined_mixed_batch(G):
    mats = [goe(40, 1), goe(260, 2), goe(128, 3)]
    ws, Vs, info = solve_refined(G, mats)
    assert (info == 0).all()
    for A, w, V in zip(mats, ws, Vs):
        assert np.max(np.abs(w - np.linalg.eigvalsh(A))) <= 1e-13 * np.linalg.norm(A, 2)
        assert residual(A, V, w) <= 1e-13
