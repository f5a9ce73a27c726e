"""eigen2 (src/eigenSelfAdjoint.jl:633-668, tested at
test/eigenselfadjoint.jl:18-24 and :45-51), the host-buffer adjoint entry and
the tridiagonal entry gla_dstev at orders above the batched bound (the
divide-and-conquer path), against the CPU oracle.
Tolerances: eigen2 on a SymTridiagonal (and above order 128) returns rows
bit-identical to eigen's; on dense input of order <= 128 (the cheap form:
rows 1 and n of Q from the reflectors, rotations on two rows) its
eigenvalues are bit-identical to eigen's and its rows agree with eigen's
within 100 n eps64 ||A|| / gap per column, as the reference's own test
(:45-51) compares them with isapprox; eigenvalues within 8 n eps64 ||T|| of
the oracle's, residual and ||V'V - I|| <= 1e-13."""
import numpy as np
import pytest

from helpers import goe, golden, orth, residual, sym_from
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


def tridiag_dense(d, e):
    return np.diag(d) + np.diag(e, 1) + np.diag(e, -1)


def test_eigen2_symtridiagonal_rows_equal(G):
    # test/eigenselfadjoint.jl:18-24: vecs[[1, n], :] == vecs2, vecs2 vecs2' ~ I
    g = golden()["symtridiagonal"]
    dv = np.array([float.fromhex(v) for v in g["dv"]])
    ev = np.array([float.fromhex(v) for v in g["ev"]])
    n = len(dv)
    r = G.eigen(G.SymTridiagonal(dv, ev))
    r2 = G.eigen2(G.SymTridiagonal(dv, ev))
    assert np.all(np.diff(r2.values) >= 0)
    assert np.array_equal(r.values, r2.values)
    assert r2.vectors.shape == (2, n)
    assert np.array_equal(r.vectors[[0, n - 1]], r2.vectors)
    assert np.abs(r2.vectors @ r2.vectors.T - np.eye(2)).max() < 1e-13


def rows_close(A, w, V, V2):
    # columns of the two rows agree within 100 n eps ||A|| / gap
    n = len(w)
    nA = max(np.linalg.norm(A, 2), 1e-300)
    for j in range(n):
        gap = np.abs(np.delete(w, j) - w[j]).min() if n > 1 else np.inf
        if gap <= 1e-10 * nA:
            continue
        bound = 100 * n * EPS64 * nA / gap
        assert np.abs(V[[0, n - 1], j] - V2[:, j]).max() <= max(bound, 1e-15), (j, gap)


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_eigen2_symmetric_rows_equal(G, uplo):
    # test/eigenselfadjoint.jl:45-51 on a full symmetric matrix
    for n in (1, 2, 7, 50, 128, 200):
        A = goe(n, 700 + n)
        r = G.eigen(A, uplo=uplo)
        r2 = G.eigen2(A, uplo=uplo)
        assert r2.vectors.shape == (2, n)
        assert np.array_equal(r.values, r2.values)
        if n <= 128:
            rows_close(sym_from(A, uplo), r.values, r.vectors, r2.vectors)
        else:
            assert np.array_equal(r.vectors[[0, n - 1]], r2.vectors)
        if n > 1:
            assert np.abs(r2.vectors @ r2.vectors.T - np.eye(2)).max() < 1e-13
        wo, _, _ = O.syev(sym_from(A, uplo), jobz="N")
        assert np.abs(r2.values - wo).max() <= 8 * n * EPS64 * max(np.linalg.norm(A, 2), 1.0)


def test_eigen2_device_tensor(G):
    import torch
    A = goe(60, 11)
    At = torch.tensor(A, device="cuda")
    r = G.eigen(At)
    r2 = G.eigen2(At)
    assert r2.vectors.shape == (2, 60) and r2.vectors.is_cuda
    assert torch.equal(r.values, r2.values)
    rows_close(A, r.values.cpu().numpy(), r.vectors.cpu().numpy(), r2.vectors.cpu().numpy())


@pytest.mark.parametrize("precision,alg", [("f64", "QL"), ("f64", "QR"), ("f32", "QL")])
def test_eigen2_batched_plan(G, precision, alg):
    # gla_plan_execute_eigen2 over a batch of mixed orders (the 2 x n row
    # blocks at twice the eigenvalue offsets) against the full eigen of the
    # same plan configuration, row for row
    import torch
    rng = np.random.default_rng(31)
    sizes = [int(x) for x in rng.integers(1, 129, size=40)] + [1, 2, 3, 128]
    mats = [goe(n, 800 + i) for i, n in enumerate(sizes)]
    plan = G.Plan(sizes, precision=precision, alg=alg)
    dt = torch.float32 if precision == "f32" else torch.float64
    A = plan.pack(mats, device="cuda")
    w = torch.empty(plan.w_elems, dtype=dt, device="cuda")
    V = torch.empty(plan.a_elems, dtype=dt, device="cuda")
    w2 = torch.empty_like(w)
    V2 = torch.empty(2 * plan.w_elems, dtype=dt, device="cuda")
    info = torch.zeros(len(sizes), dtype=torch.int32, device="cuda")
    plan.execute(A, w, V, info)
    info2 = torch.zeros_like(info)
    plan.execute_eigen2(A, w2, V2, info2)
    torch.cuda.synchronize()
    assert (info.cpu() == 0).all() and (info2.cpu() == 0).all()
    assert torch.equal(w, w2)
    ws, Vs = plan.unpack(w.cpu().numpy().astype(np.float64), V.cpu().numpy().astype(np.float64))
    V2h = V2.cpu().numpy().astype(np.float64)
    eps = 2.0 ** -23 if precision == "f32" else EPS64
    off = 0
    for A_, wv, Vv, n in zip(mats, ws, Vs, sizes):
        rows = V2h[2 * off: 2 * off + 2 * n].reshape(n, 2).T
        off += n
        nA = np.linalg.norm(A_, 2)
        for j in range(n):
            gap = np.abs(np.delete(wv, j) - wv[j]).min() if n > 1 else np.inf
            if gap <= 1e-4 * nA:
                continue
            assert np.abs(Vv[[0, n - 1], j] - rows[:, j]).max() <= max(100 * n * eps * nA / gap, 1e-15)


def test_adjoint_host_matches_device(G):
    import torch
    rng = np.random.default_rng(5)
    mats = [goe(int(n), 900 + i) for i, n in enumerate(rng.integers(8, 97, size=9))]
    plan = G.Plan([m.shape[0] for m in mats])
    A = plan.pack(mats, device="cuda")
    w = torch.empty(plan.w_elems, dtype=torch.float64, device="cuda")
    V = torch.empty(plan.a_elems, dtype=torch.float64, device="cuda")
    info = torch.zeros(len(mats), dtype=torch.int32, device="cuda")
    plan.execute(A, w, V, info)
    wbar = torch.tensor(rng.standard_normal(plan.w_elems), device="cuda")
    Vbar = torch.tensor(rng.standard_normal(plan.a_elems), device="cuda")
    Abar = torch.empty_like(V)
    plan.adjoint(w, V, wbar, Vbar, Abar)
    torch.cuda.synchronize()
    Ah = np.empty(plan.a_elems)
    plan.adjoint_host(w.cpu().numpy(), V.cpu().numpy(), wbar.cpu().numpy(), Vbar.cpu().numpy(), Ah)
    assert np.array_equal(Ah, Abar.cpu().numpy())


def test_adjoint_host_large_plan_matches_device(G):
    import torch
    rng = np.random.default_rng(8)
    plan = G.Plan([300])
    A = plan.pack([goe(300, 3)], device="cuda")
    w = torch.empty(plan.w_elems, dtype=torch.float64, device="cuda")
    V = torch.empty(plan.a_elems, dtype=torch.float64, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    plan.execute(A, w, V, info)
    wbar = torch.tensor(rng.standard_normal(plan.w_elems), device="cuda")
    Vbar = torch.tensor(rng.standard_normal(plan.a_elems), device="cuda")
    Abar = torch.empty_like(V)
    plan.adjoint(w, V, wbar, Vbar, Abar)
    torch.cuda.synchronize()
    Ah = np.empty(plan.a_elems)
    plan.adjoint_host(w.cpu().numpy(), V.cpu().numpy(), wbar.cpu().numpy(), Vbar.cpu().numpy(), Ah)
    assert np.array_equal(Ah, Abar.cpu().numpy())


def wilkinson_plus(n):
    m = (n - 1) / 2.0
    return np.abs(np.arange(n) - m), np.ones(n - 1)


@pytest.mark.parametrize("case", ["random", "wilkinson", "graded", "split"])
def test_large_symtridiagonal_dc(G, case):
    # orders above the batched bound go through gla_dstev's divide and conquer
    rng = np.random.default_rng(17)
    if case == "random":
        n = 300
        d, e = rng.standard_normal(n), rng.standard_normal(n - 1)
    elif case == "wilkinson":  # W+_n: pairs of eigenvalues agreeing to many digits
        n = 401
        d, e = wilkinson_plus(n)
    elif case == "graded":
        n = 520
        d = 10.0 ** np.linspace(0, -12, n)
        e = 0.5 * np.sqrt(d[:-1] * d[1:])
    else:  # exact zeros on the off-diagonal split the matrix into blocks
        n = 700
        d, e = rng.standard_normal(n), rng.standard_normal(n - 1)
        e[rng.choice(n - 1, 25, replace=False)] = 0.0
    T = tridiag_dense(d, e)
    nT = np.linalg.norm(T, 2)
    # the oracle's QL-with-vectors values: its root-free PWK variant (jobz 'N',
    # src/eigenSelfAdjoint.jl:163-219) loses ~4e-9 on W+_401's near-integer pairs
    wo, _, _ = O.stev(d, e, "V")
    r = G.eigen(G.SymTridiagonal(d, e))
    assert np.all(np.diff(r.values) >= 0)
    assert np.abs(r.values - wo).max() <= 8 * n * EPS64 * nT
    assert residual(T, r.vectors, r.values) <= 1e-13
    assert orth(r.vectors) <= 1e-13
    w = G.eigvals(G.SymTridiagonal(d, e))
    assert np.abs(w - wo).max() <= 8 * n * EPS64 * nT
    r2 = G.eigen2(G.SymTridiagonal(d, e))
    assert np.array_equal(r2.vectors, r.vectors[[0, n - 1]])


def test_large_symtridiagonal_device_inputs(G):
    import torch
    n = 1000
    rng = np.random.default_rng(23)
    d, e = rng.standard_normal(n), rng.standard_normal(n - 1)
    r = G.eigen(G.SymTridiagonal(torch.tensor(d, device="cuda"), torch.tensor(e, device="cuda")))
    assert r.values.is_cuda and r.vectors.shape == (n, n)
    T = tridiag_dense(d, e)
    wo, _, _ = O.stev(d, e, "V")
    assert np.abs(r.values.cpu().numpy() - wo).max() <= 8 * n * EPS64 * np.linalg.norm(T, 2)
    assert residual(T, r.vectors.cpu().numpy(), r.values.cpu().numpy()) <= 1e-13


def test_eigen2_host_matches_device(G):
    # gla_plan_execute_eigen2_host (host arenas, the Julia glue's entry) gives
    # the device entry's bits, including orders 1 and 2 whose 2 x n block is
    # larger than n^2
    import torch
    sizes = [1, 2, 5, 64, 128, 3]
    mats = [goe(n, 1200 + n) for n in sizes]
    plan = G.Plan(sizes)
    Ah = plan.pack(mats)
    w = np.empty(plan.w_elems)
    V2 = np.empty(2 * plan.w_elems)
    info = np.zeros(len(sizes), dtype=np.int32)
    assert plan.execute_eigen2_host(Ah, w, V2, info) == 0
    A = plan.pack(mats, device="cuda")
    wd = torch.empty(plan.w_elems, dtype=torch.float64, device="cuda")
    V2d = torch.empty(2 * plan.w_elems, dtype=torch.float64, device="cuda")
    infod = torch.zeros(len(sizes), dtype=torch.int32, device="cuda")
    plan.execute_eigen2(A, wd, V2d, infod)
    torch.cuda.synchronize()
    assert np.array_equal(w, wd.cpu().numpy()) and np.array_equal(V2, V2d.cpu().numpy())
    assert (info == 0).all()
