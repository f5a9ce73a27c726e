"""GPU parity: libglagpu.so (through the C ABI, via the glagpu host mirror)
against the CPU oracle on the same seeded inputs, plus the reference's own
known-answer cases (test/eigenselfadjoint.jl).

Tolerances (eigenvalues to a relative tolerance, eigenvectors by residual,
orthogonality and sign-normalised comparison):
  FP64        |w - w_oracle| <= 8 n eps64 ||A||, residual and ||V'V - I|| <= 1e-13,
              vectors within 100 n eps ||A|| / gap of the oracle's
  FP32        |w - w_oracle32| <= 8 n eps32 ||A||, residual, orthogonality <= 32 n eps32
  F32_REFINED |w - w_oracle64| <= 1e-13 ||A||, residual and orthogonality <= 1e-13
"""
import numpy as np
import pytest

from helpers import from_hex, goe, golden, golden_large, orth, prescribed, residual, sym_from, vec_parity
from oracle import oracle as O

pytestmark = pytest.mark.gpu

EPS64 = 2.0 ** -52
EPS32 = 2.0 ** -23


@pytest.fixture(scope="module")
def G():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import glagpu
    return glagpu


def batch_mats(seed, sizes):
    return [goe(int(n), seed * 1000 + i) for i, n in enumerate(sizes)]


def check_f64(A, w, V, wo, Vo, uplo="L"):
    S = sym_from(A, uplo)
    n = len(w)
    nA = max(np.linalg.norm(S, 2), 1e-300)
    assert np.all(np.diff(w) >= 0)
    assert np.abs(w - wo).max() <= 8 * n * EPS64 * nA
    if V is not None:
        assert residual(S, V, w) <= 1e-13
        assert orth(V) <= 1e-13
        assert vec_parity(S, V, Vo, wo) <= 1.0


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_batched_f64_vs_oracle(G, uplo):
    rng = np.random.default_rng(2)
    sizes = list(rng.integers(1, 129, size=60)) + [1, 2, 3, 4, 31, 32, 33, 64, 65, 96, 97, 127, 128]
    mats = batch_mats(2, sizes)
    res = G.eigen_batched([__import__("torch").tensor(m, device="cuda") for m in mats], uplo=uplo)
    for A, r in zip(mats, res):
        wo, Vo, info = O.syev(A, "V", uplo)
        check_f64(A, r.values.cpu().numpy(), r.vectors.cpu().numpy(), wo, Vo, uplo)


def test_batched_f64_qr_variant(G):
    mats = batch_mats(3, [5, 16, 50, 100, 128])
    res = G.eigen_batched(mats, alg="QR")
    for A, r in zip(mats, res):
        wo, Vo, info = O.syev(A, "V", use_qr=True)
        check_f64(A, r.values, r.vectors, wo, Vo)


def test_batched_eigvals_pwk(G):
    rng = np.random.default_rng(4)
    sizes = list(rng.integers(1, 129, size=40)) + [1, 2, 3, 128]
    mats = batch_mats(4, sizes)
    ws = G.eigvals_batched(mats)
    for A, w in zip(mats, ws):
        wo = O.syev(A, "N")[0]
        check_f64(A, w, None, wo, None)


def test_host_and_device_paths_identical(G):
    import torch
    mats = batch_mats(5, [7, 40, 128, 3])
    rh = G.eigen_batched(mats)
    rd = G.eigen_batched([torch.tensor(m, device="cuda") for m in mats])
    for a, b in zip(rh, rd):
        assert np.array_equal(a.values, b.values.cpu().numpy())
        assert np.array_equal(a.vectors, b.vectors.cpu().numpy())


def test_deterministic(G):
    mats = batch_mats(6, [128, 77, 12])
    r1 = G.eigen_batched(mats)
    r2 = G.eigen_batched(mats)
    for a, b in zip(r1, r2):
        assert np.array_equal(a.values, b.values) and np.array_equal(a.vectors, b.vectors)


def test_batched_f32_vs_oracle(G):
    rng = np.random.default_rng(7)
    sizes = list(rng.integers(1, 129, size=40)) + [1, 2, 128]
    mats = [m.astype(np.float32) for m in batch_mats(7, sizes)]
    res = G.eigen_batched(mats, precision="f32")
    for A, r in zip(mats, res):
        wo, Vo, info = O.syev(A, "V", dtype=np.float32)
        A64 = A.astype(np.float64)
        n = len(wo)
        nA = max(np.linalg.norm(A64, 2), 1e-30)
        w = r.values.astype(np.float64)
        V = r.vectors.astype(np.float64)
        assert np.abs(w - wo).max() <= 8 * n * EPS32 * nA
        assert residual(A64, V, w) <= 32 * n * EPS32
        assert orth(V) <= 32 * n * EPS32


def test_f32_refined_reaches_1e13(G):
    rng = np.random.default_rng(8)
    sizes = list(rng.integers(1, 129, size=40)) + [1, 2, 3, 128, 128]
    mats = batch_mats(8, sizes)
    res = G.eigen_batched(mats, precision="f32_refined")
    for A, r in zip(mats, res):
        wo, Vo, info = O.syev(A, "V")
        nA = max(np.linalg.norm(A, 2), 1e-300)
        assert np.abs(r.values - wo).max() <= 1e-13 * nA
        assert residual(A, r.vectors, r.values) <= 1e-13
        assert orth(r.vectors) <= 1e-13


def test_f32_refined_prescribed_spectrum(G):
    # cond 1e6 spectrum with random signs (the large-n precision configuration, at n <= 128)
    rng = np.random.default_rng(9)
    mats = []
    for n in (64, 100, 128):
        lam = np.logspace(-6, 0, n) * rng.choice([-1.0, 1.0], n)
        mats.append(prescribed(lam, 30 + n))
    res = G.eigen_batched(mats, precision="f32_refined")
    for A, r in zip(mats, res):
        wo, Vo, _ = O.syev(A, "V")
        nA = np.linalg.norm(A, 2)
        assert np.abs(r.values - wo).max() <= 1e-13 * nA
        assert residual(A, r.vectors, r.values) <= 1e-13


def test_f32_refined_cond1e8_clusters(G):
    # lam = +-logspace(-8, 0) (the mixed workload's prescribed half): a run of
    # eigenvalues below the FP32 resolution forms one cluster whose end-to-end
    # gap exceeds delta; the refinement must neither stall nor report success
    # on an unconverged iterate
    rng = np.random.default_rng(235)
    mats, lams = [], []
    for n in (16, 21, 33, 47, 80, 128):
        for rep in range(3):
            lam = np.logspace(-8, 0, n) * rng.choice([-1.0, 1.0], n)
            mats.append(prescribed(lam, 1000 * n + rep))
            lams.append(np.sort(lam))
    plan = G.Plan([m.shape[0] for m in mats], precision="f32_refined")
    w = np.empty(plan.w_elems)
    V = np.empty(plan.a_elems)
    info = np.zeros(len(mats), dtype=np.int32)
    plan.execute_host(plan.pack(mats), w, V, info)
    ws, Vs = plan.unpack(w, V)
    assert (info == 0).all(), info
    for A, lam, wg, Vg in zip(mats, lams, ws, Vs):
        assert np.abs(wg - lam).max() <= 1e-13
        assert residual(A, Vg, wg) <= 1e-13
        assert orth(Vg) <= 1e-13


def test_reference_known_answers(G):
    # 1x1 (:100-105), issue 52 (:108-117, exact), #139 (:164-170, exact)
    r = G.eigen(np.array([[1.0]]))
    assert r.values.tolist() == [1.0] and r.vectors.tolist() == [[1.0]]
    for pos in (0, 2):
        M = np.zeros((3, 3))
        M[pos, pos] = 0.01
        assert G.eigvals(M).tolist() == [0.0, 0.0, 0.01]
        assert G.eigen(M).values.tolist() == [0.0, 0.0, 0.01]
    assert G.eigvals(np.diag([1.0, 2.0])).tolist() == [1.0, 2.0]
    assert G.eigen(np.diag([1.0, 2.0])).values.tolist() == [1.0, 2.0]
    # issue 123 (:125-133) against the 256-bit oracle
    import mpmath
    g = golden()["issue123"]
    M = np.array([[float(v) for v in row] for row in g["A"]])
    r = G.eigen(M)
    w256 = np.array([float(mpmath.mpf(v)) for v in g["w"]])
    assert residual(M, r.vectors, r.values) <= 1e-14
    assert np.abs(r.values - w256).max() <= 1e-14 * np.linalg.norm(M, 2)


def test_goe_against_256bit(G):
    import mpmath
    for g in golden()["goe"]:
        A = from_hex(g["A"])
        w256 = np.array([float(mpmath.mpf(v)) for v in g["w"]])
        r = G.eigen(A)
        n = len(w256)
        assert np.abs(r.values - w256).max() <= 8 * n * EPS64 * np.linalg.norm(A, 2)
        assert vec_parity(A, r.vectors, np.array(g["V"]), w256) <= 1.0


def test_symtridiagonal_ql_qr_pwk(G):
    # test/eigenselfadjoint.jl:5-32
    import mpmath
    g = golden()["symtridiagonal"]
    dv = np.array([float.fromhex(v) for v in g["dv"]])
    ev = np.array([float.fromhex(v) for v in g["ev"]])
    T = np.diag(dv) + np.diag(ev, 1) + np.diag(ev, -1)
    w256 = np.array([float(mpmath.mpf(v)) for v in g["w"]])
    nT = np.linalg.norm(T, 2)
    for alg in ("QL", "QR"):
        r = G.eigen(G.SymTridiagonal(dv, ev), alg=alg)
        assert np.all(np.diff(r.values) >= 0)
        assert np.abs(r.values - w256).max() <= 200 * EPS64 * nT
        assert residual(T, r.vectors, r.values) < 1e-13 and orth(r.vectors) < 1e-13
    w = G.eigvals(G.SymTridiagonal(dv, ev))
    wp256 = np.array([float(mpmath.mpf(v)) for v in g["w_pwk"]])
    assert np.abs(w - wp256).max() <= 200 * EPS64 * nT


def test_two_by_two_table_as_tridiagonal(G):
    # test/eigenselfadjoint.jl:135-149 through the tridiagonal entry (n = 2)
    for case in golden()["eig2x2_cases"]:
        d, e = case["d"], case["e"]
        r = G.eigen(G.SymTridiagonal(np.array(d), np.array(e)))
        wo, Vo, _ = O.stev(d, e, "V")
        assert np.allclose(r.values, wo, rtol=1e-15, atol=0)
        assert orth(r.vectors) < 1e-15


def test_nonfinite_input_flags(G):
    import torch
    A = goe(9, 3)
    A[4, 2] = np.nan
    with pytest.raises(G.NonFiniteError):
        G.eigen(A)
    B = goe(9, 4)
    B[1, 7] = np.inf  # upper triangle: ignored for uplo 'L', flagged for 'U'
    r = G.eigen(B, uplo="L")
    assert np.isfinite(r.values).all()
    with pytest.raises(G.NonFiniteError):
        G.eigen(B, uplo="U")
    # batched: only the bad matrix is flagged, the others are solved
    mats = [goe(10, 5), A, goe(12, 6)]
    res, info = G._solve_batched([torch.tensor(m, device="cuda") for m in mats], "V", "L", None, "f64", "QL", False)
    assert info.tolist() == [0, -1, 0]
    assert np.isnan(res[1].values.cpu().numpy()).all()
    assert residual(mats[2], res[2].vectors.cpu().numpy(), res[2].values.cpu().numpy()) < 1e-13


def test_dimension_mismatch(G):
    with pytest.raises(G.DimensionMismatch):
        G.eigen(np.zeros((3, 4)))
    with pytest.raises(G.DimensionMismatch):
        G.SymTridiagonal(np.zeros(4), np.zeros(4))
    with pytest.raises(G.DimensionMismatch):
        G.Plan([G.GLA_MAX_N + 1])


def test_empty_batch_and_zero_order(G):
    assert G.eigen_batched([]) == []
    r = G.eigen_batched([np.zeros((0, 0)), goe(3, 1)])
    assert len(r[0].values) == 0 and len(r[1].values) == 3


def test_plan_stats_rotation_count(G):
    import torch
    mats = batch_mats(10, [64, 128])
    plan = G.Plan([64, 128])
    A = plan.pack(mats, device="cuda")
    w = torch.empty(plan.w_elems, dtype=torch.float64, device="cuda")
    V = torch.empty(plan.a_elems, dtype=torch.float64, device="cuda")
    info = torch.zeros(2, dtype=torch.int32, device="cuda")
    plan.execute(A, w, V, info)
    st = plan.stats()
    nrot = sum(O.syev(m, return_stats=True)[3]["nrot"] for m in mats)
    assert abs(st["rotations"] - nrot) <= 0.05 * nrot
    assert st["passes"] <= 2  # the second, asynchronous pass only finishes overflowed logs


def test_multi_pass_chase_identical(G):
    # a tiny rotation log forces the chase to stop and resume between sweeps
    import torch
    mats = batch_mats(11, [128, 100, 60, 9, 2])
    outs = []
    for small in (False, True):
        plan = G.Plan([m.shape[0] for m in mats], small_log=small)
        A = plan.pack(mats, device="cuda")
        w = torch.empty(plan.w_elems, dtype=torch.float64, device="cuda")
        V = torch.empty(plan.a_elems, dtype=torch.float64, device="cuda")
        info = torch.zeros(len(mats), dtype=torch.int32, device="cuda")
        plan.execute(A, w, V, info)
        outs.append((w.cpu().numpy(), V.cpu().numpy(), plan.stats()["passes"]))
        plan.close()
    assert outs[0][2] <= 2 and outs[1][2] > 3
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("precision", ["f64", "f32_refined"])
def test_cuda_graph_capture_and_replay(G, precision):
    # the batched solve captured once, replayed on two different inputs:
    # bit-identical to the uncaptured execute of each input
    import torch
    rng = np.random.default_rng(12)
    sizes = list(rng.integers(1, 129, size=50))
    mats1 = batch_mats(12, sizes)
    mats2 = batch_mats(13, sizes)
    ref = G.Plan(sizes, precision=precision)
    gp = G.Plan(sizes, precision=precision, graph=True)
    A = gp.pack(mats1, device="cuda")
    w = torch.empty(gp.w_elems, dtype=torch.float64, device="cuda")
    V = torch.empty(gp.a_elems, dtype=torch.float64, device="cuda")
    info = torch.zeros(len(sizes), dtype=torch.int32, device="cuda")
    g = gp.capture(A, w, V, info)
    for mats in (mats2, mats1):
        A.copy_(gp.pack(mats, device="cuda"))
        g.replay()
        torch.cuda.synchronize()
        A2 = ref.pack(mats, device="cuda")
        w2 = torch.empty_like(w)
        V2 = torch.empty_like(V)
        info2 = torch.zeros_like(info)
        ref.execute(A2, w2, V2, info2)
        torch.cuda.synchronize()
        assert (info.cpu().numpy() == 0).all()
        assert torch.equal(w, w2) and torch.equal(V, V2)


@pytest.mark.parametrize("precision", ["f64", "f32_refined"])
def test_goe_large_against_256bit(G, precision):
    # the single-matrix workload (GOE n = 64, seed 1) and a GOE n = 128, solved
    # alone and together in one batch, against the 256-bit restatement
    import torch
    cases = [golden_large(64), golden_large(128)]
    single = [G.eigen(torch.tensor(A, device="cuda"), precision=precision) for A, _, _, _ in cases]
    batched = G.eigen_batched([torch.tensor(A, device="cuda") for A, _, _, _ in cases], precision=precision)
    for (A, w256, V256, _), r1, r2 in zip(cases, single, batched):
        n = A.shape[0]
        nA = np.linalg.norm(A, 2)
        tol = 8 * n * EPS64 * nA if precision == "f64" else 1e-13 * nA
        for r in (r1, r2):
            w, V = r.values.cpu().numpy(), r.vectors.cpu().numpy()
            assert np.abs(w - w256).max() <= tol
            assert residual(A, V, w) <= 1e-13 and orth(V) <= 1e-13
            assert vec_parity(A, V, V256, w256, tol_factor=1.0 if precision == "f64" else 10.0) <= 1.0
