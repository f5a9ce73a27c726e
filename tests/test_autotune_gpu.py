"""The autotuner (GLA_FLAG_AUTOTUNE): per size bucket it measures the
tridiagonalisation's threads per CTA and the chase's matrices per warp on
synthetic matrices, keeps the fastest, and plans reuse the table; results
stay within the batched path's tolerances (eigenvalues within 8 n eps ||A||
of the oracle, residual and orthogonality <= 1e-13; refined <= 1e-13)."""
import numpy as np
import pytest

from helpers import goe, orth, residual
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


def batch(seed, count):
    rng = np.random.default_rng(seed)
    ns = rng.integers(8, 129, size=count)
    return [goe(int(n), seed * 1000 + i) for i, n in enumerate(ns)]


def solve(G, plan, mats):
    w = np.empty(plan.w_elems)
    V = np.empty(plan.a_elems)
    info = np.zeros(len(mats), dtype=np.int32)
    plan.execute_host(plan.pack(mats), w, V, info)
    assert (info == 0).all()
    return plan.unpack(w, V)


@pytest.mark.parametrize("precision", ["f64", "f32_refined"])
def test_autotuned_plan_configs_and_accuracy(G, precision):
    G.autotune_clear()
    mats = batch(3, 300)
    plan = G.Plan([m.shape[0] for m in mats], precision=precision, autotune=True)
    cfgs = plan.bucket_configs()
    assert len(cfgs) == 8
    for c in cfgs:
        nt = max(32, (c["nmax"] + 31) // 32 * 32)
        assert c["nt_tri"] in {nt, min(256, 2 * nt), min(256, 4 * nt)}
        assert c["lanes_per_warp"] in (4, 8, 16, 32)
    ws, Vs = solve(G, plan, mats)
    for A, w, V in zip(mats, ws, Vs):
        n = A.shape[0]
        wo, _, _ = O.syev(A, jobz="N")
        tol = 1e-13 * np.linalg.norm(A, 2) if precision == "f32_refined" else 8 * n * EPS64 * np.linalg.norm(A, 2)
        assert np.abs(w - wo).max() <= tol
        assert residual(A, V, w) <= 1e-13 and orth(V) <= 1e-13


def test_autotune_table_reused_and_saved(G, tmp_path):
    G.autotune_clear()
    mats = batch(4, 200)
    ns = [m.shape[0] for m in mats]
    p1 = G.Plan(ns, autotune=True)
    c1 = p1.bucket_configs()
    path = tmp_path / "tune.txt"
    G.autotune_save(path)
    G.autotune_clear()
    assert G.autotune_load(path) == len(c1)
    p2 = G.Plan(ns, autotune=True)  # every bucket found in the loaded table: no measurement
    assert p2.bucket_configs() == c1
    ws1, _ = solve(G, p1, mats)
    ws2, _ = solve(G, p2, mats)
    for a, b in zip(ws1, ws2):
        assert np.array_equal(a, b)
