"""gla_plan_execute_host pipelined over contiguous chunks of the batch
(FP32 + refinement plans of orders <= 128, page-locked host buffers): the
copy of one chunk's A and of another's w and V overlap the persistent solve
of a third. The results equal, bit for bit, those of gla_plan_execute on
device buffers of the same plan, including matrices the persistent kernel
leaves to the QL chase (finished, and copied out again, after their chunk's
copy), non-finite input and empty orders. Pageable buffers take the
unpipelined path, with the same results. A sample and every hard matrix are
also checked against the oracle (eigenvalues within 1e-13 ||A||, residual
and orthogonality <= 1e-13)."""
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


def wilkinson(n):
    m = (n - 1) // 2
    return np.diag(np.abs(np.arange(-m, m + 1)).astype(float)) + np.diag(np.ones(n - 1), 1) + np.diag(np.ones(n - 1), -1)


def batch(seed, count):
    """GOE matrices of orders 0 .. 40, with matrices the FP32 solver hands to
    the QL chase spread over the chunks, and one matrix holding a NaN."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(0, 41, size=count)
    mats = [goe(int(n), seed + i) for i, n in enumerate(ns)]
    hard = [wilkinson(21), np.eye(7), np.kron(np.eye(3), goe(12, seed + 1)),
            prescribed(np.repeat(rng.standard_normal(8), 4), seed + 2), wilkinson(101)]
    pos = [3, count // 3, count // 2, (2 * count) // 3, count - 2]
    for p, H in zip(pos, hard):
        mats[p] = H
    bad = goe(9, seed + 3)
    bad[2, 3] = bad[3, 2] = np.nan
    mats[count // 4] = bad
    return mats, pos, count // 4


_keep = []  # the page-locked tensors behind the arrays below stay alive


def pinned(torch, x):
    t = torch.from_numpy(np.ascontiguousarray(x)).pin_memory()
    _keep.append(t)
    return t.numpy()


@pytest.mark.parametrize("jobz", ["V", "N"])
def test_pipelined_host_execute_matches_device_execute(G, jobz):
    import torch
    mats, hard_pos, nan_pos = batch(3100, 4000)
    ns = [m.shape[0] for m in mats]
    plan = G.Plan(ns, precision="f32_refined", jobz=jobz)
    chunks, _ = plan.host_pipeline()
    assert chunks >= 2
    A = plan.pack(mats)
    nW, nA = max(plan.w_elems, 1), max(plan.a_elems, 1)
    # device buffers (gla_plan_execute)
    dA = torch.from_numpy(A).cuda()
    dw = torch.empty(nW, dtype=torch.float64, device="cuda")
    dV = torch.empty(nA, dtype=torch.float64, device="cuda") if jobz == "V" else None
    dinfo = torch.zeros(len(ns), dtype=torch.int32, device="cuda")
    plan.execute(dA, dw, dV, dinfo)
    torch.cuda.synchronize()
    w_ref = dw.cpu().numpy()
    V_ref = dV.cpu().numpy() if jobz == "V" else None
    info_ref = dinfo.cpu().numpy()
    # page-locked host buffers: the pipeline
    hA = pinned(torch, A)
    hw = pinned(torch, np.full(nW, -7.0))
    hV = pinned(torch, np.full(nA, -7.0)) if jobz == "V" else None
    hinfo = pinned(torch, np.full(len(ns), 99, dtype=np.int32))
    plan.execute_host(hA, hw, hV, hinfo)
    assert plan.host_pipeline() == (chunks, True)
    assert plan.stats()["rotations"] > 0  # the hard matrices went through the chase
    assert np.array_equal(hinfo, info_ref)
    assert np.array_equal(hw, w_ref, equal_nan=True)
    if jobz == "V":
        assert np.array_equal(hV, V_ref, equal_nan=True)
    # pageable host buffers: copied in and out whole, same results
    w2 = np.full(nW, -7.0)
    V2 = np.full(nA, -7.0) if jobz == "V" else None
    info2 = np.full(len(ns), 99, dtype=np.int32)
    plan.execute_host(A, w2, V2, info2)
    assert plan.host_pipeline() == (chunks, False)
    assert np.array_equal(info2, info_ref)
    assert np.array_equal(w2, w_ref, equal_nan=True)
    if jobz == "V":
        assert np.array_equal(V2, V_ref, equal_nan=True)
    # against the oracle: the hard matrices and a sample
    assert info_ref[nan_pos] != 0
    assert np.isnan(hw[plan.w_off[nan_pos]:plan.w_off[nan_pos] + ns[nan_pos]]).all()
    ws, Vs = plan.unpack(hw, hV if jobz == "V" else np.zeros(nA))
    rng = np.random.default_rng(5)
    sample = sorted(set(hard_pos) | set(int(i) for i in rng.choice(len(ns), 60, replace=False)) - {nan_pos})
    for i in sample:
        Ai = mats[i]
        assert info_ref[i] == 0, i
        if ns[i] == 0:
            continue
        wo = O.syev(Ai, "V")[0]
        nA_i = max(np.linalg.norm(Ai, 2), 1e-300)
        assert np.abs(ws[i] - wo).max() <= 1e-13 * nA_i, i
        if jobz == "V":
            assert residual(Ai, Vs[i], ws[i]) <= 1e-13, i
            assert orth(Vs[i]) <= 1e-13, i
    plan.close()


def test_small_batches_and_other_plans_do_not_pipeline(G):
    import torch
    mats = [goe(n, 3200 + n) for n in (5, 17, 64, 128)]
    ns = [m.shape[0] for m in mats]
    for kw in ({"precision": "f32_refined"}, {"precision": "f64"}, {"precision": "f32_refined", "graph": True}):
        plan = G.Plan(ns, **kw)
        assert plan.host_pipeline() == (0, False)
        A = pinned(torch, plan.pack(mats))
        w = pinned(torch, np.zeros(plan.w_elems))
        V = pinned(torch, np.zeros(plan.a_elems))
        info = pinned(torch, np.zeros(len(ns), dtype=np.int32))
        plan.execute_host(A, w, V, info)
        assert plan.host_pipeline() == (0, False)
        assert (info == 0).all()
        ws, _ = plan.unpack(w, V)
        for Ai, wi in zip(mats, ws):
            assert np.abs(wi - O.syev(Ai, "V")[0]).max() <= 1e-12 * np.linalg.norm(Ai, 2)
        plan.close()
