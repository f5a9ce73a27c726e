"""Adjoint of the batched eigen-decomposition (gla_plan_adjoint): against the
analytic gradient built from the CPU oracle's eigenpairs, against central
finite differences of L = sum(wt * lambda) + sum(C o V) (h = 1e-6, 1e-6
relative), and through the torch autograd wrapper. Matrices follow the
differentiation configuration: n in [32, 96], Q diag(lambda) Q' with lambda
sorted on [-1, 1] and gaps >= 1e-3."""
import numpy as np
import pytest

from helpers import analytic_adjoint, gapped_spectrum, prescribed
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import glagpu
    return glagpu


def c4_batch(seed, count):
    rng = np.random.default_rng(seed)
    mats = []
    for _ in range(count):
        n = int(rng.integers(32, 97))
        mats.append(prescribed(gapped_spectrum(n, rng), int(rng.integers(1 << 30))))
    return mats


def solve(G, plan, mats):
    import torch
    A = plan.pack(mats, device="cuda")
    w = torch.empty(plan.w_elems, dtype=torch.float64, device="cuda")
    V = torch.empty(plan.a_elems, dtype=torch.float64, device="cuda")
    info = torch.zeros(len(mats), dtype=torch.int32, device="cuda")
    plan.execute(A, w, V, info)
    assert (info.cpu().numpy() == 0).all()
    return w, V


def test_adjoint_matches_analytic_from_oracle_eigenpairs(G):
    import torch
    mats = c4_batch(1, 12)
    ns = [m.shape[0] for m in mats]
    plan = G.Plan(ns)
    w, V = solve(G, plan, mats)
    rng = np.random.default_rng(2)
    wbar = torch.tensor(rng.standard_normal(plan.w_elems), device="cuda")
    Vbar = torch.tensor(rng.standard_normal(plan.a_elems), device="cuda")
    Abar = torch.empty_like(V)
    plan.adjoint(w, V, wbar, Vbar, Abar)
    ws, Vs = plan.unpack(w.cpu().numpy(), V.cpu().numpy())
    wbs, Vbs = plan.unpack(wbar.cpu().numpy(), Vbar.cpu().numpy())
    _, Abs = plan.unpack(w.cpu().numpy(), Abar.cpu().numpy())
    for A, wg, Vg, wb, Vb, Ab in zip(mats, ws, Vs, wbs, Vbs, Abs):
        wo, Vo, _ = O.syev(A)
        Vo = Vo * np.sign(np.sum(Vo * Vg, axis=0))  # align the oracle's signs with the GPU's
        ref = analytic_adjoint(Vo, wo, wb, Vb)
        assert np.linalg.norm(Ab - ref) <= 1e-10 * np.linalg.norm(ref)
        assert np.allclose(Ab, Ab.T, rtol=0, atol=1e-14 * np.abs(Ab).max())


def test_adjoint_central_finite_differences(G):
    import torch
    mats = c4_batch(3, 6)
    rng = np.random.default_rng(4)
    ns = [m.shape[0] for m in mats]
    wt = [rng.standard_normal(n) for n in ns]
    Cs = [rng.standard_normal((n, n)) for n in ns]
    Es = []
    for n in ns:
        E = rng.standard_normal((n, n))
        E = (E + E.T) / 2
        Es.append(E / np.linalg.norm(E))
    h = 1e-6
    # base point, +h and -h in one batch
    plan = G.Plan(ns * 3)
    w, V = solve(G, plan, mats + [A + h * E for A, E in zip(mats, Es)] + [A - h * E for A, E in zip(mats, Es)])
    ws, Vs = plan.unpack(w.cpu().numpy(), V.cpu().numpy())
    k = len(mats)
    piv = [np.argmax(np.abs(Vs[b]), axis=0) for b in range(k)]  # sign convention fixed at the base point

    def loss(b, wv, Vv):
        s = np.sign(Vv[piv[b], np.arange(Vv.shape[1])])
        return float(wt[b] @ wv + np.sum(Cs[b] * (Vv * s)))

    # adjoint at the base point with the sign-normalised V
    bp = G.Plan(ns)
    Vn = [Vs[b] * np.sign(Vs[b][piv[b], np.arange(ns[b])]) for b in range(k)]
    wd = torch.tensor(np.concatenate(ws[:k]), device="cuda")
    Vd = bp.pack(Vn, device="cuda")
    wbar = torch.tensor(np.concatenate(wt), device="cuda")
    Vbar = bp.pack(Cs, device="cuda")
    Abar = torch.empty_like(Vd)
    bp.adjoint(wd, Vd, wbar, Vbar, Abar)
    _, Abs = bp.unpack(wd.cpu().numpy(), Abar.cpu().numpy())
    for b in range(k):
        fd = (loss(b, ws[k + b], Vs[k + b]) - loss(b, ws[2 * k + b], Vs[2 * k + b])) / (2 * h)
        ad = float(np.sum(Abs[b] * Es[b]))
        assert abs(fd - ad) <= 1e-6 * max(abs(ad), 1.0), (b, fd, ad)


def test_torch_autograd_wrapper(G):
    import torch
    mats = c4_batch(5, 5)
    ns = [m.shape[0] for m in mats]
    plan = G.Plan(ns)
    A = plan.pack(mats, device="cuda").requires_grad_(True)
    w, V = G.eigh_autograd(A, plan)
    rng = np.random.default_rng(6)
    wt = torch.tensor(rng.standard_normal(plan.w_elems), device="cuda")
    Ct = torch.tensor(rng.standard_normal(plan.a_elems), device="cuda")
    (w * wt).sum().add((V * Ct).sum()).backward()
    ws, Vs = plan.unpack(w.detach().cpu().numpy(), V.detach().cpu().numpy())
    wts, Cts = plan.unpack(wt.cpu().numpy(), Ct.cpu().numpy())
    _, grads = plan.unpack(ws, A.grad.cpu().numpy())
    for wv, Vv, wb, Vb, g in zip(ws, Vs, wts, Cts, grads):
        ref = analytic_adjoint(Vv, wv, wb, Vb)
        assert np.linalg.norm(g - ref) <= 1e-10 * np.linalg.norm(ref)


@pytest.mark.parametrize("precision", ["f64", "f32_refined"])
def test_forward_and_adjoint_in_one_graph(G, precision):
    # the solve plus its backward captured once (Plan.capture_step), replayed
    # on two inputs and two cotangent pairs: bit-identical to eager execute
    # followed by adjoint on the same data
    import torch
    mats1 = c4_batch(21, 40)
    rng = np.random.default_rng(22)
    mats2 = [prescribed(gapped_spectrum(m.shape[0], rng), 900 + i) for i, m in enumerate(mats1)]
    sizes = [m.shape[0] for m in mats1]
    ref = G.Plan(sizes, precision=precision)
    gp = G.Plan(sizes, precision=precision, graph=True)
    A = gp.pack(mats1, device="cuda")
    w = torch.empty(gp.w_elems, dtype=torch.float64, device="cuda")
    V = torch.empty(gp.a_elems, dtype=torch.float64, device="cuda")
    info = torch.zeros(len(sizes), dtype=torch.int32, device="cuda")
    wbar = torch.randn(gp.w_elems, dtype=torch.float64, device="cuda")
    Vbar = torch.randn(gp.a_elems, dtype=torch.float64, device="cuda")
    Abar = torch.empty_like(V)
    g = gp.capture_step(A, w, V, info, wbar, Vbar, Abar)
    for k, mats in enumerate((mats2, mats1)):
        A.copy_(gp.pack(mats, device="cuda"))
        wbar.copy_(torch.randn(gp.w_elems, dtype=torch.float64, device="cuda"))
        Vbar.copy_(torch.randn(gp.a_elems, dtype=torch.float64, device="cuda"))
        g.replay()
        torch.cuda.synchronize()
        A2 = ref.pack(mats, device="cuda")
        w2, V2 = torch.empty_like(w), torch.empty_like(V)
        info2 = torch.zeros_like(info)
        Abar2 = torch.empty_like(Abar)
        ref.execute(A2, w2, V2, info2)
        ref.adjoint(w2, V2, wbar, Vbar, Abar2)
        torch.cuda.synchronize()
        assert (info.cpu().numpy() == 0).all()
        assert torch.equal(w, w2) and torch.equal(V, V2)
        assert torch.equal(Abar, Abar2)
    gp.close()
    ref.close()


def test_adjoint_tensor_core_products_all_orders(G):
    # the batched adjoint's tensor-core products at every slab and pass
    # boundary of the order (1 .. 128, the 32-column passes, a 1e6 scaling):
    # the kernel's Abar against the closed form on the same (w, V)
    import torch
    from helpers import goe
    ns = [1, 2, 3, 17, 31, 32, 33, 63, 64, 65, 96, 127, 128]
    mats = [goe(n, 300 + n) * (1e6 if n == 65 else 1.0) for n in ns]
    plan = G.Plan(ns)
    w, V = solve(G, plan, mats)
    rng = np.random.default_rng(5)
    wbar = torch.tensor(rng.standard_normal(plan.w_elems), device="cuda")
    Vbar = torch.tensor(rng.standard_normal(plan.a_elems), device="cuda")
    Abar = torch.empty_like(V)
    plan.adjoint(w, V, wbar, Vbar, Abar)
    ws, Vs = plan.unpack(w.cpu().numpy(), V.cpu().numpy())
    wbs, Vbs = plan.unpack(wbar.cpu().numpy(), Vbar.cpu().numpy())
    _, Abs = plan.unpack(w.cpu().numpy(), Abar.cpu().numpy())
    for wg, Vg, wb, Vb, Ab in zip(ws, Vs, wbs, Vbs, Abs):
        ref = analytic_adjoint(Vg, wg, wb, Vb, gap_rel=1e-10)
        assert np.all(np.isfinite(Ab))
        assert np.linalg.norm(Ab - ref) <= 1e-11 * max(np.linalg.norm(ref), 1e-300)
        assert np.array_equal(Ab, Ab.T)
