"""Spectrum slicing (the reference's numnegevals, src/tridiag.jl:20-36, tested
at test/tridiag.jl:3-7) and eigenvalue subsets by Sturm-count multisection
(gla_dstebz), against the CPU oracle.
Tolerances: counts bit-identical to the oracle's recurrence; subset
eigenvalues within 32 eps ||T|| of LAPACK (scipy eigh_tridiagonal, itself
off by ~2e-14 on these cases) and within 4 eps |lambda| of a 200-bit Sturm
bisection for spot checks."""
import numpy as np
import pytest
import scipy.linalg as sl

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


def test_numnegevals_reference_case(G):
    # test/tridiag.jl:3-7
    for seed in range(5):
        rng = np.random.default_rng(seed)
        d, e = rng.standard_normal(20), rng.standard_normal(19)
        w = np.linalg.eigvalsh(np.diag(d) + np.diag(e, 1) + np.diag(e, -1))
        assert G.numnegevals(G.SymTridiagonal(d, e)) == int((w < 0).sum())


@pytest.mark.parametrize("n", [1, 2, 50, 300, 2000])
def test_numnegevals_counts_bit_identical(G, n):
    rng = np.random.default_rng(n)
    d, e = rng.standard_normal(n), rng.standard_normal(max(n - 1, 0))
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    w = np.linalg.eigvalsh(T)
    # shifts at the eigenvalues themselves, between them, on the diagonal
    # entries (zero pivots), at 0 and far outside the spectrum
    sig = np.concatenate([w, (w[:-1] + w[1:]) / 2, d, [0.0, -1e3, 1e3, np.nextafter(w[0], -np.inf)]])
    got = G.numnegevals(G.SymTridiagonal(d, e), sig)
    ref = O.numnegevals(d, e, sig)
    assert np.array_equal(got, ref)


def test_numnegevals_zero_pivot(G):
    d, e = np.array([0.0, 0.0, 2.0]), np.array([1.0, 0.5])
    for s in (0.0, 2.0, 1.0):
        assert G.numnegevals(G.SymTridiagonal(d, e), s) == O.numnegevals(d, e, s)


@pytest.mark.parametrize("case", ["random", "clustered", "wilkinson"])
def test_dstebz_subsets(G, case):
    rng = np.random.default_rng(7)
    if case == "random":
        n = 500
        d, e = rng.standard_normal(n), rng.standard_normal(n - 1)
    elif case == "clustered":  # eigenvalues in tight groups
        n = 300
        d = np.repeat(np.arange(10.0), 30) + 1e-9 * rng.standard_normal(n)
        e = 1e-7 * rng.standard_normal(n - 1)
    else:
        n = 201
        d, e = np.abs(np.arange(n) - (n - 1) / 2.0), np.ones(n - 1)
    nT = np.abs(np.linalg.eigvalsh(np.diag(d) + np.diag(e, 1) + np.diag(e, -1))).max()
    T = G.SymTridiagonal(d, e)
    for il, iu in [(1, n), (1, 1), (n, n), (n // 3, n // 3 + 17)]:
        w = G.eigvals(T, irange=(il, iu))
        ref = sl.eigh_tridiagonal(d, e, eigvals_only=True, select="i", select_range=(il - 1, iu - 1))
        assert w.shape == ref.shape
        assert np.all(np.diff(w) >= 0)
        assert np.abs(w - ref).max() <= 32 * EPS64 * nT


def test_dstebz_value_range_and_device(G):
    import torch
    rng = np.random.default_rng(9)
    n = 400
    d, e = rng.standard_normal(n), rng.standard_normal(n - 1)
    ref = sl.eigh_tridiagonal(d, e, eigvals_only=True)  # tridiagonal LAPACK: a few eps |lambda|
    vl, vu = -0.5, 1.25
    w = G.eigvals(G.SymTridiagonal(d, e), vl=vl, vu=vu)
    sel = ref[(ref > vl) & (ref <= vu)]
    assert w.shape == sel.shape and np.abs(w - sel).max() <= 32 * EPS64 * np.abs(ref).max()
    wt = G.eigvals(G.SymTridiagonal(torch.tensor(d, device="cuda"), torch.tensor(e, device="cuda")), irange=(3, 9))
    assert wt.is_cuda and np.abs(wt.cpu().numpy() - ref[2:9]).max() <= 32 * EPS64 * np.abs(ref).max()
    # eigenvalues 5 and 7 against a 200-bit Sturm bisection
    true = [mp_eigenvalue(d, e, k, ref[k]) for k in (4, 6)]
    assert abs(wt[2].item() - true[0]) <= 4 * EPS64 * abs(true[0])
    assert abs(wt[4].item() - true[1]) <= 4 * EPS64 * abs(true[1])


def mp_eigenvalue(d, e, k, guess):
    """Eigenvalue k (0-based) of SymTridiagonal(d, e) by bisection on Sturm
    counts in 200-bit arithmetic, from a bracket of +-1e-12 around guess."""
    import mpmath
    with mpmath.workprec(200):
        D = [mpmath.mpf(float(x)) for x in d]
        E2 = [mpmath.mpf(float(x)) ** 2 for x in e]

        def count(x):
            q = D[0] - x
            c = 1 if q < 0 else 0
            for j in range(len(D) - 1):
                q = (D[j + 1] - x) - E2[j] / q
                c += 1 if q < 0 else 0
            return c

        lo, hi = mpmath.mpf(float(guess)) - mpmath.mpf("1e-12"), mpmath.mpf(float(guess)) + mpmath.mpf("1e-12")
        assert count(lo) <= k < count(hi)
        for _ in range(64):
            m = (lo + hi) / 2
            if count(m) <= k:
                lo = m
            else:
                hi = m
        return float((lo + hi) / 2)


def test_host_buffer_entries(G):
    import ctypes as C
    from glagpu import _lib
    L = _lib.load()
    rng = np.random.default_rng(12)
    n = 150
    d, e = rng.standard_normal(n), rng.standard_normal(n - 1)
    sig = np.linspace(-3, 3, 41)
    counts = np.empty(len(sig), dtype=np.int64)
    p = lambda a: C.c_void_p(a.ctypes.data)
    assert L.gla_numnegevals_host(n, p(d), p(e), len(sig), p(sig), p(counts)) == 0
    assert np.array_equal(counts, O.numnegevals(d, e, sig))
    w = np.empty(10)
    assert L.gla_dstebz_host(n, p(d), p(e), 20, 29, 0.0, p(w)) == 0
    ref = sl.eigh_tridiagonal(d, e, eigvals_only=True)[19:29]
    assert np.abs(w - ref).max() <= 32 * EPS64 * 4
    assert L.gla_dstebz_host(n, p(d), p(e), 0, 3, 0.0, p(w)) == -4  # il < 1
