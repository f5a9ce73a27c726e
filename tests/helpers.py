"""Shared test helpers: seeded inputs and comparison metrics."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.json")


def golden():
    with open(GOLDEN) as f:
        return json.load(f)


def goe(n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    B = rng.standard_normal((n, n))
    return (B + B.T) / 2


def haar(n, rng):
    Q, R = np.linalg.qr(rng.standard_normal((n, n)))
    return Q * np.sign(np.diag(R))


def prescribed(lam, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    Q = haar(len(lam), rng)
    A = (Q * lam) @ Q.T
    return (A + A.T) / 2


def from_hex(rows):
    return np.array([[float.fromhex(v) for v in row] for row in rows])


def sym_from(A, uplo):
    """The symmetric matrix the solver sees when only the uplo triangle is read."""
    L = np.tril(A) if uplo == "L" else np.triu(A)
    return L + L.T - np.diag(np.diag(A))


def residual(A, V, w):
    nA = np.linalg.norm(A, 2)
    if nA == 0:
        return float(np.linalg.norm(A @ V - V * w, 2))
    return float(np.linalg.norm(A @ V - V * w, 2) / nA)


def orth(V):
    return float(np.linalg.norm(V.T @ V - np.eye(V.shape[1]), 2))


def signfix(V):
    V = np.array(V, dtype=np.float64, copy=True)
    idx = np.argmax(np.abs(V), axis=0)
    s = np.sign(V[idx, np.arange(V.shape[1])])
    s[s == 0] = 1
    return V * s


def vec_parity(A, V1, V2, w, tol_factor=1.0):
    """Columns of V1, V2 agree (after sign normalisation) wherever the
    eigenvalue is separated; returns the worst ratio error/bound (<= 1 ok).
    Bound: 100 * n * eps * ||A|| / gap (first-order perturbation theory)."""
    n = len(w)
    nA = max(np.linalg.norm(A, 2), 1e-300)
    worst = 0.0
    V1 = signfix(V1)
    V2 = signfix(V2)
    for j in range(n):
        gaps = np.abs(np.delete(w, j) - w[j]) if n > 1 else np.array([np.inf])
        gap = gaps.min() if len(gaps) else np.inf
        if gap <= 1e-10 * nA:
            continue
        bound = tol_factor * 100 * n * 2.2e-16 * nA / gap
        err = min(np.linalg.norm(V1[:, j] - V2[:, j]), np.linalg.norm(V1[:, j] + V2[:, j]))
        worst = max(worst, err / max(bound, 1e-15))
    return worst


def gapped_spectrum(n, rng, gap=1e-3):
    """Sorted values in [-1, 1] with consecutive gaps >= gap (the adjoint configuration)."""
    u = np.sort(rng.random(n))
    return -1.0 + (2.0 - (n - 1) * gap) * u + gap * np.arange(n)


def analytic_adjoint(V, w, wbar, Vbar, gap_rel=1e-10):
    """Abar = V (diag(wbar) + sym(F o V'Vbar)) V' in numpy (FP64)."""
    n = len(w)
    G = V.T @ Vbar
    dl = w[None, :] - w[:, None]  # lam_j - lam_i
    with np.errstate(divide="ignore"):
        F = np.where(np.abs(dl) > gap_rel * np.abs(w).max(), 1.0 / np.where(dl == 0, 1, dl), 0.0)
    np.fill_diagonal(F, 0.0)
    M = 0.5 * (F * G + (F * G).T) + np.diag(wbar)
    return V @ M @ V.T
