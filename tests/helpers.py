"""Shared test helpers: seeded inputs and comparison metrics."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.json")
GOLDEN_LARGE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_large.json")


def golden():
    with open(GOLDEN) as f:
        return json.load(f)


def golden_large(n):
    """The 256-bit fixture of order n in golden_large.json: (A, w256, V256),
    w256 the eigenvalues rounded to float64, V256 the eigenvectors."""
    import mpmath
    with open(GOLDEN_LARGE) as f:
        g = [c for c in json.load(f)["goe"] if c["n"] == n][0]
    A = from_hex(g["A"])
    return A, np.array([float(mpmath.mpf(v)) for v in g["w"]]), np.array(g["V"]), g["seed"]


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


# ---- quaternion matrices as (m, n, 4) arrays of (s, i, j, k) components ----

def qmul(A, B):
    """Quaternion matrix product (m, k, 4) x (k, n, 4), Hamilton's rules."""
    a0, a1, a2, a3 = (A[..., m] for m in range(4))
    b0, b1, b2, b3 = (B[..., m] for m in range(4))
    return np.stack([a0 @ b0 - a1 @ b1 - a2 @ b2 - a3 @ b3,
                     a0 @ b1 + a1 @ b0 + a2 @ b3 - a3 @ b2,
                     a0 @ b2 - a1 @ b3 + a2 @ b0 + a3 @ b1,
                     a0 @ b3 + a1 @ b2 - a2 @ b1 + a3 @ b0], -1)


def qH(A):
    B = np.swapaxes(A, 0, 1).copy()
    B[..., 1:] *= -1
    return B


def qeye(n):
    Z = np.zeros((n, n, 4))
    Z[..., 0] = np.eye(n)
    return Z


def chi(A):
    Z1 = A[..., 0] + 1j * A[..., 1]
    Z2 = A[..., 2] + 1j * A[..., 3]
    return np.block([[Z1, Z2], [-Z2.conj(), Z1.conj()]])


def qnorm(A):
    return np.linalg.norm(chi(A), 2)


def qunitary(n, rng):
    """A random unitary quaternion matrix (Gram-Schmidt on Gaussian columns)."""
    X = rng.standard_normal((n, n, 4))
    Q = np.zeros_like(X)
    for j in range(n):
        r = X[:, j:j + 1]
        for _ in range(2):
            for q in range(j):
                v = Q[:, q:q + 1]
                r = r - qmul(v, qmul(qH(v), r))
        Q[:, j:j + 1] = r / np.sqrt((r ** 2).sum())
    return Q


def qherm_spectrum(lam, rng):
    n = len(lam)
    U = qunitary(n, rng)
    D = np.zeros((n, n, 4))
    D[..., 0] = np.diag(lam)
    A = qmul(qmul(U, D), qH(U))
    return (A + qH(A)) / 2


def qherm_random(n, rng):
    B = rng.standard_normal((n, n, 4))
    return (B + qH(B)) / 2
