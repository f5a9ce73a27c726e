"""CPU model (numpy, FP64) of a two-stage symmetric tridiagonal reduction,
the form planned for the FP32 large-order path in place of the one-stage
reduction that follows the reference's symtriLower!
(src/eigenSelfAdjoint.jl:450-504). Test infrastructure: it fixes the task
structure and the intermediate results (the band matrix, the tridiagonal,
the reflectors) that GPU kernels of that form are to be checked against.

1. Dense -> band of half-width b (sy2sb): per panel of b columns, a
   Householder QR of the rows below the band (compact WY: Q = I - V T V',
   T upper triangular as LAPACK's larft forms it), then the two-sided
   update of the trailing matrix as a symmetric rank-2b update
   A22 <- A22 - V W' - W V', W = A22 V T - V (T' V' A22 V T) / 2.
2. Band -> tridiagonal (sb2st) by Householder bulge chasing: sweep j
   annihilates column j below the subdiagonal; each task of a sweep applies
   one reflector of length <= b to rows and columns r0 .. r1 - 1
   two-sidedly, which fills a bulge b rows further down that the next task
   of the sweep removes.
3. Back-transform X = Q1 Q2 Z for the tridiagonal's eigenvectors Z.

Reflectors follow LAPACK's dlarfg convention (Golub and Van Loan 5.1):
v[0] = 1, beta = -sign(x0) ||x||, tau = (beta - x0) / beta, as the
reference's reflector! does.
"""
import numpy as np


def house(x):
    """(v, tau, beta) with (I - tau v v') x = beta e1 and v[0] = 1."""
    alpha = x[0]
    sigma = float(np.dot(x[1:], x[1:]))
    v = np.zeros_like(x)
    v[0] = 1.0
    if sigma == 0.0:
        return v, 0.0, alpha
    beta = -np.copysign(np.sqrt(alpha * alpha + sigma), alpha)
    v[1:] = x[1:] / (alpha - beta)
    return v, (beta - alpha) / beta, beta


def panel_qr(P):
    """Householder QR of an m x b panel: V (m x b, unit lower), T (b x b,
    upper, Q = I - V T V'), R (b x b upper)."""
    m, b = P.shape
    P = P.copy()
    V = np.zeros((m, b))
    taus = np.zeros(b)
    for j in range(min(b, m)):
        v, tau, _ = house(P[j:, j])
        V[j:, j] = v
        taus[j] = tau
        P[j:, j:] -= tau * np.outer(v, v @ P[j:, j:])
    T = np.zeros((b, b))
    for j in range(b):  # forward accumulation (larft, direct 'F', storev 'C')
        T[j, j] = taus[j]
        if j:
            T[:j, j] = -taus[j] * T[:j, :j] @ (V[:, :j].T @ V[:, j])
    return V, T, np.triu(P[:b, :b])


def mirror_lower(S):
    """The lower triangle of S mirrored: the matrix a kernel storing only the
    lower triangle holds."""
    L = np.tril(S)
    return L + np.tril(S, -1).T


def sy2sb(A, b):
    """Dense symmetric A -> band of half-width b (returned dense), and the
    panels (row offset r0, V, T): Q1 = prod_k (I - V_k T_k V_k') on rows r0..."""
    A = np.array(A, dtype=float)
    n = A.shape[0]
    panels = []
    for k in range(0, n - b - 1, b):
        r0 = k + b
        V, T, R = panel_qr(A[r0:, k:k + b])
        A[r0:, k:k + b] = 0.0
        A[r0:r0 + b, k:k + b] = R
        A[k:k + b, r0:] = A[r0:, k:k + b].T
        A22 = A[r0:, r0:]
        W = A22 @ V @ T
        W -= 0.5 * V @ (T.T @ (V.T @ W))
        A[r0:, r0:] = mirror_lower(A22 - V @ W.T - W @ V.T)
        panels.append((r0, V, T))
    return A, panels


def sb2st_tasks(n, b):
    """The bulge-chasing tasks in program order: (sweep j, task t, r0, r1,
    lo, hi). Task (j, t) applies a reflector on rows r0 .. r1 - 1; it reads
    and writes rows and columns lo .. hi - 1 (the annihilated column r0 - b,
    or j for t = 0, through the bulge it fills down to r1 + b)."""
    for j in range(n - 2):
        r0, t = j + 1, 0
        while r0 < n and min(r0 + b, n) - r0 >= 2:
            r1 = min(r0 + b, n)
            yield j, t, r0, r1, max(0, r0 - b), min(n, r1 + b)
            r0 = r1
            t += 1


def sb2st(B, b):
    """Band (half-width b) -> tridiagonal by Householder bulge chasing.
    Returns the tridiagonal (dense) and the reflectors (j, t, r0, v, tau)."""
    B = np.array(B, dtype=float)
    n = B.shape[0]
    refl = []
    for j, t, r0, r1, lo, hi in sb2st_tasks(n, b):
        c = j if t == 0 else r0 - b  # the column this task annihilates
        v, tau, _ = house(B[r0:r1, c].copy())
        if tau != 0.0:
            H = np.eye(r1 - r0) - tau * np.outer(v, v)
            B[r0:r1, lo:hi] = H @ B[r0:r1, lo:hi]
            B[lo:hi, r0:r1] = B[lo:hi, r0:r1] @ H
            B[lo:hi, lo:hi] = mirror_lower(B[lo:hi, lo:hi])
        B[r0 + 1:r1, c] = 0.0
        B[c, r0 + 1:r1] = 0.0
        refl.append((j, t, r0, v, tau))
    return B, refl


def q1_apply(panels, Z):
    """Q1 Z (the last panel's reflectors first)."""
    Z = np.array(Z, dtype=float)
    for r0, V, T in reversed(panels):
        Z[r0:] -= V @ (T @ (V.T @ Z[r0:]))
    return Z


def q2_apply(refl, Z):
    """Q2 Z, Q2 the product of the sweeps' reflectors in program order."""
    Z = np.array(Z, dtype=float)
    for _, _, r0, v, tau in reversed(refl):
        r1 = r0 + len(v)
        Z[r0:r1] -= tau * np.outer(v, v @ Z[r0:r1])
    return Z


def q2_apply_blocked(refl, Z, b, nb):
    """Q2 Z with the reflectors grouped in compact-WY blocks: group (J, t)
    holds task t of sweeps J .. J + nb - 1 (nb <= b), rows J + 1 + t b ..
    J + nb + t b + b - 1, one (b + nb - 1) x nb block V and nb x nb T.
    Groups are applied for J descending and, within J, t ascending, each as
    I - V T V' (its sweeps descending). Two reflectors whose order this
    changes against q2_apply act on disjoint rows (nb <= b), so the result
    is the same up to rounding; each group is one GEMM pair over all of Z's
    columns instead of nb rank-1 updates."""
    assert nb <= b
    Z = np.array(Z, dtype=float)
    n = Z.shape[0]
    by = {}
    for j, t, r0, v, tau in refl:
        by[(j, t)] = (r0, v, tau)
    nsweep = max(j for j, _, _, _, _ in refl) + 1 if refl else 0
    for J in reversed(range(0, nsweep, nb)):
        ts = sorted({t for (j, t) in by if J <= j < J + nb})
        for t in ts:
            members = [(j,) + by[(j, t)] for j in range(J, min(J + nb, nsweep)) if (j, t) in by]
            lo = min(r0 for _, r0, _, _ in members)
            hi = max(r0 + len(v) for _, r0, v, _ in members)
            k = len(members)
            V = np.zeros((hi - lo, k))
            taus = np.zeros(k)
            for c, (_, r0, v, tau) in enumerate(members):  # sweeps ascending
                V[r0 - lo:r0 - lo + len(v), c] = v
                taus[c] = tau
            T = np.zeros((k, k))
            for c in range(k):
                T[c, c] = taus[c]
                if c:
                    T[:c, c] = -taus[c] * T[:c, :c] @ (V[:, :c].T @ V[:, c])
            Z[lo:hi] -= V @ (T @ (V.T @ Z[lo:hi]))
    return Z


def critical_path(n, b):
    """(tasks, critical path in tasks, widest step) of the bulge chase with
    unit-time tasks, each after every earlier task that touched one of the
    lower-band entries it touches: the latency floor of a GPU schedule of
    the sweeps. Task (j, t) reads and writes rows r0 .. r1 - 1, columns
    c .. r1 - 1 (c the column it annihilates: its left update and the
    diagonal block) and rows r1 .. r1 + b - 1, columns r0 .. r1 - 1 (its
    right update, which fills the bulge)."""
    last = np.zeros((n, n), dtype=np.int64)
    count, width = 0, {}
    for j, t, r0, r1, _, _ in sb2st_tasks(n, b):
        c = j if t == 0 else r0 - b
        r2 = min(n, r1 + b)
        s = int(last[r0:r1, c:r1].max())
        if r2 > r1:
            s = max(s, int(last[r1:r2, r0:r1].max()))
            last[r1:r2, r0:r1] = s + 1
        last[r0:r1, c:r1] = s + 1
        count += 1
        width[s] = width.get(s, 0) + 1
    return count, int(last.max()), max(width.values()) if width else 0
