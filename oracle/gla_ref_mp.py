"""CPU ORACLE (test infrastructure only): the self-adjoint eigensolver of
GenericLinearAlgebra.jl v0.4.0 restated over mpmath at 256 bits — the
counterpart of running the reference on BigFloat (precision 256, Julia's
default). Pure Python: use for n <= ~40; results are cached as golden
fixtures by tests/golden/make_golden.py.

Follows src/eigenSelfAdjoint.jl: symtriLower! :450-504 (reflector! and the
symv/rank-2 loops), Array(EigenQ) :101 / lmul! :23-41, eigQL! :221-288 with
singleShiftQL! :377-409, eig2x2! :136-161, eigvalsPWK! :163-219 with
singleShiftQLPWK! :343-374, sorteig! (stable ascending). Givens rotations
use the stdlib dlartg convention (r = +-sqrt(f^2+g^2), sign fixed so that
c > 0 when |f| > |g|); tol = eps(BigFloat) = 2^-255.
"""
import mpmath

PREC = 256


def _ctx():
    ctx = mpmath.mp.clone()
    ctx.prec = PREC
    return ctx


def eps(ctx):
    return ctx.mpf(2) ** (1 - PREC)


def _reflector(ctx, x):
    """LinearAlgebra.reflector!: in place on list x, returns tau."""
    if not x:
        return ctx.mpf(0)
    xi1 = x[0]
    normu = ctx.sqrt(ctx.fsum(v * v for v in x))
    if normu == 0:
        return ctx.mpf(0)
    nu = normu if xi1 >= 0 else -normu
    xi1 = xi1 + nu
    x[0] = -nu
    for i in range(1, len(x)):
        x[i] = x[i] / xi1
    return xi1 / nu


def symtri_lower(ctx, A):
    """A: list of lists (n x n, lower triangle used), modified in place.
    Returns (tau, d, e)."""
    n = len(A)
    tau = [ctx.mpf(0)] * max(n - 1, 0)
    for k in range(n - 2):
        m = n - k - 1
        x = [A[k + 1 + i][k] for i in range(m)]
        tk = _reflector(ctx, x)
        tau[k] = tk
        beta = x[0]
        x[0] = ctx.mpf(1)
        for i in range(1, m):
            A[k + 1 + i][k] = x[i]
        # u = tk * At * x with At the lower-triangle symmetric trailing block
        u = []
        for i in range(m):
            s = ctx.mpf(0)
            for j in range(m):
                a = A[k + 1 + i][k + 1 + j] if j <= i else A[k + 1 + j][k + 1 + i]
                s += a * x[j]
            u.append(tk * s)
        xi = tk * ctx.fsum(x[i] * u[i] for i in range(m))
        for j in range(m):
            for i in range(j, m):
                A[k + 1 + i][k + 1 + j] += x[i] * (xi * x[j]) - x[i] * u[j] - u[i] * x[j]
        A[k + 1][k] = beta
    d = [A[i][i] for i in range(n)]
    e = [A[i + 1][i] for i in range(n - 1)]
    return tau, d, e


def form_q(ctx, A, tau):
    """Array(EigenQ('L', A, tau)) = H_1 ... H_{n-2} applied to I (lmul!)."""
    n = len(A)
    Q = [[ctx.mpf(1) if i == j else ctx.mpf(0) for j in range(n)] for i in range(n)]
    for k in range(n - 1, 0, -1):  # 1-based k = n-1 .. 1
        t = tau[k - 1]
        h = [ctx.mpf(1)] + [A[i][k - 1] for i in range(k + 1, n)]
        for j in range(n):
            tmp = t * ctx.fsum(h[i] * Q[k + i][j] for i in range(n - k))
            for i in range(n - k):
                Q[k + i][j] -= h[i] * tmp
    return Q


def _givens(ctx, f, g):
    if g == 0:
        return ctx.mpf(1), ctx.mpf(0), f
    if f == 0:
        return ctx.mpf(0), ctx.mpf(1), g
    r = ctx.sqrt(f * f + g * g)
    c, s = f / r, g / r
    if abs(f) > abs(g) and c < 0:
        c, s, r = -c, -s, -r
    return c, s, r


def _update(V, c, s, j):
    for row in V:
        v1, v2 = row[j + 1], row[j]
        row[j + 1] = c * v1 + s * v2
        row[j] = c * v2 - s * v1


def _blockend(ctx, d, e, n, bs, tol):
    for be in range(bs + 1, n):
        if abs(e[be - 1]) <= tol * ctx.sqrt(abs(d[be - 1])) * ctx.sqrt(abs(d[be])):
            return be - 1
    return n - 1


def eig_ql(ctx, d, e, V, tol, max_sweeps=None):
    n = len(d)
    cap = max_sweeps if max_sweeps is not None else 30 * n
    bs, sweeps = 0, 0
    if n <= 1:
        return 0
    while True:
        be = _blockend(ctx, d, e, n, bs, tol)
        if bs == be:
            bs += 1
        elif bs + 1 == be:
            dj, dj1, ej = d[bs], d[be], e[bs]
            r1 = (dj + dj1) / 2
            r2 = ctx.hypot(dj - dj1, 2 * ej) / 2
            lp, lm = r1 + r2, r1 - r2
            d[bs], d[be], e[bs] = lp, lm, ctx.mpf(0)
            if ej == 0:
                c, s = ctx.mpf(1), ctx.mpf(0)
            elif abs(lp - dj) > abs(lm - dj):
                c = -ej / ctx.hypot(ej, lp - dj)
                s = ctx.sqrt(1 - c * c)
            else:
                s = abs(ej) / ctx.hypot(ej, lm - dj)
                c = ctx.sqrt(1 - s * s)
                c = c if -ej >= 0 else -c
            _update(V, c, s, bs)
            bs += 2
        else:
            if sweeps >= cap:
                return 1
            mu = (d[bs + 1] - d[bs]) / (2 * e[bs])
            r = ctx.hypot(mu, 1)
            mu = d[bs] - e[bs] / (mu + (r if mu >= 0 else -r))
            g = d[be] - mu
            p = g
            ci, si = ctx.mpf(1), ctx.mpf(0)
            for i in range(be - 1, bs - 1, -1):
                ei = e[i]
                ci1, si1 = ci, si
                ci, si, zeta = _givens(ctx, p, ei)
                if i < be - 1:
                    e[i + 1] = si1 * zeta
                di = d[i]
                g1 = g
                g = ci * ci * (di - mu) - si * si * g1
                d[i + 1] = g1 + di - g
                p = -ei * ci1 if ci == 0 else g / ci
                _update(V, ci, si, i)
            e[bs] = si * p
            d[bs] = mu + g
            sweeps += 1
        if bs >= n - 1:
            return 0


def eigvals_pwk(ctx, d, e, tol, max_sweeps=None):
    n = len(d)
    cap = max_sweeps if max_sweeps is not None else 30 * n
    e[:] = [v * v for v in e]
    bs, sweeps = 0, 0
    if n <= 1:
        return 0
    while True:
        be = _blockend(ctx, d, e, n, bs, tol)
        if bs == be:
            bs += 1
        elif bs + 1 == be:
            r1 = (d[bs] + d[be]) / 2
            r2 = ctx.hypot(d[bs] - d[be], 2 * ctx.sqrt(e[bs])) / 2
            d[bs], d[be] = r1 + r2, r1 - r2
            e[bs] = ctx.mpf(0)
            bs += 1
        else:
            if sweeps >= cap:
                return 1
            sq = ctx.sqrt(e[bs])
            mu = (d[bs + 1] - d[bs]) / (2 * sq)
            r = ctx.hypot(mu, 1)
            mu = d[bs] - sq / (mu + (r if mu >= 0 else -r))
            g = d[be] - mu
            p = g * g
            ci, s = ctx.mpf(1), ctx.mpf(0)
            for i in range(be - 1, bs - 1, -1):
                ei = e[i]
                zeta = p + ei
                if i < be - 1:
                    e[i + 1] = s * zeta
                ci1 = ci
                ci = p / zeta
                s = ei / zeta
                di = d[i]
                g1 = g
                g = ci * (di - mu) - s * g1
                d[i + 1] = g1 + di - g
                p = ei * ci1 if ci == 0 else g * g / ci
            e[bs] = s * p
            d[bs] = mu + g
            sweeps += 1
        if bs >= n - 1:
            return 0


def syev(A_rows, jobz="V"):
    """_eigen!/_eigvals!(Hermitian(A, :L)) at 256 bits. A_rows: n x n nested
    sequence of numbers or decimal strings. Returns (w, V) as lists of mpf
    (V[i][j], column j = eigenvector j), ascending."""
    ctx = _ctx()
    A = [[ctx.mpf(v) for v in row] for row in A_rows]
    n = len(A)
    tol = eps(ctx)
    tau, d, e = symtri_lower(ctx, A)
    if jobz == "N":
        eigvals_pwk(ctx, d, e, tol)
        return sorted(d), None
    V = form_q(ctx, A, tau)
    eig_ql(ctx, d, e, V, tol)
    order = sorted(range(n), key=lambda i: d[i])
    w = [d[i] for i in order]
    Vs = [[V[r][i] for i in order] for r in range(n)]
    return w, Vs
