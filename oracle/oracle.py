"""CPU ORACLE (test infrastructure only): ctypes front end of the C++
restatement of GenericLinearAlgebra.jl's self-adjoint eigensolver
(src/eigenSelfAdjoint.jl). Imported only by tests/, the smoke check and the
CPU-baseline leg of bench.py; the shipped GPU path never calls it.

Functions mirror the reference entry points:
  syev(A, jobz, uplo)   -> _eigen!/_eigvals!(Hermitian(A, uplo))   :566-618
  heev(A, jobz, uplo)   -> the same for complex Hermitian A (T <: Complex, :462)
  heev_quaternion(...)  -> the same for quaternion Hermitian A ((n, n, 4) arrays)
  stev(d, e, jobz)      -> _eigen!/_eigvals!(SymTridiagonal(d, e)) :566,602-612
  eigql(d, e, V)        -> eigQL!/eigQR! on explicit vectors       :221-340
  symtri(A, uplo)       -> symtri!                                  :446-564
  eigenq_lmul/rmul      -> lmul!/rmul!(::EigenQ)                    :23-99
  eig2x2(d, e)          -> eig2x2!                                  :136-161
  givens(f, g)          -> givensAlgorithm (stdlib dlartg / :706-709)
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="F_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="F_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_vp = C.c_void_p
_i64 = C.c_int64
_d = C.c_double
_f = C.c_float
_ch = C.c_char
_int = C.c_int


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.gla_oracle_syev_d.argtypes = [_ch, _ch, _i64, _vp, _i64, _vp, _vp, _i64, _d, _int, _int, _i64, _vp, _vp]
        L.gla_oracle_syev_s.argtypes = [_ch, _ch, _i64, _vp, _i64, _vp, _vp, _i64, _f, _int, _int, _i64, _vp, _vp]
        L.gla_oracle_syev_q.argtypes = [_ch, _ch, _i64, _vp, _i64, _vp, _vp, _vp, _vp, _i64, _int, _int, _vp]
        L.gla_oracle_stev_d.argtypes = [_ch, _i64, _vp, _vp, _vp, _i64, _d, _int, _int, _i64, _vp]
        L.gla_oracle_stev_s.argtypes = [_ch, _i64, _vp, _vp, _vp, _i64, _f, _int, _int, _i64, _vp]
        L.gla_oracle_eigql_d.argtypes = [_i64, _vp, _vp, _vp, _i64, _i64, _d, _int, _int, _vp]
        L.gla_oracle_symtri_d.argtypes = [_ch, _i64, _vp, _i64, _vp, _vp, _vp]
        L.gla_oracle_symtri_d.restype = None
        L.gla_oracle_eigenq_lmul_d.argtypes = [_ch, _i64, _vp, _i64, _vp, _vp, _i64, _i64]
        L.gla_oracle_eigenq_lmul_d.restype = None
        L.gla_oracle_eigenq_rmul_d.argtypes = [_ch, _i64, _vp, _i64, _vp, _vp, _i64, _i64]
        L.gla_oracle_eigenq_rmul_d.restype = None
        L.gla_oracle_eig2x2_d.argtypes = [_vp, _vp, _vp, _vp, _vp]
        L.gla_oracle_eig2x2_d.restype = None
        L.gla_oracle_givens_d.argtypes = [_d, _d, _int, _vp, _vp, _vp]
        L.gla_oracle_givens_d.restype = None
        L.gla_oracle_hypot_d.argtypes = [_d, _d]
        L.gla_oracle_hypot_d.restype = _d
        L.gla_oracle_syev_batched_d.argtypes = [_ch, _ch, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _d, _int]
        L.gla_oracle_syev_batched_s.argtypes = [_ch, _ch, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _f, _int]
        L.gla_oracle_max_threads.argtypes = []
        L.gla_oracle_numnegevals_d.argtypes = [_i64, _vp, _vp, _i64, _vp, _vp]
        L.gla_oracle_numnegevals_d.restype = None
        L.gla_oracle_heev_z.argtypes = [_ch, _ch, _i64, _vp, _i64, _vp, _vp, _i64, _d]
        L.gla_oracle_symtri_z.argtypes = [_ch, _i64, _vp, _i64, _vp, _vp, _vp]
        L.gla_oracle_symtri_z.restype = None
        L.gla_oracle_heev_q.argtypes = [_ch, _ch, _i64, _vp, _i64, _vp, _vp, _i64, _d]
        L.gla_oracle_symtri_qt.argtypes = [_ch, _i64, _vp, _i64, _vp, _vp, _vp]
        L.gla_oracle_symtri_qt.restype = None
        L.gla_oracle_eigenq_lmul_qt.argtypes = [_ch, _i64, _vp, _i64, _vp, _vp, _i64, _i64]
        L.gla_oracle_eigenq_lmul_qt.restype = None
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_vp)


class OracleError(RuntimeError):
    pass


def syev(A, jobz="V", uplo="L", tol=0.0, use_qr=False, generic_givens=False, max_sweeps=-1, dtype=np.float64,
         return_stats=False):
    """_eigen!(Hermitian(A, uplo)) (jobz='V') or _eigvals!(...) (jobz='N').

    Returns (w, V, info) with w ascending; V is None for jobz='N'. A is
    copied, not overwritten."""
    A = np.array(A, dtype=dtype, order="F", copy=True)
    n = A.shape[0]
    assert A.shape == (n, n)
    w = np.zeros(n, dtype=dtype)
    V = np.zeros((n, n), dtype=dtype, order="F") if jobz == "V" else np.zeros((1, 1), dtype=dtype, order="F")
    nrot = np.zeros(1, np.int64)
    nsw = np.zeros(1, np.int64)
    fn = lib().gla_oracle_syev_d if dtype == np.float64 else lib().gla_oracle_syev_s
    info = fn(jobz.encode(), uplo.encode(), n, _p(A), max(n, 1), _p(w), _p(V), max(n, 1), tol, int(use_qr),
              int(generic_givens), max_sweeps, _p(nrot), _p(nsw))
    out = (w, V if jobz == "V" else None, info)
    if return_stats:
        return out + ({"nrot": int(nrot[0]), "nsweeps": int(nsw[0])},)
    return out


def heev(A, jobz="V", uplo="L", tol=0.0):
    """_eigen!/_eigvals!(Hermitian(A, uplo)) for complex A (the T <: Complex
    path: n-1 reflectors, complex Q, real QL rotations on complex vectors).
    Returns (w, V, info); A is copied."""
    A = np.array(A, dtype=np.complex128, order="F", copy=True)
    n = A.shape[0]
    assert A.shape == (n, n)
    w = np.zeros(n)
    V = np.zeros((n, n), dtype=np.complex128, order="F") if jobz == "V" else np.zeros((1, 1), np.complex128)
    info = lib().gla_oracle_heev_z(jobz.encode(), uplo.encode(), n, _p(A), max(n, 1), _p(w), _p(V), max(n, 1), tol)
    return w, (V if jobz == "V" else None), info


def symtri_complex(A, uplo="L"):
    """symtri!(Hermitian(A, uplo)) for complex A: returns (factors, tau, d, e)."""
    F = np.array(A, dtype=np.complex128, order="F", copy=True)
    n = F.shape[0]
    tau = np.zeros(max(n - 1, 1), dtype=np.complex128)
    d = np.zeros(n)
    e = np.zeros(max(n - 1, 1))
    lib().gla_oracle_symtri_z(uplo.encode(), n, _p(F), max(n, 1), _p(tau), _p(d), _p(e))
    return F, tau[: n - 1], d, e[: n - 1]


def _qcols(A):
    """(n, m, 4) quaternion array -> column-major storage, 4 doubles per entry."""
    return np.ascontiguousarray(np.asarray(A, dtype=np.float64).transpose(1, 0, 2))


def heev_quaternion(A, jobz="V", uplo="L", tol=0.0):
    """_eigen!/_eigvals!(Hermitian(A, uplo)) for a quaternion matrix A given
    as an (n, n, 4) array of (s, i, j, k) components. Returns (w, V, info),
    V as (n, n, 4); A is copied."""
    X = _qcols(A)
    n = X.shape[0]
    w = np.zeros(n)
    V = np.zeros((max(n, 1), max(n, 1), 4))
    info = lib().gla_oracle_heev_q(jobz.encode(), uplo.encode(), n, _p(X), max(n, 1), _p(w), _p(V), max(n, 1), tol)
    return w, (V[:n, :n].transpose(1, 0, 2).copy() if jobz == "V" else None), info


def symtri_quaternion(A, uplo="L"):
    """symtri!(Hermitian(A, uplo)) for a quaternion (n, n, 4) array: returns
    (factors (n, n, 4), tau (n-1, 4), d, e)."""
    X = _qcols(A)
    n = X.shape[0]
    tau = np.zeros((max(n - 1, 1), 4))
    d = np.zeros(n)
    e = np.zeros(max(n - 1, 1))
    lib().gla_oracle_symtri_qt(uplo.encode(), n, _p(X), max(n, 1), _p(tau), _p(d), _p(e))
    return X.transpose(1, 0, 2).copy(), tau[: n - 1], d, e[: n - 1]


def eigenq_lmul_quaternion(uplo, F, tau, B):
    """lmul!(EigenQ(uplo, F, tau), B) for quaternion factors and B ((n, m, 4)
    arrays); returns Q*B."""
    Fc = _qcols(F)
    Bc = _qcols(B)
    n, m = Bc.shape[1], Bc.shape[0]
    t = np.zeros((max(n - 1, 1), 4))
    t[: n - 1] = tau
    lib().gla_oracle_eigenq_lmul_qt(uplo.encode(), n, _p(Fc), max(n, 1), _p(t), _p(Bc), max(n, 1), m)
    return Bc.transpose(1, 0, 2).copy()


def syev_quad(A, jobz="V", uplo="L", use_qr=False, generic_givens=False):
    """Same algorithm in IEEE binary128. Returns (w_hi, w_lo, V_hi, V_lo, info)."""
    A = np.array(A, dtype=np.float64, order="F", copy=True)
    n = A.shape[0]
    whi = np.zeros(n)
    wlo = np.zeros(n)
    Vhi = np.zeros((n, n), order="F")
    Vlo = np.zeros((n, n), order="F")
    nrot = np.zeros(1, np.int64)
    info = lib().gla_oracle_syev_q(jobz.encode(), uplo.encode(), n, _p(A), max(n, 1), _p(whi), _p(wlo), _p(Vhi),
                                   _p(Vlo), max(n, 1), int(use_qr), int(generic_givens), _p(nrot))
    return whi, wlo, (Vhi if jobz == "V" else None), (Vlo if jobz == "V" else None), info


def stev(d, e, jobz="V", tol=0.0, use_qr=False, generic_givens=False, max_sweeps=-1, dtype=np.float64):
    """_eigen!/_eigvals!(SymTridiagonal(d, e)). Returns (w, V, info)."""
    d = np.array(d, dtype=dtype, copy=True)
    n = d.shape[0]
    e = np.array(e, dtype=dtype, copy=True) if n > 1 else np.zeros(1, dtype=dtype)
    V = np.zeros((n, n), dtype=dtype, order="F") if jobz == "V" else np.zeros((1, 1), dtype=dtype, order="F")
    nrot = np.zeros(1, np.int64)
    fn = lib().gla_oracle_stev_d if dtype == np.float64 else lib().gla_oracle_stev_s
    info = fn(jobz.encode(), n, _p(d), _p(e), _p(V), max(n, 1), tol, int(use_qr), int(generic_givens), max_sweeps,
              _p(nrot))
    return d, (V if jobz == "V" else None), info


def eigql(d, e, V, tol=0.0, use_qr=False, generic_givens=False):
    """eigQL!(SymTridiagonal(d, e); vectors=V) without sorting (V: m x n, m <= n).
    Returns (d, e, V, info), all copies."""
    d = np.array(d, dtype=np.float64, copy=True)
    n = d.shape[0]
    e = np.array(e, dtype=np.float64, copy=True) if n > 1 else np.zeros(1)
    V = np.array(V, dtype=np.float64, order="F", copy=True)
    m = V.shape[0]
    nrot = np.zeros(1, np.int64)
    info = lib().gla_oracle_eigql_d(n, _p(d), _p(e), _p(V), max(m, 1), m, tol, int(use_qr), int(generic_givens),
                                    _p(nrot))
    return d, e, V, info


def symtri(A, uplo="L"):
    """symtri!(Hermitian(A, uplo)): returns (factors, tau, d, e)."""
    F = np.array(A, dtype=np.float64, order="F", copy=True)
    n = F.shape[0]
    tau = np.zeros(max(n - 1, 1))
    d = np.zeros(n)
    e = np.zeros(max(n - 1, 1))
    lib().gla_oracle_symtri_d(uplo.encode(), n, _p(F), max(n, 1), _p(tau), _p(d), _p(e))
    return F, tau[: n - 1], d, e[: n - 1]


def eigenq_lmul(uplo, F, tau, B):
    """lmul!(EigenQ(uplo, F, tau), B) on copies; returns (Q*B, F_after)."""
    F = np.array(F, dtype=np.float64, order="F", copy=True)
    B = np.array(B, dtype=np.float64, order="F", copy=True)
    n = F.shape[0]
    t = np.zeros(max(n - 1, 1))
    t[: n - 1] = tau
    lib().gla_oracle_eigenq_lmul_d(uplo.encode(), n, _p(F), max(n, 1), _p(t), _p(B), max(n, 1), B.shape[1])
    return B, F


def eigenq_rmul(uplo, F, tau, B):
    """rmul!(B, EigenQ(uplo, F, tau)) on copies; returns (B*Q, F_after)."""
    F = np.array(F, dtype=np.float64, order="F", copy=True)
    B = np.array(B, dtype=np.float64, order="F", copy=True)
    n = F.shape[0]
    t = np.zeros(max(n - 1, 1))
    t[: n - 1] = tau
    lib().gla_oracle_eigenq_rmul_d(uplo.encode(), n, _p(F), max(n, 1), _p(t), _p(B), max(B.shape[0], 1),
                                   B.shape[0])
    return B, F


def eig2x2(d, e):
    """eig2x2!(d, e, 1, I(2)): returns (d_after, e_after, V, c, s)."""
    d = np.array(d, dtype=np.float64, copy=True)
    e = np.array(e, dtype=np.float64, copy=True)
    V = np.eye(2, order="F")
    c = np.zeros(1)
    s = np.zeros(1)
    lib().gla_oracle_eig2x2_d(_p(d), _p(e), _p(V), _p(c), _p(s))
    return d, e, V, float(c[0]), float(s[0])


def givens(f, g, generic=False):
    c = np.zeros(1)
    s = np.zeros(1)
    r = np.zeros(1)
    lib().gla_oracle_givens_d(f, g, int(generic), _p(c), _p(s), _p(r))
    return float(c[0]), float(s[0]), float(r[0])


def hypot(x, y):
    return lib().gla_oracle_hypot_d(x, y)


def syev_batched(mats, jobz="V", uplo="L", dtype=np.float64, nthreads=0):
    """Batched _eigen! over a list of square matrices, one matrix per OpenMP
    thread. Returns (list of w, list of V or None, info array)."""
    ns = np.array([m.shape[0] for m in mats], dtype=np.int64)
    aoff = np.zeros(len(mats), np.int64)
    woff = np.zeros(len(mats), np.int64)
    if len(mats) > 1:
        aoff[1:] = np.cumsum(ns * ns)[:-1]
        woff[1:] = np.cumsum(ns)[:-1]
    A = np.concatenate([np.asarray(m, dtype=dtype).ravel(order="F") for m in mats]) if mats else np.zeros(1, dtype)
    w = np.zeros(max(int(ns.sum()), 1), dtype)
    V = np.zeros(max(int((ns * ns).sum()), 1), dtype) if jobz == "V" else None
    info = np.zeros(max(len(mats), 1), np.int32)
    fn = lib().gla_oracle_syev_batched_d if dtype == np.float64 else lib().gla_oracle_syev_batched_s
    fn(jobz.encode(), uplo.encode(), len(mats), _p(ns), _p(aoff), _p(A), _p(w), _p(woff),
       _p(V) if V is not None else None, _p(info), 0.0, nthreads)
    ws = [w[woff[b]: woff[b] + ns[b]].copy() for b in range(len(mats))]
    Vs = None
    if V is not None:
        Vs = [V[aoff[b]: aoff[b] + ns[b] * ns[b]].reshape(ns[b], ns[b], order="F").copy() for b in range(len(mats))]
    return ws, Vs, info[: len(mats)]


def batched_raw(jobz, uplo, ns, aoff, A, w, woff, V, info, dtype=np.float64, nthreads=0):
    """Zero-copy batched call on caller-owned packed numpy arenas (for timing)."""
    fn = lib().gla_oracle_syev_batched_d if dtype == np.float64 else lib().gla_oracle_syev_batched_s
    return fn(jobz.encode(), uplo.encode(), len(ns), _p(ns), _p(aoff), _p(A), _p(w), _p(woff),
              _p(V) if V is not None else None, _p(info), 0.0, nthreads)


def numnegevals(d, e, sigma=0.0):
    """numnegevals(SymTridiagonal(d, e), sigma) (src/tridiag.jl:20-36); sigma
    may be a scalar or an array of shifts (one count per shift)."""
    d = np.ascontiguousarray(d, dtype=np.float64)
    e = np.ascontiguousarray(e, dtype=np.float64)
    sig = np.atleast_1d(np.ascontiguousarray(sigma, dtype=np.float64))
    out = np.zeros(len(sig), dtype=np.int64)
    lib().gla_oracle_numnegevals_d(len(d), _p(d), _p(e), len(sig), _p(sig), _p(out))
    return int(out[0]) if np.ndim(sigma) == 0 else out


def max_threads():
    return lib().gla_oracle_max_threads()
