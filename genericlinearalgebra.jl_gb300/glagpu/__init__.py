"""glagpu — Python host mirror of GenericLinearAlgebra.jl's self-adjoint
eigensolver API, running on the GB300 kernels of libglagpu.so.

Reference interface (GenericLinearAlgebra.jl v0.4.0, src/eigenSelfAdjoint.jl)
and the functions here that mirror it:

  eigen!(Hermitian/Symmetric)   :626-630   -> eigen(A, uplo=...)       (copying)
  eigvals!(Hermitian/Symmetric) :584-588   -> eigvals(A, uplo=...)
  eigen!(SymTridiagonal)        :623       -> eigen(SymTridiagonal(dv, ev))
  eigvals!(SymTridiagonal)      :581       -> eigvals(SymTridiagonal(dv, ev))
  eigQR!                        :290-340   -> alg="QR"
  eigen2                        :633-668   -> eigen2(A)
  symtri! / EigenQ              :6-118, :446-564 -> symtri(A, uplo) / EigenQ.lmul, rmul, array
  eigen!(Hermitian{<:Complex})  :462       -> eigen(A) with complex A
  eigen!(Hermitian{Quaternion}) (test/eigenselfadjoint.jl:54-84) -> eigen(QuaternionMatrix(A))
  numnegevals                   src/tridiag.jl:20-36 -> numnegevals(T, sigma)
  keyword tol = eps(T)          :566-630   -> tol=None (eps of the precision)
  keyword sortby = eigsortby    :592-599   -> sortby=eigsortby (ascending), any key function,
                                              or None (no particular order)
  LinearAlgebra.Eigen                      -> Eigen(values, vectors)

Beside the reference's plain path, precision="f32_refined" runs the FP32
solve plus FP64 Ogita-Aishima refinement, and Plan / eigen_batched solve
thousands of matrices per launch sequence.

Inputs are torch CUDA tensors (results stay on the device) or numpy arrays
(host buffers: copied in and out by the library, results as numpy). Errors:
DimensionMismatch for shape errors (as the reference raises at :230-243),
NonConvergenceError(info) when a chase hits its sweep cap (the reference
would loop forever; LAPACK-style info as in src/lapack.jl:62) and
NonFiniteError for NaN/Inf input.
"""
import ctypes as C
from collections import namedtuple

import numpy as np

from . import _lib
from ._lib import GLA_ALG_QL, GLA_ALG_QR, GLA_MAX_N, GLA_MAX_SMALL_N, GLAError

Eigen = namedtuple("Eigen", ["values", "vectors"])

PRECISIONS = {"f64": _lib.GLA_PREC_F64, "f32": _lib.GLA_PREC_F32, "f32_refined": _lib.GLA_PREC_F32_REFINED}


class DimensionMismatch(ValueError):
    pass


class NonConvergenceError(RuntimeError):
    """Raised when info > 0 for some matrix (sweep cap reached)."""

    def __init__(self, info):
        self.info = info
        super().__init__(f"eigensolver did not converge (info = {info})")


class NonFiniteError(ValueError):
    """Raised when the referenced triangle holds NaN or Inf (info == -1)."""


def _torch():
    import torch
    return torch


def _is_torch(x):
    try:
        import torch
    except ImportError:
        return False
    return isinstance(x, torch.Tensor)


def _stream_ptr(stream=None):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


class SymTridiagonal:
    """SymTridiagonal(dv, ev): diagonal (n) and off-diagonal (n-1)."""

    def __init__(self, dv, ev):
        self.dv = dv
        self.ev = ev
        n = len(dv)
        if len(ev) != max(n - 1, 0):
            raise DimensionMismatch(f"off-diagonal has length {len(ev)}, expected {max(n - 1, 0)}")


def _raise_for_info(info):
    info = np.asarray(info)
    if (info == -1).any():
        raise NonFiniteError("input contains NaN or Inf")
    if (info > 0).any():
        raise NonConvergenceError(int(info[info > 0][0]))


class Plan:
    """Batched solver plan over matrices of orders `ns` (each <= GLA_MAX_N;
    orders above GLA_MAX_SMALL_N = 128 run the blocked large-matrix path).

    Arena layout: matrix b is column-major n_b x n_b at offset sum(n_c^2, c<b);
    its eigenvalues at sum(n_c, c<b). precision: "f64", "f32", "f32_refined".
    refine_ql: for "f32_refined", run the FP32 stage with the QL chase instead
    of the per-eigenvalue solver (GLA_FLAG_REFINE_QL). bisect: for "f32", use
    that per-eigenvalue solver instead of the QL chase (GLA_FLAG_F32_BISECT).
    refine_simt: for "f32_refined", the refinement's double-float products on
    the FP32 pipe instead of the tensor cores (GLA_FLAG_REFINE_SIMT).
    """

    def __init__(self, ns, precision="f64", jobz="V", uplo="L", tol=None, alg="QL", small_log=False,
                 timing=False, graph=False, autotune=False, refine_ql=False, bisect=False,
                 refine_simt=False):
        L = _lib.load()
        ns = np.ascontiguousarray(np.asarray(ns, dtype=np.int64))
        if (ns < 0).any() or (ns > GLA_MAX_N).any():
            raise DimensionMismatch(f"orders must lie in [0, {GLA_MAX_N}]")
        self.ns = ns
        self.precision = precision
        self.jobz = jobz
        self.uplo = uplo
        self.dtype = np.float32 if precision == "f32" else np.float64
        flags = (GLA_ALG_QR if alg == "QR" else GLA_ALG_QL) | (_lib.GLA_FLAG_SMALL_LOG if small_log else 0) | \
            (_lib.GLA_FLAG_TIMING if timing else 0) | (_lib.GLA_FLAG_GRAPH if graph else 0) | \
            (_lib.GLA_FLAG_AUTOTUNE if autotune else 0) | (_lib.GLA_FLAG_REFINE_QL if refine_ql else 0) | \
            (_lib.GLA_FLAG_F32_BISECT if bisect else 0) | (_lib.GLA_FLAG_REFINE_SIMT if refine_simt else 0)
        self.graph = graph
        h = C.c_void_p()
        _lib.check(L.gla_plan_create(C.byref(h), PRECISIONS[precision], jobz.encode(), uplo.encode(), len(ns),
                                     ns.ctypes.data_as(C.POINTER(C.c_int64)), float(tol or 0.0), flags),
                   "gla_plan_create")
        self._h = h
        a = C.c_int64()
        w = C.c_int64()
        L.gla_plan_arena_sizes(h, C.byref(a), C.byref(w))
        self.a_elems = a.value
        self.w_elems = w.value
        self.a_off = np.zeros(len(ns), np.int64)
        self.w_off = np.zeros(len(ns), np.int64)
        if len(ns) > 1:
            self.a_off[1:] = np.cumsum(ns * ns)[:-1]
            self.w_off[1:] = np.cumsum(ns)[:-1]

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().gla_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def bucket_configs(self):
        """Launch shapes of the size buckets: list of dicts (nmax, matrices,
        threads per CTA of the tridiagonalisation, chase matrices per warp)."""
        L = _lib.load()
        nb = C.c_int()
        _lib.check(L.gla_plan_buckets(self._h, C.byref(nb)), "gla_plan_buckets")
        out = []
        for b in range(nb.value):
            v = [C.c_int() for _ in range(4)]
            _lib.check(L.gla_plan_bucket_config(self._h, b, *[C.byref(x) for x in v]), "gla_plan_bucket_config")
            out.append(dict(zip(("nmax", "matrices", "nt_tri", "lanes_per_warp"), [x.value for x in v])))
        return out

    def workspace_bytes(self):
        b = C.c_size_t()
        _lib.check(_lib.load().gla_plan_workspace_size(self._h, C.byref(b)))
        return b.value

    def execute(self, A, w, V, info, stream=None):
        """Device run: A, w, V (may be None for jobz 'N'), info are torch CUDA
        tensors holding the packed arenas. Asynchronous on `stream`."""
        rc = _lib.load().gla_plan_execute(self._h, C.c_void_p(A.data_ptr()), C.c_void_p(w.data_ptr()),
                                          C.c_void_p(V.data_ptr()) if V is not None else None,
                                          C.c_void_p(info.data_ptr()), _stream_ptr(stream))
        return _lib.check(rc, "gla_plan_execute")

    def execute_eigen2(self, A, w, V2, info, stream=None):
        """eigen2 over the batch (gla_plan_execute_eigen2): eigenvalues and
        rows 1 and n of each eigenvector matrix, 2 x n_b column-major at
        twice the eigenvalue offset (V2 holds 2 w_elems). Device tensors."""
        rc = _lib.load().gla_plan_execute_eigen2(self._h, C.c_void_p(A.data_ptr()), C.c_void_p(w.data_ptr()),
                                                 C.c_void_p(V2.data_ptr()), C.c_void_p(info.data_ptr()),
                                                 _stream_ptr(stream))
        return _lib.check(rc, "gla_plan_execute_eigen2")

    def execute_eigen2_host(self, A, w, V2, info, stream=None):
        """execute_eigen2 from and to numpy arenas (gla_plan_execute_eigen2_host);
        synchronizes. Returns the number of matrices with nonzero info."""
        rc = _lib.load().gla_plan_execute_eigen2_host(self._h, C.c_void_p(A.ctypes.data), C.c_void_p(w.ctypes.data),
                                                      C.c_void_p(V2.ctypes.data), C.c_void_p(info.ctypes.data),
                                                      _stream_ptr(stream) if stream is not None else None)
        return _lib.check(rc, "gla_plan_execute_eigen2_host")

    def capture(self, A, w, V, info):
        """Capture execute(A, w, V, info) into a torch.cuda.CUDAGraph (plan made
        with graph=True). Replaying it re-solves whatever A holds at replay."""
        if not self.graph:
            raise ValueError("plan was not created with graph=True")
        torch = _torch()
        self.execute(A, w, V, info)  # warm-up outside the capture
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.execute(A, w, V, info)
        return g

    def capture_step(self, A, w, V, info, wbar, Vbar, Abar, gap_rel=0.0):
        """Capture the forward solve and its adjoint, execute(A, w, V, info)
        then adjoint(w, V, wbar, Vbar, Abar), into one torch.cuda.CUDAGraph
        (plan made with graph=True). Replaying it re-solves whatever A holds
        and back-propagates whatever wbar and Vbar hold."""
        if not self.graph:
            raise ValueError("plan was not created with graph=True")
        torch = _torch()
        # warm-up outside the capture: the first adjoint allocates its workspace
        self.execute(A, w, V, info)
        self.adjoint(w, V, wbar, Vbar, Abar, gap_rel)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.execute(A, w, V, info)
            self.adjoint(w, V, wbar, Vbar, Abar, gap_rel)
        return g

    def execute_host(self, A, w, V, info, stream=None):
        """Host-buffer run (numpy arenas); copies in/out and synchronizes.
        Returns the number of matrices with nonzero info."""
        rc = _lib.load().gla_plan_execute_host(self._h, C.c_void_p(A.ctypes.data), C.c_void_p(w.ctypes.data),
                                               C.c_void_p(V.ctypes.data) if V is not None else None,
                                               C.c_void_p(info.ctypes.data),
                                               _stream_ptr(stream) if stream is not None else None)
        return _lib.check(rc, "gla_plan_execute_host")

    def host_pipeline(self):
        """(chunks, last_pipelined): the chunks execute_host overlaps its copies
        with (0: never), and whether its last call did."""
        c, u = C.c_int(0), C.c_int(0)
        _lib.check(_lib.load().gla_plan_host_pipeline(self._h, C.byref(c), C.byref(u)))
        return c.value, bool(u.value)

    def adjoint(self, w, V, wbar, Vbar, Abar, gap_rel=0.0, stream=None):
        """Abar = V (diag(wbar) + sym(F o V'Vbar)) V' for every matrix (torch CUDA
        arenas, FP64, packed like execute's outputs). Asynchronous."""
        rc = _lib.load().gla_plan_adjoint(self._h, C.c_void_p(w.data_ptr()), C.c_void_p(V.data_ptr()),
                                          C.c_void_p(wbar.data_ptr()), C.c_void_p(Vbar.data_ptr()),
                                          C.c_void_p(Abar.data_ptr()), float(gap_rel), _stream_ptr(stream))
        return _lib.check(rc, "gla_plan_adjoint")

    def adjoint_host(self, w, V, wbar, Vbar, Abar, gap_rel=0.0, stream=None):
        """adjoint() on host numpy arenas (float64, C-contiguous); the library
        stages them on the device and synchronizes."""
        arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in (w, V, wbar, Vbar)]
        if not (Abar.dtype == np.float64 and Abar.flags.c_contiguous):
            raise ValueError("Abar must be a C-contiguous float64 array")
        rc = _lib.load().gla_plan_adjoint_host(self._h, *[C.c_void_p(x.ctypes.data) for x in arrs],
                                               C.c_void_p(Abar.ctypes.data), float(gap_rel),
                                               _stream_ptr(stream) if stream is not None else None)
        return _lib.check(rc, "gla_plan_adjoint_host")

    def stats(self):
        """Work counters of the last execute (rotations, sweeps, row_rotations,
        refine_n3, passes)."""
        c = (C.c_int64 * len(_lib.COUNTERS))()
        _lib.check(_lib.load().gla_plan_counters(self._h, c))
        return dict(zip(_lib.COUNTERS, [int(x) for x in c]))

    def phase_times(self):
        """Milliseconds per phase of the last execute (plan made with timing=True)."""
        ms = (C.c_float * len(_lib.PHASES))()
        _lib.check(_lib.load().gla_plan_phase_times(self._h, ms))
        return dict(zip(_lib.PHASES, [float(x) for x in ms]))

    # -- packing helpers (column-major arenas)
    def pack(self, mats, device=None):
        """Pack square matrices into the column-major A arena (numpy, or torch on `device`)."""
        if device is None:
            return np.concatenate([np.asarray(m, dtype=self.dtype).ravel(order="F") for m in mats]) \
                if len(mats) else np.zeros(1, self.dtype)
        torch = _torch()
        dt = torch.float32 if self.dtype == np.float32 else torch.float64
        return torch.cat([torch.as_tensor(m, dtype=dt, device=device).t().contiguous().reshape(-1) for m in mats])

    def unpack(self, w, V=None):
        vals, vecs = [], []
        for b, n in enumerate(self.ns):
            vals.append(w[self.w_off[b]: self.w_off[b] + n])
            if V is not None:
                seg = V[self.a_off[b]: self.a_off[b] + n * n]
                vecs.append(seg.reshape(n, n).T if not _is_torch(seg) else seg.reshape(n, n).t())
        return vals, (vecs if V is not None else None)


def _solve_batched(mats, jobz, uplo, tol, precision, alg, check):
    if len(mats) == 0:
        return []
    for m in mats:
        if m.ndim != 2 or m.shape[0] != m.shape[1]:
            raise DimensionMismatch(f"matrix is not square: dimensions are {tuple(m.shape)}")
    ns = [int(m.shape[0]) for m in mats]
    plan = Plan(ns, precision=precision, jobz=jobz, uplo=uplo, tol=tol, alg=alg)
    try:
        if _is_torch(mats[0]):
            torch = _torch()
            dev = mats[0].device
            A = plan.pack(mats, device=dev)
            dt = A.dtype
            w = torch.empty(max(plan.w_elems, 1), dtype=dt, device=dev)
            V = torch.empty(max(plan.a_elems, 1), dtype=dt, device=dev) if jobz == "V" else None
            info = torch.zeros(len(mats), dtype=torch.int32, device=dev)
            plan.execute(A, w, V, info)
            info_h = info.cpu().numpy()
        else:
            A = plan.pack(mats)
            w = np.zeros(max(plan.w_elems, 1), plan.dtype)
            V = np.zeros(max(plan.a_elems, 1), plan.dtype) if jobz == "V" else None
            info_h = np.zeros(len(mats), np.int32)
            plan.execute_host(A, w, V, info_h)
        if check:
            _raise_for_info(info_h)
        vals, vecs = plan.unpack(w, V)
        if jobz == "V":
            return [Eigen(v, x) for v, x in zip(vals, vecs)], info_h
        return vals, info_h
    finally:
        plan.close()


def eigen_batched(mats, uplo="L", tol=None, precision="f64", alg="QL", check=True):
    """[eigen(Hermitian(A, uplo)) for A in mats] in one batched launch sequence."""
    r = _solve_batched(list(mats), "V", uplo, tol, precision, alg, check)
    return r[0] if r else []


def eigvals_batched(mats, uplo="L", tol=None, precision="f64", check=True):
    r = _solve_batched(list(mats), "N", uplo, tol, precision, "QL", check)
    return r[0] if r else []


def _tridiag(T, jobz, alg, tol):
    if tol is not None:
        raise ValueError("tol for SymTridiagonal input: only the default eps(Float64) is supported")
    L = _lib.load()
    torch = _torch()
    on_dev = _is_torch(T.dv)
    dev = T.dv.device if on_dev else torch.device("cuda")
    d = torch.as_tensor(T.dv, dtype=torch.float64, device=dev).clone()
    e = torch.as_tensor(T.ev, dtype=torch.float64, device=dev).clone()
    n = d.numel()
    if e.numel() == 0:
        e = torch.zeros(1, dtype=torch.float64, device=dev)
    Z = torch.empty((n, n), dtype=torch.float64, device=dev) if jobz == "V" else None
    info = C.c_int()
    rc = L.gla_dstev(jobz.encode(), n, C.c_void_p(d.data_ptr()), C.c_void_p(e.data_ptr()),
                     C.c_void_p(Z.data_ptr()) if Z is not None else None, max(n, 1),
                     GLA_ALG_QR if alg == "QR" else GLA_ALG_QL, C.byref(info), _stream_ptr())
    _lib.check(rc, "gla_dstev")
    _raise_for_info([info.value])
    if jobz == "V":
        Zt = Z.t()  # column-major buffer -> row-major view
        if on_dev:
            return Eigen(d, Zt)
        return Eigen(d.cpu().numpy(), Zt.cpu().numpy())
    return d if on_dev else d.cpu().numpy()


class _EighFunction:
    """torch.autograd.Function for the batched eigen-decomposition of a list of
    same-plan symmetric matrices (the Python counterpart of an rrule for
    eigen): forward = gla_plan_execute, backward = gla_plan_adjoint."""

    @staticmethod
    def build():
        torch = _torch()

        class Eigh(torch.autograd.Function):
            @staticmethod
            def forward(ctx, A, plan):
                w = torch.empty(plan.w_elems, dtype=torch.float64, device=A.device)
                V = torch.empty(plan.a_elems, dtype=torch.float64, device=A.device)
                info = torch.zeros(len(plan.ns), dtype=torch.int32, device=A.device)
                plan.execute(A, w, V, info)
                _raise_for_info(info.cpu().numpy())
                ctx.plan = plan
                ctx.save_for_backward(w, V)
                return w, V

            @staticmethod
            def backward(ctx, wbar, Vbar):
                w, V = ctx.saved_tensors
                wbar = torch.zeros_like(w) if wbar is None else wbar.contiguous()
                Vbar = torch.zeros_like(V) if Vbar is None else Vbar.contiguous()
                Abar = torch.empty_like(V)
                ctx.plan.adjoint(w, V, wbar, Vbar, Abar)
                return Abar, None

        return Eigh


_eigh_fn = None


def eigh_autograd(A, plan):
    """Differentiable batched eigen-decomposition: A is the packed FP64 arena
    (torch CUDA tensor, requires_grad allowed), plan a Plan with jobz 'V'.
    Returns packed (w, V); gradients flow back through gla_plan_adjoint."""
    global _eigh_fn
    if _eigh_fn is None:
        _eigh_fn = _EighFunction.build()
    return _eigh_fn.apply(A, plan)


def _is_complex(A):
    if _is_torch(A):
        return A.is_complex()
    return np.iscomplexobj(A)


def _zheev(A, jobz, uplo):
    """Complex Hermitian input through gla_zheev (FP64 only)."""
    torch = _torch()
    on_dev = _is_torch(A)
    X = A.to(torch.complex128) if on_dev else torch.as_tensor(np.asarray(A, dtype=np.complex128), device="cuda")
    n = X.shape[0]
    if X.dim() != 2 or X.shape[1] != n:
        raise DimensionMismatch("A must be square")
    Xc = X.t().contiguous()  # column-major, interleaved (re, im)
    w = torch.empty(max(n, 1), dtype=torch.float64, device=X.device)
    V = torch.empty((max(n, 1), max(n, 1)), dtype=torch.complex128, device=X.device) if jobz == "V" else None
    info = C.c_int()
    rc = _lib.load().gla_zheev(jobz.encode(), uplo.encode(), n, C.c_void_p(Xc.data_ptr()), max(n, 1),
                               C.c_void_p(w.data_ptr()), C.c_void_p(V.data_ptr()) if V is not None else None,
                               max(n, 1), C.byref(info), _stream_ptr())
    _lib.check(rc, "gla_zheev")
    _raise_for_info([info.value])
    w = w[:n]
    if jobz == "V":
        Vt = V[:n, :n].t()  # column-major buffer -> row-major view
        return Eigen(w, Vt) if on_dev else Eigen(w.cpu().numpy(), Vt.cpu().numpy())
    return w if on_dev else w.cpu().numpy()


class QuaternionMatrix:
    """A quaternion matrix as an (n, n, 4) float64 array or tensor of
    components (s, i, j, k), the field order of Julia's Quaternion{Float64}:
    eigen(QuaternionMatrix(A)) is the reference's eigen(Hermitian(A)) on
    quaternion input. Its eigenvectors come back in the same (n, n, 4) form
    (right eigenvectors, A v = v lambda)."""

    def __init__(self, data):
        if tuple(data.shape[2:]) != (4,) or len(data.shape) != 3 or data.shape[0] != data.shape[1]:
            raise DimensionMismatch(f"a quaternion matrix is (n, n, 4), got {tuple(data.shape)}")
        self.data = data


def _qheev(Q, jobz, uplo):
    """Quaternion Hermitian input through gla_qheev (FP64 only)."""
    torch = _torch()
    A = Q.data
    on_dev = _is_torch(A)
    X = A.to(torch.float64) if on_dev else torch.as_tensor(np.asarray(A, dtype=np.float64), device="cuda")
    n = X.shape[0]
    Xc = X.permute(1, 0, 2).contiguous()  # column-major, 4 doubles per entry
    w = torch.empty(max(n, 1), dtype=torch.float64, device=X.device)
    V = torch.empty((max(n, 1), max(n, 1), 4), dtype=torch.float64, device=X.device) if jobz == "V" else None
    info = C.c_int()
    rc = _lib.load().gla_qheev(jobz.encode(), uplo.encode(), n, C.c_void_p(Xc.data_ptr()), max(n, 1),
                               C.c_void_p(w.data_ptr()), C.c_void_p(V.data_ptr()) if V is not None else None,
                               max(n, 1), C.byref(info), _stream_ptr())
    _lib.check(rc, "gla_qheev")
    _raise_for_info([info.value])
    w = w[:n]
    if jobz == "V":
        Vt = V[:n, :n].permute(1, 0, 2)  # column-major buffer -> (row, column, component)
        return Eigen(w, Vt) if on_dev else Eigen(w.cpu().numpy(), Vt.cpu().numpy())
    return w if on_dev else w.cpu().numpy()


def eigsortby(x):
    """The default sort key of eigen!/eigvals! (LinearAlgebra.eigsortby for
    real eigenvalues): the value itself, i.e. ascending order."""
    return x


def _sorted_by(vals, vecs, sortby):
    """sorteig!(vals, vecs, sortby) (src/eigenSelfAdjoint.jl:598): a stable
    permutation of the device's ascending output by the key sortby(value)
    (ties keep their ascending order), applied to the values and to the
    eigenvector columns. sortby None or eigsortby leaves the ascending order
    (None asks for no particular order)."""
    if sortby is None or sortby is eigsortby:
        return vals, vecs
    host = vals.cpu().numpy() if _is_torch(vals) else np.asarray(vals)
    keys = [sortby(float(x)) for x in host]
    perm = sorted(range(len(keys)), key=lambda i: keys[i])  # Python's sort is stable
    if _is_torch(vals):
        torch = _torch()
        p = torch.tensor(perm, dtype=torch.long, device=vals.device)
        return vals[p], (vecs[:, p] if vecs is not None else None)
    p = np.asarray(perm, dtype=np.int64)
    return vals[p], (vecs[:, p] if vecs is not None else None)


def eigen(A, uplo="L", tol=None, precision="f64", alg="QL", sortby=eigsortby):
    """eigen(Hermitian(A, uplo)) / eigen(SymTridiagonal): eigenvalues and the
    matching orthonormal eigenvectors (columns), ascending unless sortby
    names another key (as the reference's sortby keyword). Complex input is
    a complex Hermitian matrix (FP64, gla_zheev); a QuaternionMatrix a
    quaternion Hermitian one (FP64, gla_qheev)."""
    if isinstance(A, SymTridiagonal):
        r = _tridiag(A, "V", alg, tol)
    elif isinstance(A, QuaternionMatrix):
        if precision != "f64" or tol is not None:
            raise ValueError("quaternion Hermitian input: FP64 with the default tolerance only")
        r = _qheev(A, "V", uplo)
    elif _is_complex(A):
        if precision != "f64" or tol is not None:
            raise ValueError("complex Hermitian input: FP64 with the default tolerance only")
        r = _zheev(A, "V", uplo)
    else:
        r = eigen_batched([A], uplo=uplo, tol=tol, precision=precision, alg=alg)[0]
    if sortby is None or sortby is eigsortby:
        return r
    return Eigen(*_sorted_by(r.values, r.vectors, sortby))


def eigvals(A, uplo="L", tol=None, precision="f64", irange=None, vl=None, vu=None, abstol=0.0, sortby=eigsortby):
    """eigvals(Hermitian(A, uplo)) / eigvals(SymTridiagonal): the eigenvalues,
    ascending unless sortby names another key. For SymTridiagonal input,
    irange = (il, iu) (1-based, inclusive, as Julia's eigvals(T, il:iu)) or
    vl < lambda <= vu (eigvals(T, vl, vu)) select a subset, computed by
    Sturm-count multisection (gla_dstebz)."""
    if isinstance(A, SymTridiagonal):
        if irange is not None or vl is not None or vu is not None:
            return _tridiag_subset(A, irange, vl, vu, abstol)
        w = _tridiag(A, "N", "QL", tol)
    elif irange is not None or vl is not None or vu is not None:
        raise ValueError("eigenvalue subsets are available for SymTridiagonal input")
    elif isinstance(A, QuaternionMatrix):
        if precision != "f64" or tol is not None:
            raise ValueError("quaternion Hermitian input: FP64 with the default tolerance only")
        w = _qheev(A, "N", uplo)
    elif _is_complex(A):
        if precision != "f64" or tol is not None:
            raise ValueError("complex Hermitian input: FP64 with the default tolerance only")
        w = _zheev(A, "N", uplo)
    else:
        w = eigvals_batched([A], uplo=uplo, tol=tol, precision=precision)[0]
    return _sorted_by(w, None, sortby)[0]


def release_workspaces():
    """Free the device workspaces the single-call entry points cache per order
    (gla_release_workspaces); waits for the device first."""
    _lib.check(_lib.load().gla_release_workspaces(), "gla_release_workspaces")


def _tridiag_dev(T):
    torch = _torch()
    on_dev = _is_torch(T.dv)
    dev = T.dv.device if on_dev else torch.device("cuda")
    d = torch.as_tensor(T.dv, dtype=torch.float64, device=dev).contiguous()
    e = torch.as_tensor(T.ev, dtype=torch.float64, device=dev).contiguous()
    if e.numel() == 0:
        e = torch.zeros(1, dtype=torch.float64, device=dev)
    return d, e, on_dev, dev


class EigenQ:
    """The orthogonal factor of symtri (src/eigenSelfAdjoint.jl:6-21): Householder
    reflectors stored in `factors` (a torch CUDA float64 tensor, n x n, in the
    reference's symtriLower! layout for uplo 'L' and symtriUpper!'s for 'U')
    with scalars `tau`. lmul(B) = Q B and rmul(B) = B Q (lmul!/rmul!, :23-99),
    array() = Q (Array(::EigenQ), :101); the trans forms apply Q'."""

    def __init__(self, factors, tau, uplo="L"):
        if uplo not in ("L", "U"):
            raise ValueError("uplo must be 'L' or 'U'")
        self.uplo = uplo
        self.factors = factors
        self.tau = tau
        self.n = factors.shape[0]

    def _apply(self, side, trans, B):
        # the operand's shape is checked before any device work (lmul!/rmul!
        # raise DimensionMismatch, src/eigenSelfAdjoint.jl:25-27, :64-66)
        shape = tuple(B.shape) if hasattr(B, "shape") else np.shape(B)
        if len(shape) != 2:
            raise DimensionMismatch("B must be a matrix")
        m, k = shape
        if (side == "L" and m != self.n) or (side == "R" and k != self.n):
            raise DimensionMismatch(f"Q has order {self.n}, B is {m} x {k}")
        torch = _torch()
        on_dev = _is_torch(B)
        X = (B.to(torch.float64) if on_dev else torch.as_tensor(np.asarray(B, dtype=np.float64), device="cuda"))
        Xc = X.t().contiguous().clone()  # column-major storage of X
        F = self.factors.t().contiguous()
        _lib.check(_lib.load().gla_dormtr(side.encode(), self.uplo.encode(), trans.encode(), m, k,
                                          C.c_void_p(F.data_ptr()), self.n, C.c_void_p(self.tau.data_ptr()),
                                          C.c_void_p(Xc.data_ptr()), max(m, 1), _stream_ptr()), "gla_dormtr")
        out = Xc.t()
        return out if on_dev else out.cpu().numpy()

    def lmul(self, B, trans=False):
        return self._apply("L", "T" if trans else "N", B)

    def rmul(self, B, trans=False):
        return self._apply("R", "T" if trans else "N", B)

    def array(self):
        torch = _torch()
        return self.lmul(torch.eye(self.n, dtype=torch.float64, device="cuda"))


SymmetricTridiagonalFactorization = namedtuple("SymmetricTridiagonalFactorization", ["reflectors", "diagonals"])


def symtri(A, uplo="L"):
    """symtri!(Hermitian(A, uplo)) (src/eigenSelfAdjoint.jl:446-564) on the GPU:
    A = Q T Q'. Returns SymmetricTridiagonalFactorization(EigenQ, SymTridiagonal)
    with device tensors; the factors follow symtriLower!'s layout for uplo 'L'
    and symtriUpper!'s for 'U'."""
    torch = _torch()
    X = A.to(torch.float64) if _is_torch(A) else torch.as_tensor(np.asarray(A, dtype=np.float64), device="cuda")
    n = X.shape[0]
    if X.dim() != 2 or X.shape[1] != n:
        raise DimensionMismatch("A must be square")
    F = X.t().contiguous().clone()  # column-major working storage
    d = torch.empty(max(n, 1), dtype=torch.float64, device=X.device)
    e = torch.empty(max(n - 1, 1), dtype=torch.float64, device=X.device)
    tau = torch.empty(max(n - 1, 1), dtype=torch.float64, device=X.device)
    _lib.check(_lib.load().gla_dsytrd(uplo.encode(), n, C.c_void_p(F.data_ptr()), max(n, 1), C.c_void_p(d.data_ptr()),
                                      C.c_void_p(e.data_ptr()), C.c_void_p(tau.data_ptr()), _stream_ptr()),
               "gla_dsytrd")
    return SymmetricTridiagonalFactorization(EigenQ(F.t(), tau, uplo), SymTridiagonal(d[:n], e[:max(n - 1, 0)]))


def numnegevals(T, sigma=0.0):
    """numnegevals(T::SymTridiagonal, sigma) (src/tridiag.jl:20-36): the number
    of negative eigenvalues of T - sigma I. sigma may be an array of shifts
    (one count per shift, computed in parallel); counts equal the reference's
    recurrence bit for bit."""
    torch = _torch()
    d, e, on_dev, dev = _tridiag_dev(T)
    n = d.numel()
    sig = torch.as_tensor(np.atleast_1d(np.asarray(sigma, dtype=np.float64)) if not _is_torch(sigma) else sigma,
                          dtype=torch.float64, device=dev).reshape(-1).contiguous()
    counts = torch.empty(sig.numel(), dtype=torch.int64, device=dev)
    _lib.check(_lib.load().gla_numnegevals(n, C.c_void_p(d.data_ptr()), C.c_void_p(e.data_ptr()), sig.numel(),
                                           C.c_void_p(sig.data_ptr()), C.c_void_p(counts.data_ptr()),
                                           _stream_ptr()), "gla_numnegevals")
    if not _is_torch(sigma) and np.ndim(sigma) == 0:
        return int(counts[0].item())
    return counts if on_dev else counts.cpu().numpy()


def _tridiag_subset(T, irange, vl, vu, abstol):
    torch = _torch()
    d, e, on_dev, dev = _tridiag_dev(T)
    n = d.numel()
    if irange is not None:
        il, iu = int(irange[0]), int(irange[1])
    else:
        lo = -np.inf if vl is None else float(vl)
        hi = np.inf if vu is None else float(vu)
        # vl < lambda <= vu through counts of eigenvalues below each end
        il = 1 if lo == -np.inf else numnegevals(T, lo) + 1
        iu = n if hi == np.inf else numnegevals(T, hi)
    if iu < il:
        w = torch.empty(0, dtype=torch.float64, device=dev)
        return w if on_dev else w.cpu().numpy()
    w = torch.empty(iu - il + 1, dtype=torch.float64, device=dev)
    _lib.check(_lib.load().gla_dstebz(n, C.c_void_p(d.data_ptr()), C.c_void_p(e.data_ptr()), il, iu, float(abstol),
                                      C.c_void_p(w.data_ptr()), _stream_ptr()), "gla_dstebz")
    return w if on_dev else w.cpu().numpy()


def eigen2(A, uplo="L", tol=None, precision="f64", alg="QL"):
    """eigen2 (src/eigenSelfAdjoint.jl:633-668): ascending eigenvalues and the
    FIRST and LAST rows of the eigenvector matrix (a 2 x n array; for n = 1
    both rows are the single entry). Dense real input of order <= 128 in
    FP64 or FP32 takes the reference's cheap form (gla_plan_execute_eigen2:
    rows 1 and n of Q from the reflectors, the rotations replayed on two
    rows); its rows agree with eigen(A)'s to rounding. Other input (a
    SymTridiagonal, whose rows equal eigen's exactly, larger orders, the
    refined precision) keeps two rows of eigen(A)."""
    dense = not isinstance(A, (SymTridiagonal, QuaternionMatrix)) and not _is_complex(A)
    if dense and precision in ("f64", "f32") and A.shape[0] == A.shape[1] and 1 <= A.shape[0] <= GLA_MAX_SMALL_N:
        torch = _torch()
        on_dev = _is_torch(A)
        n = int(A.shape[0])
        plan = Plan([n], precision=precision, jobz="V", uplo=uplo, tol=tol, alg=alg)
        try:
            dt = torch.float32 if precision == "f32" else torch.float64
            dev = A.device if on_dev else torch.device("cuda")
            Ad = plan.pack([A], device=dev).to(dt)
            w = torch.empty(n, dtype=dt, device=dev)
            V2 = torch.empty(2 * n, dtype=dt, device=dev)
            info = torch.zeros(1, dtype=torch.int32, device=dev)
            plan.execute_eigen2(Ad, w, V2, info)
            _raise_for_info(info.cpu().numpy())
        finally:
            plan.close()
        vecs = V2.reshape(n, 2).t()  # column-major 2 x n
        return Eigen(w, vecs.clone()) if on_dev else Eigen(w.cpu().numpy(), vecs.cpu().numpy().copy())
    r = eigen(A, uplo=uplo, tol=tol, precision=precision, alg=alg)
    vals, vecs = r
    n = vecs.shape[0]
    rows = [0, n - 1]
    if _is_torch(vecs):
        torch = _torch()
        return Eigen(vals, vecs[torch.tensor(rows, device=vecs.device)].clone())
    return Eigen(vals, vecs[rows].copy())


def autotune_clear():
    """Drop every entry of the process-wide autotune table."""
    _lib.check(_lib.load().gla_autotune_clear(), "gla_autotune_clear")


def autotune_save(path):
    """Write the autotune table to a text file."""
    _lib.check(_lib.load().gla_autotune_save(str(path).encode()), "gla_autotune_save")


def autotune_load(path):
    """Merge the entries of an autotune file; returns how many were loaded."""
    rc = _lib.load().gla_autotune_load(str(path).encode())
    if rc < 0:
        raise OSError(f"cannot read autotune file {path}")
    return rc


__all__ = ["Eigen", "Plan", "SymTridiagonal", "eigen", "eigen2", "eigvals", "eigen_batched", "eigvals_batched", "eigh_autograd",
           "autotune_clear", "autotune_save", "autotune_load", "numnegevals", "symtri", "EigenQ", "eigsortby",
           "release_workspaces",
           "SymmetricTridiagonalFactorization", "QuaternionMatrix",
           "DimensionMismatch", "NonConvergenceError", "NonFiniteError", "GLAError", "GLA_MAX_SMALL_N", "GLA_MAX_N"]
