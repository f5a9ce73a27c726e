"""ctypes binding of libglagpu.so (include/glagpu.h).

The library must have been built (genericlinearalgebra.jl_gb300/build.py, or
__graft_entry__.build()); there is no fallback: importing the solver without
it raises ImportError.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "build", "libglagpu.so")

GLA_PREC_F64 = 0
GLA_PREC_F32 = 1
GLA_PREC_F32_REFINED = 2
GLA_ALG_QL = 0
GLA_ALG_QR = 1
GLA_MAX_SMALL_N = 128
GLA_MAX_N = 16384
GLA_STATIC_MAX_N = 128
GLA_ERR_STATIC_TOO_LARGE = -2001
GLA_ERR_UNSUPPORTED = -2002
GLA_FLAG_SMALL_LOG = 4
GLA_FLAG_TIMING = 8
GLA_FLAG_GRAPH = 16
GLA_FLAG_AUTOTUNE = 32
GLA_FLAG_REFINE_QL = 64
GLA_FLAG_F32_BISECT = 128
GLA_FLAG_REFINE_SIMT = 256
PHASES = ("tridiag", "chase", "apply", "refine")
COUNTERS = ("rotations", "sweeps", "row_rotations", "refine_n3", "passes")

# Every symbol include/glagpu.h declares, with its ctypes signature.
_i64 = C.c_int64
_vp = C.c_void_p
_ch = C.c_char
_int = C.c_int
_d = C.c_double
SIGNATURES = {
    "gla_version": ([], _int),
    "gla_gemm_df": ([_i64, _i64, _i64, _vp, _vp, _i64, _vp, _vp, _i64, _vp, _vp, _i64, _vp], _int),
    "gla_gemm_df_last_ms": ([C.POINTER(C.c_float), C.POINTER(C.c_float)], _int),
    "gla_autotune_clear": ([], _int),
    "gla_autotune_save": ([C.c_char_p], _int),
    "gla_autotune_load": ([C.c_char_p], _int),
    "gla_plan_buckets": ([_vp, C.POINTER(_int)], _int),
    "gla_plan_bucket_config": ([_vp, _int, C.POINTER(_int), C.POINTER(_int), C.POINTER(_int), C.POINTER(_int)], _int),
    "gla_numnegevals": ([_i64, _vp, _vp, _i64, _vp, _vp, _vp], _int),
    "gla_dstebz": ([_i64, _vp, _vp, _i64, _i64, _d, _vp, _vp], _int),
    "gla_numnegevals_host": ([_i64, _vp, _vp, _i64, _vp, _vp], _int),
    "gla_dstebz_host": ([_i64, _vp, _vp, _i64, _i64, _d, _vp], _int),
    "gla_dsytrd": ([_ch, _i64, _vp, _i64, _vp, _vp, _vp, _vp], _int),
    "gla_dormtr": ([_ch, _ch, _ch, _i64, _i64, _vp, _i64, _vp, _vp, _i64, _vp], _int),
    "gla_dsytrd_host": ([_ch, _i64, _vp, _i64, _vp, _vp, _vp], _int),
    "gla_dormtr_host": ([_ch, _ch, _ch, _i64, _i64, _vp, _i64, _vp, _vp, _i64], _int),
    "gla_zheev": ([_ch, _ch, _i64, _vp, _i64, _vp, _vp, _i64, C.POINTER(_int), _vp], _int),
    "gla_zheev_host": ([_ch, _ch, _i64, _vp, _i64, _vp, _vp, _i64, C.POINTER(_int)], _int),
    "gla_qheev": ([_ch, _ch, _i64, _vp, _i64, _vp, _vp, _i64, C.POINTER(_int), _vp], _int),
    "gla_qheev_host": ([_ch, _ch, _i64, _vp, _i64, _vp, _vp, _i64, C.POINTER(_int)], _int),
    "gla_status_string": ([_int], C.c_char_p),
    "gla_plan_create": ([C.POINTER(_vp), _int, _ch, _ch, _i64, C.POINTER(_i64), _d, _int], _int),
    "gla_plan_destroy": ([_vp], _int),
    "gla_plan_workspace_size": ([_vp, C.POINTER(C.c_size_t)], _int),
    "gla_plan_arena_sizes": ([_vp, C.POINTER(_i64), C.POINTER(_i64)], _int),
    "gla_plan_execute": ([_vp, _vp, _vp, _vp, _vp, _vp], _int),
    "gla_plan_execute_host": ([_vp, _vp, _vp, _vp, _vp, _vp], _int),
    "gla_plan_host_pipeline": ([_vp, C.POINTER(_int), C.POINTER(_int)], _int),
    "gla_plan_execute_eigen2": ([_vp, _vp, _vp, _vp, _vp, _vp], _int),
    "gla_plan_execute_eigen2_host": ([_vp, _vp, _vp, _vp, _vp, _vp], _int),
    "gla_plan_stats": ([_vp, C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_int)], _int),
    "gla_plan_phase_times": ([_vp, C.POINTER(C.c_float)], _int),
    "gla_plan_counters": ([_vp, C.POINTER(_i64)], _int),
    "gla_plan_adjoint": ([_vp, _vp, _vp, _vp, _vp, _vp, _d, _vp], _int),
    "gla_plan_adjoint_host": ([_vp, _vp, _vp, _vp, _vp, _vp, _d, _vp], _int),
    "gla_dsyev": ([_ch, _ch, _i64, _vp, _i64, _vp, C.POINTER(_int), _vp], _int),
    "gla_ssyev": ([_ch, _ch, _i64, _vp, _i64, _vp, C.POINTER(_int), _vp], _int),
    "gla_dstev": ([_ch, _i64, _vp, _vp, _vp, _i64, _int, C.POINTER(_int), _vp], _int),
    "gla_dsyev_static": ([_ch, _ch, _i64, _vp, _i64, _vp, C.POINTER(_int), _vp], _int),
    "gla_release_workspaces": ([], _int),
    "gla_sgemm_3xtf32": ([_i64, _i64, _i64, C.c_float, _vp, _i64, _vp, _i64, C.c_float, _vp, _i64, _vp], _int),
}

_lib = None


def load():
    """Load libglagpu.so and bind every exported entry point."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"libglagpu.so not found at {LIB_PATH}; build it with "
            "`python genericlinearalgebra.jl_gb300/build.py` (no CPU fallback exists)")
    lib = C.CDLL(LIB_PATH)
    for name, (args, res) in SIGNATURES.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _lib = lib
    return lib


class GLAError(RuntimeError):
    """Nonzero status from the C ABI (argument error or CUDA error)."""

    def __init__(self, status, what=""):
        self.status = status
        msg = load().gla_status_string(status).decode()
        super().__init__(f"{what}: status {status}: {msg}" if what else f"status {status}: {msg}")


def check(status, what=""):
    if status < 0:
        raise GLAError(status, what)
    return status
