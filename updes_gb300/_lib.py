"""ctypes binding of the C ABI in ``include/updes_gb300.h``.

The shared library is built in-tree by ``updes_gb300/build.py`` into
``updes_gb300/_lib/libupdes_gb300.so``.  There is no fallback: if the library
is missing or fails to load, every solver entry point raises.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libupdes_gb300.so")

# status codes
OK, ERR_INVALID, ERR_CUDA, ERR_SINGULAR, ERR_NOT_CONVERGED, ERR_TIMEOUT, ERR_UNSUPPORTED, ERR_WORKSPACE, \
    ERR_TOO_LARGE = range(9)
NOALLOC_MAX_N = 24576  # UPDES_NOALLOC_MAX_N
# kernels
RBF_POLYHARMONIC, RBF_GAUSSIAN, RBF_MULTIQUADRIC, RBF_INVERSE_MULTIQUADRIC, RBF_THIN_PLATE = range(5)
# boundary rows
ROW_DIRICHLET, ROW_NEUMANN, ROW_ROBIN, ROW_PERIODIC_VALUE, ROW_PERIODIC_FLUX = range(5)
# precisions
PREC_FP64, PREC_FP32 = 0, 1


class UpdesError(RuntimeError):
    """A non-zero status returned by the C ABI."""

    def __init__(self, status: int, what: str):
        self.status = status
        msg = f"{what}: {status_string(status)} (status {status})"
        if status == ERR_CUDA:
            try:
                msg += f": {_lib.updes_last_error().decode()}"
            except Exception:  # pragma: no cover
                pass
        super().__init__(msg)


class Problem(ctypes.Structure):
    _fields_ = [
        ("N", ctypes.c_int32), ("Ni", ctypes.c_int32), ("M", ctypes.c_int32), ("rbf", ctypes.c_int32),
        ("rbf_param", ctypes.c_double), ("self_term", ctypes.c_int32), ("support_width", ctypes.c_int32),
        ("nodes", ctypes.c_void_p), ("op_weights", ctypes.c_void_p), ("bd_kind", ctypes.c_void_p),
        ("bd_node", ctypes.c_void_p), ("bd_geom", ctypes.c_void_p), ("supports", ctypes.c_void_p),
    ]


class SolveOpts(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int32), ("max_iters", ctypes.c_int32), ("restart", ctypes.c_int32),
                ("fallback_fp64", ctypes.c_int32), ("tol", ctypes.c_double)]


class SolveInfo(ctypes.Structure):
    _fields_ = [("iters", ctypes.c_int32), ("fell_back", ctypes.c_int32), ("lu_info", ctypes.c_int32),
                ("converged", ctypes.c_int32), ("rel_residual", ctypes.c_double),
                ("backward_error", ctypes.c_double),
                ("t_assemble_ms", ctypes.c_double), ("t_factor_ms", ctypes.c_double),
                ("t_refine_ms", ctypes.c_double), ("t_eval_ms", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


NSTAT = 7
STAT_NAMES = ["trailing_update", "panel", "trsm", "trsv", "gemv", "assemble", "other"]


class Stats(ctypes.Structure):
    _fields_ = [("launches", ctypes.c_int64), ("count", ctypes.c_int64 * NSTAT), ("ms", ctypes.c_double * NSTAT),
                ("flops", ctypes.c_double * NSTAT), ("bytes", ctypes.c_double * NSTAT)]

    def as_dict(self):
        return {"launches": int(self.launches),
                "by_class": {STAT_NAMES[i]: {"count": int(self.count[i]), "ms": self.ms[i], "flops": self.flops[i],
                                             "bytes": self.bytes[i]} for i in range(NSTAT)}}


_vp, _i32, _i64, _f64, _sz = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_size_t

# name -> (restype, argtypes); every symbol declared in include/updes_gb300.h
SIGNATURES = {
    "updes_version": (ctypes.c_int, []),
    "updes_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "updes_last_error": (ctypes.c_char_p, []),
    "updes_matrix_ld": (_i64, [_i64, _i32]),
    "updes_assemble": (ctypes.c_int, [ctypes.POINTER(Problem), _vp, _i64, _vp, _i64, _vp]),
    "updes_assemble_df_scratch": (ctypes.c_int, [ctypes.POINTER(Problem), ctypes.POINTER(ctypes.c_size_t)]),
    "updes_assemble_df": (ctypes.c_int, [ctypes.POINTER(Problem), _vp, _vp, _i64, _vp, _vp, _vp, ctypes.c_size_t,
                                         _vp]),
    "updes_eval_values": (ctypes.c_int, [ctypes.POINTER(Problem), _vp, _vp, _vp]),
    "updes_eval_field": (ctypes.c_int, [_i32, _vp, _i32, _vp, _i32, _i32, _f64, _vp, _i32, _vp, _vp]),
    "updes_lu_workspace": (ctypes.c_int, [_i32, _i32, ctypes.POINTER(_sz)]),
    "updes_lu_factor": (ctypes.c_int, [_i32, _vp, _i64, _i32, _vp, _i64, _vp, _vp, _sz,
                                       ctypes.POINTER(_i32), _vp]),
    "updes_lu_solve": (ctypes.c_int, [_i32, _vp, _i64, _i32, _vp, _vp, _i32, _i64, _i32, _vp, _sz, _vp]),
    "updes_lu_solve_noalloc": (ctypes.c_int, [_i32, _vp, _i64, _i32, _vp, _vp, _i32, _i64, _i32, _vp]),
    "updes_residual": (ctypes.c_int, [_i32, _vp, _i64, _vp, _vp, _vp, _i32, _vp]),
    "updes_solve_workspace": (ctypes.c_int, [ctypes.POINTER(Problem), ctypes.POINTER(SolveOpts),
                                             ctypes.POINTER(_sz)]),
    "updes_solve": (ctypes.c_int, [ctypes.POINTER(Problem), _vp, _vp, _vp, ctypes.POINTER(SolveOpts),
                                   ctypes.POINTER(SolveInfo), _vp, _sz, _vp]),
    "updes_factor": (ctypes.c_int, [ctypes.POINTER(Problem), ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveInfo),
                                    _vp, _sz, _vp]),
    "updes_solve_factored": (ctypes.c_int, [ctypes.POINTER(Problem), _i32, _vp, _i64, _vp, _i64, _vp, _i64,
                                            ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveInfo), _vp, _sz, _vp]),
    "updes_batch_workspace": (ctypes.c_int, [_i32, ctypes.POINTER(_sz)]),
    "updes_batch_prepare": (ctypes.c_int, [ctypes.POINTER(Problem), _vp, _sz, _vp, _sz, _vp]),
    "updes_solve_batch": (ctypes.c_int, [ctypes.POINTER(Problem), _i32, _vp, _i64, _vp, _i64, _i32, _vp, _sz, _vp,
                                         _sz, _vp]),
    "updes_workspace_status": (ctypes.c_int, [ctypes.POINTER(Problem), _vp, _sz, ctypes.POINTER(_i32), _vp]),
    "updes_eval_values_batch": (ctypes.c_int, [ctypes.POINTER(Problem), _i32, _vp, _i64, _vp, _i64, _vp]),
    "updes_solve_many_workspace": (ctypes.c_int, [ctypes.POINTER(Problem), _i32, ctypes.POINTER(SolveOpts), _i32,
                                                  ctypes.POINTER(_sz)]),
    "updes_solve_many": (ctypes.c_int, [ctypes.POINTER(Problem), _i32, _vp, _vp, _vp, ctypes.POINTER(SolveOpts),
                                        ctypes.POINTER(SolveInfo), _vp, _sz, _i32]),
    "updes_solve_batched_workspace": (ctypes.c_int, [ctypes.POINTER(Problem), _i32, _i32, ctypes.POINTER(_sz)]),
    "updes_solve_batched": (ctypes.c_int, [ctypes.POINTER(Problem), _i32, _vp, _vp, _vp, _vp, _vp, _i32, _i32,
                                           ctypes.POINTER(SolveInfo), _vp, _sz, _vp]),
    "updes_eval_values_t": (ctypes.c_int, [ctypes.POINTER(Problem), _vp, _vp, _vp]),
    "updes_solve_transpose": (ctypes.c_int, [ctypes.POINTER(Problem), _vp, _vp, ctypes.POINTER(SolveOpts),
                                             ctypes.POINTER(SolveInfo), _vp, _sz, _vp]),
    "updes_coeff_grad": (ctypes.c_int, [ctypes.POINTER(Problem), _vp, _vp, _vp, _vp]),
    "updes_set_spin_limit": (ctypes.c_int, [_i64]),
    "updes_stats_reset": (None, [_i32]),
    "updes_stats_read": (None, [ctypes.POINTER(Stats)]),
}


def set_spin_limit(iterations: int = 0) -> None:
    """Polls before a wait between CTAs gives up with ERR_TIMEOUT, on the current device (0: the default)."""
    check(load().updes_set_spin_limit(int(iterations)), "updes_set_spin_limit")


def stats_reset(timing: bool = False) -> None:
    load().updes_stats_reset(int(timing))


def stats_read() -> dict:
    st = Stats()
    load().updes_stats_read(ctypes.byref(st))
    return st.as_dict()

_lib = None


def load() -> ctypes.CDLL:
    """Load the in-tree library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python updes_gb300/build.py` "
                          "(the GB300 solver has no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def status_string(status: int) -> str:
    return load().updes_status_string(status).decode()


def check(status: int, what: str) -> None:
    if status != OK:
        raise UpdesError(status, what)
