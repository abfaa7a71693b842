"""ctypes binding of the ctgpu C ABI (``include/ctgpu.h``).

This is the same boundary a jax.ffi handler or a cgo/JNI stub would bind:
plain pointers, sizes, a stream handle and an integer status.  The library
is loaded from ``scico_gb300/_lib/libctgpu.so`` (built in-tree by
``scico_gb300.build``).  There is no fallback: if the library is missing
every operation raises.
"""

from __future__ import annotations

import ctypes
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libctgpu.so"

c_int32 = ctypes.c_int32
c_int64 = ctypes.c_int64
c_float = ctypes.c_float
c_double = ctypes.c_double
c_size_t = ctypes.c_size_t
c_void_p = ctypes.c_void_p
c_char_p = ctypes.c_char_p

CT_OK = 0
CT_ERR_INVALID_ARG = 1
CT_ERR_SHAPE = 2
CT_ERR_UNSUPPORTED = 3
CT_ERR_CUDA = 4
CT_ERR_TIMEOUT = 5
CT_ERR_NONFINITE = 6
CT_ERR_WORKSPACE = 7
CT_ERR_NO_DEVICE = 8

CT_VIEW2D_STRIDE = 8
CT_VIEW3D_STRIDE = 12
CT_PROJ3D_ORDER = 256
CT_PROJ3D_GENERAL = 0
CT_PROJ3D_AXIS0 = 1

# CG scalar slots (double[16])
CT_CG_NUM = 0
CT_CG_PAP = 1
CT_CG_ALPHA = 2
CT_CG_BETA = 3
CT_CG_BNORM = 4
CT_CG_TOL2 = 5
CT_CG_ITERS = 6
CT_CG_DONE = 7
CT_CG_MAXITER = 8
CT_CG_RAN = 9
CT_CG_NSCALARS = 16

# itstat record fields
CT_ITSTAT_OBJECTIVE = 0
CT_ITSTAT_PRIMAL = 1
CT_ITSTAT_DUAL = 2
CT_ITSTAT_CG_ITERS = 3
CT_ITSTAT_CG_RELRES = 4
CT_ITSTAT_FIELDS = 8


class CtError(RuntimeError):
    """A ctgpu call returned a non-OK status."""

    def __init__(self, status: int, func: str, message: str):
        self.status = status
        self.func = func
        super().__init__(f"{func}: {message}")


class Proj2dSchedule(ctypes.Structure):
    _fields_ = [
        ("views_per_cta", c_int32),
        ("adj_splits", c_int32),
        ("fwd_us", ctypes.c_float),
        ("adj_us", ctypes.c_float),
        ("tuned", c_int32),
    ]


class Geom2D(ctypes.Structure):
    _fields_ = [
        ("rows", c_int32),
        ("cols", c_int32),
        ("n_views", c_int32),
        ("det_count", c_int32),
        ("views", c_void_p),
        ("max_width", c_float),
    ]


class Geom3D(ctypes.Structure):
    _fields_ = [
        ("shape", c_int32 * 3),
        ("det_shape", c_int32 * 2),
        ("n_views", c_int32),
        ("kind", c_int32),
        ("row_offset", c_int32),
        ("views", c_void_p),
        ("order", c_void_p),
    ]


class FdDesc(ctypes.Structure):
    _fields_ = [
        ("ndim", c_int32),
        ("shape", c_int32 * 3),
        ("naxes", c_int32),
        ("axes", c_int32 * 3),
        ("prepend", c_int32),
        ("append", c_int32),
        ("circular", c_int32),
    ]


class AdmmTvDesc(ctypes.Structure):
    _fields_ = [
        ("geom", Geom2D),
        ("maxiter", c_int32),
        ("cg_maxiter", c_int32),
        ("cg_tol", c_double),
        ("cg_atol", c_double),
        ("lam_l21", c_double),
        ("lam_l1", c_double),
        ("rho", c_double),
        ("loss_scale", c_double),
        ("alpha", c_double),
        ("use_graph", c_int32),
    ]


class Proj3dSchedule(ctypes.Structure):
    _fields_ = [
        ("tile_groups", c_int32),
        ("adj_splits", c_int32),
        ("fwd_us", c_float),
        ("adj_us", c_float),
        ("tuned", c_int32),
    ]


class AdmmTv3dDesc(ctypes.Structure):
    _fields_ = [
        ("geom", Geom3D),
        ("maxiter", c_int32),
        ("cg_maxiter", c_int32),
        ("cg_tol", c_double),
        ("cg_atol", c_double),
        ("lam_l21", c_double),
        ("lam_l1", c_double),
        ("rho", c_double),
        ("loss_scale", c_double),
        ("alpha", c_double),
        ("use_graph", c_int32),
    ]


class CgBlockDesc(ctypes.Structure):
    _fields_ = [
        ("geom", Geom2D),
        ("nsys", c_int32),
        ("maxiter", c_int32),
        ("recompute", c_int32),
        ("gram_scale", c_float),
    ]


class PadmmTvDesc(ctypes.Structure):
    _fields_ = [
        ("nd", c_int32),
        ("geom2", Geom2D),
        ("geom3", Geom3D),
        ("maxiter", c_int32),
        ("lam", c_double),
        ("alpha", c_double),
        ("rho", c_double),
        ("mu", c_double),
        ("nu", c_double),
        ("loss_scale", c_double),
        ("use_graph", c_int32),
    ]


P = c_void_p
_SIGNATURES = {
    "ct_version": (c_char_p, []),
    "ct_status_string": (c_char_p, [ctypes.c_int]),
    "ct_last_error": (c_char_p, []),
    "ct_proj2d_views": (ctypes.c_int, [P, c_int32, c_float, c_float, c_float, c_float, c_float, P, P]),
    "ct_proj2d_workspace": (ctypes.c_int, [P, c_int32, P, P]),
    "ct_proj2d_fwd": (ctypes.c_int, [P, P, P, c_int32, P, c_size_t, P]),
    "ct_proj2d_fwd_noalloc": (ctypes.c_int, [P, P, P, c_int32, P]),
    "ct_proj2d_adj": (ctypes.c_int, [P, P, P, c_int32, P, c_size_t, P]),
    "ct_proj2d_check": (ctypes.c_int, [P]),
    "ct_proj2d_errflag": (ctypes.c_int, []),
    "ct_proj3d_errflag": (ctypes.c_int, []),
    "ct_set_wait_poll_limit": (None, [ctypes.c_uint32]),
    "ct_set_solver_fast_forward": (None, [ctypes.c_int32]),
    "ct_solver_fast_forward": (ctypes.c_int32, []),
    "ct_wait_poll_limit": (ctypes.c_uint32, []),
    "ct_proj2d_autotune": (ctypes.c_int, [P, c_int32, P, P, P, c_size_t, c_int32, P, P]),
    "ct_proj2d_schedule_get": (ctypes.c_int, [P, c_int32, P]),
    "ct_proj2d_schedule_clear": (None, []),
    "ct_fbp_filter": (ctypes.c_int, [P, P, c_int32, c_int32, P]),
    "ct_proj3d_views": (ctypes.c_int, [P, c_int32, P, P, P, P, P, P]),
    "ct_proj3d_workspace": (ctypes.c_int, [P, c_int32, P, P]),
    "ct_proj3d_fwd": (ctypes.c_int, [P, P, P, c_int32, P, c_size_t, P]),
    "ct_proj3d_adj": (ctypes.c_int, [P, P, P, c_int32, P, c_size_t, P]),
    "ct_proj3d_autotune": (ctypes.c_int, [P, P, P, P, c_size_t, c_int32, P, P]),
    "ct_proj3d_schedule_get": (ctypes.c_int, [P, P]),
    "ct_proj3d_schedule_clear": (None, []),
    "ct_fd_out_count": (ctypes.c_int, [P, P]),
    "ct_fd_fwd": (ctypes.c_int, [P, P, P, c_int32, P]),
    "ct_fd_adj": (ctypes.c_int, [P, P, P, c_int32, P]),
    "ct_haar_fwd": (ctypes.c_int, [P, P, P, c_int32, P]),
    "ct_haar_adj": (ctypes.c_int, [P, P, P, c_int32, P]),
    "ct_l21_prox": (ctypes.c_int, [P, P, c_int32, c_int64, c_float, P]),
    "ct_l1_prox": (ctypes.c_int, [P, P, c_int64, c_float, P]),
    "ct_l21_norm": (ctypes.c_int, [P, c_int32, c_int64, P, P, c_size_t, P]),
    "ct_reduce_workspace": (c_size_t, []),
    "ct_dot": (ctypes.c_int, [P, P, c_int64, P, P, c_size_t, P]),
    "ct_cg_init": (ctypes.c_int, [P, P, P, P, c_int64, c_double, c_double, c_int32, P, P, c_size_t, P]),
    "ct_cg_update": (ctypes.c_int, [P, P, P, P, c_int64, P, P, c_size_t, P]),
    "ct_cg_direction": (ctypes.c_int, [P, P, c_int64, P, P, c_size_t, P]),
    "ct_admm_tv_workspace": (ctypes.c_int, [P, P]),
    "ct_admm_tv_state": (ctypes.c_int, [P, P, P, P]),
    "ct_admm_tv_solve": (ctypes.c_int, [P, P, P, P, c_int32, P, c_size_t, P]),
    "ct_admm_tv_solve_batch": (ctypes.c_int, [P, c_int32, P, P, P, c_int32, P, P, c_int32, P]),
    "ct_admm_tv3d_workspace": (ctypes.c_int, [P, P]),
    "ct_admm_tv3d_state": (ctypes.c_int, [P, P, P, P]),
    "ct_admm_tv3d_solve": (ctypes.c_int, [P, P, P, P, c_int32, P, c_size_t, P]),
    "ct_cg_block_workspace": (ctypes.c_int, [P, P, P]),
    "ct_cg_block_fwd": (ctypes.c_int, [P, P, c_float, P, P, P, c_size_t, P, c_size_t, P]),
    "ct_cg_block_bwd": (ctypes.c_int, [P, P, P, c_float, P, P, c_size_t, P, P, P, P, c_size_t, P]),
    "ct_padmm_tv_workspace": (ctypes.c_int, [P, P]),
    "ct_padmm_tv_state": (ctypes.c_int, [P, P, P, P, P]),
    "ct_padmm_tv_solve": (ctypes.c_int, [P, P, P, P, c_int32, P, c_size_t, P]),
}

_lock = threading.Lock()
_lib: ctypes.CDLL | None = None


def load() -> ctypes.CDLL:
    """Load the library (once) and declare every exported signature."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"ctgpu library not built ({LIB_PATH} missing); run "
                "`python -c 'import __graft_entry__ as g; g.build()'` or `python -m scico_gb300.build`"
            )
        lib = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def exported_symbols() -> list[str]:
    """Names of the C ABI functions this binding declares."""
    return sorted(_SIGNATURES)


def call(name: str, *args) -> None:
    """Call a status-returning ctgpu function; raise on failure."""
    lib = load()
    st = getattr(lib, name)(*args)
    if st != CT_OK:
        msg = (lib.ct_last_error() or b"").decode(errors="replace")
        text = (lib.ct_status_string(st) or b"").decode()
        exc = CtError(st, name, f"{text}: {msg}")
        if st == CT_ERR_SHAPE:
            raise ValueError(str(exc)) from exc
        raise exc


def check_device(stream) -> None:
    """Raise CtError if a projector's device-side check fired since the last
    check (a bounded wait ran out, or a span exceeded the plan: the guarded
    work was skipped).  Synchronises `stream`."""
    call("ct_proj2d_check", stream)
    w3 = load().ct_proj3d_errflag()
    if w3:
        raise CtError(CT_ERR_UNSUPPORTED, "ct_proj3d_errflag", f"3D projector device check word {w3:#x}")


def ptr(x) -> int:
    """Device (or host) address of a torch tensor / ctypes object / int."""
    if x is None:
        return 0
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    return ctypes.addressof(x)
