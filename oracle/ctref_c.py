"""ctypes wrapper of the C/OpenMP restatement (oracle/ctref.c).

TEST INFRASTRUCTURE ONLY (CPU baseline of bench.py, mid-size checks in
tests).  The geometry table is the oracle's float32 view parameters
(oracle/ctref.py:xray2d_view_params)."""

from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build
from . import ctref

_lib = None


class _Geom(ctypes.Structure):
    _fields_ = [("rows", ctypes.c_int), ("cols", ctypes.c_int), ("nv", ctypes.c_int), ("det", ctypes.c_int),
                ("views", ctypes.c_void_p)]


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(_build.build()))
        P = ctypes.c_void_p
        _lib.ref_proj2d_fwd.argtypes = [P, P, P]
        _lib.ref_proj2d_adj.argtypes = [P, P, P]
        _lib.ref_fd_fwd.argtypes = [ctypes.c_int, ctypes.c_int, P, P]
        _lib.ref_fd_adj.argtypes = [ctypes.c_int, ctypes.c_int, P, P]
        _lib.ref_set_threads.argtypes = [ctypes.c_int]
        _lib.ref_get_threads.restype = ctypes.c_int
        _lib.ref_admm_tv.argtypes = [P, P, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_float, P, P, P, P]
        _lib.ref_admm_tv.restype = ctypes.c_int
        _lib.ref_set_dot64.argtypes = [ctypes.c_int]
        _lib.ref_set_proj64.argtypes = [ctypes.c_int]
        _lib.ref_proj3d_fwd.argtypes = [P, P, ctypes.c_int, P, P, P]
        _lib.ref_proj3d_adj.argtypes = [P, P, ctypes.c_int, P, P, P]
    return _lib


class Geometry:
    """XRayTransform2D geometry in the form the C restatement takes."""

    def __init__(self, input_shape, angles, x0=None, dx=None, y0=None, det_count=None):
        self.g = ctref.xray2d_defaults(input_shape, angles, x0=x0, dx=dx, y0=y0, det_count=det_count)
        Pxmin, Pd0, Pd1, width = ctref.xray2d_view_params(self.g, np.float32)
        nv = len(Pxmin)
        self.table = np.zeros((nv, 8), dtype=np.float32)
        self.table[:, 0], self.table[:, 1], self.table[:, 2], self.table[:, 3] = Pxmin, Pd0, Pd1, width
        self.shape = tuple(input_shape)
        self.nv, self.det = nv, self.g["ny"]
        self.cg = _Geom(self.shape[0], self.shape[1], nv, self.det, self.table.ctypes.data)

    def project(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.empty((self.nv, self.det), dtype=np.float32)
        lib().ref_proj2d_fwd(ctypes.addressof(self.cg), x.ctypes.data, y.ctypes.data)
        return y

    def back_project(self, y: np.ndarray) -> np.ndarray:
        y = np.ascontiguousarray(y, dtype=np.float32)
        x = np.empty(self.shape, dtype=np.float32)
        lib().ref_proj2d_adj(ctypes.addressof(self.cg), y.ctypes.data, x.ctypes.data)
        return x

    def admm_tv(self, y, lam, rho, maxiter, cg_maxiter=10, cg_tol=1e-4, scale=0.5, state=None, dot64=False,
                proj64=False):
        """Run `maxiter` ADMM-TV iterations; returns (x, z, u, itstat (maxiter, 5)).

        dot64=False: float32 CG scalars as the reference; True: float64 dot
        products (the GPU solver's precision policy).  proj64: projector sums
        accumulated in float64 and rounded once (rounding-sensitivity probe)."""
        lib().ref_set_dot64(1 if dot64 else 0)
        lib().ref_set_proj64(1 if proj64 else 0)
        y = np.ascontiguousarray(y, dtype=np.float32)
        R, C = self.shape
        if state is None:
            x = np.zeros(self.shape, dtype=np.float32)
            z = np.zeros((2, R, C), dtype=np.float32)
            lib().ref_fd_fwd(R, C, x.ctypes.data, z.ctypes.data)
            u = np.zeros((2, R, C), dtype=np.float32)
        else:
            x, z, u = (np.ascontiguousarray(a, dtype=np.float32).copy() for a in state)
        it = np.zeros((maxiter, 5), dtype=np.float64)
        lib().ref_admm_tv(ctypes.addressof(self.cg), y.ctypes.data, lam, rho, scale, maxiter, cg_maxiter, cg_tol,
                          x.ctypes.data, z.ctypes.data, u.ctypes.data, it.ctypes.data)
        return x, z, u, it


class Geometry3D:
    """XRayTransform3D geometry (float32 (V, 2, 4) matrices) for the C
    restatement of the 3D projector."""

    def __init__(self, input_shape, matrices, det_shape):
        self.shape = tuple(int(n) for n in input_shape)
        self.det = tuple(int(n) for n in det_shape)
        self.mats = np.ascontiguousarray(matrices, dtype=np.float32).reshape(-1, 2, 4)
        self.nv = len(self.mats)
        self._shape = np.asarray(self.shape, dtype=np.int32)
        self._det = np.asarray(self.det, dtype=np.int32)

    def project(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.empty((self.nv,) + self.det, dtype=np.float32)
        lib().ref_proj3d_fwd(self._shape.ctypes.data, self._det.ctypes.data, self.nv, self.mats.ctypes.data,
                             x.ctypes.data, y.ctypes.data)
        return y

    def back_project(self, y: np.ndarray) -> np.ndarray:
        y = np.ascontiguousarray(y, dtype=np.float32)
        x = np.empty(self.shape, dtype=np.float32)
        lib().ref_proj3d_adj(self._shape.ctypes.data, self._det.ctypes.data, self.nv, self.mats.ctypes.data,
                             y.ctypes.data, x.ctypes.data)
        return x


def set_threads(n: int) -> int:
    lib().ref_set_threads(int(n))
    return lib().ref_get_threads()


def default_threads() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
