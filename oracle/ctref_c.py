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

_libs = {}


class _Geom(ctypes.Structure):
    _fields_ = [("rows", ctypes.c_int), ("cols", ctypes.c_int), ("nv", ctypes.c_int), ("det", ctypes.c_int),
                ("views", ctypes.c_void_p)]


def lib(f64: bool = False):
    """The float32 build of the restatement, or the float64 one (f64=True)."""
    key = bool(f64)
    if key not in _libs:
        L = ctypes.CDLL(str(_build.build(f64=key)))
        P = ctypes.c_void_p
        f = ctypes.c_double if key else ctypes.c_float
        L.ref_proj2d_fwd.argtypes = [P, P, P]
        L.ref_proj2d_adj.argtypes = [P, P, P]
        L.ref_fd_fwd.argtypes = [ctypes.c_int, ctypes.c_int, P, P]
        L.ref_fd_adj.argtypes = [ctypes.c_int, ctypes.c_int, P, P]
        L.ref_set_threads.argtypes = [ctypes.c_int]
        L.ref_get_threads.restype = ctypes.c_int
        L.ref_admm_tv.argtypes = [P, P, f, f, f, ctypes.c_int, ctypes.c_int, f, P, P, P, P]
        L.ref_admm_tv.restype = ctypes.c_int
        L.ref_set_dot64.argtypes = [ctypes.c_int]
        L.ref_set_proj64.argtypes = [ctypes.c_int]
        L.ref_proj3d_fwd.argtypes = [P, P, ctypes.c_int, P, P, P]
        L.ref_proj3d_adj.argtypes = [P, P, ctypes.c_int, P, P, P]
        L.ref_admm_tv3d.argtypes = [P, P, ctypes.c_int, P, P, f, f, f, f, ctypes.c_int, ctypes.c_int, f, P, P, P, P]
        L.ref_admm_tv3d.restype = ctypes.c_int
        _libs[key] = L
    return _libs[key]


class Geometry:
    """XRayTransform2D geometry in the form the C restatement takes.

    f64=False: the float32 restatement (geometry, weights, sums and solver
    in float32, as the reference's default precision); f64=True: the float64
    build (the restatement of an x64 run: view parameters, weights, sums and
    solver in float64; arrays are passed and returned as float64)."""

    def __init__(self, input_shape, angles, x0=None, dx=None, y0=None, det_count=None, f64=False):
        self.f64 = bool(f64)
        self.dt = np.float64 if self.f64 else np.float32
        self.g = ctref.xray2d_defaults(input_shape, angles, x0=x0, dx=dx, y0=y0, det_count=det_count)
        Pxmin, Pd0, Pd1, width = ctref.xray2d_view_params(self.g, self.dt)
        nv = len(Pxmin)
        self.table = np.zeros((nv, 8), dtype=self.dt)
        self.table[:, 0], self.table[:, 1], self.table[:, 2], self.table[:, 3] = Pxmin, Pd0, Pd1, width
        self.shape = tuple(input_shape)
        self.nv, self.det = nv, self.g["ny"]
        self.cg = _Geom(self.shape[0], self.shape[1], nv, self.det, self.table.ctypes.data)

    def project(self, x: np.ndarray, proj64: bool = False) -> np.ndarray:
        """A x; proj64: sums accumulated in float64 and rounded once."""
        x = np.ascontiguousarray(x, dtype=self.dt)
        y = np.empty((self.nv, self.det), dtype=self.dt)
        lib(self.f64).ref_set_proj64(1 if proj64 else 0)
        lib(self.f64).ref_proj2d_fwd(ctypes.addressof(self.cg), x.ctypes.data, y.ctypes.data)
        return y

    def back_project(self, y: np.ndarray, proj64: bool = False) -> np.ndarray:
        """A^T y; proj64 as for project."""
        y = np.ascontiguousarray(y, dtype=self.dt)
        x = np.empty(self.shape, dtype=self.dt)
        lib(self.f64).ref_set_proj64(1 if proj64 else 0)
        lib(self.f64).ref_proj2d_adj(ctypes.addressof(self.cg), y.ctypes.data, x.ctypes.data)
        return x

    def admm_tv(self, y, lam, rho, maxiter, cg_maxiter=10, cg_tol=1e-4, scale=0.5, state=None, dot64=False,
                proj64=False):
        """Run `maxiter` ADMM-TV iterations; returns (x, z, u, itstat (maxiter, 5)).

        dot64=False: float32 CG scalars as the reference; True: float64 dot
        products (the GPU solver's precision policy).  proj64: projector sums
        accumulated in float64 and rounded once (rounding-sensitivity probe)."""
        L, dt = lib(self.f64), self.dt
        L.ref_set_dot64(1 if dot64 else 0)
        L.ref_set_proj64(1 if proj64 else 0)
        y = np.ascontiguousarray(y, dtype=dt)
        R, C = self.shape
        if state is None:
            x = np.zeros(self.shape, dtype=dt)
            z = np.zeros((2, R, C), dtype=dt)
            L.ref_fd_fwd(R, C, x.ctypes.data, z.ctypes.data)
            u = np.zeros((2, R, C), dtype=dt)
        else:
            x, z, u = (np.ascontiguousarray(a, dtype=dt).copy() for a in state)
        it = np.zeros((maxiter, 5), dtype=np.float64)
        L.ref_admm_tv(ctypes.addressof(self.cg), y.ctypes.data, lam, rho, scale, maxiter, cg_maxiter, cg_tol,
                          x.ctypes.data, z.ctypes.data, u.ctypes.data, it.ctypes.data)
        return x, z, u, it


class Geometry3D:
    """XRayTransform3D geometry ((V, 2, 4) matrices) for the C restatement
    of the 3D projector; f64 as for Geometry (float64 matrices, weights,
    sums and solver)."""

    def __init__(self, input_shape, matrices, det_shape, f64=False):
        self.f64 = bool(f64)
        self.dt = np.float64 if self.f64 else np.float32
        self.shape = tuple(int(n) for n in input_shape)
        self.det = tuple(int(n) for n in det_shape)
        self.mats = np.ascontiguousarray(matrices, dtype=self.dt).reshape(-1, 2, 4)
        self.nv = len(self.mats)
        self._shape = np.asarray(self.shape, dtype=np.int32)
        self._det = np.asarray(self.det, dtype=np.int32)

    def project(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=self.dt)
        y = np.empty((self.nv,) + self.det, dtype=self.dt)
        lib(self.f64).ref_proj3d_fwd(self._shape.ctypes.data, self._det.ctypes.data, self.nv, self.mats.ctypes.data,
                             x.ctypes.data, y.ctypes.data)
        return y

    def back_project(self, y: np.ndarray) -> np.ndarray:
        y = np.ascontiguousarray(y, dtype=self.dt)
        x = np.empty(self.shape, dtype=self.dt)
        lib(self.f64).ref_proj3d_adj(self._shape.ctypes.data, self._det.ctypes.data, self.nv, self.mats.ctypes.data,
                             y.ctypes.data, x.ctypes.data)
        return x

    def admm_tv(self, y, lam_l21, lam_l1, rho, maxiter, cg_maxiter=8, cg_tol=1e-4, scale=0.5, state=None,
                dot64=False):
        """Run `maxiter` iterations of ADMM-TV with g = lam_l21 ||Dx||_{2,1}
        + lam_l1 ||Dx||_1 (terms with a zero weight left out, one z/u block
        each, L2,1 first); returns (x, z, u, itstat (maxiter, 5)).  dot64 as
        for the 2D solve."""
        L, dt = lib(self.f64), self.dt
        L.ref_set_dot64(1 if dot64 else 0)
        L.ref_set_proj64(0)
        y = np.ascontiguousarray(y, dtype=dt)
        nt = int(lam_l21 != 0) + int(lam_l1 != 0)
        if state is None:
            x = np.zeros(self.shape, dtype=dt)
            z = np.zeros((nt, 3) + self.shape, dtype=dt)
            u = np.zeros_like(z)
        else:
            x, z, u = (np.ascontiguousarray(a, dtype=dt).copy() for a in state)
        it = np.zeros((maxiter, 5), dtype=np.float64)
        rc = L.ref_admm_tv3d(self._shape.ctypes.data, self._det.ctypes.data, self.nv, self.mats.ctypes.data,
                                 y.ctypes.data, lam_l21, lam_l1, rho, scale, maxiter, cg_maxiter, cg_tol,
                                 x.ctypes.data, z.ctypes.data, u.ctypes.data, it.ctypes.data)
        if rc != 0:
            raise RuntimeError(f"ref_admm_tv3d failed ({rc})")
        return x, z, u, it


def set_threads(n: int) -> int:
    for f64 in (False, True):
        lib(f64).ref_set_threads(int(n))
    return lib().ref_get_threads()


def default_threads() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
