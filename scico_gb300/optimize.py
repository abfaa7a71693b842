"""ADMM with LinearSubproblemSolver, mirroring scico.optimize.

* :class:`ADMM` -- scico/optimize/_admm.py:34-378 with the solve loop,
  nanstop, iteration statistics and save/load of scico/optimize/_common.py:
  86-320.
* :class:`LinearSubproblemSolver` -- scico/optimize/_admmaux.py:118-269.

Two execution paths, same results (within float32 rounding):

* generic: ``ADMM.step`` composes the operators exactly as the reference
  does (every operator application is a ctgpu kernel launch);
* fused: when the problem is the CT TV pattern -- ``f = SquaredL2Loss(y,
  A=XRayTransform2D or XRayTransform3D)``, every ``C_i`` a
  ``FiniteDifference(append=0)`` over all image axes, ``g_i`` a scaled
  ``L21Norm()`` and/or ``L1Norm()``, equal ``rho_i``,
  ``LinearSubproblemSolver`` -- ``solve()`` runs ``ct_admm_tv_solve`` (2D)
  or ``ct_admm_tv3d_solve`` (3D): the whole outer iteration (x-update CG
  with device-side stopping test, z/u updates, iteration statistics)
  replayed as one CUDA graph.
"""

from __future__ import annotations

import collections
import math
import time
import weakref
from typing import Any, Callable, List, Optional

import numpy as np
import torch

from . import _device, _lib, linop
from .functional import Functional, L1Norm, L21Norm, ScaledFunctional, SeparableFunctional, ZeroFunctional
from .loss import SquaredL2Loss, _sqnorm
from .solver import cg as scico_cg

ITSTAT_FIELDS = ("Iter", "Time", "Objective", "Prml_Rsdl", "Dual_Rsdl", "CG_It", "CG_Res")
IterationRecord = collections.namedtuple("IterationRecord", ITSTAT_FIELDS)


class LinearSubproblemSolver:
    """x-update by CG on ``(A^T W A + sum_i rho_i C_i^T C_i) x = rhs``."""

    def __init__(self, cg_kwargs: Optional[dict] = None, cg_function: str = "scico", device=None):
        default = {"tol": 1e-4, "maxiter": 100}  # _admmaux.py:189
        if cg_kwargs:
            default.update(cg_kwargs)
        self.cg_kwargs = default
        if cg_function != "scico":
            raise ValueError(f"Argument 'cg_function' must be 'scico' here; got {cg_function}.")
        self.cg_function = cg_function
        self.cg = scico_cg
        self.info = None
        self.device = device

    def internal_init(self, admm: "ADMM"):
        if not isinstance(admm.f, SquaredL2Loss):
            raise TypeError(f"LinearSubproblemSolver requires f to be a SquaredL2Loss; got {type(admm.f)}.")
        if not isinstance(admm.f.A, linop.LinearOperator):
            raise TypeError(f"LinearSubproblemSolver requires f.A to be a LinearOperator; got {type(admm.f.A)}.")
        # a weak reference: the solver owns its subproblem solver, and a cycle
        # would keep a finished solver's device buffers alive until the
        # garbage collector runs
        self.admm = weakref.proxy(admm)
        lhs = None
        for rho, C in zip(admm.rho_list, admm.C_list):  # :222-224
            t = rho * C.gram_op
            lhs = t if lhs is None else lhs + t
        self.lhs_op = lhs + admm.f.hessian  # :225-227

    def compute_rhs(self):
        """``2 scale A^T y + sum_i rho_i C_i^T (z_i - u_i)`` (:231-256)."""
        admm = self.admm
        C0 = admm.C_list[0]
        rhs = _device.zeros(C0.input_shape)
        rhs = rhs + 2.0 * admm.f.scale * admm.f.A.adj(admm.f.y)
        for rho, C, z, u in zip(admm.rho_list, admm.C_list, admm.z_list, admm.u_list):
            rhs = rhs + rho * C.adj(_sub(z, u))
        return rhs

    def solve(self, x0):
        rhs = self.compute_rhs()
        x, self.info = self.cg(self.lhs_op, rhs, x0, **self.cg_kwargs)
        return x


def _sub(a, b):
    if isinstance(a, tuple):
        return tuple(u - v for u, v in zip(a, b))
    return a - b


def _g_kind(g: Functional):
    """('l21' | 'l1', weight) of a supported regulariser, else None."""
    scale = 1.0
    base = g
    if isinstance(g, ScaledFunctional):
        scale, base = g.scale, g.functional
    if isinstance(base, L21Norm) and base.l2_axis == 0:
        return "l21", scale
    if isinstance(base, L1Norm):
        return "l1", scale
    return None


class ADMM:
    """Alternating direction method of multipliers (scico/optimize/_admm.py:34)."""

    def __init__(self, f: Functional, g_list: List[Functional], C_list: List[linop.LinearOperator],
                 rho_list: List[float], alpha: float = 1.0, x0=None, subproblem_solver=None, **kwargs):
        N = len(g_list)
        if len(C_list) != N:
            raise ValueError(f"len(C_list)={len(C_list)} not equal to len(g_list)={N}.")
        if len(rho_list) != N:
            raise ValueError(f"len(rho_list)={len(rho_list)} not equal to len(g_list)={N}.")
        self.f, self.g_list, self.C_list = f, g_list, C_list
        self.rho_list = [float(r) for r in rho_list]
        self.alpha = float(alpha)
        if subproblem_solver is None:
            raise NotImplementedError("only LinearSubproblemSolver is implemented on the device path")
        self.subproblem_solver = subproblem_solver
        self.subproblem_solver.internal_init(self)
        if x0 is None:
            self.x = _device.zeros(C_list[0].input_shape)
        else:
            self.x = _device.to_device(x0, shape=C_list[0].input_shape, name="x0").clone()
        # z_list = z_init (:297-315), z_list_old, u_list = u_init (:317-332):
        # made on first use (the fused solver initialises its own state)
        self._zu = {}
        # Optimizer.__init__ (_common.py:117-135)
        self.itnum = kwargs.pop("iter0", 0)
        self.maxiter = kwargs.pop("maxiter", 100)
        self.nanstop = kwargs.pop("nanstop", False)
        itstat_options = kwargs.pop("itstat_options", None) or {}
        self.fused = kwargs.pop("fused", "auto")
        if kwargs:
            raise TypeError(f"Unrecognized keyword argument(s) {', '.join(kwargs)}")
        self.itstat_display = bool(itstat_options.get("display", False))
        self.itstat_period = int(itstat_options.get("period", 1))
        self._iters: List[IterationRecord] = []
        self._pending_records = []  # fused solves' itstat arrays, turned into records on first use
        self._fused_state = None
        self._elapsed = 0.0

    @property
    def iterations(self) -> List[IterationRecord]:
        for rec, it0, el0, dt in self._pending_records:
            m = len(rec)
            for k in range(m):
                r = rec[k]
                self._iters.append(IterationRecord(it0 + k, el0 + dt * (k + 1) / m, float(r[_lib.CT_ITSTAT_OBJECTIVE]),
                                                   float(r[_lib.CT_ITSTAT_PRIMAL]), float(r[_lib.CT_ITSTAT_DUAL]),
                                                   int(r[_lib.CT_ITSTAT_CG_ITERS]),
                                                   float(r[_lib.CT_ITSTAT_CG_RELRES])))
        self._pending_records = []
        return self._iters

    @iterations.setter
    def iterations(self, v: List[IterationRecord]):
        self._pending_records = []
        self._iters = list(v)

    # -- z and u state (made on first use) --------------------------------------
    def _zu_get(self, key):
        zu = self._zu
        if "z_list" not in zu:
            zu["z_list"] = [C(self.x) for C in self.C_list]  # before any step: x = x0
        if key == "u_list" and key not in zu:
            zu[key] = [_zeros_like(z) for z in zu["z_list"]]
        if key == "z_list_old" and key not in zu:
            zu[key] = list(zu["z_list"])
        return zu[key]

    z_list = property(lambda self: self._zu_get("z_list"), lambda self, v: self._zu.__setitem__("z_list", v))
    z_list_old = property(lambda self: self._zu_get("z_list_old"),
                          lambda self, v: self._zu.__setitem__("z_list_old", v))
    u_list = property(lambda self: self._zu_get("u_list"), lambda self, v: self._zu.__setitem__("u_list", v))

    def objective(self, x=None, z_list=None) -> float:
        if (x is None) != (z_list is None):
            raise ValueError("Both or neither of arguments 'x' and 'z_list' must be supplied.")
        if x is None:
            x, z_list = self.x, self.z_list
        out = self.f(x)
        for g, z in zip(self.g_list, z_list):
            out += g(z)
        return out

    def norm_primal_residual(self, x=None) -> float:
        x = self.x if x is None else x
        s = 0.0
        for rho, C, z in zip(self.rho_list, self.C_list, self.z_list):
            s += rho * _sqnorm(_flat(_sub(C(x), z)))
        return math.sqrt(s)

    def norm_dual_residual(self) -> float:
        acc = None
        for rho, z, zo, C in zip(self.rho_list, self.z_list, self.z_list_old, self.C_list):
            t = rho * C.adj(_sub(z, zo))
            acc = t if acc is None else acc + t
        return math.sqrt(_sqnorm(acc))

    def minimizer(self):
        return self.x

    # -- generic step (:334-378) ---------------------------------------------
    def step(self):
        self.x = self.subproblem_solver.solve(self.x)
        self.z_list_old = list(self.z_list)
        for i, (rho, g, C, z, u) in enumerate(zip(self.rho_list, self.g_list, self.C_list, self.z_list,
                                                  self.u_list)):
            Cx = C(self.x)
            if self.alpha != 1.0:
                Cx = _lin(self.alpha, Cx, 1.0 - self.alpha, z)
            z = g.prox(_add(Cx, u), 1.0 / rho, v0=z)
            u = _sub(_add(u, Cx), z)
            self.z_list[i] = z
            self.u_list[i] = u

    def _working_vars_finite(self) -> bool:
        for v in [self.x] + list(self.z_list) + list(self.u_list):
            for t in (v if isinstance(v, tuple) else (v,)):
                if not bool(torch.isfinite(t).all()):
                    return False
        return True

    def _record(self, rec: IterationRecord):
        self.iterations.append(rec)  # (pending fused records first, in order)
        if self.itstat_display and (rec.Iter % self.itstat_period == 0):
            print("  ".join(f"{k}={v:.4g}" if isinstance(v, float) else f"{k}={v}" for k, v in rec._asdict().items()))

    def solve(self, callback: Optional[Callable] = None):
        """Run ``maxiter`` iterations (Optimizer.solve, _common.py:287-320)."""
        use_fused = self.fused is True or (self.fused == "auto" and callback is None and self._fused_plan() is not None)
        if self.fused is True and self._fused_plan() is None:
            raise ValueError("fused=True but the problem is not the fused ADMM-TV pattern")
        if use_fused:
            self._solve_fused()
        else:
            t0 = time.perf_counter()
            for self.itnum in range(self.itnum, self.itnum + self.maxiter):
                self.step()
                if self.nanstop and not self._working_vars_finite():
                    raise ValueError(f"NaN or Inf value encountered in working variable in iteration {self.itnum}.")
                info = self.subproblem_solver.info or {}
                self._record(IterationRecord(self.itnum, self._elapsed + time.perf_counter() - t0,
                                             self.objective(), self.norm_primal_residual(),
                                             self.norm_dual_residual(), info.get("num_iter", 0),
                                             info.get("rel_res", float("nan"))))
                if callback:
                    callback(self)
            self._elapsed += time.perf_counter() - t0
            self.itnum += 1
        return self.minimizer()

    def history(self, transpose: bool = False):
        if transpose:
            return IterationRecord(*[list(col) for col in zip(*self.iterations)]) if self.iterations else \
                IterationRecord(*[[] for _ in ITSTAT_FIELDS])
        return list(self.iterations)

    # -- fused native path ------------------------------------------------------
    def _fused_plan(self):
        f = self.f
        if not isinstance(f, SquaredL2Loss) or not isinstance(f.A, (linop.XRayTransform2D, linop.XRayTransform3D)):
            return None
        if not isinstance(self.subproblem_solver, LinearSubproblemSolver):
            return None
        if len(set(self.rho_list)) != 1 or not (1 <= len(self.g_list) <= 2):
            return None
        shape = f.A.input_shape
        for C in self.C_list:
            if not isinstance(C, linop.FiniteDifference) or C.input_shape != shape:
                return None
            if C.axes != tuple(range(len(shape))) or C.append != 0 or C.prepend is not None or C.circular:
                return None
        kinds = [_g_kind(g) for g in self.g_list]
        if any(k is None for k in kinds) or len({k[0] for k in kinds}) != len(kinds):
            return None
        lam = {k: w for k, w in kinds}
        if any(w == 0 for w in lam.values()):
            return None
        # the native solver keeps its terms in the order L2,1 then L1
        native = [k for k in ("l21", "l1") if k in lam]
        order = [native.index(k) for k, _ in kinds]
        return dict(lam21=lam.get("l21", 0.0), lam1=lam.get("l1", 0.0), order=order)

    def _fused_prepare(self):
        """Descriptor, workspace (kept across calls) and output buffers of one
        fused solve of ``maxiter`` iterations."""
        plan = self._fused_plan()
        A = self.f.A
        cgk = self.subproblem_solver.cg_kwargs
        g = A.geometry()
        three = isinstance(A, linop.XRayTransform3D)
        Desc, fn = (_lib.AdmmTv3dDesc, "ct_admm_tv3d") if three else (_lib.AdmmTvDesc, "ct_admm_tv")
        desc = Desc(g, int(self.maxiter), int(cgk.get("maxiter", 100)), float(cgk.get("tol", 1e-4)),
                    float(cgk.get("atol", 0.0)), float(plan["lam21"]), float(plan["lam1"]),
                    float(self.rho_list[0]), float(self.f.scale), float(self.alpha), 1)
        st = self._fused_state
        first = st is None
        if first:
            nbytes = _lib.c_size_t()
            _lib.call(fn + "_workspace", _lib.ctypes.addressof(desc), _lib.ctypes.addressof(nbytes))
            ws = _device.workspace(nbytes.value)
            zoff, uoff, nt = _lib.c_size_t(), _lib.c_size_t(), _lib.c_int32()
            _lib.call(fn + "_state", _lib.ctypes.addressof(desc), _lib.ctypes.addressof(zoff),
                      _lib.ctypes.addressof(uoff), _lib.ctypes.addressof(nt))
            st = self._fused_state = dict(ws=ws, zoff=zoff.value, uoff=uoff.value, nt=nt.value, y=self.f.y)
        itstat = _device.zeros((max(1, self.maxiter), _lib.CT_ITSTAT_FIELDS), dtype=torch.float64)
        x = self.x.contiguous()
        return dict(plan=plan, desc=desc, fn=fn, st=st, first=first, itstat=itstat, x=x)

    def _fused_finish(self, run, dt):
        """Take over x, the z/u state and the iteration records of a fused solve."""
        A = self.f.A
        plan, st, itstat = run["plan"], run["st"], run["itstat"]
        self.x = run["x"]
        # expose z_list / u_list as views of the solver state (in g_list order)
        N = int(np.prod(A.input_shape))
        nd = len(A.input_shape)
        ws = st["ws"]
        zs = ws[st["zoff"]:st["zoff"] + st["nt"] * nd * N * 4].view(torch.float32).view(st["nt"], nd, *A.input_shape)
        us = ws[st["uoff"]:st["uoff"] + st["nt"] * nd * N * 4].view(torch.float32).view(st["nt"], nd, *A.input_shape)
        self.z_list = [zs[k] for k in plan["order"]]
        self.u_list = [us[k] for k in plan["order"]]
        rec = itstat.cpu().numpy()[: self.maxiter]
        if self.itstat_display:
            for k in range(self.maxiter):
                r = rec[k]
                self._record(IterationRecord(self.itnum + k, self._elapsed + dt * (k + 1) / self.maxiter,
                                             float(r[_lib.CT_ITSTAT_OBJECTIVE]), float(r[_lib.CT_ITSTAT_PRIMAL]),
                                             float(r[_lib.CT_ITSTAT_DUAL]), int(r[_lib.CT_ITSTAT_CG_ITERS]),
                                             float(r[_lib.CT_ITSTAT_CG_RELRES])))
        else:
            self._pending_records.append((rec, self.itnum, self._elapsed, dt))
        self._elapsed += dt
        self.itnum += self.maxiter
        if self.nanstop and not self._working_vars_finite():
            raise ValueError("NaN or Inf value encountered in a working variable during the fused solve.")

    def _solve_fused(self):
        run = self._fused_prepare()
        st = run["st"]
        t0 = time.perf_counter()
        _lib.call(run["fn"] + "_solve", _lib.ctypes.addressof(run["desc"]), st["y"].data_ptr(), run["x"].data_ptr(),
                  run["itstat"].data_ptr(), 0 if run["first"] else 1, st["ws"].data_ptr(), st["ws"].numel(),
                  _device.stream())
        _lib.check_device(_device.stream())  # synchronises; raises if a device check skipped work
        self._fused_finish(run, time.perf_counter() - t0)

    # -- state (_common.py:222-258) --------------------------------------------
    def save_state(self, path: str):
        def host(v):
            return np.stack([t.cpu().numpy() for t in v]) if isinstance(v, (list, tuple)) else v.cpu().numpy()

        np.savez(path, opt_class=np.array(type(self).__name__), itnum=self.itnum, x=host(self.x),
                 z_list=host(self.z_list), z_list_old=host(self.z_list_old), u_list=host(self.u_list),
                 history=np.array([tuple(r) for r in self.iterations], dtype=np.float64))

    def load_state(self, path: str):
        npz = np.load(path, allow_pickle=False)
        if str(npz["opt_class"]) != type(self).__name__:
            raise TypeError(f"Cannot load state for {npz['opt_class']} into optimizer of type {type(self)}.")
        self.itnum = int(npz["itnum"])
        self.x = _device.to_device(npz["x"])
        self.z_list = [_device.to_device(z) for z in npz["z_list"]]
        self.z_list_old = [_device.to_device(z) for z in npz["z_list_old"]]
        self.u_list = [_device.to_device(u) for u in npz["u_list"]]
        self.iterations = [IterationRecord(int(r[0]), *[float(v) for v in r[1:5]], int(r[5]), float(r[6]))
                           for r in npz["history"]]
        self._fused_state = None
        self.fused = False  # the fused solver state lives in its workspace; continue generically


def solve_batch(solvers: List["ADMM"], n_streams: int = 0) -> List[torch.Tensor]:
    """Run ``solve()`` of many independent 2D CT-TV ADMM problems at once.

    Each solver must be the fused pattern with an XRayTransform2D (see
    :class:`ADMM`); sizes, view counts, regularization weights and iteration
    counts may all differ.  The solves run concurrently through
    ``ct_admm_tv_solve_batch`` (each scan replays its own iteration graph on
    one of ``n_streams`` internal streams, 0 = automatic) and give the same
    iterates as calling ``solve()`` on each.  No counterpart in the
    reference, whose scripts solve one scan after another.  Returns the
    solutions in order.
    """
    if not solvers:
        return []
    for s in solvers:
        if s._fused_plan() is None or not isinstance(s.f.A, linop.XRayTransform2D):
            raise ValueError("solve_batch needs 2D problems of the fused ADMM-TV pattern")
        if s.fused is False:
            raise ValueError("solve_batch runs the fused solver; a solver has fused=False")
    runs = [s._fused_prepare() for s in solvers]
    if len({r["first"] for r in runs}) != 1:
        raise ValueError("solve_batch: all solvers must be fresh, or all continuing")
    n = len(runs)
    P = _lib.ctypes.c_void_p
    descs = (_lib.AdmmTvDesc * n)(*[r["desc"] for r in runs])
    ys = (P * n)(*[r["st"]["y"].data_ptr() for r in runs])
    xs = (P * n)(*[r["x"].data_ptr() for r in runs])
    its = (P * n)(*[r["itstat"].data_ptr() for r in runs])
    wss = (P * n)(*[r["st"]["ws"].data_ptr() for r in runs])
    nbs = (_lib.c_size_t * n)(*[r["st"]["ws"].numel() for r in runs])
    t0 = time.perf_counter()
    _lib.call("ct_admm_tv_solve_batch", _lib.ctypes.addressof(descs), n, _lib.ctypes.addressof(ys),
              _lib.ctypes.addressof(xs), _lib.ctypes.addressof(its), 0 if runs[0]["first"] else 1,
              _lib.ctypes.addressof(wss), _lib.ctypes.addressof(nbs), int(n_streams), _device.stream())
    _lib.check_device(_device.stream())  # synchronises; raises if a device check skipped work
    dt = time.perf_counter() - t0
    for s, r in zip(solvers, runs):
        s._fused_finish(r, dt)
    return [s.x for s in solvers]


def _zeros_like(z):
    if isinstance(z, tuple):
        return tuple(torch.zeros_like(t) for t in z)
    return torch.zeros_like(z)


def _add(a, b):
    if isinstance(a, tuple):
        return tuple(u + v for u, v in zip(a, b))
    return a + b


def _lin(a, x, b, y):
    if isinstance(x, tuple):
        return tuple(a * u + b * v for u, v in zip(x, y))
    return a * x + b * y


def _flat(v):
    if isinstance(v, tuple):
        return torch.cat([t.reshape(-1) for t in v])
    return v.reshape(-1)


def _zeros_of(shape):
    """Zeros of an array shape or of a block shape (tuple of shapes)."""
    if len(shape) and isinstance(shape[0], tuple):
        return tuple(_device.zeros(s) for s in shape)
    return _device.zeros(shape)


def _axpy(a: float, x, y):
    """a * x + y, blockwise."""
    if isinstance(x, tuple):
        return tuple(a * u + v for u, v in zip(x, y))
    return a * x + y


def _minus_c(v, c):
    if isinstance(c, (int, float)):
        if c == 0:
            return v
        return tuple(t - c for t in v) if isinstance(v, tuple) else v - c
    return _sub(v, c)


PADMMRecord = collections.namedtuple("PADMMRecord", ("Iter", "Time", "Objective", "Prml_Rsdl", "Dual_Rsdl"))


class ProximalADMM:
    r"""Proximal ADMM (scico/optimize/_padmm.py:180-411) for
    ``argmin f(x) + g(z)  s.t.  A x + B z = c``:

        x <- prox_{f / (rho mu)}(x - A^T(2u - u_old) / mu)
        z <- prox_{g / (rho nu)}(z - B^T(A x + B z - c + u) / nu)
        u <- u + A x + B z - c

    with ``mu > ||A||^2``, ``nu > ||B||^2`` (:meth:`estimate_parameters`).
    ``B = None`` means ``-I``, ``c = None`` zero.  Variables may be block
    variables (tuples of tensors), as with ``VerticalStack`` A and a
    ``SeparableFunctional`` g -- the CG-free 3D TV reconstruction of the
    reference's ct_3d_tv_padmm example.  Every operator application runs in
    the ctgpu kernels; ``A x`` is computed once per step and used for both
    the z-update and the u-update.

    ``fused`` ("auto", True, False): that example's pattern -- f =
    ZeroFunctional, A = VerticalStack((C, alpha * D)) with C an
    XRayTransform2D/3D and D = FiniteDifference(append=0) over all axes,
    g = SeparableFunctional((SquaredL2Loss(y), w * L21Norm())), B = None,
    c = None, fast dual residual -- runs in the native solver
    ``ct_padmm_tv_solve`` (one iteration captured as a CUDA graph, replayed
    ``maxiter`` times, residuals and objective computed in its kernels);
    every other problem runs the generic step loop.
    """

    def __init__(self, f: Functional, g: Functional, A: linop.LinearOperator, rho: float, mu: float, nu: float,
                 B: Optional[linop.LinearOperator] = None, c=None, x0=None, z0=None, u0=None,
                 fast_dual_residual: bool = True, fused="auto", **kwargs):
        self.fused = fused
        self._fused_state = None
        self._fused_ok = B is None and c is None and z0 is None and u0 is None and fast_dual_residual
        self.f, self.g, self.A = f, g, A
        self.B = -linop.Identity(A.output_shape) if B is None else B
        self.c = 0.0 if c is None else c
        self.rho, self.mu, self.nu = float(rho), float(mu), float(nu)
        self.fast_dual_residual = bool(fast_dual_residual)
        self.x = _zeros_of(A.input_shape) if x0 is None else _device.to_device(x0, shape=A.input_shape, name="x0")
        self.z = _zeros_of(self.B.input_shape) if z0 is None else z0
        self.z_old = self.z
        self.u = _zeros_of(A.output_shape) if u0 is None else u0
        self.u_old = self.u
        self.itnum = kwargs.pop("iter0", 0)
        self.maxiter = kwargs.pop("maxiter", 100)
        self.nanstop = kwargs.pop("nanstop", False)
        itstat_options = kwargs.pop("itstat_options", None) or {}
        if kwargs:
            raise TypeError(f"Unrecognized keyword argument(s) {', '.join(kwargs)}")
        self.itstat_display = bool(itstat_options.get("display", False))
        self.itstat_period = int(itstat_options.get("period", 1))
        self.iterations: List[PADMMRecord] = []
        self._elapsed = 0.0
        self._Ax = None

    # -- reference quantities (:121-176, 294-347) -----------------------------
    def objective(self, x=None, z=None) -> float:
        if (x is None) != (z is None):
            raise ValueError("Both or neither of arguments 'x' and 'z' must be supplied")
        if x is None:
            x, z = self.x, self.z
        return self.f(x) + self.g(z)

    def norm_primal_residual(self, x=None, z=None) -> float:
        if (x is None) != (z is None):
            raise ValueError("Both or neither of arguments 'x' and 'z' must be supplied")
        Ax = self.A(self.x) if x is None and self._Ax is None else (self._Ax if x is None else self.A(x))
        z = self.z if z is None else z
        return math.sqrt(_sqnorm(_flat(_minus_c(_add(Ax, self.B(z)), self.c))))

    def norm_dual_residual(self) -> float:
        d = _sub(self.z, self.z_old)
        if not self.fast_dual_residual:
            d = self.A.adj(self.B(d))
        return math.sqrt(_sqnorm(_flat(d)))

    def minimizer(self):
        return self.x

    def _working_vars_finite(self) -> bool:
        for v in (self.x, self.z, self.u):
            for t in (v if isinstance(v, tuple) else (v,)):
                if not bool(torch.isfinite(t).all()):
                    return False
        return True

    # -- iteration (:349-363) ---------------------------------------------------
    def step(self):
        proxarg = _axpy(-1.0 / self.mu, self.A.adj(_lin(2.0, self.u, -1.0, self.u_old)), self.x)
        self.x = self.f.prox(proxarg, 1.0 / (self.rho * self.mu), v0=self.x)
        Ax = self.A(self.x)
        proxarg = _axpy(-1.0 / self.nu, self.B.adj(_add(_minus_c(_add(Ax, self.B(self.z)), self.c), self.u)),
                        self.z)
        self.z_old = self.z
        self.z = self.g.prox(proxarg, 1.0 / (self.rho * self.nu), v0=self.z)
        self.u_old = self.u
        self.u = _add(self.u, _minus_c(_add(Ax, self.B(self.z)), self.c))
        self._Ax = Ax

    # -- fused native solver ------------------------------------------------
    def _fused_plan(self):
        """The ct_3d_tv_padmm pattern's parameters, or None."""
        if not self._fused_ok or not isinstance(self.f, ZeroFunctional):
            return None
        A = self.A
        if not isinstance(A, linop.VerticalStack) or len(A.ops) != 2:
            return None
        C, aD = A.ops
        if not isinstance(C, (linop.XRayTransform2D, linop.XRayTransform3D)):
            return None
        if not isinstance(aD, linop.ScaledLinearOperator) or not isinstance(aD.base, linop.FiniteDifference):
            return None
        D = aD.base
        shape = C.input_shape
        if D.input_shape != shape or D.axes != tuple(range(len(shape))) or D.append != 0 or \
                D.prepend is not None or D.circular or aD.scale == 0.0:
            return None
        g = self.g
        if not isinstance(g, SeparableFunctional) or len(g.functional_list) != 2:
            return None
        g0, g1 = g.functional_list
        if not isinstance(g0, SquaredL2Loss) or not g0.has_prox:
            return None
        if not isinstance(g1, ScaledFunctional) or not isinstance(g1.functional, L21Norm) or \
                g1.functional.l2_axis != 0:
            return None
        return dict(C=C, alpha=aD.scale, lam=g1.scale * aD.scale, y=g0.y, scale=g0.scale)

    def _solve_fused(self, plan):
        C = plan["C"]
        three = isinstance(C, linop.XRayTransform3D)
        desc = _lib.PadmmTvDesc()
        desc.nd = 3 if three else 2
        if three:
            desc.geom3 = C.geometry()
        else:
            desc.geom2 = C.geometry()
        desc.maxiter = int(self.maxiter)
        desc.lam, desc.alpha = float(plan["lam"]), float(plan["alpha"])
        desc.rho, desc.mu, desc.nu = self.rho, self.mu, self.nu
        desc.loss_scale = float(plan["scale"])
        desc.use_graph = 1
        first = self._fused_state is None
        if first:
            nb = _lib.c_size_t()
            _lib.call("ct_padmm_tv_workspace", _lib.ctypes.addressof(desc), _lib.ctypes.addressof(nb))
            offs = [_lib.c_size_t() for _ in range(4)]
            _lib.call("ct_padmm_tv_state", _lib.ctypes.addressof(desc), *[_lib.ctypes.addressof(o) for o in offs])
            self._fused_state = dict(ws=_device.workspace(nb.value), offs=[o.value for o in offs])
            self.x = self.x.contiguous().clone()
        st = self._fused_state
        y = plan["y"].contiguous()
        itstat = _device.zeros((max(1, self.maxiter), 3), dtype=torch.float64)
        t0 = time.perf_counter()
        _lib.call("ct_padmm_tv_solve", _lib.ctypes.addressof(desc), y.data_ptr(), self.x.data_ptr(),
                  itstat.data_ptr(), 0 if first else 1, st["ws"].data_ptr(), st["ws"].numel(), _device.stream())
        _lib.check_device(_device.stream())
        dt = time.perf_counter() - t0
        # z and u as views of the solver state (sinogram block, difference block)
        ws, (oz0, oz1, ou0, ou1) = st["ws"], st["offs"]
        S, M = int(np.prod(C.output_shape)), len(C.input_shape) * int(np.prod(C.input_shape))

        def view(off, n, shape):
            return ws[off:off + 4 * n].view(torch.float32).view(shape)

        dshape = (len(C.input_shape),) + tuple(C.input_shape)
        self.z = (view(oz0, S, C.output_shape), view(oz1, M, dshape))
        self.u = (view(ou0, S, C.output_shape), view(ou1, M, dshape))
        self._Ax = None
        rec = itstat.cpu().numpy()
        for k in range(self.maxiter):
            self.iterations.append(PADMMRecord(self.itnum + k, self._elapsed + dt * (k + 1) / self.maxiter,
                                               float(rec[k, 0]), float(rec[k, 1]), float(rec[k, 2])))
        self._elapsed += dt
        self.itnum += self.maxiter
        if self.nanstop and not self._working_vars_finite():
            raise ValueError("NaN or Inf value encountered in a working variable during the fused solve.")
        return self.x

    def solve(self, callback: Optional[Callable] = None):
        """Run ``maxiter`` iterations (Optimizer.solve, _common.py:287-320)."""
        if self.fused is not False and callback is None:
            plan = self._fused_plan()
            if plan is None and self.fused is True:
                raise ValueError("fused=True: the problem is not the fused CT-TV proximal ADMM pattern")
            if plan is not None:
                return self._solve_fused(plan)
        t0 = time.perf_counter()
        evaluatable = getattr(self.f, "has_eval", False) and getattr(self.g, "has_eval", False)
        for self.itnum in range(self.itnum, self.itnum + self.maxiter):
            self.step()
            if self.nanstop and not self._working_vars_finite():
                raise ValueError(f"NaN or Inf value encountered in working variable in iteration {self.itnum}.")
            rec = PADMMRecord(self.itnum, self._elapsed + time.perf_counter() - t0,
                              self.objective() if evaluatable else float("nan"), self.norm_primal_residual(),
                              self.norm_dual_residual())
            self.iterations.append(rec)
            if self.itstat_display and rec.Iter % self.itstat_period == 0:
                print("  ".join(f"{k}={v:.4g}" if isinstance(v, float) else f"{k}={v}"
                                for k, v in rec._asdict().items()))
            if callback:
                callback(self)
        self._elapsed += time.perf_counter() - t0
        self.itnum += 1
        return self.minimizer()

    def history(self, transpose: bool = False):
        if transpose:
            return PADMMRecord(*[list(col) for col in zip(*self.iterations)]) if self.iterations else \
                PADMMRecord(*[[] for _ in PADMMRecord._fields])
        return list(self.iterations)

    @staticmethod
    def estimate_parameters(A: linop.LinearOperator, B: Optional[linop.LinearOperator] = None,
                            factor: Optional[float] = 1.01, maxiter: int = 100, seed: Optional[int] = None):
        """(mu, nu) = factor * (||A||^2, ||B||^2) by power iteration, nu = 1
        for B = -I (:365-411)."""
        mu = linop.operator_norm(A, maxiter=maxiter, seed=seed) ** 2
        nu = 1.0 if B is None else linop.operator_norm(B, maxiter=maxiter, seed=seed) ** 2
        return (mu, nu) if factor is None else (factor * mu, factor * nu)


PGMRecord = collections.namedtuple("PGMRecord", ("Iter", "Time", "Objective", "L", "Residual"))


class PGMStepSize:
    """Constant step size 1/L0 (scico/optimize/_pgmaux.py PGMStepSize)."""

    def internal_init(self, solver):
        self.solver = solver

    def update(self, v) -> float:
        return self.solver.L


class PGM:
    r"""Proximal gradient method (scico/optimize/_pgm.py:30-180) for
    ``f(x) + g(x)``: ``x <- prox_{g/L}(x - grad f(x) / L)``."""

    def __init__(self, f: Functional, g: Functional, L0: float, x0, step_size: Optional[PGMStepSize] = None,
                 **kwargs):
        self.f = f
        if g.has_prox is not True:
            raise ValueError(f"Functional 'g' ({type(g)}) must have a prox method.")
        self.g = g
        self.step_size = PGMStepSize() if step_size is None else step_size
        self.step_size.internal_init(self)
        self.L = float(L0)
        self.fixed_point_residual = float("inf")
        self.x = _device.to_device(x0, name="x0").clone()
        self.itnum = kwargs.pop("iter0", 0)
        self.maxiter = kwargs.pop("maxiter", 100)
        self.nanstop = kwargs.pop("nanstop", False)
        itstat_options = kwargs.pop("itstat_options", None) or {}
        if kwargs:
            raise TypeError(f"Unrecognized keyword argument(s) {', '.join(kwargs)}")
        self.itstat_display = bool(itstat_options.get("display", False))
        self.itstat_period = int(itstat_options.get("period", 1))
        self.iterations: List[PGMRecord] = []
        self._elapsed = 0.0

    def x_step(self, v, L: float):
        return self.g.prox(v - (1.0 / L) * self.f.grad(v), 1.0 / L)

    def objective(self, x=None) -> float:
        x = self.x if x is None else x
        return self.f(x) + self.g(x)

    def norm_residual(self) -> float:
        return self.fixed_point_residual

    def minimizer(self):
        return self.x

    def step(self):
        self.L = self.step_size.update(self.x)
        x = self.x_step(self.x, self.L)
        self.fixed_point_residual = math.sqrt(_sqnorm((self.x - x).reshape(-1)))
        self.x = x

    def solve(self, callback: Optional[Callable] = None):
        t0 = time.perf_counter()
        evaluatable = getattr(self.f, "has_eval", False) and getattr(self.g, "has_eval", False)
        for self.itnum in range(self.itnum, self.itnum + self.maxiter):
            self.step()
            if self.nanstop and not bool(torch.isfinite(self.x).all()):
                raise ValueError(f"NaN or Inf value encountered in working variable in iteration {self.itnum}.")
            rec = PGMRecord(self.itnum, self._elapsed + time.perf_counter() - t0,
                            self.objective() if evaluatable else float("nan"), self.L, self.norm_residual())
            self.iterations.append(rec)
            if self.itstat_display and rec.Iter % self.itstat_period == 0:
                print("  ".join(f"{k}={v:.4g}" if isinstance(v, float) else f"{k}={v}"
                                for k, v in rec._asdict().items()))
            if callback:
                callback(self)
        self._elapsed += time.perf_counter() - t0
        self.itnum += 1
        return self.minimizer()

    def history(self, transpose: bool = False):
        if transpose:
            return PGMRecord(*[list(col) for col in zip(*self.iterations)]) if self.iterations else \
                PGMRecord(*[[] for _ in PGMRecord._fields])
        return list(self.iterations)


class AcceleratedPGM(PGM):
    r"""Accelerated PGM / FISTA (scico/optimize/_pgm.py:183-252):
    ``x <- prox step at v``, ``t' = (1 + sqrt(1 + 4 t^2)) / 2``,
    ``v <- x + (t - 1)/t' (x - x_old)``."""

    def __init__(self, f: Functional, g: Functional, L0: float, x0, step_size: Optional[PGMStepSize] = None,
                 **kwargs):
        super().__init__(f=f, g=g, L0=L0, x0=x0, step_size=step_size, **kwargs)
        self.v = self.x.clone()
        self.t = 1.0

    def step(self):
        x_old = self.x
        self.L = self.step_size.update(self.v)
        self.x = self.x_step(self.v, self.L)
        self.fixed_point_residual = math.sqrt(_sqnorm((self.x - self.v).reshape(-1)))
        t_old = self.t
        self.t = 0.5 * (1.0 + math.sqrt(1.0 + 4.0 * t_old ** 2))
        self.v = self.x + ((t_old - 1.0) / self.t) * (self.x - x_old)
