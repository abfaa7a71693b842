"""Full-length ADMM-TV solves at the benchmark configurations against the
oracle: the 256^2 / 180-view problem for its 50 iterations, the 512^2 /
360-view problem for its 100, and the 3D L2,1 + L1 problem for its 30 (on a
128^3 / 180-view volume: the C restatement of the 3D projector takes about
1.5 minutes of 16 cores for that solve, 25 minutes at the full 256^3 / 360
views).

What full-length parity can mean here.  With CG capped at 10 (3D: 8) steps
and a stopping test relative to ||b|| (dominated by c A^T y), the x-update
is an unconverged, rounding-sensitive map, and on the 512^2 problem the
stopping test starts to pass at its first step somewhere between iteration
11 and 20, after which x does not change.  Where that happens depends on
float32 rounding alone: equally valid evaluations of the same algorithm
(the oracle with its projector summed in float32 or in float64, this GPU
path on the sinogram perturbed by one ulp per bin) end 1e-3 .. 5e-2 apart
in x.  The bar is therefore a floor measured in the test from those
evaluations: x, the objective trajectory and the SNR to the phantom must
lie within 3x that floor of the oracle run with the GPU's own precision
policy (float32 vectors, float64 dot products).  The oracle with the
reference's float32 CG scalars and the float64 restatement (an x64 run)
are evaluated beside it and reported; against them the bar is 3x the
largest spread among all the evaluations.  Each test prints one FULLSOLVE
line with every distance and the CG step counts.
"""

import json

import numpy as np
import pytest
import torch

from oracle import ctref, ctref_c
from scico_gb300 import functional, linop, loss, workloads
from scico_gb300.optimize import ADMM, LinearSubproblemSolver

pytestmark = pytest.mark.gpu


def _perturb(y, seed=7):
    """y with every bin moved by one float32 ulp (relative 2^-23) up or down."""
    sign = np.where(np.random.default_rng(seed).random(y.shape) < 0.5, -1.0, 1.0).astype(np.float32)
    return (y * (np.float32(1.0) + sign * np.float32(2.0**-23))).astype(np.float32)


def _rel(a, b):
    return float(ctref.rel_l2(np.asarray(a, np.float64), np.asarray(b, np.float64)))


def _orel(a, b):
    return float(np.max(np.abs(np.asarray(a) / np.asarray(b) - 1)))


def _gpu_2d(cuda, c, y):
    A = linop.XRayTransform2D((c.n, c.n), c.angles, det_count=c.det_count)
    s = ADMM(f=loss.SquaredL2Loss(y=torch.from_numpy(y).to(cuda), A=A), g_list=[c.lam * functional.L21Norm()],
             C_list=[linop.FiniteDifference((c.n, c.n), append=0)], rho_list=[c.rho], maxiter=c.maxiter,
             subproblem_solver=LinearSubproblemSolver(cg_kwargs={"tol": c.cg_tol, "maxiter": c.cg_maxiter}),
             fused=True)
    x = s.solve().cpu().numpy()
    h = s.history(transpose=True)
    return x, np.array(h.Objective), np.array(h.CG_It, dtype=int)


_CACHE = {}


def _case_2d(cuda, name):
    """GPU solves (sinogram and its one-ulp perturbation) and the oracle
    solves of one 2D configuration, computed once per test session."""
    if name in _CACHE:
        return _CACHE[name]
    c = {"c1": workloads.C1, "c2": workloads.C2}[name]
    G = ctref_c.Geometry((c.n, c.n), c.angles, det_count=c.det_count)
    ctref_c.set_threads(ctref_c.default_threads())
    x_gt = c.phantom()
    y = workloads.noisy(G.project(x_gt), c.noise, c.noise_seed)
    r = {"c": c, "x_gt": x_gt, "y": y}
    r["gpu"] = _gpu_2d(cuda, c, y)
    r["gpu_q"] = _gpu_2d(cuda, c, _perturb(y))
    kw = dict(cg_maxiter=c.cg_maxiter, cg_tol=c.cg_tol)
    for key, opts in (("dot64", dict(dot64=True)), ("dot64_proj64", dict(dot64=True, proj64=True))):
        xo, _, _, it = G.admm_tv(y, c.lam, c.rho, c.maxiter, **kw, **opts)
        r[key] = (xo, it[:, 0], it[:, 3].astype(int))
    _CACHE[name] = r
    return r


def _report(tag, d):
    print("FULLSOLVE " + tag + " " + json.dumps(d), flush=True)


def _diverging(k1, k2):
    return [int(i) for i in np.nonzero(np.asarray(k1) != np.asarray(k2))[0]]


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_full_solve_vs_oracle(cuda, name):
    """The whole benchmark solve against the oracle under the GPU's precision
    policy, within 3x the measured rounding floor (x, objective, SNR)."""
    r = _case_2d(cuda, name)
    x, obj, k = r["gpu"]
    xq, objq, kq = r["gpu_q"]
    xm, om, km = r["dot64"]
    xp, op, kp = r["dot64_proj64"]
    snr = lambda v: float(ctref.snr(r["x_gt"], v))
    fx = max(_rel(xp, xm), _rel(xq, x))
    fo = max(_orel(op, om), _orel(objq, obj))
    fs = max(abs(snr(xp) - snr(xm)), abs(snr(xq) - snr(x)))
    ex, eo, es = _rel(x, xm), _orel(obj, om), abs(snr(x) - snr(xm))
    _report(name, {"iterations": len(obj), "rel_l2_x_vs_oracle": ex, "floor_x": fx, "objective_max_rel": eo,
                   "floor_objective": fo, "snr_gpu": snr(x), "snr_oracle": snr(xm), "floor_snr": fs,
                   "final_objective_gpu": float(obj[-1]), "final_objective_oracle": float(om[-1]),
                   "cg_steps_gpu": int(k.sum()), "cg_steps_oracle": int(km.sum()),
                   "cg_steps_oracle_proj64": int(kp.sum()), "cg_steps_gpu_perturbed": int(kq.sum()),
                   "iterations_where_cg_counts_differ": _diverging(k, km)})
    assert len(obj) == r["c"].maxiter
    assert ex <= 3 * fx + 1e-4, (ex, fx)
    assert eo <= 3 * fo + 1e-5, (eo, fo)
    assert es <= 3 * fs + 0.02, (es, fs)


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_full_solve_vs_reference_precisions(cuda, name):
    """The same solve against the oracle with the reference's own float32 CG
    scalars and against the float64 restatement (an x64 run of the
    reference); the distances are reported, and each must stay within 3x
    the largest spread among all the evaluations of the problem."""
    r = _case_2d(cuda, name)
    c = r["c"]
    x, obj, k = r["gpu"]
    kw = dict(cg_maxiter=c.cg_maxiter, cg_tol=c.cg_tol)
    G = ctref_c.Geometry((c.n, c.n), c.angles, det_count=c.det_count)
    xr, _, _, itr = G.admm_tv(r["y"], c.lam, c.rho, c.maxiter, dot64=False, **kw)
    G64 = ctref_c.Geometry((c.n, c.n), c.angles, det_count=c.det_count, f64=True)
    x64, _, _, it64 = G64.admm_tv(r["y"].astype(np.float64), c.lam, c.rho, c.maxiter, dot64=True, **kw)
    evals = {"gpu": x, "gpu_perturbed": r["gpu_q"][0], "oracle_dot64": r["dot64"][0],
             "oracle_dot64_proj64": r["dot64_proj64"][0], "oracle_f32_scalars": xr, "oracle_f64": x64}
    names = list(evals)
    spread = max(_rel(evals[a], evals[b]) for i, a in enumerate(names) for b in names[i + 1:])
    e32, e64 = _rel(x, xr), _rel(x, x64)
    snr = lambda v: float(ctref.snr(r["x_gt"], v))
    _report(name + "_precisions", {"rel_l2_x_vs_f32_scalars": e32, "rel_l2_x_vs_f64": e64,
                                   "largest_spread": spread, "objective_max_rel_vs_f32_scalars": _orel(obj, itr[:, 0]),
                                   "objective_max_rel_vs_f64": _orel(obj, it64[:, 0]),
                                   "snr_gpu": snr(x), "snr_f32_scalars": snr(xr), "snr_f64": snr(x64),
                                   "cg_steps_gpu": int(k.sum()), "cg_steps_f32_scalars": int(itr[:, 3].sum()),
                                   "cg_steps_f64": int(it64[:, 3].sum())})
    assert e32 <= 3 * spread and e64 <= 3 * spread, (e32, e64, spread)


def test_full_solve_3d_vs_oracle(cuda):
    """The 3D benchmark problem's solve (L2,1 + L1 on one FiniteDifference,
    lambda 0.005 each, rho 1, 30 iterations, CG <= 8, rotation about axis 0)
    on a 128^3 volume with 180 views, against the C restatement with float64
    dot products, within 3x the floor measured against the oracle with the
    reference's float32 CG scalars and this path on a one-ulp-perturbed
    projection set."""
    c5 = workloads.C5
    n, nv = 128, 180
    det = (n, int(np.ceil(np.sqrt(2.0) * n)) + 1)
    ang = np.linspace(0, np.pi, nv, endpoint=False)
    M = linop.XRayTransform3D.matrices_from_euler_angles((n, n, n), det, "X", ang[:, None])
    G = ctref_c.Geometry3D((n, n, n), np.asarray(M, np.float32), det)
    ctref_c.set_threads(ctref_c.default_threads())
    x_gt = workloads.random_ellipsoids(n, c5.n_ellipsoids, c5.phantom_seed)
    y0 = G.project(x_gt)
    y = (y0 + c5.noise * np.abs(y0).max() * np.random.default_rng(c5.noise_seed).standard_normal(y0.shape)).astype(
        np.float32)

    def gpu(yv):
        A = linop.XRayTransform3D((n, n, n), M, det)
        C = linop.FiniteDifference((n, n, n), append=0)
        s = ADMM(f=loss.SquaredL2Loss(y=torch.from_numpy(yv).to(cuda), A=A),
                 g_list=[c5.lam_l21 * functional.L21Norm(), c5.lam_l1 * functional.L1Norm()], C_list=[C, C],
                 rho_list=[c5.rho] * 2, maxiter=c5.maxiter,
                 subproblem_solver=LinearSubproblemSolver(cg_kwargs={"tol": c5.cg_tol, "maxiter": c5.cg_maxiter}),
                 fused=True)
        xs = s.solve().cpu().numpy()
        h = s.history(transpose=True)
        return xs, np.array(h.Objective), np.array(h.CG_It, dtype=int)

    x, obj, k = gpu(y)
    xq, objq, _ = gpu(_perturb(y))
    kw = dict(cg_maxiter=c5.cg_maxiter, cg_tol=c5.cg_tol)
    xm, _, _, itm = G.admm_tv(y, c5.lam_l21, c5.lam_l1, c5.rho, c5.maxiter, dot64=True, **kw)
    xr, _, _, itr = G.admm_tv(y, c5.lam_l21, c5.lam_l1, c5.rho, c5.maxiter, dot64=False, **kw)
    fx = max(_rel(xr, xm), _rel(xq, x))
    fo = max(_orel(itr[:, 0], itm[:, 0]), _orel(objq, obj))
    ex, eo = _rel(x, xm), _orel(obj, itm[:, 0])
    _report("3d_128", {"iterations": len(obj), "rel_l2_x_vs_oracle": ex, "floor_x": fx, "objective_max_rel": eo,
                      "floor_objective": fo, "rel_l2_x_vs_f32_scalars": _rel(x, xr),
                      "cg_steps_gpu": int(k.sum()), "cg_steps_oracle": int(itm[:, 3].sum()),
                      "cg_steps_f32_scalars": int(itr[:, 3].sum()),
                      "iterations_where_cg_counts_differ": _diverging(k, itm[:, 3].astype(int))})
    assert len(obj) == c5.maxiter
    assert ex <= 3 * fx + 1e-4, (ex, fx)
    assert eo <= 3 * fo + 1e-5, (eo, fo)
