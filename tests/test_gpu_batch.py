"""Concurrent solves of many 2D scans (ct_admm_tv_solve_batch through
optimize.solve_batch): every scan's result is bit-identical to solving it
alone, for any number of internal streams; continuation and argument checks;
the 64-scan uneven workload runs."""

import numpy as np
import pytest
import torch

from oracle import ctref
from scico_gb300 import _lib, functional, linop, loss, workloads
from scico_gb300.optimize import ADMM, LinearSubproblemSolver, solve_batch

pytestmark = pytest.mark.gpu


def _scan(cuda, n, nv, lam, seed, maxiter=4, cg_maxiter=6, l1=0.0):
    ang = np.linspace(0, np.pi, nv, endpoint=False)
    det = int(np.ceil(np.sqrt(2.0) * n)) + 1
    A = linop.XRayTransform2D((n, n), ang, det_count=det)
    x_gt = torch.from_numpy(workloads.random_ellipses(n, 5, seed)).to(cuda)
    y = A(x_gt)
    y = y + 0.01 * y.abs().max() * torch.randn(y.shape, generator=torch.Generator().manual_seed(seed)).to(cuda)
    C = linop.FiniteDifference((n, n), append=0)
    gl, Cl = [lam * functional.L21Norm()], [C]
    if l1:
        gl.append(l1 * functional.L1Norm())
        Cl.append(C)
    return ADMM(f=loss.SquaredL2Loss(y=y, A=A), g_list=gl, C_list=Cl, rho_list=[1.0] * len(gl), maxiter=maxiter,
                subproblem_solver=LinearSubproblemSolver(cg_kwargs={"tol": 1e-4, "maxiter": cg_maxiter}))


SPECS = [(32, 24, 0.01, 1), (96, 60, 0.005, 2), (48, 90, 0.02, 3), (64, 45, 0.01, 4, 0.005), (40, 30, 0.003, 5),
         (80, 120, 0.008, 6)]


def _make(cuda, **kw):
    return [_scan(cuda, s[0], s[1], s[2], s[3], l1=(s[4] if len(s) > 4 else 0.0), **kw) for s in SPECS]


@pytest.mark.parametrize("n_streams", [0, 1, 3])
def test_batch_equals_individual(cuda, n_streams):
    ref = [s.solve().clone() for s in _make(cuda)]
    batch = _make(cuda)
    xs = solve_batch(batch, n_streams=n_streams)
    for a, b, s in zip(ref, xs, batch):
        assert torch.equal(a, b)
        assert len(s.history()) == 4
    ind = _make(cuda)
    for s in ind:
        s.solve()
    for s, t in zip(batch, ind):
        assert s.history(transpose=True).Objective == t.history(transpose=True).Objective
        for za, zb in zip(s.z_list, t.z_list):
            assert torch.equal(za, zb)


def test_batch_continuation(cuda):
    full = _make(cuda, maxiter=4)
    xs_full = solve_batch(full)
    half = _make(cuda, maxiter=2)
    solve_batch(half)
    xs = solve_batch(half)  # continues from the workspaces
    for a, b in zip(xs_full, xs):
        assert ctref.rel_l2(b.cpu().numpy(), a.cpu().numpy()) <= 1e-6


def test_batch_argument_checks(cuda):
    s = _make(cuda)[:2]
    with pytest.raises(_lib.CtError, match="n_streams"):
        solve_batch(s, n_streams=99)
    A3 = linop.XRayTransform3D((8, 8, 8), linop.XRayTransform3D.matrices_from_euler_angles(
        (8, 8, 8), (8, 13), "X", [[0.1], [0.6]]), (8, 13))
    y3 = torch.zeros(A3.output_shape, device=cuda)
    C3 = linop.FiniteDifference((8, 8, 8), append=0)
    s3 = ADMM(f=loss.SquaredL2Loss(y=y3, A=A3), g_list=[0.01 * functional.L21Norm()], C_list=[C3], rho_list=[1.0],
              maxiter=1, subproblem_solver=LinearSubproblemSolver())
    with pytest.raises(ValueError, match="2D problems"):
        solve_batch([s3])
    assert solve_batch([]) == []


def test_c3_workload_batch(cuda):
    """The 64 uneven scans (N 128..768, 90..720 views, det ceil(sqrt2 N)+1,
    lambda per scan): two iterations batched equal two iterations solved one
    by one, for a sample of the scans."""
    cfgs = workloads.batched_configs()
    assert len(cfgs) == 64

    def build():
        out = []
        for c in cfgs:
            A = linop.XRayTransform2D((c.n, c.n), c.angles, det_count=c.det_count)
            x_gt = torch.from_numpy(c.phantom()).to(cuda)
            y = A(x_gt)
            y = y + c.noise * y.abs().max() * torch.randn(
                y.shape, generator=torch.Generator().manual_seed(c.noise_seed)).to(cuda)
            C = linop.FiniteDifference((c.n, c.n), append=0)
            out.append(ADMM(f=loss.SquaredL2Loss(y=y, A=A), g_list=[c.lam * functional.L21Norm()], C_list=[C],
                            rho_list=[c.rho], maxiter=2,
                            subproblem_solver=LinearSubproblemSolver(cg_kwargs={"tol": c.cg_tol,
                                                                                "maxiter": c.cg_maxiter})))
        return out

    batch = build()
    xs = solve_batch(batch)
    alone = build()
    for k in range(0, 64, 7):
        assert torch.equal(xs[k], alone[k].solve())
