"""3D ADMM-TV on the GPU (generic drop-in path and the fused graph solver,
ct_admm_tv3d_solve) against the oracle.

Converged regime only (each CG reaches its tolerance): float32, and float32
with float64 dots, agree with the float64 oracle to a few 1e-6 there, so the
bar is rel l2 <= 1e-4 for x and the objective, as for 2D.  The oracle's
projector uses the reference's float32 weights with float64 sums (float64
weights would move voxels at the model's integer-`left` discontinuity).
The full 256^3 x 360-view workload is checked through properties.
"""

import numpy as np
import pytest
import torch

from oracle import ctref
from scico_gb300 import functional, linop, loss, workloads
from scico_gb300.optimize import ADMM, LinearSubproblemSolver

pytestmark = pytest.mark.gpu
X3 = linop.XRayTransform3D


def _problem(shape=(12, 16, 16), det=(12, 23), seq="X", nv=16, seed=3, noise=0.01):
    rng = np.random.default_rng(seed)
    x_gt = np.zeros(shape, np.float32)
    for _ in range(4):  # a few boxes of random value
        lo = [rng.integers(0, n // 2) for n in shape]
        hi = [lo[k] + rng.integers(2, shape[k] // 2 + 1) for k in range(3)]
        x_gt[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]] += rng.uniform(0.2, 1.0)
    if len(seq) == 1:
        ang = np.linspace(0, np.pi, nv, endpoint=False)[:, None]
    else:
        ang = rng.uniform(0, np.pi, (nv, len(seq)))
    M = X3.matrices_from_euler_angles(shape, det, seq, ang).astype(np.float32)
    y = ctref.xray3d_project(x_gt, M, det, np.float32, np.float64).astype(np.float32)
    return x_gt, M, workloads.noisy(y, noise, seed + 1)


def _solver(cuda, M, y, shape, det, lam21=0.02, lam1=0.0, rho=50.0, maxiter=4, cg_maxiter=30, cg_tol=1e-5,
            fused="auto"):
    A = X3(shape, M, det)
    f = loss.SquaredL2Loss(y=torch.from_numpy(y).to(cuda), A=A)
    C = linop.FiniteDifference(shape, append=0)
    gl, Cl = [], []
    if lam21:
        gl.append(lam21 * functional.L21Norm())
        Cl.append(C)
    if lam1:
        gl.append(lam1 * functional.L1Norm())
        Cl.append(C)
    return ADMM(f=f, g_list=gl, C_list=Cl, rho_list=[rho] * len(gl), maxiter=maxiter,
                subproblem_solver=LinearSubproblemSolver(cg_kwargs={"tol": cg_tol, "maxiter": cg_maxiter}),
                fused=fused), A


def _oracle(y, M, shape, det, **kw):
    fwd = lambda v: ctref.xray3d_project(v, M, det, np.float32, np.float64)
    adj = lambda v: ctref.xray3d_back_project(v, M, shape, np.float32, np.float64)
    return ctref.admm_tv(fwd, adj, y.astype(np.float64), shape, dtype=np.float64, **kw)


@pytest.mark.parametrize("fused", [False, True])
@pytest.mark.parametrize("terms", ["l21", "l1", "both"])
def test_admm3d_converged_vs_oracle(cuda, fused, terms):
    shape, det = (12, 16, 16), (12, 23)
    x_gt, M, y = _problem(shape, det)
    lam21 = 0.02 if terms in ("l21", "both") else 0.0
    lam1 = 0.01 if terms in ("l1", "both") else 0.0
    s, A = _solver(cuda, M, y, shape, det, lam21=lam21, lam1=lam1, fused=fused)
    assert A.kind == "axis0"
    x = s.solve().cpu().numpy()
    x64, hist, z64, _ = _oracle(y, M, shape, det, lam_l21=lam21, lam_l1=lam1, rho=50.0, maxiter=4,
                                cg_maxiter=30, cg_tol=1e-5)
    assert ctref.rel_l2(x, x64) <= 1e-4
    h = s.history(transpose=True)
    np.testing.assert_allclose(h.Objective, [r["Objective"] for r in hist], rtol=1e-4)
    np.testing.assert_allclose(h.Prml_Rsdl, [r["Prml_Rsdl"] for r in hist], rtol=1e-3)
    np.testing.assert_allclose(h.Dual_Rsdl, [r["Dual_Rsdl"] for r in hist], rtol=1e-3)
    assert all(abs(a - b) <= 1 for a, b in zip(h.CG_It, [r["CG_It"] for r in hist]))
    for zk, zo in zip(s.z_list, z64):
        assert zk.shape == (3,) + shape
        assert ctref.rel_l2(zk.cpu().numpy(), zo) <= 1e-3


@pytest.mark.parametrize("fused", [False, True])
def test_admm3d_general_geometry(cuda, fused):
    shape, det = (10, 12, 14), (18, 20)
    x_gt, M, y = _problem(shape, det, seq="XYZ", nv=12, seed=9)
    s, A = _solver(cuda, M, y, shape, det, lam21=0.02, lam1=0.01, fused=fused)
    assert A.kind == "general"
    x = s.solve().cpu().numpy()
    x64, hist, _, _ = _oracle(y, M, shape, det, lam_l21=0.02, lam_l1=0.01, rho=50.0, maxiter=4,
                              cg_maxiter=30, cg_tol=1e-5)
    assert ctref.rel_l2(x, x64) <= 1e-4
    np.testing.assert_allclose(s.history(transpose=True).Objective, [r["Objective"] for r in hist], rtol=1e-4)


def test_admm3d_fused_matches_generic(cuda):
    shape, det = (20, 24, 24), (20, 35)
    x_gt, M, y = _problem(shape, det, nv=24, seed=5)
    xa = _solver(cuda, M, y, shape, det, lam21=0.01, lam1=0.01, maxiter=5, rho=1.0, cg_maxiter=8,
                 cg_tol=1e-4, fused=False)[0].solve()
    xb = _solver(cuda, M, y, shape, det, lam21=0.01, lam1=0.01, maxiter=5, rho=1.0, cg_maxiter=8,
                 cg_tol=1e-4, fused=True)[0].solve()
    assert ctref.rel_l2(xb.cpu().numpy(), xa.cpu().numpy()) <= 1e-4


def test_admm3d_c5_size(cuda):
    """256^3 volume, 360 views about axis 0, 256 x 363 detector, lambda 0.005
    on both L1 and L2,1 of one FD, rho 1, CG <= 8: two fused iterations
    plus one continued from the workspace state match a three-iteration run;
    repeated runs are bit-identical; the objective falls and CG stays
    within its cap."""
    c = workloads.C5
    x_gt = torch.from_numpy(workloads.random_ellipsoids(c.n, 6, seed=c.phantom_seed)).to(cuda)
    A = X3(c.shape, c.matrices(), c.det_shape)
    assert A.kind == "axis0"
    y = A(x_gt)
    y = y + 0.01 * y.abs().max() * torch.randn(y.shape, generator=torch.Generator().manual_seed(1)).to(cuda)

    def run(iters):
        f = loss.SquaredL2Loss(y=y, A=A)
        C = linop.FiniteDifference(c.shape, append=0)
        return ADMM(f=f, g_list=[c.lam_l21 * functional.L21Norm(), c.lam_l1 * functional.L1Norm()],
                    C_list=[C, C], rho_list=[c.rho] * 2, maxiter=iters,
                    subproblem_solver=LinearSubproblemSolver(cg_kwargs={"tol": c.cg_tol, "maxiter": c.cg_maxiter}),
                    fused=True)

    a = run(3)
    xa = a.solve()
    h = a.history(transpose=True)
    assert torch.isfinite(xa).all()
    assert h.Objective[-1] < h.Objective[0]
    assert all(k <= c.cg_maxiter for k in h.CG_It)
    b = run(2)
    b.solve()
    b.maxiter = 1
    xb = b.solve()
    assert ctref.rel_l2(xb.cpu().numpy(), xa.cpu().numpy()) <= 1e-6
    assert len(b.history()) == 3
    assert torch.equal(xa, run(3).solve())
