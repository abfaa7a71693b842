"""The solve graphs' fast-forward CG start (k_init_ffwd,
ct_set_solver_fast_forward).  Once CG's stopping test passes at its first
step, one cooperative launch runs the CG-free ADMM iterations back to back
(z/u update, next rhs, next CG start), its blocks meeting at bounded grid
barriers.  It must give the same bits as the separate kernels: x, the z/u
state and every itstat record (objective, residuals, CG step counts and
relative residuals), in 2D and 3D, with one and two g terms, across
continued solves, when the call's last iterations are CG-free and when CG
has steps to run again after a CG-free stretch.  A barrier wait that runs
out is reported (bit 3 of the device error word, CT_ERR_TIMEOUT) instead of
hanging; tests/test_gpu_failure.py covers the projector's waits the same
way."""

import numpy as np
import pytest
import torch

from scico_gb300 import _lib, functional, linop, loss, workloads
from scico_gb300.optimize import ADMM, LinearSubproblemSolver

pytestmark = pytest.mark.gpu


def _both(fn):
    """fn() with the fast-forward CG start off, then on."""
    lib = _lib.load()
    old = lib.ct_solver_fast_forward()
    out = []
    try:
        for on in (0, 1):
            lib.ct_set_solver_fast_forward(on)
            out.append(fn())
    finally:
        lib.ct_set_solver_fast_forward(old)
    return out


def _admm(A, y, shape, lam21, lam1, rho, maxiter, cg_tol, cg_maxiter):
    C = linop.FiniteDifference(shape, append=0)
    gl, Cl = [], []
    if lam21:
        gl.append(lam21 * functional.L21Norm())
        Cl.append(C)
    if lam1:
        gl.append(lam1 * functional.L1Norm())
        Cl.append(C)
    return ADMM(f=loss.SquaredL2Loss(y=y, A=A), g_list=gl, C_list=Cl, rho_list=[rho] * len(gl), maxiter=maxiter,
                subproblem_solver=LinearSubproblemSolver(cg_kwargs={"tol": cg_tol, "maxiter": cg_maxiter}),
                fused=True)


def _run(s, calls):
    for _ in range(calls):
        x = s.solve()
    recs = [tuple(r)[2:] for r in s.history()]  # all fields but Iter and the host time
    return x.clone(), [z.clone() for z in s.z_list], [u.clone() for u in s.u_list], recs


def _same(a, b):
    xa, za, ua, ra = a
    xb, zb, ub, rb = b
    assert torch.equal(xa, xb)
    assert all(torch.equal(p, q) for p, q in zip(za, zb))
    assert all(torch.equal(p, q) for p, q in zip(ua, ub))
    assert ra == rb


def _problem2d(cuda, n, nv, seed):
    x_gt = workloads.random_ellipses(n, 10, seed)
    A = linop.XRayTransform2D((n, n), np.linspace(0, np.pi, nv, endpoint=False))
    y = A(torch.from_numpy(x_gt).to(cuda))
    noise = torch.randn(y.shape, generator=torch.Generator().manual_seed(seed + 1)).to(cuda)
    return A, (y + 0.005 * float(y.abs().max()) * noise).contiguous()


@pytest.mark.parametrize("terms", ["l21", "both"])
def test_fast_forward_2d_bit_identical(cuda, terms):
    n, nv = 128, 90
    A, y = _problem2d(cuda, n, nv, 7)
    lam1 = 0.002 if terms == "both" else 0.0

    def go():
        return _run(_admm(A, y, (n, n), 0.005, lam1, 2.0, 40, 1e-4, 10), calls=2)

    off, on = _both(go)
    _same(off, on)
    cg = [r[3] for r in on[3]]
    assert len(cg) == 80 and cg.count(0) >= 10, cg  # CG-free iterations were fast-forwarded


def test_fast_forward_cg_resumes(cuda):
    """Problems whose CG has steps to run again after CG-free iterations (the
    kernel hands back to the graph's CG loop mid-solve, many times)."""
    n, nv = 64, 40
    x_gt = workloads.random_ellipses(n, 10, 11)
    A = linop.XRayTransform2D((n, n), np.linspace(0, np.pi, nv, endpoint=False))
    y0 = A(torch.from_numpy(x_gt).to(cuda)).cpu().numpy()
    y = torch.from_numpy(workloads.noisy(y0, 0.005, 12)).to(cuda)
    resumes = 0
    for lam, rho in ((0.02, 2.0), (0.05, 0.5)):

        def go():
            return _run(_admm(A, y, (n, n), lam, 0.0, rho, 60, 1e-4, 10), calls=1)

        off, on = _both(go)
        _same(off, on)
        cg = [r[3] for r in on[3]]
        resumes += sum(1 for k in range(len(cg) - 1) if cg[k] == 0 and cg[k + 1] > 0)
    assert resumes >= 3, resumes


def test_fast_forward_odd_shape_scalar_path(cuda):
    """A 45-column image: the element passes take their scalar path."""
    x_gt = workloads.random_ellipses(64, 6, 3)[:40, :45].copy()
    A = linop.XRayTransform2D(x_gt.shape, np.linspace(0, np.pi, 50, endpoint=False))
    y = A(torch.from_numpy(x_gt).to(cuda))

    def go():
        return _run(_admm(A, y, x_gt.shape, 0.01, 0.0, 2.0, 30, 1e-4, 10), calls=1)

    off, on = _both(go)
    _same(off, on)


def test_fast_forward_3d_bit_identical(cuda):
    shape, det, nv = (20, 24, 24), (20, 35), 24
    ang = np.linspace(0, np.pi, nv, endpoint=False)[:, None]
    M = linop.XRayTransform3D.matrices_from_euler_angles(shape, det, "X", ang).astype(np.float32)
    A = linop.XRayTransform3D(shape, M, det)
    x_gt = np.zeros(shape, np.float32)
    x_gt[4:14, 6:18, 5:15] = 1.0
    y = A(torch.from_numpy(x_gt).to(cuda))

    def go():
        return _run(_admm(A, y, shape, 0.01, 0.01, 1.0, 25, 1e-3, 8), calls=1)

    off, on = _both(go)
    _same(off, on)
    assert [r[3] for r in on[3]].count(0) >= 1


def test_barrier_timeout_reports_and_recovers(cuda):
    lib = _lib.load()
    if not lib.ct_solver_fast_forward():
        pytest.skip("fast-forward CG start switched off in this environment")
    n, nv = 64, 40
    A, y = _problem2d(cuda, n, nv, 5)

    def solve():
        return _admm(A, y, (n, n), 0.01, 0.0, 2.0, 6, 1e-4, 10).solve().clone()

    x_ref = solve()
    assert lib.ct_proj2d_errflag() == 0
    default = lib.ct_wait_poll_limit()
    lib.ct_set_wait_poll_limit(0)  # every bounded wait gives up at its first poll
    try:
        with pytest.raises(_lib.CtError) as ei:
            solve()
    finally:
        lib.ct_set_wait_poll_limit(default)
    assert ei.value.status == _lib.CT_ERR_TIMEOUT
    assert "grid barrier" in str(ei.value)
    assert lib.ct_proj2d_errflag() == 0  # reported once, then cleared
    x_again = solve()  # the default limit: clean and exact again
    assert lib.ct_proj2d_errflag() == 0
    assert torch.equal(x_again, x_ref)


@pytest.mark.parametrize("n", [64, 45])
def test_plain_launches_match_the_graph(cuda, n):
    """ct_admm_tv_solve with use_graph = 0 (every kernel a plain launch, each
    after the first of the call a programmatic dependent launch) against the
    solve graph (with its cooperative kernels): the same x and itstat
    records, bit for bit; n = 45 takes the kernels' scalar paths."""
    x_gt = workloads.random_ellipses(64, 6, 9)[:n, :n].copy()
    A = linop.XRayTransform2D((n, n), np.linspace(0, np.pi, 40, endpoint=False))
    y = A(torch.from_numpy(x_gt).to(cuda)).contiguous()
    g = A.geometry()
    out = []
    for use_graph in (0, 1):
        desc = _lib.AdmmTvDesc(g, 25, 10, 1e-4, 0.0, 0.01, 0.0, 2.0, 0.5, 1.0, use_graph)
        nb = _lib.c_size_t()
        _lib.call("ct_admm_tv_workspace", _lib.ctypes.addressof(desc), _lib.ctypes.addressof(nb))
        ws = torch.empty(nb.value, dtype=torch.uint8, device=cuda)
        x = torch.zeros((n, n), device=cuda)
        it = torch.zeros((25, _lib.CT_ITSTAT_FIELDS), dtype=torch.float64, device=cuda)
        _lib.call("ct_admm_tv_solve", _lib.ctypes.addressof(desc), y.data_ptr(), x.data_ptr(), it.data_ptr(), 0,
                  ws.data_ptr(), ws.numel(), torch.cuda.current_stream().cuda_stream)
        _lib.check_device(torch.cuda.current_stream().cuda_stream)
        out.append((x.clone(), it.cpu()))
    assert torch.equal(out[0][0], out[1][0])
    assert torch.equal(out[0][1], out[1][1])
    assert int((out[1][1][:, _lib.CT_ITSTAT_CG_ITERS] == 0).sum()) >= 1  # CG-free iterations in both


def test_fast_forward_c2_size(cuda):
    """The benchmark's workload (512^2, 360 views, 725 bins, lambda 0.005,
    rho 2, 100 iterations, CG <= 10): one quad per thread of the 304 x 256
    grid; the same bits with the cooperative kernels on and off."""
    c = workloads.C2
    A = linop.XRayTransform2D((c.n, c.n), c.angles, det_count=c.det_count)
    y0 = A(torch.from_numpy(c.phantom()).to(cuda)).cpu().numpy()
    y = torch.from_numpy(workloads.noisy(y0, c.noise, c.noise_seed)).to(cuda)

    def go():
        return _run(_admm(A, y, (c.n, c.n), c.lam, 0.0, c.rho, c.maxiter, c.cg_tol, c.cg_maxiter), calls=1)

    off, on = _both(go)
    _same(off, on)
    assert [r[3] for r in on[3]].count(0) >= 50


def test_fast_forward_3d_several_quads_per_thread(cuda):
    """A 64^3 volume: 65,536 quads, so the grid-stride passes give most
    threads several quads (the 3D path of the passes at size)."""
    shape, det, nv = (64, 64, 64), (64, 91), 48
    ang = np.linspace(0, np.pi, nv, endpoint=False)[:, None]
    M = linop.XRayTransform3D.matrices_from_euler_angles(shape, det, "X", ang).astype(np.float32)
    A = linop.XRayTransform3D(shape, M, det)
    x_gt = np.zeros(shape, np.float32)
    x_gt[10:40, 20:50, 15:45] = 1.0
    x_gt[30:55, 5:25, 30:60] += 0.5
    y = A(torch.from_numpy(x_gt).to(cuda))

    def go():
        return _run(_admm(A, y, shape, 0.01, 0.01, 1.0, 20, 1e-3, 8), calls=1)

    off, on = _both(go)
    _same(off, on)
    assert [r[3] for r in on[3]].count(0) >= 1
