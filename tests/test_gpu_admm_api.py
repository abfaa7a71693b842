"""The ADMM object as scico code uses it, around the fused solver: its z/u
state made on first use (z_init = C x0, u_init = 0, _admm.py:297-332), the
itstat records of fused solves turned into records on first read, and a
finished solver releasing its device buffers when its last reference goes
(no reference cycle): its workspace goes back to the allocator at once,
where the next solver of the same problem can pick it up and, with it, the
cached graph."""

import gc
import weakref

import numpy as np
import pytest
import torch

from scico_gb300 import functional, linop, loss, workloads
from scico_gb300.optimize import ADMM, LinearSubproblemSolver

pytestmark = pytest.mark.gpu


def _solver(cuda, x0=None, maxiter=6, display=False):
    n, nv = 48, 40
    ang = np.linspace(0, np.pi, nv, endpoint=False)
    A = linop.XRayTransform2D((n, n), ang)
    x_gt = torch.from_numpy(workloads.random_ellipses(n, 5, 3)).to(cuda)
    y = A(x_gt)
    opts = {"display": True} if display else None
    return ADMM(f=loss.SquaredL2Loss(y=y, A=A), g_list=[0.01 * functional.L21Norm()],
                C_list=[linop.FiniteDifference((n, n), append=0)], rho_list=[2.0], x0=x0, maxiter=maxiter,
                subproblem_solver=LinearSubproblemSolver(cg_kwargs={"tol": 1e-4, "maxiter": 10}),
                itstat_options=opts)


def test_state_made_on_first_use(cuda):
    x0 = torch.rand((48, 48), generator=torch.Generator().manual_seed(5)).to(cuda)
    s = _solver(cuda, x0=x0)
    C = s.C_list[0]
    z, u, zo = s.z_list, s.u_list, s.z_list_old
    assert torch.equal(z[0], C(x0))
    assert float(u[0].abs().max()) == 0.0
    assert zo[0] is z[0]
    assert torch.equal(s.x, x0) and s.x.data_ptr() != x0.data_ptr()  # a copy of x0


def test_fused_records_and_continuation(cuda):
    s = _solver(cuda)
    s.solve()
    h = s.history()
    assert [r.Iter for r in h] == list(range(6))
    assert all(np.isfinite(r.Objective) and r.Prml_Rsdl >= 0 for r in h)
    t = s.history(transpose=True)
    assert len(t.Objective) == 6
    s.solve()  # continues from the fused state
    assert [r.Iter for r in s.history()] == list(range(12))
    # the same solves with itstat display on give the same records
    d = _solver(cuda, display=True)
    d.solve()
    d.solve()
    assert [tuple(r)[2:] for r in d.history()] == [tuple(r)[2:] for r in s.history()]


def test_finished_solver_is_freed(cuda):
    def solve_once():
        s = _solver(cuda)
        x = s.solve().clone()
        return x, weakref.ref(s), weakref.ref(s._fused_state["ws"])

    gc.disable()
    try:
        x1, r1, w1 = solve_once()
        assert r1() is None and w1() is None  # freed by reference counting alone
        x2, r2, w2 = solve_once()
        assert r2() is None and w2() is None
    finally:
        gc.enable()
    assert torch.equal(x1, x2)
