"""Projector autotuner (ct_proj2d_autotune): measured schedules are recorded
per geometry, used by later projections and fused solves, and change no
forward result and only the adjoint's split summation order."""

import numpy as np
import pytest
import torch

from oracle import ctref
from scico_gb300 import _lib, functional, linop, loss
from scico_gb300.optimize import ADMM, LinearSubproblemSolver

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def clear_schedules():
    _lib.load().ct_proj2d_schedule_clear()
    yield
    _lib.load().ct_proj2d_schedule_clear()


def _op(shape=(96, 80), nv=50):
    ang = np.linspace(0, np.pi, nv, endpoint=False)
    return linop.XRayTransform2D(shape, ang)


def test_autotune_records_and_keeps_results(cuda):
    H = _op()
    g = torch.Generator().manual_seed(0)
    x = torch.rand(H.input_shape, generator=g).to(cuda)
    y = torch.rand(H.output_shape, generator=g).to(cuda)
    ws0 = H.workspace_bytes()
    d = H.schedule()
    assert not d["tuned"] and d["views_per_cta"] >= 2 and d["adj_splits"] >= 1
    ax0, aty0 = H.project(x), H.back_project(y)

    t = H.autotune(reps=3)
    assert t["tuned"] and t["fwd_us"] > 0 and t["adj_us"] > 0
    assert t["views_per_cta"] in (2, 3, 4, 5, 6, 7, 8, 10, 12, 16) and t["adj_splits"] >= 1
    s = H.schedule()
    assert (s["views_per_cta"], s["adj_splits"], s["tuned"]) == (t["views_per_cta"], t["adj_splits"], True)
    assert H.workspace_bytes() == ws0  # sized for every schedule the tuner may pick

    ax1, aty1 = H.project(x), H.back_project(y)
    assert torch.equal(ax0, ax1)  # views per CTA do not change the arithmetic
    assert ctref.rel_l2(aty1.cpu().numpy(), aty0.cpu().numpy()) <= 1e-6
    lhs = float((ax1.double() * y.double()).sum())
    rhs = float((x.double() * aty1.double()).sum())
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)


def test_autotune_batch_is_its_own_entry(cuda):
    H = _op((64, 64), 40)
    H.autotune(batch=2, reps=2)
    assert H.schedule(batch=2)["tuned"] and not H.schedule(batch=1)["tuned"]


def test_fused_solve_after_autotune(cuda):
    H = _op((64, 64), 60)
    rng = np.random.default_rng(3)
    x_gt = np.zeros((64, 64), np.float32)
    x_gt[16:40, 20:50] = 1.0
    y = H(torch.from_numpy(x_gt).to(cuda))
    y = y + 0.01 * torch.from_numpy(rng.standard_normal(tuple(y.shape)).astype(np.float32)).to(cuda)

    def solve():
        f = loss.SquaredL2Loss(y=y, A=H)
        s = ADMM(f=f, g_list=[0.02 * functional.L21Norm()], C_list=[linop.FiniteDifference((64, 64), append=0)],
                 rho_list=[50.0], maxiter=4,
                 subproblem_solver=LinearSubproblemSolver(cg_kwargs={"tol": 1e-5, "maxiter": 30}), fused=True)
        return s.solve()

    xa = solve()
    H.autotune(reps=2)
    xb = solve()  # the iteration graph is captured again with the recorded schedule
    assert ctref.rel_l2(xb.cpu().numpy(), xa.cpu().numpy()) <= 1e-5


def test_autotune_refused_inside_capture(cuda):
    H = _op((64, 64), 30)
    H.project(torch.zeros(H.input_shape, device=cuda))  # function attributes set outside the capture
    graph = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        graph.capture_begin()
        try:
            with pytest.raises(_lib.CtError, match="stream capture"):
                H.autotune(reps=1)
        finally:
            graph.capture_end()


def test_schedule_clear_restores_default(cuda):
    H = _op((64, 64), 30)
    d = H.schedule()
    H.autotune(reps=2)
    _lib.load().ct_proj2d_schedule_clear()
    assert H.schedule() == d
