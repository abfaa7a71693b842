"""3D projector autotuner (ct_proj3d_autotune): AXIS0 forward tile groups
and adjoint view splits chosen by measurement, recorded per geometry, used
by later projections and fused 3D solves; results change only in summation
order (rel l2 <= 1e-6 for nonnegative data)."""

import numpy as np
import pytest
import torch

from oracle import ctref
from scico_gb300 import _device, _lib, functional, linop, loss
from scico_gb300.optimize import ADMM, LinearSubproblemSolver

pytestmark = pytest.mark.gpu
X3 = linop.XRayTransform3D


@pytest.fixture(autouse=True)
def clear_schedules():
    _lib.load().ct_proj3d_schedule_clear()
    yield
    _lib.load().ct_proj3d_schedule_clear()


def _op(shape=(64, 96, 80), det=(64, 126), nv=48, seq="X"):
    ang = np.linspace(0, np.pi, nv, endpoint=False)
    M = X3.matrices_from_euler_angles(shape, det, seq, ang[:, None] if seq == "X" else np.stack([ang] * 3, 1))
    return X3(shape, M, det)


def _rel(a, b):
    return float((a.double() - b.double()).norm() / b.double().norm())


def test_autotune3d_records_and_keeps_results(cuda):
    H = _op()
    assert H.kind == "axis0"
    gen = torch.Generator().manual_seed(0)
    x = torch.rand(H.input_shape, generator=gen).to(cuda)
    y = torch.rand(H.output_shape, generator=gen).to(cuda)
    ws0 = H.workspace_bytes()
    d = H.schedule()
    assert not d["tuned"] and 1 <= d["tile_groups"] <= 8 and d["adj_splits"] >= 1
    ax0, aty0 = H.project(x), H.back_project(y)
    t = H.autotune(reps=3)
    assert t["tuned"] and t["fwd_us"] > 0 and t["adj_us"] > 0
    assert 1 <= t["tile_groups"] <= 8 and t["adj_splits"] in (1, 2, 3, 4)
    assert H.schedule() == t
    assert H.workspace_bytes() == ws0  # the workspace query covers every schedule
    assert _rel(H.project(x), ax0) <= 1e-6
    assert _rel(H.back_project(y), aty0) <= 1e-6
    assert _lib.load().ct_proj3d_errflag() == 0


def test_autotune3d_general_geometry(cuda):
    H = _op(shape=(24, 28, 20), det=(40, 44), nv=12, seq="XYZ")
    assert H.kind == "general"
    t = H.autotune(reps=2)
    assert t["tuned"] and t["tile_groups"] == 0 and t["adj_splits"] >= 1 and t["fwd_us"] == 0.0
    y = torch.rand(H.output_shape, generator=torch.Generator().manual_seed(2)).to(cuda)
    M = H.matrices.astype(np.float32)
    b = H.back_project(y).cpu().numpy()
    assert ctref.rel_l2(b, ctref.xray3d_back_project(y.cpu().numpy(), M, H.input_shape, np.float32)) <= 1e-5


def test_fused_3d_solve_after_autotune(cuda):
    """A converged-regime 3D solve gives the same result (to 1e-5) before
    and after tuning: the solver's graph picks up the recorded schedule."""
    H = _op(shape=(32, 40, 48), det=(32, 64), nv=24)
    x_gt = torch.rand(H.input_shape, generator=torch.Generator().manual_seed(4)).to(cuda)
    y = H(x_gt)

    def solve():
        C = linop.FiniteDifference(H.input_shape, append=0)
        s = ADMM(f=loss.SquaredL2Loss(y=y, A=H), g_list=[0.01 * functional.L21Norm(), 0.01 * functional.L1Norm()],
                 C_list=[C, C], rho_list=[20.0, 20.0], maxiter=4,
                 subproblem_solver=LinearSubproblemSolver(cg_kwargs={"tol": 1e-5, "maxiter": 40}), fused=True)
        return s.solve()

    x0 = solve()
    H.autotune(reps=2)
    x1 = solve()
    assert _rel(x1, x0) <= 1e-5


def test_autotune3d_refused_inside_capture(cuda):
    H = _op(shape=(16, 16, 16), det=(16, 23), nv=9)
    g = H.geometry()
    fb, ab = H.workspace_bytes()
    ws = _device.workspace(max(fb, ab, 256))
    vol = torch.zeros(H.input_shape, device=cuda)
    proj = torch.zeros(H.output_shape, device=cuda)
    s = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        graph.capture_begin()
        try:
            st = _lib.load().ct_proj3d_autotune(_lib.ctypes.addressof(g), vol.data_ptr(), proj.data_ptr(),
                                                ws.data_ptr(), ws.numel(), 1, s.cuda_stream, None)
        finally:
            graph.capture_end()
    assert st == _lib.CT_ERR_INVALID_ARG
