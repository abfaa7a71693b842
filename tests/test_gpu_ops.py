"""Finite differences, proximal operators, norms and CG on the GPU against
the oracle (bit-exact where the operation sequence is the same)."""

import numpy as np
import pytest
import torch

from oracle import ctref
from scico_gb300 import functional, linop, solver

pytestmark = pytest.mark.gpu

MODES = dict(none={}, pre0=dict(prepend=0), pre1=dict(prepend=1), app0=dict(append=0), app1=dict(append=1),
             both01=dict(prepend=0, append=1), circ=dict(circular=True))


@pytest.mark.parametrize("shape", [(16,), (16, 24), (5, 6, 7), (64, 64)])
@pytest.mark.parametrize("mode", list(MODES))
def test_fd_vs_oracle(cuda, shape, mode):
    kw = MODES[mode]
    rng = np.random.default_rng(0)
    x = rng.standard_normal(shape).astype(np.float32)
    A = linop.FiniteDifference(shape, **kw)
    y = A(torch.from_numpy(x).to(cuda))
    ref = ctref.fd_eval(x, **kw)
    if isinstance(ref, list):
        for yb, rb in zip(y, ref):
            np.testing.assert_array_equal(yb.cpu().numpy(), rb)
        d = [rng.standard_normal(b.shape).astype(np.float32) for b in ref]
        back = A.adj(tuple(torch.from_numpy(b).to(cuda) for b in d)).cpu().numpy()
    else:
        np.testing.assert_array_equal(y.cpu().numpy(), ref)
        d = rng.standard_normal(ref.shape).astype(np.float32)
        back = A.adj(torch.from_numpy(d).to(cuda)).cpu().numpy()
    np.testing.assert_array_equal(back, ctref.fd_adj(d, shape, **kw))  # the same float32 sums
    # dot test (test_diff.py:68-78)
    d64 = [np.asarray(b, np.float64) for b in (d if isinstance(d, list) else list(d))]
    r64 = [np.asarray(b, np.float64) for b in (ref if isinstance(ref, list) else list(ref))]
    lhs = sum(float(np.sum(a * b)) for a, b in zip(r64, d64))
    rhs = float(np.sum(x.astype(np.float64) * back))
    assert abs(lhs - rhs) <= 1e-4 * max(abs(lhs), 1.0)


def test_fd_kat(cuda):
    """scico/test/linop/test_diff.py:11-31 through the GPU operator."""
    import json
    from pathlib import Path

    k = json.loads((Path(__file__).parent / "golden" / "reference_kat.json").read_text())
    c = k["fd_eval_append1"]
    A = linop.FiniteDifference((2, 3), append=1)
    Ax = A(torch.tensor(c["x"], dtype=torch.float32, device=cuda))
    np.testing.assert_array_equal(Ax[0].cpu().numpy(), np.array(c["axis0"]))
    np.testing.assert_array_equal(Ax[1].cpu().numpy(), np.array(c["axis1"]))
    for case in k["fd_1d"]["cases"]:
        B = linop.SingleAxisFiniteDifference((5,), prepend=case["prepend"], append=case["append"])
        y = B(torch.arange(1, 6, dtype=torch.float32, device=cuda)).cpu().numpy()
        np.testing.assert_array_equal(y, np.array(case["truth"]))


@pytest.mark.parametrize("axis", [0, 1, (0, 2)])
def test_l21_kat(cuda, axis):
    """scico/test/functional/test_norm.py:9-28 through the GPU kernels."""
    x = torch.ones((3, 4, 5), device=cuda)
    F = functional.L21Norm(l2_axis=axis)
    l2axis = (axis,) if isinstance(axis, int) else axis
    l2 = np.sqrt(np.prod([x.shape[k] for k in l2axis]))
    l1 = np.prod([x.shape[k] for k in set(range(3)) - set(l2axis)])
    np.testing.assert_allclose(F(x), l2 * l1, rtol=1e-5)
    np.testing.assert_allclose(F.prox(x, 1.0).cpu().numpy(), (l2 - 1.0) / l2 * np.ones((3, 4, 5)), rtol=1e-5)


@pytest.mark.parametrize("ncomp", [2, 3])
def test_prox_bit_exact(cuda, ncomp):
    rng = np.random.default_rng(ncomp)
    v = rng.standard_normal((ncomp, 50, 60)).astype(np.float32)
    v[:, :3, :3] = 0.0  # zero-length groups (no_nan_divide)
    lam = 0.37
    g = functional.L21Norm()
    out = g.prox(torch.from_numpy(v).to(cuda), lam).cpu().numpy()
    np.testing.assert_array_equal(out, ctref.l21_prox(v, np.float32(lam)))
    out1 = functional.L1Norm().prox(torch.from_numpy(v).to(cuda), lam).cpu().numpy()
    np.testing.assert_array_equal(out1, ctref.l1_prox(v, np.float32(lam)))
    np.testing.assert_allclose(g(torch.from_numpy(v).to(cuda)), ctref.l21_norm(v), rtol=1e-6)
    np.testing.assert_allclose(functional.L1Norm()(torch.from_numpy(v).to(cuda)), ctref.l1_norm(v), rtol=1e-6)
    sg = 0.5 * g
    np.testing.assert_array_equal(sg.prox(torch.from_numpy(v).to(cuda), 2 * lam).cpu().numpy(),
                                  ctref.l21_prox(v, np.float32(lam)))


def test_cg_spd(cuda):
    """scico/test/test_solver.py:28-60 style: CG on an SPD matrix."""
    rng = np.random.default_rng(6)
    n = 64
    M = rng.standard_normal((n, n)).astype(np.float32)
    M = M.T @ M + n * np.eye(n, dtype=np.float32)
    Mt = torch.from_numpy(M).to(cuda)
    b = rng.standard_normal(n).astype(np.float32)
    x, info = solver.cg(lambda v: Mt @ v, torch.from_numpy(b).to(cuda), torch.zeros(n, device=cuda),
                        tol=1e-6, maxiter=200)
    res = np.linalg.norm(b - M @ x.cpu().numpy()) / np.linalg.norm(b)
    assert res < 1e-5
    assert info["num_iter"] < 200
    assert info["rel_res"] < 1e-6


def test_cg_ct_normal_equations(cuda):
    """CG on (A^T A + D^T D) x = A^T y, 15 steps, against the same-precision
    oracle CG (float32 vectors, float64 dots), within the float32 rounding
    floor of the problem (the spread between that oracle with its float32
    projector and with a float64 projector rounded to float32)."""
    from scico_gb300 import workloads

    x_gt = workloads.random_ellipses(48, 5, 21)
    ang = np.linspace(0, np.pi, 30, endpoint=False)
    H = linop.XRayTransform2D(x_gt.shape, ang)
    D = linop.FiniteDifference(x_gt.shape, append=0)
    lhs = H.gram_op + D.gram_op
    g = ctref.xray2d_defaults(x_gt.shape, ang)
    y = ctref.xray2d_project(x_gt, g, np.float64).astype(np.float32)
    b = H.adj(torch.from_numpy(y).to(cuda))
    x, info = solver.cg(lhs, b, torch.zeros_like(b), tol=1e-4, maxiter=15)
    D = lambda v: ctref.fd_adj(ctref.fd_eval(v, append=0), x_gt.shape, append=0)
    runs = []
    for pdt in (np.float32, np.float64):
        fwd = lambda v: ctref.xray2d_project(v, g, pdt).astype(np.float32)
        adj = lambda v: ctref.xray2d_back_project(v, g, pdt).astype(np.float32)
        bb = b.cpu().numpy()
        runs.append(ctref.cg(lambda v: adj(fwd(v)) + D(v), bb, np.zeros_like(bb), tol=1e-4, maxiter=15,
                             dot_dtype=np.float64))
    (xm, im), (xp, _) = runs
    floor = ctref.rel_l2(xp, xm)
    assert abs(info["num_iter"] - im["num_iter"]) <= 1
    assert ctref.rel_l2(x.cpu().numpy(), xm) <= 3 * floor + 1e-5, (ctref.rel_l2(x.cpu().numpy(), xm), floor)
