"""ProximalADMM (scico/optimize/_padmm.py) with VerticalStack, operator_norm
and the separable data + TV functional of the reference's ct_3d_tv_padmm
example, on the GPU against the oracle.  The iteration has no inner solver,
so float32 and float64 stay close: rel l2 <= 1e-4 after 30 iterations."""

import numpy as np
import pytest
import torch

from oracle import ctref
from scico_gb300 import functional, linop, loss, workloads
from scico_gb300.optimize import ProximalADMM

pytestmark = pytest.mark.gpu


def test_operator_norm_vs_dense(cuda):
    n, nv = 16, 12
    ang = np.linspace(0, np.pi, nv, endpoint=False)
    A = linop.XRayTransform2D((n, n), ang)
    g = ctref.xray2d_defaults((n, n), ang)
    cols = []
    for k in range(n * n):
        e = np.zeros((n, n))
        e.flat[k] = 1.0
        cols.append(ctref.xray2d_project(e, g, np.float64).ravel())
    sigma = np.linalg.norm(np.stack(cols, axis=1), 2)
    est = linop.operator_norm(A, maxiter=300, seed=1)
    assert abs(est - sigma) <= 1e-3 * sigma
    D = linop.FiniteDifference((n, n), append=0)
    V = linop.VerticalStack((A, 10.0 * D))
    assert V.output_shape == (A.output_shape, D.output_shape)
    x = torch.rand((n, n), device=cuda)
    yv = (torch.rand(A.output_shape, device=cuda), torch.rand(D.output_shape, device=cuda))
    lhs = sum(float((a.double() * b.double()).sum()) for a, b in zip(V(x), yv))
    rhs = float((x.double() * V.adj(yv).double()).sum())
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)


def _padmm_case(cuda, H, fwd, adj, y, shape, lam=0.5, alpha=10.0, rho=0.05, iters=30):
    D = linop.FiniteDifference(shape, append=0)
    A = linop.VerticalStack((H, alpha * D))
    mu, nu = ProximalADMM.estimate_parameters(A, maxiter=100, seed=0)
    g = functional.SeparableFunctional((loss.SquaredL2Loss(y=torch.from_numpy(y).to(cuda)),
                                        (lam / alpha) * functional.L21Norm()))
    s = ProximalADMM(f=functional.ZeroFunctional(), g=g, A=A, rho=rho, mu=mu, nu=nu, maxiter=iters)
    x = s.solve().cpu().numpy()
    x64, hist = ctref.padmm_tv(fwd, adj, y.astype(np.float64), shape, lam, alpha, rho, mu, nu, iters)
    return s, x, x64, hist


def test_padmm_2d_vs_oracle(cuda):
    n, nv = 32, 30
    ang = np.linspace(0, np.pi, nv, endpoint=False)
    H = linop.XRayTransform2D((n, n), ang)
    g = ctref.xray2d_defaults((n, n), ang)
    x_gt = workloads.random_ellipses(n, 5, 2)
    y = workloads.noisy(ctref.xray2d_project(x_gt, g, np.float64).astype(np.float32), 0.01, 3)
    s, x, x64, hist = _padmm_case(cuda, H, lambda v: ctref.xray2d_project(v, g, np.float64),
                                  lambda v: ctref.xray2d_back_project(v, g, np.float64), y, (n, n))
    assert ctref.rel_l2(x, x64) <= 1e-4
    h = s.history(transpose=True)
    np.testing.assert_allclose(h.Prml_Rsdl, [p for p, _ in hist], rtol=1e-3)
    np.testing.assert_allclose(h.Dual_Rsdl, [d for _, d in hist], rtol=1e-3)
    assert h.Prml_Rsdl[-1] < h.Prml_Rsdl[0]


def test_padmm_3d_vs_oracle(cuda):
    shape, det, nv = (8, 16, 16), (8, 23), 12
    M = linop.XRayTransform3D.matrices_from_euler_angles(shape, det, "X",
                                                         np.linspace(0, np.pi, nv, endpoint=False)[:, None])
    H = linop.XRayTransform3D(shape, M, det)
    M32 = M.astype(np.float32)
    rng = np.random.default_rng(4)
    x_gt = np.zeros(shape, np.float32)
    x_gt[2:6, 4:12, 3:11] = 1.0
    x_gt[3:5, 6:9, 5:13] += rng.uniform(0.2, 0.8)
    y = ctref.xray3d_project(x_gt, M32, det, np.float32, np.float64).astype(np.float32)
    fwd = lambda v: ctref.xray3d_project(v, M32, det, np.float32, np.float64)
    adj = lambda v: ctref.xray3d_back_project(v, M32, shape, np.float32, np.float64)
    s, x, x64, _ = _padmm_case(cuda, H, fwd, adj, y, shape, iters=20)
    assert ctref.rel_l2(x, x64) <= 1e-4


def _padmm_solver(cuda, H, y, shape, fused, lam=0.5, alpha=10.0, rho=0.05, iters=30, mu_nu=None):
    D = linop.FiniteDifference(shape, append=0)
    A = linop.VerticalStack((H, alpha * D))
    mu, nu = mu_nu if mu_nu else ProximalADMM.estimate_parameters(A, maxiter=100, seed=0)
    g = functional.SeparableFunctional((loss.SquaredL2Loss(y=torch.from_numpy(y).to(cuda)),
                                        (lam / alpha) * functional.L21Norm()))
    return ProximalADMM(f=functional.ZeroFunctional(), g=g, A=A, rho=rho, mu=mu, nu=nu, maxiter=iters,
                        fused=fused), (mu, nu)


@pytest.mark.parametrize("three", [False, True])
def test_padmm_fused_matches_generic(cuda, three):
    """The native solver (ct_padmm_tv_solve) against the generic step loop on
    the same operators: the same arithmetic up to float32 rounding order."""
    if three:
        shape, det, nv = (8, 16, 16), (8, 23), 12
        M = linop.XRayTransform3D.matrices_from_euler_angles(shape, det, "X",
                                                             np.linspace(0, np.pi, nv, endpoint=False)[:, None])
        H = linop.XRayTransform3D(shape, M, det)
        x_gt = np.zeros(shape, np.float32)
        x_gt[2:6, 4:12, 3:11] = 1.0
    else:
        shape = (32, 32)
        H = linop.XRayTransform2D(shape, np.linspace(0, np.pi, 30, endpoint=False))
        x_gt = workloads.random_ellipses(32, 5, 2)
    y = H(torch.from_numpy(x_gt).to(cuda)).cpu().numpy()
    a, mn = _padmm_solver(cuda, H, y, shape, fused=True)
    xa = a.solve().cpu().numpy()
    assert a._fused_state is not None  # the native path ran
    b, _ = _padmm_solver(cuda, H, y, shape, fused=False, mu_nu=mn)
    xb = b.solve().cpu().numpy()
    assert ctref.rel_l2(xa, xb) <= 1e-5
    ha, hb = a.history(transpose=True), b.history(transpose=True)
    np.testing.assert_allclose(ha.Prml_Rsdl, hb.Prml_Rsdl, rtol=1e-4)
    np.testing.assert_allclose(ha.Dual_Rsdl, hb.Dual_Rsdl, rtol=1e-4, atol=1e-9)
    np.testing.assert_allclose(ha.Objective, hb.Objective, rtol=1e-5)
    for za, zb in zip(a.z, b.z):
        assert ctref.rel_l2(za.cpu().numpy(), zb.cpu().numpy()) <= 1e-5


def test_padmm_fused_continuation(cuda):
    """Two calls of 10 iterations continue from the solver state and give
    exactly the iterates of one call of 20."""
    shape = (32, 32)
    H = linop.XRayTransform2D(shape, np.linspace(0, np.pi, 30, endpoint=False))
    y = H(torch.from_numpy(workloads.random_ellipses(32, 5, 2)).to(cuda)).cpu().numpy()
    a, mn = _padmm_solver(cuda, H, y, shape, fused=True, iters=20)
    xa = a.solve()
    b, _ = _padmm_solver(cuda, H, y, shape, fused=True, iters=10, mu_nu=mn)
    b.solve()
    xb = b.solve()
    assert torch.equal(xa, xb)
    assert len(b.history()) == 20
    assert [r.Prml_Rsdl for r in a.history()] == [r.Prml_Rsdl for r in b.history()]


@pytest.mark.parametrize("fused", [False, True])
def test_padmm_reference_code_vectors(cuda, fused):
    """Against scico's own ProximalADMM.step and prox code run under the
    float32 jax.numpy stand-in (tests/golden/padmm_reference_code.npz), with
    the vectors' mu and nu: x within 1e-4 after the last iteration, through
    the fused solver and the generic composition."""
    from pathlib import Path

    z = np.load(Path(__file__).resolve().parent / "golden" / "padmm_reference_code.npz")
    for k in range(2):
        p = f"c{k}_"
        n, nv = int(z[p + "n"]), int(z[p + "nv"])
        H = linop.XRayTransform2D((n, n), np.linspace(0, np.pi, nv, endpoint=False).astype(np.float32))
        alpha, lam = float(z[p + "alpha"]), float(z[p + "lam"])
        D = linop.FiniteDifference((n, n), append=0)
        A = linop.VerticalStack((H, alpha * D))
        g = functional.SeparableFunctional((loss.SquaredL2Loss(y=torch.from_numpy(z[p + "y"]).to(cuda)),
                                            (lam / alpha) * functional.L21Norm()))
        X = z[p + "x"]
        s = ProximalADMM(f=functional.ZeroFunctional(), g=g, A=A, rho=float(z[p + "rho"]), mu=float(z[p + "mu"]),
                         nu=float(z[p + "nu"]), maxiter=len(X), fused=fused)
        x = s.solve().cpu().numpy()
        assert ctref.rel_l2(x, X[-1]) <= 1e-4, (k, ctref.rel_l2(x, X[-1]))

