"""TV norms with the shift-invariant Haar prox and AcceleratedPGM
(scico/functional/_tvnorm.py, scico/optimize/_pgm.py) on the GPU: Haar
transform identities and the TV prox against the oracle restatement, and the
reference's own cross-check (test_tvnorm.py:63-119): TV denoising by ADMM
and by AcceleratedPGM with the approximate prox agree to SNR > 50 dB, and
the TV norm equals the norm of the finite differences to 1e-6."""

import numpy as np
import pytest
import torch

from oracle import ctref
from scico_gb300 import functional, linop, loss, workloads
from scico_gb300.optimize import ADMM, AcceleratedPGM, LinearSubproblemSolver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,axes", [((17,), (0,)), ((12, 9), (0, 1)), ((12, 9), (1,)), ((5, 6, 7), (0, 1, 2)),
                                        ((5, 6, 7), (2, 0))])
def test_haar_kernels_vs_oracle(cuda, shape, axes):
    """ct_haar_fwd / ct_haar_adj against the oracle's float32 Haar transform
    and its adjoint (the same float32 operations): bit for bit."""
    rng = np.random.default_rng(4)
    x = rng.standard_normal(shape).astype(np.float32)
    w = functional.haar_transform(torch.from_numpy(x).to(cuda), axes=axes)
    np.testing.assert_array_equal(w.cpu().numpy(), ctref.haar_fwd(x, axes))
    wr = rng.standard_normal((len(axes), 2) + shape).astype(np.float32)
    back = functional.haar_transform(torch.from_numpy(wr).to(cuda), axes=axes, adjoint=True)
    np.testing.assert_array_equal(back.cpu().numpy(), ctref.haar_adj(wr, axes))


def test_haar_identities(cuda):
    x = torch.randn((3, 4), generator=torch.Generator().manual_seed(1)).to(cuda)
    for ax in (0, 1):
        w = functional.haar_transform(x, axes=(ax,))
        assert torch.allclose(functional.haar_transform(w, axes=(ax,), adjoint=True), 2 * x, rtol=1e-6, atol=1e-6)
    w = functional.haar_transform(x)
    assert torch.allclose(functional.haar_transform(w, adjoint=True), 4 * x, rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("iso", [True, False])
@pytest.mark.parametrize("circular", [True, False])
@pytest.mark.parametrize("shape", [(16, 20), (6, 8, 10), (50,)])
def test_tv_prox_vs_oracle(cuda, iso, circular, shape):
    v = np.random.default_rng(len(shape)).standard_normal(shape).astype(np.float32)
    h = (functional.IsotropicTVNorm if iso else functional.AnisotropicTVNorm)(circular=circular)
    got = h.prox(torch.from_numpy(v).to(cuda), 0.05).cpu().numpy()
    assert ctref.rel_l2(got, ctref.tv_prox(v, 0.05, iso, circular)) <= 1e-6


def _phantom(N, depth=None):
    x = workloads.circular_phantom((N, N), [0.6 * N, 0.4 * N, 0.2 * N, 0.1 * N], [0.25, 1, 0, 0.5])
    gr, gc = np.ogrid[0:N, 0:N]
    x = (x + (gr + gc) / (4 * N)).astype(np.float32)
    if depth:
        x = np.stack((0.9 * x, np.zeros(x.shape), 1.1 * x)).astype(np.float32)
    return x


def _cross_check(cuda, x_gt, tvtype, circular, L0, pgm_iter, admm_iter=150, axes=None):
    y = (x_gt + 0.02 * np.random.default_rng(0).standard_normal(x_gt.shape)).astype(np.float32)
    yt = torch.from_numpy(y).to(cuda)
    lam = 5e-2
    f = loss.SquaredL2Loss(y=yt)
    g = lam * (functional.L1Norm() if tvtype == "aniso" else functional.L21Norm())
    C = linop.FiniteDifference(x_gt.shape, axes=axes, circular=circular, append=None if circular else 0)
    admm = ADMM(f=f, g_list=[g], C_list=[C], rho_list=[1e1], x0=yt, maxiter=admm_iter,
                subproblem_solver=LinearSubproblemSolver(cg_kwargs={"tol": 1e-4, "maxiter": 25}))
    x_tvdn = admm.solve()
    h = lam * (functional.AnisotropicTVNorm(circular=circular, axes=axes) if tvtype == "aniso"
               else functional.IsotropicTVNorm(circular=circular, axes=axes))
    x_aprx = AcceleratedPGM(f=f, g=h, L0=L0, x0=yt, maxiter=pgm_iter).solve()
    a, b = x_tvdn.cpu().numpy(), x_aprx.cpu().numpy()
    assert ctref.snr(a, b) > 50, ctref.snr(a, b)
    gv, hv = g(C(x_tvdn)), h(x_tvdn)
    assert abs(gv - hv) / abs(gv) < 1e-6


@pytest.mark.parametrize("circular", [True, False])
def test_aniso_1d(cuda, circular):
    N = 128
    t = np.linspace(0, 2 * np.pi, N, dtype=np.float32)
    x_gt = np.clip(np.sin(2 * t), -0.5, 0.5).astype(np.float32)
    _cross_check(cuda, x_gt, "aniso", circular, L0=5e2, pgm_iter=100, admm_iter=50)


@pytest.mark.parametrize("circular", [True, False])
@pytest.mark.parametrize("tvtype", ["aniso", "iso"])
def test_2d(cuda, tvtype, circular):
    _cross_check(cuda, _phantom(32), tvtype, circular, L0=1e3, pgm_iter=400)


@pytest.mark.parametrize("tvtype", ["aniso", "iso"])
def test_3d(cuda, tvtype):
    """Three slices, differences along axes 1 and 2 only, non-circular."""
    _cross_check(cuda, _phantom(32, depth=3), tvtype, False, L0=1e3, pgm_iter=400, axes=(1, 2))
