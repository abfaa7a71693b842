"""The native unrolled-CG block with its hand-written backward
(inverse.cg_block: ct_cg_block_fwd / ct_cg_block_bwd) against the same
fixed-iteration CG run by torch autograd over the vector operations
(inverse.cg_solver, scico/flax/inverse.py:113-158), on the GPU projector.

Values and gradients (of b, lam and x0) agree to 1e-5 / 1e-4 while the
residual stays well above float32 rounding (4 steps at lam 10, 3 steps at
lam 0.1).  Where it does not -- 10 unconverged steps at lam 0.1, or 10
steps at lam 10, by which CG has reached float32 round-off and the reverse
recurrence divides by residual norms at the rounding floor -- any float32
implementation's gradients are rounding-dominated, so the bar there is 3x
the distance of the autograd float32 recurrence from a float64 run of the
same recurrence on the float64 oracle matrix.
Recomputation from the block's inputs reproduces the taped backward bit
for bit; a second backward on the same tape gives the same gradients."""

import numpy as np
import pytest
import torch

from oracle import ctref
from scico_gb300 import inverse, linop, workloads
from test_gpu_inverse import DenseOp

pytestmark = pytest.mark.gpu


def _op(n=32, nv=24):
    ang = np.linspace(0, np.pi, nv, endpoint=False)
    return linop.XRayTransform2D((n, n), ang), ctref.xray2d_defaults((n, n), ang)


def _rel(a, b):
    return float((a.double() - b.double()).norm() / b.double().norm())


def _both(H, b, lam_val, iters, x0=None, w_seed=3):
    """x and the gradients of <w, x> w.r.t. (b, lam, x0) by the native block
    and by autograd."""
    w = torch.randn(b.shape, generator=torch.Generator().manual_seed(w_seed)).to(b.device)
    out = []
    for native in (True, False):
        bb = b.clone().requires_grad_()
        lam = torch.full((1,), lam_val, device=b.device, requires_grad=True)
        xx0 = None if x0 is None else x0.clone().requires_grad_()
        if native:
            x = inverse.cg_block(H, bb, lam, x0=xx0, maxiter=iters)
        else:
            gram = lambda v: inverse.back_project(H, inverse.project(H, v)) + lam * v
            x = inverse.cg_solver(gram, bb, x0=xx0, maxiter=iters, batch_dims=1)
        params = [bb, lam] + ([xx0] if xx0 is not None else [])
        grads = torch.autograd.grad((w * x).sum(), params)
        out.append((x.detach(), grads))
    return out


@pytest.mark.parametrize("lam,iters", [(10.0, 4), (0.1, 3)])
@pytest.mark.parametrize("with_x0", [False, True])
def test_cg_block_matches_autograd(cuda, lam, iters, with_x0):
    H, _ = _op()
    gen = torch.Generator().manual_seed(1)
    b = torch.randn((3,) + H.input_shape, generator=gen).to(cuda)
    x0 = torch.randn((3,) + H.input_shape, generator=gen).to(cuda) if with_x0 else None
    (xn, gn), (xa, ga) = _both(H, b, lam, iters, x0)
    assert _rel(xn, xa) <= 1e-5
    for a, c in zip(gn, ga):
        assert _rel(a, c) <= 1e-4, (_rel(a, c), a.shape)


@pytest.mark.parametrize("lam", [0.1, 10.0])
def test_cg_block_ten_steps_vs_float64(cuda, lam):
    """10 steps (unconverged at lam 0.1, at round-off at lam 10): both
    float32 recurrences against float64."""
    H, g = _op(n=24, nv=16)
    gen = torch.Generator().manual_seed(2)
    b = torch.randn((2,) + H.input_shape, generator=gen).to(cuda)
    (xn, gn), (xa, ga) = _both(H, b, lam, 10)
    D = DenseOp(H, g, cuda)
    b64 = b.double().requires_grad_()
    lam64 = torch.full((1,), lam, dtype=torch.float64, device=cuda, requires_grad=True)
    gram64 = lambda v: inverse.back_project(D, inverse.project(D, v)) + lam64 * v
    x64 = inverse.cg_solver(gram64, b64, maxiter=10, batch_dims=1)
    w = torch.randn(b.shape, generator=torch.Generator().manual_seed(3)).to(cuda).double()
    g64 = torch.autograd.grad((w * x64).sum(), [b64, lam64])
    fx = _rel(xa, x64.detach())
    assert _rel(xn, x64.detach()) <= 3 * fx + 1e-5, (_rel(xn, x64.detach()), fx)
    for a, c, r in zip(gn, ga, g64):
        fl = _rel(c, r)
        assert _rel(a, r) <= 3 * fl + 1e-4, (_rel(a, r), fl)


def test_cg_block_recompute_and_second_backward(cuda):
    H, _ = _op()
    b = torch.randn((2,) + H.input_shape, generator=torch.Generator().manual_seed(4)).to(cuda)
    w = torch.randn(b.shape, generator=torch.Generator().manual_seed(5)).to(cuda)
    res = []
    for rc in (False, True):
        bb = b.clone().requires_grad_()
        lam = torch.full((1,), 0.3, device=cuda, requires_grad=True)
        x = inverse.cg_block(H, bb, lam, maxiter=6, recompute=rc)
        g1 = torch.autograd.grad((w * x).sum(), [bb, lam], retain_graph=True)
        g2 = torch.autograd.grad((w * x).sum(), [bb, lam])
        assert all(torch.equal(a, c) for a, c in zip(g1, g2))
        res.append((x.detach(), g1))
    assert torch.equal(res[0][0], res[1][0])
    assert all(torch.equal(a, c) for a, c in zip(res[0][1], res[1][1]))


def test_cg_block_scaled_projector(cuda):
    """A projector scaled by 1/N (the reference's training scripts) runs the
    native block with gram scale 1/N^2."""
    H, _ = _op()
    Hn = (1.0 / 32) * H
    b = torch.randn((2,) + H.input_shape, generator=torch.Generator().manual_seed(6)).to(cuda)
    (xn, gn), (xa, ga) = _both(Hn, b, 0.05, 5)
    assert _rel(xn, xa) <= 1e-5
    for a, c in zip(gn, ga):
        assert _rel(a, c) <= 1e-4


def test_modl_native_matches_autograd(cuda):
    """MoDLNet with the native CG blocks against the autograd CG blocks: loss
    and every parameter gradient (3 CG steps per block)."""
    n = 24
    H, _ = _op(n=n, nv=16)
    x_gt = torch.from_numpy(np.stack([workloads.random_ellipses(n, 4, s) for s in range(3)])).to(cuda)
    y = H.project(x_gt)
    out = []
    for impl in ("native", "autograd"):
        torch.manual_seed(5)
        net = inverse.MoDLNet(H, depth=2, channels=1, num_filters=4, block_depth=2, lmbda_ini=0.3, cg_iter=3,
                              cg_impl=impl).to(cuda)
        assert net.cg_native == (impl == "native")
        loss = ((net(y) - x_gt) ** 2).mean()
        out.append((loss.detach(), torch.autograd.grad(loss, list(net.parameters()))))
    assert abs(out[0][0].item() - out[1][0].item()) <= 1e-5 * out[1][0].item()
    num = sum(((a.double() - c.double()) ** 2).sum() for a, c in zip(out[0][1], out[1][1])).sqrt()
    den = sum((c.double() ** 2).sum() for c in out[1][1]).sqrt()
    assert (num / den).item() <= 1e-4


def test_cg_block_reference_code_vectors(cuda):
    """Against scico.flax's own cg_solver run under the float32 jax.numpy
    stand-in (tests/golden/modl_cg_reference_code.npz).  The block keeps its
    dot products in float64, the stand-in in float32: the bar is 3x the
    distance of the oracle's recurrence with float64 dots from the vectors,
    plus 1e-5 (at lambda 0.1 / 10 steps that distance is 6e-4, at 0.5 / 6
    steps 1e-4)."""
    from pathlib import Path

    z = np.load(Path(__file__).resolve().parent / "golden" / "modl_cg_reference_code.npz")
    for k in range(2):
        p = f"c{k}_"
        n, nv = int(z[p + "n"]), int(z[p + "nv"])
        ang = np.linspace(0, np.pi, nv, endpoint=False).astype(np.float32)
        H = linop.XRayTransform2D((n, n), ang)
        g = ctref.xray2d_defaults((n, n), ang)
        lm = float(z[p + "lmbda"])
        A = lambda v: ctref.xray2d_back_project(ctref.xray2d_project(v, g, np.float32), g, np.float32) + \
            np.float32(lm) * v
        floor = ctref.rel_l2(ctref.cg_fixed(A, z[p + "b"], maxiter=int(z[p + "maxiter"]), dot_dtype=np.float64),
                             z[p + "x"])
        b = torch.from_numpy(z[p + "b"]).to(cuda)[None]
        lam = torch.full((1,), lm, device=cuda)
        x = inverse.cg_block(H, b, lam, maxiter=int(z[p + "maxiter"]))[0].cpu().numpy()
        assert ctref.rel_l2(x, z[p + "x"]) <= 3 * floor + 1e-5, (k, ctref.rel_l2(x, z[p + "x"]), floor)

