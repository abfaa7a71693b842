"""Differentiable reconstruction on the GPU: projector VJPs, the
fixed-iteration cg_solver (scico/flax/inverse.py:113-158) and MoDLNet
(:35-110).

Values: cg_solver against the oracle restatement, MoDLNet's forward
against a float64 twin: the same module with the dense float64 matrix of the
oracle's projector as its operator.

Gradients: directional derivatives of the autograd gradient against central
finite differences along 20 random directions, difference <= 1e-3 relative
to the directional derivative's size (the check the benchmark definition
asks for; step 1e-3 per entry in float32, 1e-6 in float64 where the larger
step's truncation error would dominate).  The
unrolled fixed-iteration CG amplifies float32 rounding once it runs more
than a few unconverged steps (see test_cg_solver_vs_oracle), which float32
finite differences cannot resolve; so the full-length checks (10 CG steps,
lmbda 0.1) run in float64 through the identical autograd code on the dense
twin (<= 1e-3), and the float32 GPU gradients are compared with the twin's
at 3 CG steps (<= 1e-4); float32 finite differences themselves resolve only
~2e-3 here and are held to 1e-2 as a coarse check.  Convolutions run in full float32 (TF32 off, as
scico sets the highest matmul precision)."""

import numpy as np
import pytest
import torch

from oracle import ctref
from scico_gb300 import inverse, linop, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _no_tf32():
    old = (torch.backends.cudnn.allow_tf32, torch.backends.cuda.matmul.allow_tf32)
    torch.backends.cudnn.allow_tf32 = False
    torch.backends.cuda.matmul.allow_tf32 = False
    yield
    torch.backends.cudnn.allow_tf32, torch.backends.cuda.matmul.allow_tf32 = old


def _op(n=32, nv=24):
    ang = np.linspace(0, np.pi, nv, endpoint=False)
    return linop.XRayTransform2D((n, n), ang), ctref.xray2d_defaults((n, n), ang)


def test_projector_vjps(cuda):
    H, _ = _op()
    x = torch.rand((3,) + H.input_shape, device=cuda, requires_grad=True)
    g = torch.randn((3,) + H.output_shape, device=cuda)
    (inverse.project(H, x) * g).sum().backward()
    assert torch.equal(x.grad, H.back_project(g))
    y = torch.rand((2,) + H.output_shape, device=cuda, requires_grad=True)
    h = torch.randn((2,) + H.input_shape, device=cuda)
    (inverse.back_project(H, y) * h).sum().backward()
    assert torch.equal(y.grad, H.project(h))


@pytest.mark.parametrize("lam", [10.0, 0.1])
def test_cg_solver_vs_oracle(cuda, lam):
    """Three steps: rel l2 <= 1e-5 against the float64 oracle.  Ten steps:
    the fixed-iteration recurrence has no stopping test and amplifies
    rounding (the oracle's own float32 and float64 runs differ by 1e-4 ..
    6e-3 there), so the recurrence is checked against the oracle's cg_fixed
    (NumPy, float32 vectors, float64 dots) run with the GPU projector as its
    operator: the same operator values, so only the two implementations of
    the recurrence differ -- rel l2 <= 1e-5."""
    H, g = _op()
    rng = np.random.default_rng(0)
    b = rng.standard_normal((2,) + H.input_shape).astype(np.float32)
    gram = lambda v: inverse.back_project(H, inverse.project(H, v)) + lam * v
    A64 = lambda v: ctref.xray2d_back_project(ctref.xray2d_project(v, g, np.float64), g, np.float64) + lam * v

    def Agpu(v):  # the GPU operator on host arrays, float32 like the solver
        t = torch.from_numpy(np.ascontiguousarray(v, dtype=np.float32)).to(cuda)
        return (H.back_project(H.project(t)) + np.float32(lam) * t).cpu().numpy()

    bt = torch.from_numpy(b).to(cuda)
    x3 = inverse.cg_solver(gram, bt, maxiter=3, batch_dims=1).cpu().numpy()
    x10 = inverse.cg_solver(gram, bt, maxiter=10, batch_dims=1).cpu().numpy()
    for k in range(2):
        assert ctref.rel_l2(x3[k], ctref.cg_fixed(A64, b[k].astype(np.float64), maxiter=3)) <= 1e-5
        xh = ctref.cg_fixed(Agpu, b[k], maxiter=10, dot_dtype=np.float64)
        assert ctref.rel_l2(x10[k], xh) <= 1e-5, ctref.rel_l2(x10[k], xh)
        # one system at a time gives the same iterates as the batch
        xk = inverse.cg_solver(gram, bt[k], maxiter=10).cpu().numpy()
        assert ctref.rel_l2(xk, x10[k]) <= 1e-6


def _fd_check(f, params, n_dir=20, eps=1e-3, seed=0):
    """Directional derivatives of f (a scalar function of the tensors in
    `params`) by autograd and by central differences with step eps along
    random directions with unit-variance entries.  Returns the worst
    difference relative to max(|autograd|, |finite difference|, ||grad||):
    ||grad|| is the typical size of a directional derivative along such a
    direction, so directions whose contributions happen to cancel are not
    judged on their tiny total."""
    loss = f()
    grads = torch.autograd.grad(loss, params)
    gnorm = torch.sqrt(sum((gi.double() ** 2).sum() for gi in grads)).item()
    gen = torch.Generator().manual_seed(seed)
    worst = 0.0
    for _ in range(n_dir):
        # unit-variance entries: every parameter moves by about eps
        d = [torch.randn(p.shape, generator=gen, dtype=p.dtype).to(p.device) for p in params]
        ad = sum((gi.double() * di.double()).sum() for gi, di in zip(grads, d)).item()
        with torch.no_grad():
            for p, di in zip(params, d):
                p.add_(eps * di)
            fp = f().item()
            for p, di in zip(params, d):
                p.sub_(2 * eps * di)
            fm = f().item()
            for p, di in zip(params, d):
                p.add_(eps * di)
        fd = (fp - fm) / (2 * eps)
        worst = max(worst, abs(ad - fd) / max(abs(fd), abs(ad), gnorm, 1e-30))
    return worst


class DenseOp:
    """A projector given by its dense float64 matrix (built from the
    oracle's float64 projector), with the operator interface MoDLNet and
    cg_solver use."""

    def __init__(self, H, g, dev):
        n0, n1 = H.input_shape
        cols = []
        for k in range(n0 * n1):
            e = np.zeros((n0, n1))
            e.flat[k] = 1.0
            cols.append(ctref.xray2d_project(e, g, np.float64).ravel())
        self.A = torch.from_numpy(np.stack(cols, axis=1)).to(dev)
        self.input_shape, self.output_shape = H.input_shape, H.output_shape

    def project(self, v):
        return (v.reshape(v.shape[0], -1) @ self.A.T).reshape((v.shape[0],) + self.output_shape)

    def back_project(self, w):
        return (w.reshape(w.shape[0], -1) @ self.A).reshape((w.shape[0],) + self.input_shape)


def _cg_loss(H, b, lam, target, iters):
    gram = lambda v: inverse.back_project(H, inverse.project(H, v)) + lam * v
    x = inverse.cg_solver(gram, b, maxiter=iters, batch_dims=1)
    return ((x.double() - target.double()) ** 2).mean()


def test_cg_solver_gradients_float64(cuda):
    """10 CG steps on A^T A + 0.1 I (the MoDL setting), float64 dense twin."""
    H, g = _op(n=24, nv=16)
    D = DenseOp(H, g, cuda)
    gen = torch.Generator().manual_seed(3)
    b = torch.randn((2,) + H.input_shape, generator=gen, dtype=torch.float64).to(cuda).requires_grad_()
    lam = torch.full((1,), 0.1, dtype=torch.float64, device=cuda, requires_grad=True)
    target = torch.randn((2,) + H.input_shape, generator=gen, dtype=torch.float64).to(cuda)
    assert _fd_check(lambda: _cg_loss(D, b, lam, target, 10), [b, lam], eps=1e-6) <= 1e-3


def test_cg_solver_gradients(cuda):
    """3 CG steps through the GPU projector in float32; and the GPU gradient
    against the float64 twin's."""
    H, g = _op()
    gen = torch.Generator().manual_seed(4)
    b = torch.randn((2,) + H.input_shape, generator=gen).to(cuda).requires_grad_()
    lam = torch.full((1,), 0.3, device=cuda, requires_grad=True)
    target = torch.randn((2,) + H.input_shape, generator=gen).to(cuda)
    assert _fd_check(lambda: _cg_loss(H, b, lam, target, 3), [b, lam]) <= 1e-2  # float32 FD resolution
    gb, gl = torch.autograd.grad(_cg_loss(H, b, lam, target, 3), [b, lam])
    D = DenseOp(H, g, cuda)
    b64 = b.detach().double().requires_grad_()
    l64 = lam.detach().double().requires_grad_()
    hb, hl = torch.autograd.grad(_cg_loss(D, b64, l64, target.double(), 3), [b64, l64])
    assert ctref.rel_l2(gb.cpu().numpy(), hb.cpu().numpy()) <= 1e-4
    assert abs(gl.item() - hl.item()) <= 1e-4 * abs(hl.item())


def test_cg_recompute_same(cuda):
    H, _ = _op()
    out = []
    for rc in (False, True):
        b = torch.randn((2,) + H.input_shape, generator=torch.Generator().manual_seed(1)).to(cuda).requires_grad_()
        gram = lambda v: inverse.back_project(H, inverse.project(H, v)) + 0.2 * v
        x = inverse.cg_solver(gram, b, maxiter=5, batch_dims=1, recompute=rc)
        (x ** 2).sum().backward()
        out.append((x.detach(), b.grad))
    assert torch.equal(out[0][0], out[1][0])
    assert torch.allclose(out[0][1], out[1][1], rtol=1e-5, atol=1e-6)


def _small_modl(cuda, H, recompute=False):
    torch.manual_seed(5)
    net = inverse.MoDLNet(H, depth=2, channels=1, num_filters=4, block_depth=2, lmbda_ini=0.3, cg_iter=4,
                          cg_recompute=recompute).to(cuda)
    return net


def _modl_case(cuda, n=24, nv=16, batch=3):
    H, g = _op(n=n, nv=nv)
    x_gt = torch.from_numpy(np.stack([workloads.random_ellipses(n, 4, s) for s in range(batch)])).to(cuda)
    return H, g, x_gt, H.project(x_gt)


def test_modl_gradients_float64(cuda):
    """The C4 check at its full structure (CG(10) per block, lmbda 0.1) on a
    small case, float64 twin: gradients of an MSE training loss with respect
    to every parameter (lmbda, convolutions, batch norms) against central
    differences along 20 random directions."""
    H, g, x_gt, y = _modl_case(cuda)
    torch.manual_seed(5)
    net = inverse.MoDLNet(DenseOp(H, g, cuda), depth=2, channels=1, num_filters=4, block_depth=2, lmbda_ini=0.1,
                          cg_iter=10).to(cuda).double()
    yd, xd = y.double(), x_gt.double()
    assert _fd_check(lambda: ((net(yd) - xd) ** 2).mean(), list(net.parameters()), eps=1e-6) <= 1e-3


def test_modl_gradients(cuda):
    """float32 GPU MoDLNet (CG(3) per block): finite differences, and the
    gradients against the float64 twin with the same weights."""
    H, g, x_gt, y = _modl_case(cuda)
    torch.manual_seed(5)
    net = inverse.MoDLNet(H, depth=2, channels=1, num_filters=4, block_depth=2, lmbda_ini=0.3, cg_iter=3).to(cuda)
    params = list(net.parameters())
    loss = lambda: ((net(y).double() - x_gt.double()) ** 2).mean()
    assert _fd_check(loss, params) <= 1e-2  # float32 FD resolution
    grads = torch.autograd.grad(loss(), params)
    twin = inverse.MoDLNet(DenseOp(H, g, cuda), depth=2, channels=1, num_filters=4, block_depth=2, lmbda_ini=0.3,
                           cg_iter=3).to(cuda).double()
    twin.load_state_dict(net.state_dict())
    tg = torch.autograd.grad(((twin(y.double()) - x_gt.double()) ** 2).mean(), list(twin.parameters()))
    num = sum(((a.double() - b) ** 2).sum() for a, b in zip(grads, tg)).sqrt()
    den = sum((b ** 2).sum() for b in tg).sqrt()
    assert (num / den).item() <= 1e-4


def test_modl_forward_vs_dense_twin(cuda):
    """MoDLNet forward (5 blocks, lmbda 0.1, eval mode) against the same
    network run in float64 on the dense matrix of the oracle's float64
    projector.  With CG(3) per block: rel l2 <= 1e-4.  With CG(10) the five
    blocks of unconverged steps amplify float32 rounding, so the bar is 3x
    the distance between the float32 and float64 runs of the dense twin."""
    H, g, x_gt, y = _modl_case(cuda, batch=2)
    D = DenseOp(H, g, cuda)

    class Dense32(DenseOp):
        def __init__(self, d):
            self.A = d.A.float()
            self.input_shape, self.output_shape = d.input_shape, d.output_shape

    for cg_iter in (3, 10):
        torch.manual_seed(5)
        net = inverse.MoDLNet(H, depth=5, channels=1, num_filters=4, block_depth=2, lmbda_ini=0.1,
                              cg_iter=cg_iter).to(cuda).eval()
        out = net(y).detach().cpu().numpy()
        twin = inverse.MoDLNet(D, depth=5, channels=1, num_filters=4, block_depth=2, lmbda_ini=0.1,
                               cg_iter=cg_iter).to(cuda).double().eval()
        twin.load_state_dict(net.state_dict())
        ref = twin(y.double()).detach().cpu().numpy()
        if cg_iter == 3:
            assert ctref.rel_l2(out, ref) <= 1e-4, ctref.rel_l2(out, ref)
        else:
            t32 = inverse.MoDLNet(Dense32(D), depth=5, channels=1, num_filters=4, block_depth=2, lmbda_ini=0.1,
                                  cg_iter=cg_iter).to(cuda).eval()
            t32.load_state_dict(net.state_dict())
            floor = ctref.rel_l2(t32(y).detach().cpu().numpy(), ref)
            assert ctref.rel_l2(out, ref) <= 3 * floor + 1e-4, (ctref.rel_l2(out, ref), floor)


def test_modl_recompute_same(cuda):
    H, _ = _op()
    x_gt = torch.from_numpy(np.stack([workloads.random_ellipses(32, 4, s) for s in range(2)])).to(cuda)
    y = H.project(x_gt)
    res = []
    for rc in (False, True):
        net = _small_modl(cuda, H, recompute=rc)
        loss = ((net(y) - x_gt) ** 2).mean()
        loss.backward()
        res.append((loss.item(), net.lmbda.grad.item()))
    assert res[0][0] == res[1][0]
    assert abs(res[0][1] - res[1][1]) <= 1e-5 * max(1.0, abs(res[0][1]))
