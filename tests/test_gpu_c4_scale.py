"""Gradients of the unrolled MoDL network at the training benchmark's own
scale: 256^2 images, 180 views, 363 bins, 5 blocks of CG(10) on
A^T A + 0.1 I, a 3-layer 32-filter ResNet (two images of the 16-image
batch: the gradient checks do not depend on the batch size).

The float64 reference is a twin of the network whose projector is the
oracle's float64 weight matrix held as a sparse CSR matrix on the GPU
(23.6 M non-zeros; cuSPARSE products), run through the same autograd code.

* float64 twin: directional derivatives along 20 random directions against
  central finite differences, relative to the directional derivative's
  size -- the benchmark definition's check, at full size.  With the
  ResNet's ReLUs replaced by a smooth activation (SiLU) the network is
  smooth and the check holds to 1e-3 (measured ~1e-4 at step 1e-5).  With
  the ReLUs (the network as specified) tens of millions of units sit near
  their kink, and central differences straddle kinks: the worst of 20
  directions lands at 1e-3 .. 4e-3 whatever the step (1e-5 .. 1e-7, where
  rounding takes over), so that case is held to median <= 2e-3 and worst
  <= 1e-2 and its numbers are reported.
* float32 GPU network (the library's projector) with the benchmark's
  CG(10): its gradient against the float64 twin's, within 3x the distance
  of the float32 twin (the same sparse matrix rounded to float32) from the
  float64 one.  Both are far (measured 0.68 relative, output 3 %): A^T A +
  0.1 I has lambda_max ~ 6.3e4, so float32 rounding of A p (eps |A p|)
  divided by lambda_min = 0.1 moves the iterate by ~eps kappa ~ 4 % once CG
  has resolved the large eigencomponents (after ~6 steps); this holds for
  any float32 evaluation of A, with float64 CG vectors too (2.5 %).
* float32 GPU network by central finite differences (step 1e-3): reported,
  and held to 3x the same check run on the float32 twin.
* The GPU network's gradient at CG(6), where float32 is still accurate
  (float32 and float64 gradients 2e-4 apart), against central finite
  differences of the float64 twin: 1e-3.
Each test prints one C4SCALE line with its measurements.
"""

import json
import warnings

import numpy as np
import pytest
import torch

from oracle import ctref
from scico_gb300 import inverse, linop, workloads
from test_gpu_inverse import _fd_check

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _no_tf32():
    old = (torch.backends.cudnn.allow_tf32, torch.backends.cuda.matmul.allow_tf32)
    torch.backends.cudnn.allow_tf32 = False
    torch.backends.cuda.matmul.allow_tf32 = False
    yield
    torch.backends.cudnn.allow_tf32, torch.backends.cuda.matmul.allow_tf32 = old


class SparseOp:
    """A 2D projector as a sparse matrix of the oracle's float64 weights
    (scico/linop/xray/_xray2d.py:308-351): rows view * det + bin, columns
    pixels; ``project`` / ``back_project`` on batched tensors."""

    def __init__(self, g, shape, dev, dtype=torch.float64):
        nv, ny = len(g["angles"]), g["ny"]
        npx = shape[0] * shape[1]
        rows, cols, vals = [], [], []
        pix = np.arange(npx)
        for a0 in range(0, nv, 12):
            sl = slice(a0, min(nv, a0 + 12))
            inds, w = ctref.xray2d_calc_weights(g, sl, np.float64)
            a = np.arange(sl.start, sl.stop)[:, None]
            inds, w = inds.reshape(len(a), -1), w.reshape(len(a), -1)
            for shift, val in ((0, w), (1, 1.0 - w)):
                k = inds + shift
                ok = (k >= 0) & (k < ny)
                rows.append((a * ny + k)[ok])
                cols.append(np.broadcast_to(pix, k.shape)[ok])
                vals.append(val[ok])
        idx = torch.from_numpy(np.stack([np.concatenate(rows), np.concatenate(cols)]))
        v = torch.from_numpy(np.concatenate(vals)).to(dtype)
        A = torch.sparse_coo_tensor(idx, v, (nv * ny, npx), check_invariants=True).coalesce()
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")  # CSR support is labelled beta
            self.A = A.to_sparse_csr().to(dev)
            self.AT = A.t().coalesce().to_sparse_csr().to(dev)
        self.nnz = int(v.numel())
        self.input_shape, self.output_shape = tuple(shape), (nv, ny)

    def project(self, x):
        b = x.shape[0]
        return torch.sparse.mm(self.A, x.reshape(b, -1).T).T.reshape((b,) + self.output_shape)

    def back_project(self, y):
        b = y.shape[0]
        return torch.sparse.mm(self.AT, y.reshape(b, -1).T).T.reshape((b,) + self.input_shape)


_STATE = {}


def _setup(cuda):
    if _STATE:
        return _STATE
    c = workloads.C4
    shape = (c.n, c.n)
    H = linop.XRayTransform2D(shape, c.angles, det_count=c.det_count)
    g = ctref.xray2d_defaults(shape, c.angles, det_count=c.det_count)
    x_gt = torch.from_numpy(c.phantoms()[:2]).to(cuda)
    y = H.project(x_gt)
    y = y + c.noise * y.abs().max() * torch.randn(y.shape, generator=torch.Generator().manual_seed(c.phantom_seed)).to(cuda)
    S64 = SparseOp(g, shape, cuda, torch.float64)
    S32 = SparseOp(g, shape, cuda, torch.float32)
    _STATE.update(c=c, H=H, x_gt=x_gt, y=y, S64=S64, S32=S32)
    return _STATE


def _net(c, op, dtype=torch.float32, cg_iter=None, act="relu"):
    torch.manual_seed(c.weight_seed)
    net = inverse.MoDLNet(op, depth=c.depth, channels=1, num_filters=c.num_filters, block_depth=c.block_depth,
                          lmbda_ini=c.lmbda_ini, cg_iter=c.cg_iter if cg_iter is None else cg_iter)
    if act == "silu":
        for i, m in enumerate(net.resnet.body):
            if isinstance(m, torch.nn.ReLU):
                net.resnet.body[i] = torch.nn.SiLU()
    return net.to(_STATE["x_gt"].device).to(dtype)


def _report(tag, d):
    print("C4SCALE " + tag + " " + json.dumps(d), flush=True)


def _fd_errors(f, params, n_dir=20, eps=1e-6, seed=0):
    """Per-direction |autograd - central difference| / max(|fd|, |ad|, ||grad||)
    along random directions with unit-variance entries."""
    grads = torch.autograd.grad(f(), params)
    gnorm = torch.sqrt(sum((gi.double() ** 2).sum() for gi in grads)).item()
    gen = torch.Generator().manual_seed(seed)
    errs = []
    for _ in range(n_dir):
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
        errs.append(abs(ad - fd) / max(abs(fd), abs(ad), gnorm, 1e-30))
    return errs


@pytest.mark.parametrize("act", ["silu", "relu"])
def test_c4_float64_twin_finite_differences(cuda, act):
    st = _setup(cuda)
    c = st["c"]
    net = _net(c, st["S64"], torch.float64, act=act)
    yd, xd = st["y"].double(), st["x_gt"].double()
    eps = 1e-5 if act == "silu" else 1e-6
    errs = _fd_errors(lambda: ((net(yd) - xd) ** 2).mean(), list(net.parameters()), n_dir=20, eps=eps)
    worst, med = max(errs), float(np.median(errs))
    _report("f64_fd_" + act, {"worst_rel": worst, "median_rel": med, "nnz": st["S64"].nnz, "directions": 20,
                              "eps": eps})
    if act == "silu":
        assert worst <= 1e-3, worst
    else:
        assert med <= 2e-3 and worst <= 1e-2, (med, worst)


def test_c4_gpu_gradients_vs_float64(cuda):
    st = _setup(cuda)
    c = st["c"]
    y, x_gt = st["y"], st["x_gt"]
    gpu = _net(c, st["H"])
    t64 = _net(c, st["S64"], torch.float64)
    t32 = _net(c, st["S32"])
    t64.load_state_dict(gpu.state_dict())
    t32.load_state_dict(gpu.state_dict())

    def grads(net, yy, xx):
        out = net(yy)
        return torch.autograd.grad(((out - xx) ** 2).mean(), list(net.parameters())), out.detach()

    g_gpu, o_gpu = grads(gpu, y, x_gt)
    g64, o64 = grads(t64, y.double(), x_gt.double())
    g32, o32 = grads(t32, y, x_gt)

    def rel(ga, gb):
        num = sum(((a.double() - b.double()) ** 2).sum() for a, b in zip(ga, gb)).sqrt()
        return float(num / sum((b.double() ** 2).sum() for b in gb).sqrt())

    e_gpu, floor = rel(g_gpu, g64), rel(g32, g64)
    out_gpu = float((o_gpu.double() - o64).norm() / o64.norm())
    out_floor = float((o32.double() - o64).norm() / o64.norm())
    _report("f32_vs_f64", {"grad_rel_gpu": e_gpu, "grad_rel_f32_twin": floor, "output_rel_gpu": out_gpu,
                           "output_rel_f32_twin": out_floor})
    assert e_gpu <= 3 * floor + 1e-4, (e_gpu, floor)
    assert out_gpu <= 3 * out_floor + 1e-5, (out_gpu, out_floor)


def test_c4_gpu_finite_differences(cuda):
    st = _setup(cuda)
    c = st["c"]
    y, x_gt = st["y"], st["x_gt"]
    gpu = _net(c, st["H"])
    t32 = _net(c, st["S32"])
    t32.load_state_dict(gpu.state_dict())
    loss = lambda n: (lambda: ((n(y).double() - x_gt.double()) ** 2).mean())
    e_gpu = _fd_check(loss(gpu), list(gpu.parameters()), n_dir=20, eps=1e-3)
    e_32 = _fd_check(loss(t32), list(t32.parameters()), n_dir=20, eps=1e-3)
    _report("f32_fd", {"worst_rel_gpu": e_gpu, "worst_rel_f32_twin": e_32, "directions": 20, "eps": 1e-3})
    assert e_gpu <= 3 * e_32 + 1e-3, (e_gpu, e_32)


@pytest.mark.parametrize("act", ["silu", "relu"])
def test_c4_gpu_gradient_vs_float64_finite_differences(cuda, act):
    """The GPU network's own gradient (float32, native CG blocks with the
    hand-written backward) against central finite differences of the float64
    twin, along 20 random directions, at the workload's sizes with CG(6):
    the longest CG in which float32 rounding of A p (relative eps |A p|,
    divided by lambda_min = 0.1 in the small-eigenvalue directions of
    A^T A + 0.1 I, lambda_max ~ 6.3e4) has not yet taken over -- float32 and
    float64 gradients agree to ~2e-4 at CG(5..6), 6e-4 at CG(7), 8e-3 at
    CG(8) and not at all at CG(10), for any float32 evaluation of A.  Held to
    1e-3 with the smooth activation; with the ReLUs, whose kinks limit
    central differences, to median 1e-3 and worst 1e-2."""
    st = _setup(cuda)
    c = st["c"]
    y, x_gt = st["y"], st["x_gt"]
    gpu = _net(c, st["H"], cg_iter=6, act=act)
    t64 = _net(c, st["S64"], torch.float64, cg_iter=6, act=act)
    t64.load_state_dict(gpu.state_dict())
    assert gpu.cg_native
    pg, p64 = list(gpu.parameters()), list(t64.parameters())
    grads = torch.autograd.grad(((gpu(y) - x_gt) ** 2).mean(), pg)
    gnorm = torch.sqrt(sum((gi.double() ** 2).sum() for gi in grads)).item()
    yd, xd = y.double(), x_gt.double()
    f = lambda: ((t64(yd) - xd) ** 2).mean()
    eps = 1e-5 if act == "silu" else 1e-6
    gen = torch.Generator().manual_seed(0)
    errs = []
    with torch.no_grad():
        for _ in range(20):
            d = [torch.randn(p.shape, generator=gen, dtype=torch.float64).to(p.device) for p in p64]
            ad = sum((gi.double() * di).sum() for gi, di in zip(grads, d)).item()
            for p, di in zip(p64, d):
                p.add_(eps * di)
            fp = f().item()
            for p, di in zip(p64, d):
                p.sub_(2 * eps * di)
            fm = f().item()
            for p, di in zip(p64, d):
                p.add_(eps * di)
            fd = (fp - fm) / (2 * eps)
            errs.append(abs(ad - fd) / max(abs(fd), abs(ad), gnorm, 1e-30))
    worst, med = max(errs), float(np.median(errs))
    _report("gpu_vs_f64_fd_cg6_" + act, {"worst_rel": worst, "median_rel": med, "directions": 20, "eps": eps,
                                         "cg_iter": 6})
    if act == "silu":
        assert worst <= 1e-3, worst
    else:
        assert med <= 1e-3 and worst <= 1e-2, (med, worst)
