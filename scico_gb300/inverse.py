"""Differentiable reconstruction: the pieces of scico.flax.inverse on the path.

* :func:`project` / :func:`back_project` -- a projector (XRayTransform2D or
  XRayTransform3D) as torch autograd Functions whose vector-Jacobian
  products are each other, the pairing scico's external projectors declare
  with ``jax.custom_vjp`` (scico/linop/xray/astra/_astra_2d.py:139-173).
* :func:`cg_solver` -- fixed-iteration conjugate gradient
  (scico/flax/inverse.py:113-158), differentiable through the unrolled
  steps; independent systems along leading batch axes (the reference maps
  the solver over a batch with ``lax.map``); optional recomputation of each
  step in the backward pass instead of keeping its intermediates.
* :func:`cg_block` -- the same fixed-iteration CG on H^T H + lam I for a
  2D projector, in native kernels whose backward is the hand-written
  reverse recurrence of the CG steps (optionally recomputing the iterates
  from the block's inputs).
* :class:`ResNet` and :class:`MoDLNet` -- scico/flax/_models.py:121-193 and
  scico/flax/inverse.py:35-110 as torch modules on NCHW tensors.
* :class:`ODPProxDnBlock`, :class:`ODPGrDescBlock` and :class:`ODPNet` --
  the unrolled optimization with deep priors (scico/flax/inverse.py:161-462),
  with the projector's VJPs in the data-fidelity gradient.
"""

from __future__ import annotations

import math
from typing import Callable, Optional, Tuple

import torch

from . import _device


class _Project(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, H):
        ctx.H = H
        return H.project(x.contiguous())

    @staticmethod
    def backward(ctx, g):
        return ctx.H.back_project(g.contiguous()), None


class _BackProject(torch.autograd.Function):
    @staticmethod
    def forward(ctx, y, H):
        ctx.H = H
        return H.back_project(y.contiguous())

    @staticmethod
    def backward(ctx, g):
        return ctx.H.project(g.contiguous()), None


def project(H, x: torch.Tensor) -> torch.Tensor:
    """``H.project(x)`` with ``H.back_project`` as its vector-Jacobian
    product (a leading batch axis is allowed)."""
    return _Project.apply(x, H)


def back_project(H, y: torch.Tensor) -> torch.Tensor:
    """``H.back_project(y)`` with ``H.project`` as its vector-Jacobian product."""
    return _BackProject.apply(y, H)


def cg_solver(A: Callable, b: torch.Tensor, x0: Optional[torch.Tensor] = None, maxiter: int = 50,
              batch_dims: int = 0, recompute: bool = False) -> torch.Tensor:
    r"""Conjugate gradient with a fixed number of iterations.

    Solves :math:`A\mb{x} = \mb{b}` for positive definite ``A`` with
    exactly ``maxiter`` steps from ``r0 = b - A(x0)``, ``p0 = r0``:
    ``alpha = num / <p, Ap>``, ``x += alpha p``, ``r -= alpha Ap``,
    ``beta = num' / num``, ``p = r + beta p`` (scico/flax/inverse.py:
    136-157).  Differentiable: autograd runs the reverse of the unrolled
    recurrence.

    Args:
        A: Function implementing the positive definite operator.
        b: Right-hand side.
        x0: Initial solution (zeros if ``None``).
        maxiter: Number of iterations.
        batch_dims: Leading axes of ``b`` that index independent systems,
            each with its own step sizes.
        recompute: Keep only each step's inputs for the backward pass and
            recompute the step there (less memory, one more ``A`` per step).

    Returns:
        The solution after ``maxiter`` steps.
    """
    dims = tuple(range(batch_dims, b.ndim))

    def dot(u, v):  # float64 accumulation, one value per system
        return (u.double() * v.double()).sum(dim=dims)

    def bc(s, like):
        return s.to(like.dtype).reshape(s.shape + (1,) * (like.ndim - batch_dims))

    def step(x, r, p, num):
        Ap = A(p)
        alpha = num / dot(p, Ap)
        x = x + bc(alpha, x) * p
        r = r - bc(alpha, r) * Ap
        num_new = dot(r, r)
        p = r + bc(num_new / num, p) * p
        return x, r, p, num_new

    x = torch.zeros_like(b) if x0 is None else x0
    r = b - A(x)
    num = dot(r, r)
    p = r
    for _ in range(maxiter):
        if recompute and torch.is_grad_enabled():
            from torch.utils.checkpoint import checkpoint

            x, r, p, num = checkpoint(step, x, r, p, num, use_reentrant=False)
        else:
            x, r, p, num = step(x, r, p, num)
    return x


def _native_projector(H):
    """(XRayTransform2D, gram scale) when H is a 2D projector or a scalar
    multiple of one (the native CG block applies s H^T H), else None."""
    from . import linop

    if isinstance(H, linop.XRayTransform2D):
        return H, 1.0
    if isinstance(H, linop.ScaledProjector) and isinstance(H.base, linop.XRayTransform2D):
        return H.base, H.scale * H.scale
    return None


class _CGBlock(torch.autograd.Function):
    """maxiter fixed CG steps on (s H^T H + lam I) x = b in the native kernels
    (ct_cg_block_fwd), with the hand-written reverse recurrence
    (ct_cg_block_bwd) as the backward."""

    @staticmethod
    def forward(ctx, b, lam, x0, H2, gs, maxiter, recompute):
        from . import _lib

        b = b.contiguous()
        lam32 = float(lam.detach().reshape(-1)[0].float())
        desc = _lib.CgBlockDesc(H2.geometry(), b.shape[0], int(maxiter), int(bool(recompute)), float(gs))
        tb, wb = _lib.c_size_t(), _lib.c_size_t()
        _lib.call("ct_cg_block_workspace", _lib.ctypes.addressof(desc), _lib.ctypes.addressof(tb),
                  _lib.ctypes.addressof(wb))
        tape = _device.workspace(tb.value)
        ws = _device.workspace(wb.value)
        x = torch.empty_like(b)
        x0c = x0.contiguous() if x0 is not None else None
        _lib.call("ct_cg_block_fwd", _lib.ctypes.addressof(desc), b.data_ptr(), lam32,
                  x0c.data_ptr() if x0c is not None else None, x.data_ptr(), tape.data_ptr(), tape.numel(),
                  ws.data_ptr(), ws.numel(), _device.stream())
        ctx.desc, ctx.tape, ctx.lam32, ctx.wbytes = desc, tape, lam32, wb.value
        ctx.lam_shape, ctx.lam_dtype = lam.shape, lam.dtype
        ctx.has_x0 = x0c is not None
        ctx.save_for_backward(b, x0c if x0c is not None else b)
        return x

    @staticmethod
    def backward(ctx, gx):
        from . import _lib

        b, x0 = ctx.saved_tensors
        x0 = x0 if ctx.has_x0 else None
        gx = gx.contiguous()
        gb = torch.empty_like(gx)
        gx0 = torch.empty_like(gx) if (x0 is not None and ctx.needs_input_grad[2]) else None
        glam = torch.zeros(1, dtype=torch.float64, device=gx.device)
        ws = _device.workspace(ctx.wbytes)
        _lib.call("ct_cg_block_bwd", _lib.ctypes.addressof(ctx.desc), gx.data_ptr(), b.data_ptr(), ctx.lam32,
                  x0.data_ptr() if x0 is not None else None, ctx.tape.data_ptr(), ctx.tape.numel(), gb.data_ptr(),
                  gx0.data_ptr() if gx0 is not None else None, glam.data_ptr(), ws.data_ptr(), ws.numel(),
                  _device.stream())
        glam_t = glam.to(ctx.lam_dtype).reshape(ctx.lam_shape) if ctx.needs_input_grad[1] else None
        return gb, glam_t, gx0, None, None, None, None


def cg_block(H, b: torch.Tensor, lam: torch.Tensor, x0: Optional[torch.Tensor] = None, maxiter: int = 10,
             recompute: bool = False) -> torch.Tensor:
    r"""``maxiter`` fixed conjugate-gradient steps on
    :math:`(H^T H + \lambda I) \mb{x} = \mb{b}` for a batch of images
    (leading axis of ``b``), each with its own step sizes -- the
    data-consistency block of MoDL (scico/flax/inverse.py:113-158) -- in the
    native kernels with a hand-written backward (``ct_cg_block_fwd`` /
    ``ct_cg_block_bwd``): the reverse recurrence of the CG steps, not
    autograd over the vector operations.  ``H`` is an XRayTransform2D or a
    scalar multiple of one; ``lam`` a one-element tensor (a trainable
    parameter).  ``recompute``: the forward keeps only the step scalars and
    the backward recomputes the iterates from ``b``, ``lam`` and ``x0``.
    Gradients flow to ``b``, ``lam`` and ``x0``."""
    nat = _native_projector(H)
    if nat is None:
        raise TypeError("cg_block needs an XRayTransform2D (or a scalar multiple of one)")
    H2, gs = nat
    if b.ndim != 3 or tuple(b.shape[1:]) != tuple(H2.input_shape) or b.dtype != torch.float32:
        raise ValueError(f"cg_block: b must be float32 (batch, *{tuple(H2.input_shape)}), got {tuple(b.shape)}")
    return _CGBlock.apply(b, lam, x0, H2, gs, int(maxiter), bool(recompute))


class ResNet(torch.nn.Module):
    """Convolutional net with a residual connection
    (scico/flax/_models.py:121-193): ``depth - 1`` blocks of convolution
    (no bias, circular padding, Xavier-normal init), batch normalization
    (flax momentum 0.99 = torch momentum 0.01, epsilon 1e-5) and ReLU, then a
    convolution back to ``channels`` and a batch normalization, plus the
    input.  NCHW tensors."""

    def __init__(self, depth: int, channels: int, num_filters: int = 64,
                 kernel_size: Tuple[int, int] = (3, 3), strides: Tuple[int, int] = (1, 1)):
        super().__init__()
        pad = (kernel_size[0] // 2, kernel_size[1] // 2)
        layers = []
        cin = channels
        for _ in range(depth - 1):
            layers += [
                torch.nn.Conv2d(cin, num_filters, kernel_size, stride=strides, padding=pad,
                                padding_mode="circular", bias=False),
                torch.nn.BatchNorm2d(num_filters, eps=1e-5, momentum=0.01),
                torch.nn.ReLU(),
            ]
            cin = num_filters
        layers += [
            torch.nn.Conv2d(cin, channels, kernel_size, stride=strides, padding=pad, padding_mode="circular",
                            bias=False),
            torch.nn.BatchNorm2d(channels, eps=1e-5, momentum=0.01),
        ]
        self.body = torch.nn.Sequential(*layers)
        for m in self.body:
            if isinstance(m, torch.nn.Conv2d):
                torch.nn.init.xavier_normal_(m.weight)
        # NHWC (channels-last) activations and filters: cuDNN's convolution
        # and batch-norm kernels for this layout run the MoDL training step
        # (16 x 256^2 images, 32 filters) in
        # 0.82x the time of NCHW (float32 throughout, same arithmetic up to
        # the kernels' summation order)
        self.body.to(memory_format=torch.channels_last)

    def forward(self, x):
        y = self.body(x.contiguous(memory_format=torch.channels_last))
        return y.contiguous() + x


class MoDLNet(torch.nn.Module):
    r"""Model-based deep learning (MoDL) unrolled reconstruction
    (scico/flax/inverse.py:35-110).

    ``x = A^T y``; then ``depth`` times: ``z = ResNet(x)``,
    ``x = cg_solver(A^T A + lmbda I, A^T y + lmbda z, maxiter=cg_iter)`` per
    image.  The ResNet is shared by all blocks and ``lmbda`` is a trainable
    scalar, as in the reference.  Input: projections ``(batch, *A.output_shape)``;
    output: ``(batch, *A.input_shape)``.

    ``cg_impl``: "native" (default where the operator is an XRayTransform2D
    or a scalar multiple of one) runs each CG block as :func:`cg_block`, the
    native kernels with the hand-written backward; "autograd" runs
    :func:`cg_solver` (torch autograd over the unrolled vector operations),
    which also serves any other operator.
    """

    def __init__(self, operator, depth: int, channels: int, num_filters: int, block_depth: int,
                 kernel_size: Tuple[int, int] = (3, 3), strides: Tuple[int, int] = (1, 1),
                 lmbda_ini: float = 0.5, cg_iter: int = 10, cg_recompute: bool = False, cg_impl: str = "native"):
        super().__init__()
        if cg_impl not in ("native", "autograd"):
            raise ValueError(f"cg_impl must be 'native' or 'autograd', got {cg_impl!r}")
        self.cg_native = cg_impl == "native" and _native_projector(operator) is not None
        if channels != 1:
            raise ValueError("MoDLNet here reconstructs single-channel images (channels=1)")
        self.operator = operator
        self.depth = depth
        self.cg_iter = cg_iter
        self.cg_recompute = cg_recompute
        self.lmbda = torch.nn.Parameter(torch.full((1,), float(lmbda_ini)))
        self.resnet = ResNet(block_depth, channels, num_filters, kernel_size, strides)

    def forward(self, y: torch.Tensor) -> torch.Tensor:
        H = self.operator
        lm = self.lmbda.to(y.dtype)
        Ahb = back_project(H, y)
        x = Ahb

        def gram(v):
            return back_project(H, project(H, v)) + lm * v

        for _ in range(self.depth):
            z = self.resnet(x.unsqueeze(1)).squeeze(1)
            b = Ahb + lm * z
            if self.cg_native and y.dtype == torch.float32:
                x = cg_block(H, b, self.lmbda, maxiter=self.cg_iter, recompute=self.cg_recompute)
            else:
                x = cg_solver(gram, b, maxiter=self.cg_iter, batch_dims=1, recompute=self.cg_recompute)
        return x


class ODPProxDnBlock(torch.nn.Module):
    """ODP proximal-gradient denoising block (scico/flax/inverse.py:161-226):
    ``x = (ResNet(x) + alpha y) / (1 + alpha)`` with a trainable scalar
    ``alpha`` (initial ``alpha_ini``).  The operator is the identity of the
    denoising problem; :meth:`batch_op_adj` applies its adjoint."""

    def __init__(self, operator, depth: int, channels: int, num_filters: int,
                 kernel_size: Tuple[int, int] = (3, 3), strides: Tuple[int, int] = (1, 1),
                 alpha_ini: float = 0.2):
        super().__init__()
        self.operator = operator
        self.alpha = torch.nn.Parameter(torch.full((1,), float(alpha_ini)))
        self.resnet = ResNet(depth, channels, num_filters, kernel_size, strides)

    def batch_op_adj(self, y: torch.Tensor) -> torch.Tensor:
        return y if self.operator is None else back_project(self.operator, y)

    def forward(self, x: torch.Tensor, y: torch.Tensor) -> torch.Tensor:
        a = self.alpha.to(x.dtype)
        return (self.resnet(x.unsqueeze(1)).squeeze(1) + y * a) / (1.0 + a)


def _gram_norm(operator, maxiter: int = 100, seed: int = 0) -> float:
    """||A||_2 = sqrt(largest eigenvalue of A^T A) by power iteration
    (scico/linop/_util.py:27-76, 79-110) on the operator's batched
    ``project`` / ``back_project``: normalized random start, per step
    ``Av = A^T A v``, ``mu = <v, Av> / ||v||^2``, ``v = Av / ||Av||``; sums in
    float64."""
    gen = torch.Generator().manual_seed(seed)
    v = torch.randn((1,) + tuple(operator.input_shape), generator=gen)
    v = v / torch.linalg.vector_norm(v.double()).float()
    mu = 0.0
    with torch.no_grad():
        for _ in range(maxiter):
            Av = operator.back_project(operator.project(v))
            v = v.to(Av.device)
            nav = float(torch.linalg.vector_norm(Av.double()))
            if nav == 0.0:  # a zero operator
                return 0.0
            mu = float((v.double() * Av.double()).sum()) / float((v.double() ** 2).sum())
            v = Av / nav
    return math.sqrt(max(mu, 0.0))


class ODPProxDcnvBlock(torch.nn.Module):
    """ODP proximal-gradient deconvolution block (scico/flax/inverse.py:
    228-313) for an operator A with batched ``project`` / ``back_project``
    (a circular convolution in the reference's use).  ||A|| is computed once
    by power iteration on A^T A; the block returns, as the reference
    computes it, the inverse real DFT over the two image axes of the real
    DFT of ``alpha A^T y + ResNet(x)`` divided by
    ``scale = 1 / (alpha ||A||^2 + 1)``, with a trainable scalar ``alpha``
    (initial ``alpha_ini``)."""

    def __init__(self, operator, depth: int, channels: int, num_filters: int,
                 kernel_size: Tuple[int, int] = (3, 3), strides: Tuple[int, int] = (1, 1),
                 alpha_ini: float = 0.99):
        super().__init__()
        self.operator = operator
        self.operator_norm = _gram_norm(operator)
        self.alpha = torch.nn.Parameter(torch.full((1,), float(alpha_ini)))
        self.resnet = ResNet(depth, channels, num_filters, kernel_size, strides)

    def batch_op_adj(self, y: torch.Tensor) -> torch.Tensor:
        return back_project(self.operator, y)

    def forward(self, x: torch.Tensor, y: torch.Tensor) -> torch.Tensor:
        a = self.alpha.to(x.dtype)
        scale = 1.0 / (a * self.operator_norm ** 2 + 1.0)
        v = a * self.batch_op_adj(y) + self.resnet(x.unsqueeze(1)).squeeze(1)
        f = torch.fft.rfftn(v, dim=(-2, -1)) / scale
        return torch.fft.irfftn(f, s=v.shape[-2:], dim=(-2, -1))


class ODPGrDescBlock(torch.nn.Module):
    r"""ODP gradient-descent block for an :math:`\ell_2` data term
    (scico/flax/inverse.py:295-375): ``x = ResNet(x) - alpha A^T (A x - y)``
    with a trainable scalar ``alpha``; ``A`` and ``A^T`` are the projector
    and its adjoint (each other's vector-Jacobian products)."""

    def __init__(self, operator, depth: int, channels: int, num_filters: int,
                 kernel_size: Tuple[int, int] = (3, 3), strides: Tuple[int, int] = (1, 1),
                 alpha_ini: float = 0.2):
        super().__init__()
        self.operator = operator
        self.alpha = torch.nn.Parameter(torch.full((1,), float(alpha_ini)))
        self.resnet = ResNet(depth, channels, num_filters, kernel_size, strides)

    def batch_op_adj(self, y: torch.Tensor) -> torch.Tensor:
        return back_project(self.operator, y)

    def forward(self, x: torch.Tensor, y: torch.Tensor) -> torch.Tensor:
        H = self.operator
        r = project(H, x) - y
        return self.resnet(x.unsqueeze(1)).squeeze(1) - self.alpha.to(x.dtype) * back_project(H, r)


class ODPNet(torch.nn.Module):
    """Unrolled optimization with deep priors (scico/flax/inverse.py:378-462):
    ``x = A^T y``, then ``depth`` blocks, each with its own ResNet and
    ``alpha``; the first block's ``alpha`` starts at ``alpha_ini`` and each
    later one at half its predecessor's.  ``odp_block`` selects the block
    (:class:`ODPProxDnBlock` by default, :class:`ODPGrDescBlock` for CT,
    :class:`ODPProxDcnvBlock` for deconvolution).
    Input ``(batch, *A.output_shape)``, output ``(batch, *A.input_shape)``;
    single-channel images."""

    def __init__(self, operator, depth: int, channels: int, num_filters: int, block_depth: int,
                 kernel_size: Tuple[int, int] = (3, 3), strides: Tuple[int, int] = (1, 1),
                 alpha_ini: float = 0.5, odp_block=None):
        super().__init__()
        if channels != 1:
            raise ValueError("ODPNet here reconstructs single-channel images (channels=1)")
        block = ODPProxDnBlock if odp_block is None else odp_block
        self.operator = operator
        alphas = [alpha_ini / 2.0**k for k in range(depth)]
        self.blocks = torch.nn.ModuleList(
            block(operator, block_depth, channels, num_filters, kernel_size, strides, alpha_ini=a) for a in alphas)

    def forward(self, y: torch.Tensor) -> torch.Tensor:
        x = self.blocks[0].batch_op_adj(y)
        for blk in self.blocks:
            x = blk(x, y)
        return x


def to_device(module: torch.nn.Module) -> torch.nn.Module:
    """Move a module to the CUDA device the operators run on."""
    return module.to(_device.require_cuda())
