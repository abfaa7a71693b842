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
* :class:`ResNet` and :class:`MoDLNet` -- scico/flax/_models.py:121-193 and
  scico/flax/inverse.py:35-110 as torch modules on NCHW tensors.
* :class:`ODPProxDnBlock`, :class:`ODPGrDescBlock` and :class:`ODPNet` --
  the unrolled optimization with deep priors (scico/flax/inverse.py:161-462),
  with the projector's VJPs in the data-fidelity gradient.
"""

from __future__ import annotations

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

    def forward(self, x):
        return self.body(x) + x


class MoDLNet(torch.nn.Module):
    r"""Model-based deep learning (MoDL) unrolled reconstruction
    (scico/flax/inverse.py:35-110).

    ``x = A^T y``; then ``depth`` times: ``z = ResNet(x)``,
    ``x = cg_solver(A^T A + lmbda I, A^T y + lmbda z, maxiter=cg_iter)`` per
    image.  The ResNet is shared by all blocks and ``lmbda`` is a trainable
    scalar, as in the reference.  Input: projections ``(batch, *A.output_shape)``;
    output: ``(batch, *A.input_shape)``.
    """

    def __init__(self, operator, depth: int, channels: int, num_filters: int, block_depth: int,
                 kernel_size: Tuple[int, int] = (3, 3), strides: Tuple[int, int] = (1, 1),
                 lmbda_ini: float = 0.5, cg_iter: int = 10, cg_recompute: bool = False):
        super().__init__()
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
    (:class:`ODPProxDnBlock` by default, :class:`ODPGrDescBlock` for CT).
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
