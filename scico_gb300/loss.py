"""SquaredL2Loss (scico/loss.py:154-267), the data term of the CT ADMM-TV path."""

from __future__ import annotations

from typing import Optional

import torch

from . import _device, _lib, linop
from .functional import Functional


def _sqnorm(t: torch.Tensor) -> float:
    """sum(t^2), products and sums in float64 on the device."""
    t = t.reshape(-1)
    out = _device.zeros((1,), dtype=torch.float64)
    ws = _device.reduce_workspace()
    _lib.call("ct_dot", t.data_ptr(), t.data_ptr(), t.numel(), out.data_ptr(), ws.data_ptr(), ws.numel(),
              _device.stream())
    return float(out.item())


class SquaredL2Loss(Functional):
    r"""``scale * || y - A(x) ||_W^2`` with W = Identity (scico/loss.py:154).

    Only the unweighted loss (W = None / Identity) is on the CT path.
    """

    has_eval = True

    def __init__(self, y, A: Optional[linop.LinearOperator] = None, scale: float = 0.5, W=None,
                 prox_kwargs: Optional[dict] = None):
        if W is not None and not isinstance(W, linop.Identity):
            raise NotImplementedError("only W = None (identity weighting) is implemented")
        self.y = _device.to_device(y, name="y")
        self.A = linop.Identity(tuple(self.y.shape)) if A is None else A
        self.W = linop.Identity(tuple(self.y.shape))
        self.scale = float(scale)
        # closed-form prox for a diagonal (here: identity) A (scico/loss.py:220-226)
        self.has_prox = isinstance(self.A, linop.Identity)

    def prox(self, v, lam: float = 1.0, **kwargs):
        """``argmin_x 1/2 ||v - x||^2 + lam scale ||y - x||^2`` for A = I:
        ``(c y + v) / (c + 1)`` with ``c = 2 scale lam`` (scico/loss.py:220-226)."""
        if not self.has_prox:
            raise NotImplementedError("prox of SquaredL2Loss is implemented for A = Identity")
        c = 2.0 * self.scale * lam
        return (c * self.y + v) / (c + 1.0)

    def __call__(self, x) -> float:
        r = self.y - self.A(x)
        return self.scale * _sqnorm(r)

    def grad(self, x):
        """Gradient ``2 scale A^T (A x - y)`` (the reference differentiates
        scale ||y - A x||^2 with jax.grad, scico/loss.py:104)."""
        return (2.0 * self.scale) * self.A.adj(self.A(x) - self.y)

    @property
    def hessian(self) -> linop.LinearOperator:
        """``2 * scale * A^T W A`` (scico/loss.py:245-262)."""
        A = self.A
        c = 2.0 * self.scale
        return linop.LinearOperator(
            input_shape=A.input_shape,
            output_shape=A.input_shape,
            eval_fn=lambda x: c * A.adj(A(x)),
            adj_fn=lambda x: c * A.adj(A(x)),
            input_dtype=A.input_dtype,
        )
