"""Conjugate gradient solver (scico.solver.cg, scico/solver.py:326-405).

The vector steps and the float64 dot products run in the ctgpu kernels
(``ct_cg_init``, ``ct_dot``, ``ct_cg_update``, ``ct_cg_direction``); the
CG scalars stay on the device.  Like the reference, the loop test
``num > max(tol ||b||, atol)^2`` is evaluated on the host once per
iteration.
"""

from __future__ import annotations

import math
from typing import Callable, Optional

import torch

from . import _device, _lib
from .linop import LinearOperator


def cg(A: Callable, b, x0=None, *, tol: float = 1e-5, atol: float = 0.0, maxiter: int = 1000,
       info: bool = True, M: Optional[Callable] = None):
    """Solve ``A x = b`` for positive definite ``A`` (scico.solver.cg)."""
    if M is not None:
        raise NotImplementedError("preconditioned CG (M != None) is not on the device path")
    b = _device.to_device(b, name="b")
    if x0 is None:
        if isinstance(A, LinearOperator):
            x0 = torch.zeros_like(b)
        else:
            raise ValueError("Argument 'x0' must be specified if argument 'A' is not a LinearOperator.")
    x = _device.to_device(x0, name="x0").clone()
    n = b.numel()
    s = _device.zeros((_lib.CT_CG_NSCALARS,), dtype=torch.float64)
    ws = _device.reduce_workspace()
    st = _device.stream()
    r = torch.empty_like(b)
    p = torch.empty_like(b)
    Ax = A(x)
    _lib.call("ct_cg_init", b.data_ptr(), _device.to_device(Ax).data_ptr(), r.data_ptr(), p.data_ptr(), n,
              float(tol), float(atol), int(maxiter), s.data_ptr(), ws.data_ptr(), ws.numel(), st)
    pap = s.data_ptr() + 8 * _lib.CT_CG_PAP
    while s[_lib.CT_CG_DONE].item() == 0.0:
        Ap = _device.to_device(A(p))
        _lib.call("ct_dot", p.data_ptr(), Ap.data_ptr(), n, pap, ws.data_ptr(), ws.numel(), st)
        _lib.call("ct_cg_update", x.data_ptr(), r.data_ptr(), p.data_ptr(), Ap.data_ptr(), n, s.data_ptr(),
                  ws.data_ptr(), ws.numel(), st)
        _lib.call("ct_cg_direction", p.data_ptr(), r.data_ptr(), n, s.data_ptr(), ws.data_ptr(), ws.numel(), st)
    if not info:
        return x
    sc = s.cpu().numpy()
    bn = sc[_lib.CT_CG_BNORM]
    rel = math.sqrt(sc[_lib.CT_CG_NUM]) / bn if bn != 0 else float("nan")
    return x, {"num_iter": int(sc[_lib.CT_CG_ITERS]), "rel_res": rel}
