"""Device-side failure detection of the 2D projector, exercised without a
GPU fault: every device wait in the library is bounded and every device
check sets a bit of an error word and skips the work it guards.

* The forward's strip-copy wait is made to run out by setting its poll
  limit to 0 (the copies themselves complete normally; the CTA then waits
  for them with the default limit before it releases its shared memory).
  The launch returns CT_OK, ct_proj2d_check reports CT_ERR_TIMEOUT, the
  affected CTAs leave zeros, and the next call with the default limit is
  exact and clean.
* The span checks (forward tile bins, adjoint view window) are tripped by a
  geometry whose declared max_width understates its view table's pixel
  widths: the host cannot see the table (it is device memory), the plan is
  sized from the declared width, and the device checks catch every span
  that does not fit and skip it (every access stays inside the plan's
  buffers).
"""

import ctypes

import numpy as np
import pytest
import torch

from scico_gb300 import _device, _lib, linop

pytestmark = pytest.mark.gpu


def _op(n=64, nv=24):
    return linop.XRayTransform2D((n, n), np.linspace(0, np.pi, nv, endpoint=False))


def _msg(lib):
    return (lib.ct_last_error() or b"").decode()


def test_strip_wait_timeout_reports_and_recovers(cuda):
    lib = _lib.load()
    H = _op()
    g = H.geometry()
    x = torch.rand(H.input_shape, generator=torch.Generator().manual_seed(1)).to(cuda)
    fwd_b, _ = H.workspace_bytes(1)
    ws = _device.workspace(fwd_b)
    stream = _device.stream()

    def fwd():
        y = torch.full(H.output_shape, float("nan"), device=cuda)
        st = lib.ct_proj2d_fwd(ctypes.addressof(g), x.data_ptr(), y.data_ptr(), 1, ws.data_ptr(), ws.numel(),
                               stream)
        return st, y

    st, y_ref = fwd()
    assert st == _lib.CT_OK
    assert lib.ct_proj2d_check(stream) == _lib.CT_OK
    default = lib.ct_wait_poll_limit()
    assert default == 1 << 24
    lib.ct_set_wait_poll_limit(0)
    try:
        st, y_bad = fwd()
    finally:
        lib.ct_set_wait_poll_limit(default)
    assert st == _lib.CT_OK  # the launch itself succeeds; the device reports later
    assert lib.ct_proj2d_check(stream) == _lib.CT_ERR_TIMEOUT
    assert "wait ran out" in _msg(lib)
    assert torch.count_nonzero(y_bad) == 0  # every CTA skipped its strip and left zeros (no NaN survives)
    assert lib.ct_proj2d_check(stream) == _lib.CT_OK  # the word was cleared
    st, y_again = fwd()
    assert st == _lib.CT_OK
    assert lib.ct_proj2d_check(stream) == _lib.CT_OK
    assert torch.equal(y_again, y_ref)


def test_span_checks_report_and_skip(cuda):
    lib = _lib.load()
    H = _op(n=96, nv=16)
    g = H.geometry()
    true_width = g.max_width
    g.max_width = 0.25 * true_width  # the plan's spans are sized for pixels a quarter as wide
    fwd_b, adj_b = _lib.c_size_t(), _lib.c_size_t()
    _lib.call("ct_proj2d_workspace", ctypes.addressof(g), 1, ctypes.addressof(fwd_b), ctypes.addressof(adj_b))
    ws = _device.workspace(max(fwd_b.value, adj_b.value))
    stream = _device.stream()
    x = torch.rand(H.input_shape, generator=torch.Generator().manual_seed(2)).to(cuda)
    y = torch.empty(H.output_shape, device=cuda)
    assert lib.ct_proj2d_fwd(ctypes.addressof(g), x.data_ptr(), y.data_ptr(), 1, ws.data_ptr(), ws.numel(),
                             stream) == _lib.CT_OK
    assert lib.ct_proj2d_check(stream) == _lib.CT_ERR_UNSUPPORTED
    assert "forward tile" in _msg(lib)
    b = torch.empty(H.input_shape, device=cuda)
    assert lib.ct_proj2d_adj(ctypes.addressof(g), y.data_ptr(), b.data_ptr(), 1, ws.data_ptr(), ws.numel(),
                             stream) == _lib.CT_OK
    assert lib.ct_proj2d_check(stream) == _lib.CT_ERR_UNSUPPORTED
    assert "adjoint window" in _msg(lib)
    # the honest geometry is clean and exact afterwards
    g.max_width = true_width
    y2 = H(x)
    assert lib.ct_proj2d_check(stream) == _lib.CT_OK
    assert torch.isfinite(y2).all() and float(y2.sum()) > 0


def test_solver_raises_on_device_check(cuda):
    """The fused solver reads the error words after its solve and raises
    instead of returning an image built on skipped work."""
    from scico_gb300 import functional, loss
    from scico_gb300.optimize import ADMM, LinearSubproblemSolver

    lib = _lib.load()
    n = 32
    H = _op(n=n, nv=20)
    y = H(torch.rand((n, n), generator=torch.Generator().manual_seed(3)).to(cuda))
    default = lib.ct_wait_poll_limit()
    lib.ct_set_wait_poll_limit(0)
    try:
        s = ADMM(f=loss.SquaredL2Loss(y=y, A=H), g_list=[0.01 * functional.L21Norm()],
                 C_list=[linop.FiniteDifference((n, n), append=0)], rho_list=[1.0], maxiter=2,
                 subproblem_solver=LinearSubproblemSolver(cg_kwargs={"tol": 1e-4, "maxiter": 3}), fused=True)
        with pytest.raises(_lib.CtError, match="wait ran out"):
            s.solve()
    finally:
        lib.ct_set_wait_poll_limit(default)
    assert lib.ct_proj2d_check(_device.stream()) == _lib.CT_OK
