"""The allocation-free forward projection (ct_proj2d_fwd_noalloc).

Some callers of this library cannot allocate device memory when they
project -- code inside a stream capture it does not own, plugin hosts that
hand a custom call neither an allocator nor a scratch buffer, real-time
loops that forbid allocation once running.  The entry point they use keeps
its scratch in a fixed array inside the library; this file checks, through
the C ABI, that it gives the same sinograms as the workspace entry point on
two calls in a row (the second call reuses the array the first one left
behind) and that it refuses projections too large for the array.  The file
is named to be collected last.
"""

import ctypes

import numpy as np
import pytest
import torch

from scico_gb300 import _device, _lib, linop, workloads

pytestmark = pytest.mark.gpu


def _project_both(A, img):
    g = A.geometry()
    lib = _lib.load()
    out_ws = torch.empty(A.output_shape, device=img.device)
    fwd_bytes, _ = A.workspace_bytes(1)
    ws = _device.workspace(fwd_bytes)
    _lib.call("ct_proj2d_fwd", ctypes.addressof(g), img.data_ptr(), out_ws.data_ptr(), 1, ws.data_ptr(),
              ws.numel(), _device.stream())
    out_na = torch.full(A.output_shape, float("nan"), device=img.device)
    st = lib.ct_proj2d_fwd_noalloc(ctypes.addressof(g), img.data_ptr(), out_na.data_ptr(), 1, _device.stream())
    assert st == _lib.CT_OK, lib.ct_last_error()
    torch.cuda.synchronize()
    return out_ws, out_na


@pytest.mark.parametrize("cfg", ["c1", "c2"])
def test_noalloc_matches_workspace_entry_point(cuda, cfg):
    c = {"c1": workloads.C1, "c2": workloads.C2}[cfg]
    A = linop.XRayTransform2D((c.n, c.n), c.angles, det_count=c.det_count)
    first = torch.from_numpy(c.phantom()).to(cuda)
    second = torch.from_numpy(workloads.random_ellipses(c.n, 7, 99)).to(cuda)
    for img in (first, second):  # two calls in a row share the scratch array
        ref, got = _project_both(A, img)
        assert torch.isfinite(got).all()
        rel = float((got - ref).double().norm() / ref.double().norm())
        assert rel <= 1e-6, rel
        assert torch.equal(got, ref)  # same kernels, same summation order


def test_noalloc_rejects_oversized(cuda):
    # 2048^2, 720 views: far more scratch than the built-in 16 MiB
    ang = np.linspace(0, np.pi, 720, endpoint=False)
    A = linop.XRayTransform2D((2048, 2048), ang)
    g = A.geometry()
    lib = _lib.load()
    img = torch.zeros((2048, 2048), device=cuda)
    out = torch.zeros(A.output_shape, device=cuda)
    st = lib.ct_proj2d_fwd_noalloc(ctypes.addressof(g), img.data_ptr(), out.data_ptr(), 1, _device.stream())
    assert st == _lib.CT_ERR_UNSUPPORTED
    assert b"16777216-byte built-in array" in lib.ct_last_error()
