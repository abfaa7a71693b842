"""Filtered back projection (XRayTransform2D.fbp, _xray2d.py:158-221) on the
GPU: the ramp-filtered rows and the full FBP against the oracle's
FFT restatement (rel l2 <= 1e-5), and the reference's own quality test
(test_xray_2d.py:88-102: PSNR > 28 dB for a square phantom)."""

import numpy as np
import pytest
import torch

from oracle import ctref
from scico_gb300 import _lib, linop

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("det", [24, 47, 64, 725])
def test_ramp_filter_rows(cuda, det):
    rng = np.random.default_rng(det)
    y = rng.standard_normal((7, det)).astype(np.float32)
    out = torch.empty((7, det), device=cuda)
    _lib.call("ct_fbp_filter", torch.from_numpy(y).to(cuda).data_ptr(), out.data_ptr(), 7, det,
              torch.cuda.current_stream().cuda_stream)
    assert ctref.rel_l2(out.cpu().numpy(), ctref.xray2d_fbp_rows(y)) <= 1e-5


@pytest.mark.parametrize("n,nv,dx,det", [(64, 90, None, None), (48, 60, 0.5, 40), (96, 120, 1.0, 140)])
def test_fbp_vs_oracle(cuda, n, nv, dx, det):
    ang = np.linspace(0, np.pi, nv, endpoint=False)
    A = linop.XRayTransform2D((n, n), ang, dx=dx, det_count=det)
    g = ctref.xray2d_defaults((n, n), ang, dx=dx, det_count=det)
    x = np.random.default_rng(n).random((n, n)).astype(np.float32)
    y = ctref.xray2d_project(x, g, np.float64).astype(np.float32)
    got = A.fbp(torch.from_numpy(y).to(cuda)).cpu().numpy()
    assert ctref.rel_l2(got, ctref.xray2d_fbp(y, g)) <= 1e-5
    # leading batch axis
    yb = torch.from_numpy(np.stack([y, 2 * y])).to(cuda)
    gb = A.fbp(yb).cpu().numpy()
    assert np.array_equal(gb[0], got) and ctref.rel_l2(gb[1], 2 * got) <= 1e-6


@pytest.mark.parametrize("dx", [0.5, 1.0 / np.sqrt(2)])
@pytest.mark.parametrize("det_count_factor", [1.02 / np.sqrt(2.0), 1.0])
def test_fbp_reference_quality(cuda, dx, det_count_factor):
    """test_xray_2d.py:88-102: 256^2 square phantom, 360 views."""
    N = 256
    x_gt = np.zeros((N, N), dtype=np.float32)
    N4 = N // 4
    x_gt[N4:-N4, N4:-N4] = 1.0
    angles = np.linspace(0, np.pi, 360, endpoint=False)
    A = linop.XRayTransform2D(x_gt.shape, angles, det_count=int(det_count_factor * N), dx=dx)
    xt = torch.from_numpy(x_gt).to(cuda)
    x_fbp = A.fbp(A(xt)).cpu().numpy()
    assert ctref.psnr(x_gt, x_fbp) > 28
