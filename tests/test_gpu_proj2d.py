"""2D projector on the GPU (through the C ABI) against the oracle.

Tolerances: rel l2 <= 1e-5 per application against the float64 oracle
(the weights differ from the oracle's by at most one float32 ulp and the
summation order differs); dot test <Ax, y> = <x, A^T y> to 1e-6 relative.
"""

import ctypes
from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import ctref
from scico_gb300 import _device, _lib, linop

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"

GEOMS = [
    dict(shape=(24, 20), nv=7),
    dict(shape=(12, 13), nv=10),
    dict(shape=(16, 16), nv=3, dx=1 / np.sqrt(2), det=int(16 * 1.05 / np.sqrt(2.0))),
    dict(shape=(33, 47), nv=17, dx=0.5, det=40),
    dict(shape=(40, 40), nv=12, dx=1.0, det=60),  # width up to sqrt2 > 1
    dict(shape=(64, 64), nv=45),
    dict(shape=(70, 31), nv=29, det=30),  # narrow detector, many pixels off it
]


def _op(gp):
    ang = np.linspace(0, np.pi, gp["nv"], endpoint=False)
    import warnings

    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        H = linop.XRayTransform2D(gp["shape"], ang, dx=gp.get("dx"), det_count=gp.get("det"))
    g = ctref.xray2d_defaults(gp["shape"], ang, dx=gp.get("dx"), det_count=gp.get("det"))
    return H, g


@pytest.mark.parametrize("gp", GEOMS, ids=lambda g: f"{g['shape']}x{g['nv']}")
def test_fwd_adj_vs_oracle(cuda, gp):
    H, g = _op(gp)
    rng = np.random.default_rng(hash(str(gp)) % 2**32)
    x = rng.random(gp["shape"]).astype(np.float32)
    y = H(torch.from_numpy(x).to(cuda)).cpu().numpy()
    y64 = ctref.xray2d_project(x, g, np.float64)
    assert ctref.rel_l2(y, y64) <= 1e-5
    ys = rng.standard_normal(H.output_shape).astype(np.float32)
    b = H.adj(torch.from_numpy(ys).to(cuda)).cpu().numpy()
    b64 = ctref.xray2d_back_project(ys, g, np.float64)
    assert ctref.rel_l2(b, b64) <= 1e-5
    # and against the float32 restatement of the reference's own arithmetic
    assert ctref.rel_l2(y, ctref.xray2d_project(x, g, np.float32)) <= 1e-5


@pytest.mark.parametrize("gp", GEOMS, ids=lambda g: f"{g['shape']}x{g['nv']}")
def test_dot_test(cuda, gp):
    """<Ax, y> = <x, A^T y>.  Nonnegative inputs (no cancellation in the
    float32 outputs) to 1e-6; signed Gaussian inputs to the reference's own
    1e-5 (test_xray_2d.py:85), where float32 output rounding alone is of
    order sqrt(n) ulp."""
    H, _ = _op(gp)
    gen = torch.Generator().manual_seed(3)
    x = torch.rand(H.input_shape, generator=gen)
    y = torch.rand(H.output_shape, generator=gen)
    assert linop.valid_adjoint(H, H.T, eps=None, x=x, y=y) < 1e-6
    assert linop.valid_adjoint(H, H.T, eps=None, seed=3) < 1e-5


def test_golden_fixture(cuda):
    z = np.load(GOLDEN / "oracle_small.npz")
    H = linop.XRayTransform2D(z["p2_img"].shape, z["p2_angles"])
    y = H(torch.from_numpy(z["p2_img"]).to(cuda)).cpu().numpy()
    assert ctref.rel_l2(y, z["p2_sino64"]) <= 1e-5
    b = H.T(torch.from_numpy(z["p2_sino_in"]).to(cuda)).cpu().numpy()
    assert ctref.rel_l2(b, z["p2_back64"]) <= 1e-5


def test_angle0_rows_exact(cuda):
    rng = np.random.default_rng(1)
    im = rng.integers(0, 9, size=(40, 40)).astype(np.float32)
    H = linop.XRayTransform2D(im.shape, np.array([0.0]), dx=1.0, det_count=40)
    y = H(torch.from_numpy(im).to(cuda)).cpu().numpy()
    np.testing.assert_array_equal(y[0], im.sum(axis=1))


def test_batch_and_determinism(cuda):
    H, g = _op(dict(shape=(48, 48), nv=20))
    rng = np.random.default_rng(9)
    xb = torch.from_numpy(rng.random((3, 48, 48)).astype(np.float32)).to(cuda)
    yb = H.project(xb)
    for k in range(3):
        yk = H(xb[k].contiguous())
        assert torch.equal(yb[k], yk)
    assert torch.equal(H.project(xb), yb)  # bitwise reproducible
    bb = H.back_project(yb)
    assert torch.equal(H.back_project(yb), bb)
    for k in range(3):
        assert torch.equal(bb[k], H.T(yb[k].contiguous()))


def test_c1_full_size(cuda):
    """256x256, 180 views, 363 bins: parity against the float64 oracle."""
    from scico_gb300 import workloads

    c = workloads.C1
    x = c.phantom()
    H = linop.XRayTransform2D((c.n, c.n), c.angles)
    assert H.output_shape == (180, 363)
    g = ctref.xray2d_defaults((c.n, c.n), c.angles)
    y = H(torch.from_numpy(x).to(cuda)).cpu().numpy()
    y64 = ctref.xray2d_project(x, g, np.float64)
    assert ctref.rel_l2(y, y64) <= 1e-5
    b = H.T(torch.from_numpy(y64.astype(np.float32)).to(cuda)).cpu().numpy()
    assert ctref.rel_l2(b, ctref.xray2d_back_project(y64.astype(np.float32), g, np.float64)) <= 1e-5


def test_c2_properties(cuda):
    """512x512 / 360 / 725: mass conservation per view, dot test, linearity."""
    from scico_gb300 import workloads

    c = workloads.C2
    H = linop.XRayTransform2D((c.n, c.n), c.angles, det_count=c.det_count)
    x = torch.from_numpy(c.phantom()).to(cuda)
    y = H(x)
    mass = float(x.double().sum())
    np.testing.assert_allclose(y.double().sum(dim=1).cpu().numpy(), mass, rtol=2e-6)
    assert linop.valid_adjoint(H, H.T, eps=None, seed=4) < 1e-6
    x2 = torch.rand_like(x)
    lhs = H(2.0 * x + x2)
    rhs = 2.0 * y + H(x2)
    assert float((lhs - rhs).norm() / rhs.norm()) < 1e-6


def test_workspace_errors(cuda):
    H, _ = _op(dict(shape=(32, 32), nv=8))
    g = H.geometry()
    x = torch.zeros((32, 32), device=cuda)
    y = torch.zeros(H.output_shape, device=cuda)
    lib = _lib.load()
    st = lib.ct_proj2d_fwd(ctypes.addressof(g), x.data_ptr(), y.data_ptr(), 1, None, 0,
                           _device.stream())
    assert st == _lib.CT_ERR_WORKSPACE
