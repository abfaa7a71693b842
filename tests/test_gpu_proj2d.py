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


@pytest.mark.parametrize("shape", [(64, 96), (70, 130), (37, 300)])
def test_forward_staging_paths_identical(cuda, shape):
    """The forward stages its strip tiles by tensor-map loads when the image
    rows are 16-B strided and the image 16-B aligned, by plain loads into
    the same layout otherwise: both give the same bits (an image 4 bytes
    past an aligned address takes the plain path)."""
    H, g = _op(dict(shape=shape, nv=23))
    rng = np.random.default_rng(4)
    x = torch.from_numpy(rng.random(shape).astype(np.float32)).to(cuda)
    buf = torch.zeros(x.numel() + 4, device=cuda)
    xs = buf[1:1 + x.numel()].view(shape)
    xs.copy_(x)
    assert xs.data_ptr() % 16 == 4
    assert torch.equal(H(xs), H(x))


def test_reference_code_vectors(cuda):
    """The GPU projector against the reference's own _project / _back_project
    executed under a float32 jax.numpy stand-in
    (tests/golden/make_xray2d_reference.py; the oracle reproduces those
    vectors bit for bit): rel l2 <= 1e-5 on five geometries."""
    z = np.load(GOLDEN / "xray2d_reference_code.npz")
    for k in range(len([n for n in z.files if n.endswith("_image")])):
        p = f"c{k}_"
        shape = tuple(int(v) for v in z[p + "shape"])
        H = linop.XRayTransform2D(shape, z[p + "angles"], dx=tuple(float(v) for v in z[p + "dx"]),
                                  det_count=int(z[p + "det"]))
        y = H(torch.from_numpy(z[p + "image"]).to(cuda)).cpu().numpy()
        b = H.T(torch.from_numpy(z[p + "sino_in"]).to(cuda)).cpu().numpy()
        assert ctref.rel_l2(y, z[p + "project"]) <= 1e-5, k
        assert ctref.rel_l2(b, z[p + "back_project"]) <= 1e-5, k


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


def test_c2_vs_oracle(cuda):
    """512x512 / 360 / 725 (the benchmark geometry) at full size: forward of
    the benchmark phantom and of a random image, adjoint of the phantom's
    sinogram, each against the float64 oracle and against the float32 C
    restatement of the reference's arithmetic (rel l2 <= 1e-5); adjoint of a
    white-noise signed sinogram against the float32 restatement.  White noise
    is not compared with float64 weights: where float32 and float64 Px fall
    on different sides of an integer, a pixel reads a neighbouring bin, and
    white-noise neighbours are unrelated values (3.6e-5 at this size); the
    float32 restatement uses the reference's own weights."""
    from oracle import ctref_c
    from scico_gb300 import workloads

    c = workloads.C2
    H = linop.XRayTransform2D((c.n, c.n), c.angles, det_count=c.det_count)
    g = ctref.xray2d_defaults((c.n, c.n), c.angles, det_count=c.det_count)
    G = ctref_c.Geometry((c.n, c.n), c.angles, det_count=c.det_count)
    ctref_c.set_threads(ctref_c.default_threads())
    rng = np.random.default_rng(12)
    for x in (c.phantom(), rng.random((c.n, c.n)).astype(np.float32)):
        y = H(torch.from_numpy(x).to(cuda)).cpu().numpy()
        assert ctref.rel_l2(y, ctref.xray2d_project(x, g, np.float64)) <= 1e-5
        assert ctref.rel_l2(y, G.project(x)) <= 1e-5
    yp = G.project(c.phantom())
    b = H.adj(torch.from_numpy(yp).to(cuda)).cpu().numpy()
    assert ctref.rel_l2(b, ctref.xray2d_back_project(yp, g, np.float64)) <= 1e-5
    assert ctref.rel_l2(b, G.back_project(yp)) <= 1e-5
    ys = rng.standard_normal(H.output_shape).astype(np.float32)
    b = H.adj(torch.from_numpy(ys).to(cuda)).cpu().numpy()
    assert ctref.rel_l2(b, G.back_project(ys)) <= 1e-5


def test_workspace_errors(cuda):
    H, _ = _op(dict(shape=(32, 32), nv=8))
    g = H.geometry()
    x = torch.zeros((32, 32), device=cuda)
    y = torch.zeros(H.output_shape, device=cuda)
    lib = _lib.load()
    st = lib.ct_proj2d_fwd(ctypes.addressof(g), x.data_ptr(), y.data_ptr(), 1, None, 0,
                           _device.stream())
    assert st == _lib.CT_ERR_WORKSPACE


def _edge_op(shape, nv, **kw):
    ang = np.linspace(0, np.pi, nv, endpoint=False)
    import warnings

    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        H = linop.XRayTransform2D(shape, ang, **kw)
    return H, ctref.xray2d_defaults(shape, ang, **kw)


@pytest.mark.parametrize("case", [
    dict(shape=(1, 1), nv=1, det_count=3),                 # one pixel, one view
    dict(shape=(8, 600), nv=7),                            # three strip chunks, a partial tile row
    dict(shape=(20, 20), nv=9, dx=2.0, det_count=60),      # pixels 2.8 bins wide: long spans, general walk
], ids=["1x1", "8x600", "dx2"])
def test_edge_geometries_vs_oracle(cuda, case):
    """Against the oracle with the reference's float32 arithmetic to 1e-5.
    Against float64 only where the weight model is continuous (projected
    pixels at most one bin wide: wider ones jump from weight 0 to 1/width as
    Px crosses an integer, so float32 and float64 Px disagree by whole
    pixels), to 1e-4: float32 Px is rounded to ~|Px| 6e-8 bins."""
    case = dict(case)
    shape, nv = case.pop("shape"), case.pop("nv")
    H, g = _edge_op(shape, nv, **case)
    rng = np.random.default_rng(5)
    x = rng.random(shape).astype(np.float32)
    y = rng.random(H.output_shape).astype(np.float32)
    ax = H.project(torch.from_numpy(x).to(cuda)).cpu().numpy()
    aty = H.back_project(torch.from_numpy(y).to(cuda)).cpu().numpy()
    assert ctref.rel_l2(ax, ctref.xray2d_project(x, g, np.float32)) <= 1e-5
    assert ctref.rel_l2(aty, ctref.xray2d_back_project(y, g, np.float32)) <= 1e-5
    if H.max_width <= 1.0 + 1e-6:
        assert ctref.rel_l2(ax, ctref.xray2d_project(x, g, np.float64)) <= 1e-4
        assert ctref.rel_l2(aty, ctref.xray2d_back_project(y, g, np.float64)) <= 1e-4
    lhs, rhs = float((ax.astype(np.float64) * y).sum()), float((x.astype(np.float64) * aty).sum())
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)


def test_far_detector_offset_general_floor(cuda):
    """|Px| near 3e6 (beyond the fast floor's 2^21): every tile takes the
    general floor path.  Float32 Px resolves only 1/4 bin there, so the check
    is against the oracle with the reference's float32 weights."""
    H, g = _edge_op((24, 24), 3, y0=-3_000_000.0, det_count=3_000_040)
    rng = np.random.default_rng(6)
    x = rng.random((24, 24)).astype(np.float32)
    ax = H.project(torch.from_numpy(x).to(cuda)).cpu().numpy()
    ref = ctref.xray2d_project(x, g, np.float32)
    assert np.abs(ref).sum() > 0  # the image lands on the detector
    assert ctref.rel_l2(ax, ref) <= 1e-5
    ys = np.zeros(H.output_shape, np.float32)
    ys[:, 2_999_950:3_000_040] = rng.random((3, 90)).astype(np.float32)
    aty = H.back_project(torch.from_numpy(ys).to(cuda)).cpu().numpy()
    assert ctref.rel_l2(aty, ctref.xray2d_back_project(ys, g, np.float32)) <= 1e-5


def test_too_wide_pixels_rejected(cuda):
    """Projected pixels wider than the forward's partial rows hold (about 4
    bins: dx = 4 gives 5.7) are refused with CT_ERR_UNSUPPORTED, not
    computed wrongly."""
    H, _ = _edge_op((16, 16), 4, dx=4.0, det_count=100)
    with pytest.raises(_lib.CtError, match="too large"):
        H.project(torch.zeros((16, 16), device=cuda))
