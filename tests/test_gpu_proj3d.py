"""3D projector on the GPU (through the C ABI) against the oracle.

The oracle is the float32 restatement: the reference's weight model is
discontinuous where left = Px - 0.25 is an exact integer (to_next =
ceil(left) - left drops from 0.5 to 0 and the voxel's mass moves one detector
bin), so float64 weights are not a valid stand-in -- they move different
voxels.  The GPU weights are bit-identical to the float32 restatement's;
only the summation order differs.

Tolerances: rel l2 <= 1e-5 per application; dot test <Ax, y> = <x, A^T y> to
1e-6 relative for nonnegative inputs and to the reference's 1e-5
(test_xray_3d.py:25) for signed ones.  The AXIS0 and GENERAL kernels compute
the same operator; on AXIS0 geometries both are run and must agree to 1e-6.
"""

import ctypes

import numpy as np
import pytest
import torch

from oracle import ctref
from scico_gb300 import _device, _lib, linop

pytestmark = pytest.mark.gpu

X3 = linop.XRayTransform3D

GEOMS = [
    # rotation about axis 0 (AXIS0 kernels)
    dict(shape=(16, 16, 16), det=(16, 23), seq="X", nv=9, kind="axis0"),
    dict(shape=(16, 20, 24), det=(20, 30), seq="X", nv=7, kind="axis0"),  # row offset 2
    dict(shape=(40, 48, 72), det=(40, 90), seq="X", nv=11, kind="axis0"),  # 2 slice groups, 6 tiles
    dict(shape=(8, 64, 64), det=(8, 40), seq="X", nv=13, kind="axis0"),  # narrow detector
    dict(shape=(33, 35, 37), det=(33, 51), seq="X", nv=10, kind="axis0"),  # odd sizes
    # GENERAL kernels
    dict(shape=(16, 16, 16), det=(11, 11), seq="X", nv=3, kind="general"),  # test_xray_3d.py:9-26
    dict(shape=(12, 14, 16), det=(20, 22), seq="XYZ", nv=5, kind="general"),
    dict(shape=(8, 10, 12), det=(16, 16), seq="X", nv=4, vs=[2.0, 1.0, 1.0], kind="general"),
    dict(shape=(10, 9, 11), det=(12, 14), seq="Y", nv=6, ds=[1.3, 0.8], kind="general"),
    dict(shape=(14, 14, 10), det=(17, 21), seq="zyx", nv=4, kind="general"),
]


def _angles(gp):
    n = len(gp["seq"])
    if n == 1:
        return np.linspace(0, np.pi, gp["nv"], endpoint=False)[:, None]
    return np.random.default_rng(gp["nv"]).uniform(0, np.pi, (gp["nv"], n))


def _op(gp):
    M = X3.matrices_from_euler_angles(gp["shape"], gp["det"], gp["seq"], _angles(gp),
                                      voxel_spacing=gp.get("vs"), det_spacing=gp.get("ds"))
    return X3(gp["shape"], M, gp["det"]), M.astype(np.float32)


def _ids(g):
    return f"{g['kind']}-{g['shape']}-{g['seq']}{g['nv']}"


def _general_twin(H):
    """The same operator forced onto the GENERAL kernels."""
    g = H.geometry()
    t = _lib.Geom3D()
    t.shape[:] = list(g.shape)
    t.det_shape[:] = list(g.det_shape)
    t.n_views, t.kind, t.row_offset = g.n_views, _lib.CT_PROJ3D_GENERAL, 0
    t.views, t.order = g.views, g.order
    return t


def _call(name, g, src, out_shape, dev):
    out = torch.empty(out_shape, device=dev)
    fwd = _lib.c_size_t(0)
    adj = _lib.c_size_t(0)
    _lib.call("ct_proj3d_workspace", ctypes.addressof(g), 1, ctypes.addressof(fwd), ctypes.addressof(adj))
    ws = _device.workspace(max(fwd.value, adj.value))
    _lib.call(name, ctypes.addressof(g), src.data_ptr(), out.data_ptr(), 1, ws.data_ptr(), ws.numel(),
              torch.cuda.current_stream().cuda_stream)
    return out


@pytest.mark.parametrize("gp", GEOMS, ids=_ids)
def test_fwd_adj_vs_oracle(cuda, gp):
    H, M = _op(gp)
    assert H.kind == gp["kind"]
    rng = np.random.default_rng(7)
    x = rng.random(gp["shape"]).astype(np.float32)
    y = H(torch.from_numpy(x).to(cuda)).cpu().numpy()
    assert ctref.rel_l2(y, ctref.xray3d_project(x, M, gp["det"], np.float32)) <= 1e-5
    ys = rng.standard_normal(H.output_shape).astype(np.float32)
    b = H.T(torch.from_numpy(ys).to(cuda)).cpu().numpy()
    assert ctref.rel_l2(b, ctref.xray3d_back_project(ys, M, gp["shape"], np.float32)) <= 1e-5


@pytest.mark.parametrize("gp", GEOMS, ids=_ids)
def test_dot_test(cuda, gp):
    H, _ = _op(gp)
    gen = torch.Generator().manual_seed(5)
    x = torch.rand(H.input_shape, generator=gen)
    y = torch.rand(H.output_shape, generator=gen)
    assert linop.valid_adjoint(H, H.T, eps=None, x=x, y=y) < 1e-6
    assert linop.valid_adjoint(H, H.T, eps=None, seed=5) < 1e-5


@pytest.mark.parametrize("gp", [g for g in GEOMS if g["kind"] == "axis0"], ids=_ids)
def test_axis0_matches_general_kernels(cuda, gp):
    H, _ = _op(gp)
    t = _general_twin(H)
    x = torch.rand(H.input_shape, generator=torch.Generator().manual_seed(2)).to(cuda)
    y = H(x)
    y_gen = _call("ct_proj3d_fwd", t, x, H.output_shape, cuda)
    assert ctref.rel_l2(y.cpu().numpy(), y_gen.cpu().numpy()) <= 1e-6
    b = H.T(y)
    b_gen = _call("ct_proj3d_adj", t, y, H.input_shape, cuda)
    assert ctref.rel_l2(b.cpu().numpy(), b_gen.cpu().numpy()) <= 1e-6


@pytest.mark.parametrize("case", [0, 1])
def test_scaling_kat(cuda, case):
    """scico/test/linop/xray/test_xray_3d.py:29-60 (test_scaling), on the GPU."""
    import json
    from pathlib import Path

    kat = json.loads((Path(__file__).resolve().parent / "golden" / "reference_kat.json").read_text())
    c = kat["xray3d_scaling"]["cases"][case]
    x = np.zeros((4, 4, 1), np.float32)
    x[1:3, 1:3, 0] = 1.0
    M = X3.matrices_from_euler_angles(x.shape, x.shape[:2], "X", [[0.0]], voxel_spacing=c["voxel_spacing"])
    H = X3(x.shape, M, x.shape[:2])
    np.testing.assert_allclose(H(torch.from_numpy(x).to(cuda)).cpu().numpy(), np.asarray(c["truth"]))


@pytest.mark.parametrize("case", [0, 1, 2])
def test_reference_code_vectors(cuda, case):
    """The GPU 3D projector against the reference's own _project /
    _back_project executed under a float32 jax.numpy stand-in
    (tests/golden/make_xray3d_reference.py; the oracle reproduces those
    vectors bit for bit): rotation about axis 0 (AXIS0 kernels), the
    reference's tilted "XY" example geometry and random matrices (GENERAL
    kernels), rel l2 <= 1e-5."""
    from pathlib import Path

    z = np.load(Path(__file__).resolve().parent / "golden" / "xray3d_reference_code.npz")
    p = f"c{case}_"
    shape = tuple(int(v) for v in z[p + "shape"])
    det = tuple(int(v) for v in z[p + "det"])
    H = X3(shape, z[p + "matrices"], det)
    assert H.kind == ("axis0" if case == 0 else "general")
    y = H(torch.from_numpy(z[p + "volume"]).to(cuda)).cpu().numpy()
    b = H.T(torch.from_numpy(z[p + "proj_in"]).to(cuda)).cpu().numpy()
    assert ctref.rel_l2(y, z[p + "project"]) <= 1e-5
    assert ctref.rel_l2(b, z[p + "back_project"]) <= 1e-5


def test_batch_and_determinism(cuda):
    gp = GEOMS[2]
    H, _ = _op(gp)
    xs = torch.rand((2,) + H.input_shape, generator=torch.Generator().manual_seed(4)).to(cuda)
    yb = H.project(xs)  # __call__ takes the operator's own shape only, as scico's
    for k in range(2):
        assert torch.equal(yb[k], H(xs[k].contiguous()))
    assert torch.equal(H(xs[0].contiguous()), H(xs[0].contiguous()))
    bb = H.back_project(yb)
    assert torch.equal(bb[1], H.T(yb[1].contiguous()))
    assert torch.equal(H.T(yb[0].contiguous()), H.T(yb[0].contiguous()))


def test_axis0_medium_vs_oracle(cuda):
    """40 x 96 x 80 volume, 24 views: several tiles, slice groups and
    view chunks of the AXIS0 kernels."""
    shape, det = (40, 96, 80), (40, 126)
    M = X3.matrices_from_euler_angles(shape, det, "X", np.linspace(0, np.pi, 24, endpoint=False)[:, None])
    H = X3(shape, M, det)
    assert H.kind == "axis0"
    x = np.random.default_rng(3).random(shape).astype(np.float32)
    y = H(torch.from_numpy(x).to(cuda)).cpu().numpy()
    M32 = M.astype(np.float32)
    assert ctref.rel_l2(y, ctref.xray3d_project(x, M32, det, np.float32)) <= 1e-5
    b = H.T(torch.from_numpy(y).to(cuda)).cpu().numpy()
    assert ctref.rel_l2(b, ctref.xray3d_back_project(y, M32, shape, np.float32)) <= 1e-5


def test_c5_size_properties(cuda):
    """256^3 volume, 360 views about axis 0, 256 x 363 detector: the 3D
    workload's full size.  Size-independent checks: the dot test, agreement
    of the AXIS0 and GENERAL kernels on a view subset, mass conservation
    (every detector row of every view sums to its slice's mass: the two taps
    of a voxel weigh 2t + 2(0.5 - t) = 1 and the 363 columns hold the whole
    shadow), and determinism."""
    shape, det, nv = (256, 256, 256), (256, 363), 360
    M = X3.matrices_from_euler_angles(shape, det, "X", np.linspace(0, np.pi, nv, endpoint=False)[:, None])
    H = X3(shape, M, det)
    assert H.kind == "axis0"
    x = torch.rand(shape, generator=torch.Generator().manual_seed(6)).to(cuda)
    y = H(x)
    assert torch.equal(y, H(x))
    # mass: each voxel's two taps sum to 2*t + 2*(0.5 - t) = 1 when both land
    # on the detector (363 bins cover the 256*sqrt2 + 2 wide shadow)
    mass = x.double().sum(dim=(1, 2))
    rows = y.double().sum(dim=2)
    assert torch.allclose(rows, mass[None, :].expand_as(rows), rtol=1e-5, atol=0)
    gen = torch.Generator().manual_seed(8)
    yr = torch.rand(H.output_shape, generator=gen).to(cuda)
    b = H.T(yr)
    lhs = torch.sum(y.double() * yr.double())
    rhs = torch.sum(x.double() * b.double())
    assert abs(lhs - rhs) / abs(lhs) < 1e-6
    # GENERAL kernels on 8 of the views
    sub = slice(0, nv, 45)
    Hs = X3(shape, M[sub], det)
    t = _general_twin(Hs)
    ys = _call("ct_proj3d_fwd", t, x, Hs.output_shape, cuda)
    assert ctref.rel_l2(y[sub].cpu().numpy(), ys.cpu().numpy()) <= 1e-6


def test_c5_vs_oracle(cuda):
    """The 3D workload at full size (256^3, 360 views about axis 0, 256 x 363
    detector): forward of the benchmark's 30-ellipsoid phantom and adjoint of
    a random projection set, each against the C/OpenMP float32 restatement
    (rel l2 <= 1e-5; bit-identical weights, different summation order)."""
    from oracle import ctref_c
    from scico_gb300 import workloads

    c = workloads.C5
    M = c.matrices()
    H = X3(c.shape, M, c.det_shape)
    assert H.kind == "axis0"
    G = ctref_c.Geometry3D(c.shape, np.asarray(M, np.float32), c.det_shape)
    ctref_c.set_threads(ctref_c.default_threads())
    x = c.phantom()
    y = H(torch.from_numpy(x).to(cuda)).cpu().numpy()
    assert ctref.rel_l2(y, G.project(x)) <= 1e-5
    yr = np.random.default_rng(9).random(H.output_shape, dtype=np.float32)
    b = H.T(torch.from_numpy(yr).to(cuda)).cpu().numpy()
    assert ctref.rel_l2(b, G.back_project(yr)) <= 1e-5


def test_workspace_errors(cuda):
    H, _ = _op(GEOMS[0])
    g = H.geometry()
    x = torch.zeros(H.input_shape, device=cuda)
    y = torch.empty(H.output_shape, device=cuda)
    fwd, _ = H.workspace_bytes()
    assert fwd > 0
    with pytest.raises(_lib.CtError, match="need"):
        _lib.call("ct_proj3d_fwd", ctypes.addressof(g), x.data_ptr(), y.data_ptr(), 1, None, 0,
                  torch.cuda.current_stream().cuda_stream)
    assert _lib.load().ct_proj3d_errflag() == 0
