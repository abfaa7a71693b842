"""Host side of the 3D projector: geometry classification, the per-view
tables and the argument checks of the C ABI (no device needed)."""

import ctypes

import numpy as np
import pytest

from oracle import ctref
from scico_gb300 import _lib, linop

X3 = linop.XRayTransform3D


def _views(M, shape, det, with_order=True):
    M = np.ascontiguousarray(M, dtype=np.float32)
    nv = len(M)
    views = np.zeros((nv, _lib.CT_VIEW3D_STRIDE), np.float32)
    order = np.zeros((nv, _lib.CT_PROJ3D_ORDER), np.uint16)
    kind, off = ctypes.c_int32(-1), ctypes.c_int32(-7)
    st = _lib.load().ct_proj3d_views(
        M.ctypes.data_as(ctypes.c_void_p), nv, np.asarray(shape, np.int32).ctypes.data_as(ctypes.c_void_p),
        np.asarray(det, np.int32).ctypes.data_as(ctypes.c_void_p), views.ctypes.data_as(ctypes.c_void_p),
        order.ctypes.data_as(ctypes.c_void_p) if with_order else None, ctypes.byref(kind), ctypes.byref(off))
    return st, views, order, kind.value, off.value


def test_matrices_match_oracle():
    rng = np.random.default_rng(0)
    for seq, ang in [("X", np.linspace(0, np.pi, 7, endpoint=False)[:, None]), ("XYZ", rng.uniform(0, 3, (5, 3))),
                     ("zx", rng.uniform(0, 3, (4, 2)))]:
        for vs, ds in [(None, None), ([2.0, 1.0, 1.0], None), (None, [2.0, 1.0]), ([1.0, 0.7, 1.3], [0.9, 1.1])]:
            a = X3.matrices_from_euler_angles((16, 20, 24), (18, 30), seq, ang, voxel_spacing=vs, det_spacing=ds)
            b = ctref.xray3d_matrices_from_euler_angles((16, 20, 24), (18, 30), seq, ang, voxel_spacing=vs,
                                                         det_spacing=ds)
            assert np.array_equal(a.astype(np.float32), b.astype(np.float32))
            assert np.abs(a - b).max() < 1e-13


@pytest.mark.parametrize(
    "shape,det,seq,kind,off",
    [
        ((16, 16, 16), (16, 23), "X", _lib.CT_PROJ3D_AXIS0, 0),
        ((256, 256, 256), (256, 363), "X", _lib.CT_PROJ3D_AXIS0, 0),
        ((16, 20, 24), (20, 30), "X", _lib.CT_PROJ3D_AXIS0, 2),
        ((16, 16, 16), (11, 11), "X", _lib.CT_PROJ3D_GENERAL, 0),  # to_next 0.25: two rows per slice
        ((16, 16, 16), (17, 23), "X", _lib.CT_PROJ3D_GENERAL, 0),
        ((16, 16, 16), (16, 23), "Y", _lib.CT_PROJ3D_GENERAL, 0),
        ((16, 16, 16), (16, 23), "XZ", _lib.CT_PROJ3D_GENERAL, 0),
    ],
)
def test_classification(shape, det, seq, kind, off):
    ang = np.linspace(0.1, np.pi, 6, endpoint=False)[:, None].repeat(len(seq), axis=1)
    M = X3.matrices_from_euler_angles(shape, det, seq, ang)
    st, views, order, k, o = _views(M, shape, det)
    assert st == _lib.CT_OK
    assert (k, o) == (kind, off)
    M32 = M.astype(np.float32)
    assert np.array_equal(views[:, :8], M32.reshape(len(M), 8))
    # entry 8: the axis of the largest ray-direction component
    d = np.cross(M32[:, 0, :3].astype(np.float64), M32[:, 1, :3].astype(np.float64))
    assert np.array_equal(views[:, 8], np.argmax(np.abs(d), axis=1).astype(np.float32))
    if kind == _lib.CT_PROJ3D_AXIS0:
        # the walk order of each view is a permutation of the 16x16 tile,
        # non-decreasing in the tile's detector coordinate
        for v in range(len(M)):
            p = order[v].astype(np.int64)
            assert np.array_equal(np.sort(p), np.arange(_lib.CT_PROJ3D_ORDER))
            key = M32[v, 1, 1].astype(np.float64) * (p // 16) + M32[v, 1, 2].astype(np.float64) * (p % 16)
            assert np.all(np.diff(key) >= 0)
        # AXIS0 also needs the slice -> row map of the oracle's weights
        for v in range(len(M)):
            ul, w00, w10, w01, w11 = ctref.xray3d_calc_weights(shape[:1] + (1, 1), M32[v], det)
            assert np.array_equal(ul[0].ravel(), np.arange(shape[0]) + off)
            assert np.all(w10 == 0) and np.all(w11 == 0)


def test_without_order_table_is_general():
    M = X3.matrices_from_euler_angles((16, 16, 16), (16, 23), "X", [[0.3], [0.7]])
    st, _, _, k, _ = _views(M, (16, 16, 16), (16, 23), with_order=False)
    assert st == _lib.CT_OK and k == _lib.CT_PROJ3D_GENERAL


def test_views_errors():
    M = np.zeros((1, 2, 4), np.float32)
    M[0, 0, 0] = 1.0
    M[0, 1, 0] = 2.0  # rows parallel: the view maps the volume onto a line
    st, *_ = _views(M, (4, 4, 4), (4, 4))
    assert st == _lib.CT_ERR_UNSUPPORTED
    M = X3.matrices_from_euler_angles((4, 4, 4), (4, 4), "X", [[0.2]]).astype(np.float32)
    M[0, 1, 3] = np.nan
    st, *_ = _views(M, (4, 4, 4), (4, 4))
    assert st == _lib.CT_ERR_NONFINITE
    st, *_ = _views(M[:0], (4, 4, 4), (4, 4))
    assert st == _lib.CT_ERR_SHAPE
    st, *_ = _views(X3.matrices_from_euler_angles((4, 4, 4), (4, 4), "X", [[0.2]]), (4, 0, 4), (4, 4))
    assert st == _lib.CT_ERR_SHAPE


def test_operator_errors():
    with pytest.raises(ValueError, match="3D input shape"):
        X3((4, 4), np.zeros((1, 2, 4)), (4, 4))
    with pytest.raises(ValueError, match=r"\(num_views, 2, 4\)"):
        X3((4, 4, 4), np.zeros((1, 3, 4)), (4, 4))
    with pytest.raises(ValueError, match="det_shape"):
        X3((4, 4, 4), X3.matrices_from_euler_angles((4, 4, 4), (4, 4), "X", [[0.1]]), (4,))
    H = X3((6, 8, 10), X3.matrices_from_euler_angles((6, 8, 10), (6, 14), "X", [[0.1], [0.5]]), (6, 14))
    assert H.kind == "axis0" and H.output_shape == (2, 6, 14) and H.input_shape == (6, 8, 10)


def test_workspace_query_and_checks():
    H = X3((40, 48, 72), X3.matrices_from_euler_angles((40, 48, 72), (40, 90), "X", [[0.1], [0.5], [1.0]]),
           (40, 90))
    g = _lib.Geom3D()
    g.shape[:] = [40, 48, 72]
    g.det_shape[:] = [40, 90]
    g.n_views, g.kind, g.row_offset = 3, _lib.CT_PROJ3D_AXIS0, 0
    g.views = 1  # never dereferenced by the query
    g.order = 1
    fwd, adj = ctypes.c_size_t(0), ctypes.c_size_t(0)
    lib = _lib.load()
    assert lib.ct_proj3d_workspace(ctypes.byref(g), 1, ctypes.byref(fwd), ctypes.byref(adj)) == _lib.CT_OK
    # [groups][views][cols][slices padded to 32] float32
    assert fwd.value >= 3 * 90 * 64 * 4 and fwd.value % (3 * 90 * 64 * 4) == 0  # slices padded to 64
    g.order = None
    assert lib.ct_proj3d_workspace(ctypes.byref(g), 1, ctypes.byref(fwd), ctypes.byref(adj)) == \
        _lib.CT_ERR_INVALID_ARG
    g.order, g.kind = 1, 5
    assert lib.ct_proj3d_workspace(ctypes.byref(g), 1, ctypes.byref(fwd), ctypes.byref(adj)) == \
        _lib.CT_ERR_INVALID_ARG
    g.kind, g.n_views = _lib.CT_PROJ3D_GENERAL, 0
    assert lib.ct_proj3d_workspace(ctypes.byref(g), 1, ctypes.byref(fwd), ctypes.byref(adj)) == _lib.CT_ERR_SHAPE
    assert H.kind == "axis0"
