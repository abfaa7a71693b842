"""The C ABI library without a GPU: it loads, exports every symbol the
header declares, computes the host-side geometry table exactly like the
oracle, and rejects bad arguments with a status (no CUDA call made)."""

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from oracle import ctref
from scico_gb300 import _lib

HEADER = Path(__file__).resolve().parent.parent / "include" / "ctgpu.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ct_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol(ctlib):
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(ctlib, n)]
    assert not missing, missing
    # the ctypes binding declares a signature for every header function
    assert set(names) <= set(_lib.exported_symbols()), set(names) - set(_lib.exported_symbols())


def test_wait_poll_limit_setting(ctlib):
    """The strip-copy wait's poll limit is a host-side setting (no device
    needed): default 2^24, any value settable, restored afterwards."""
    old = ctlib.ct_wait_poll_limit()
    assert old == 1 << 24
    try:
        ctlib.ct_set_wait_poll_limit(5)
        assert ctlib.ct_wait_poll_limit() == 5
    finally:
        ctlib.ct_set_wait_poll_limit(old)
    assert ctlib.ct_wait_poll_limit() == old


def test_version_and_status(ctlib):
    assert b"sm_103a" in ctlib.ct_version()
    assert ctlib.ct_status_string(0) == b"ok"
    assert ctlib.ct_status_string(_lib.CT_ERR_WORKSPACE).startswith(b"workspace")


@pytest.mark.parametrize(
    "shape,nv,dx,det",
    [((256, 256), 180, None, None), ((512, 512), 360, None, 725), ((12, 13), 10, None, None),
     ((16, 16), 3, 1 / np.sqrt(2), 11), ((33, 20), 17, 0.5, 40), ((9, 9), 4, 1.0, 9)],
)
def test_view_table_matches_oracle(ctlib, shape, nv, dx, det):
    ang = np.linspace(0, np.pi, nv, endpoint=False)
    g = ctref.xray2d_defaults(shape, ang, dx=dx, det_count=det)
    Pxmin, Pd0, Pd1, width = ctref.xray2d_view_params(g, np.float32)
    table = np.zeros((nv, 8), dtype=np.float32)
    mw = ctypes.c_float()
    a32 = ang.astype(np.float32)
    _lib.call("ct_proj2d_views", a32.ctypes.data, nv, np.float32(g["x0"][0]), np.float32(g["x0"][1]),
              np.float32(g["dx"][0]), np.float32(g["dx"][1]), np.float32(g["y0"]), table.ctypes.data,
              ctypes.addressof(mw))
    np.testing.assert_array_equal(table[:, 0], Pxmin)
    np.testing.assert_array_equal(table[:, 1], Pd0)
    np.testing.assert_array_equal(table[:, 2], Pd1)
    np.testing.assert_array_equal(table[:, 3], width)
    assert mw.value == pytest.approx(float(np.max(np.maximum(np.abs(Pd0 + Pd1), np.abs(Pd0 - Pd1)))))


def test_errors_without_device(ctlib):
    g = _lib.Geom2D(0, 4, 3, 5, 0, 1.0)
    st = ctlib.ct_proj2d_fwd(ctypes.addressof(g), None, None, 1, None, 0, None)
    assert st == _lib.CT_ERR_SHAPE
    assert b"bad geometry" in ctlib.ct_last_error()
    assert ctlib.ct_proj2d_fwd(None, None, None, 1, None, 0, None) == _lib.CT_ERR_INVALID_ARG
    with pytest.raises(ValueError):
        _lib.call("ct_proj2d_workspace", ctypes.addressof(g), 1, None, None)
    d = _lib.FdDesc(2, (_lib.c_int32 * 3)(4, 5, 0), 2, (_lib.c_int32 * 3)(0, 1, 0), 0, -1, 1)
    assert ctlib.ct_fd_fwd(ctypes.addressof(d), None, None, 1, None) == _lib.CT_ERR_INVALID_ARG
    assert b"circular" in ctlib.ct_last_error()
    assert ctlib.ct_l21_prox(None, None, 2, 10, 0.1, None) == _lib.CT_ERR_INVALID_ARG
    assert ctlib.ct_dot(1, 1, 10, 1, None, 0, None) == _lib.CT_ERR_WORKSPACE


@pytest.mark.parametrize(
    "shape,axes,pre,app,circ,count",
    [((4, 5), (0, 1), -1, 0, 0, 40), ((4, 5), (0, 1), -1, -1, 0, 15 + 16), ((4, 5), (1,), 1, 1, 0, 24),
     ((3, 4, 5), (0, 1, 2), -1, -1, 1, 180), ((7,), (0,), 0, -1, 0, 7)],
)
def test_fd_out_count(ctlib, shape, axes, pre, app, circ, count):
    d = _lib.FdDesc(len(shape), (_lib.c_int32 * 3)(*(list(shape) + [0] * (3 - len(shape)))), len(axes),
                    (_lib.c_int32 * 3)(*(list(axes) + [0] * (3 - len(axes)))), pre, app, circ)
    n = ctypes.c_int64()
    _lib.call("ct_fd_out_count", ctypes.addressof(d), ctypes.addressof(n))
    assert n.value == count


def test_admm_workspace_query(ctlib):
    g = _lib.Geom2D(512, 512, 360, 725, 256, 1.0)
    d = _lib.AdmmTvDesc(g, 100, 10, 1e-4, 0.0, 0.005, 0.0, 2.0, 0.5, 1.0, 1)
    n = ctypes.c_size_t()
    _lib.call("ct_admm_tv_workspace", ctypes.addressof(d), ctypes.addressof(n))
    assert 512 * 512 * 4 * 10 < n.value < 2**31
