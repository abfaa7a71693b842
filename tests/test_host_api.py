"""Host-side behaviour of the scico-mirroring API that needs no GPU:
constructor defaults, warnings and argument errors (the reference's own
assertions in scico/test/linop/xray/test_xray_2d.py:14-49 and
scico/test/linop/test_diff.py:34-46)."""

import warnings

import numpy as np
import pytest

from scico_gb300 import linop


def test_xray2d_init_warnings():
    """test_xray_2d.py:14-30."""
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        linop.XRayTransform2D((3, 3), np.array([np.pi / 4]))
        linop.XRayTransform2D((3, 3), np.array([0.0]), dx=np.array([1, 1]))
    with pytest.warns(UserWarning):
        linop.XRayTransform2D((3, 3), np.array([0.1]), dx=np.array([1.1, 1.1]))
    with pytest.warns(UserWarning):
        linop.XRayTransform2D((3, 3), np.array([0.0]), dx=np.array([1.1, 1.1]))


def test_xray2d_shapes():
    """test_xray_2d.py:33-49 (output shapes, default and explicit det_count)."""
    ang = np.linspace(0, np.pi, 10, endpoint=False)
    H = linop.XRayTransform2D((12, 13), ang)
    assert H.output_shape == (10, int(np.ceil(np.linalg.norm((12, 13)))))
    H = linop.XRayTransform2D((12, 13), ang, det_count=14)
    assert H.output_shape == (10, 14)
    assert H.T.output_shape == (12, 13)
    assert H.gram_op.shape == ((12, 13), (12, 13))


def test_fd_errors():
    """test_diff.py:11-13, 34-46."""
    with pytest.raises(ValueError):
        linop.FiniteDifference(input_shape=(3, 4, 5), axes=(0, 3))
    with pytest.raises(TypeError):
        linop.SingleAxisFiniteDifference(input_shape=(3,), axis=2.5)
    with pytest.raises(ValueError):
        linop.SingleAxisFiniteDifference(input_shape=(3,), prepend=0, circular=True)
    with pytest.raises(ValueError):
        linop.SingleAxisFiniteDifference(input_shape=(3,), prepend=2)
    with pytest.raises(ValueError):
        linop.SingleAxisFiniteDifference(input_shape=(3,), append="a")


def test_fd_shapes():
    A = linop.FiniteDifference((4, 5), append=0)
    assert A.output_shape == (2, 4, 5)
    B = linop.FiniteDifference((4, 5))
    assert B.output_shape == ((3, 5), (4, 4))
    C = linop.SingleAxisFiniteDifference((5,), prepend=1, append=1)
    assert C.output_shape == (6,)


def test_operator_shape_errors():
    A = linop.FiniteDifference((4, 5), append=0)
    with pytest.raises(ValueError):
        A(np.zeros((5, 4), dtype=np.float32))
    H = linop.XRayTransform2D((8, 8), np.linspace(0, np.pi, 4, endpoint=False))
    with pytest.raises(ValueError):
        H + A
