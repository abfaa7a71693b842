"""Linear operators of the CT hot path, mirroring scico's interfaces.

* :class:`LinearOperator` -- scico/linop/_linop.py:123-441 (eval/adj/T/H,
  gram, gram_op, +, -, scalar *, /, @, composition) and the shape checks of
  scico/operator/_operator.py:187-225.
* :class:`XRayTransform2D` -- scico/linop/xray/_xray2d.py:29-306.
* :class:`XRayTransform3D` -- scico/linop/xray/_xray3d.py:27-327.
* :class:`FiniteDifference`, :class:`SingleAxisFiniteDifference` --
  scico/linop/_diff.py:25-272 (stacked output as VerticalStack does,
  scico/operator/_stack.py:87-88,126-129).
* :class:`Identity` -- scico/linop/_diag.py:271-305.

Arrays are float32 CUDA tensors (numpy inputs are copied to the device).
Every operator evaluation runs in the ctgpu kernels through the C ABI.
"""

from __future__ import annotations

import math
import warnings
from typing import Callable, Optional, Sequence, Tuple, Union

import numpy as np
import torch

from . import _device, _lib

Shape = Tuple[int, ...]


def _np_dtype(dt) -> np.dtype:
    if isinstance(dt, torch.dtype):
        return np.dtype(str(dt).replace("torch.", ""))
    return np.dtype(dt)


def _shape_of(x) -> tuple:
    if isinstance(x, (tuple, list)):
        return tuple(_shape_of(b) for b in x)
    return tuple(x.shape)


def _dtype_of(x) -> np.dtype:
    if isinstance(x, (tuple, list)):
        return _dtype_of(x[0])
    return _np_dtype(x.dtype)


class LinearOperator:
    """Generic linear operator (scico/linop/_linop.py:123)."""

    def __init__(
        self,
        input_shape,
        output_shape=None,
        eval_fn: Optional[Callable] = None,
        adj_fn: Optional[Callable] = None,
        input_dtype=np.float32,
        output_dtype=None,
        jit: bool = False,
    ):
        self.input_shape = (input_shape,) if isinstance(input_shape, int) else tuple(input_shape)
        self.input_dtype = _np_dtype(input_dtype)
        if eval_fn is not None:
            self._eval = eval_fn
        elif not hasattr(self, "_eval"):
            raise NotImplementedError(
                "Operator is an abstract base class when argument 'eval_fn' is not specified."
            )
        if output_shape is None:
            raise ValueError("output_shape must be given (no shape inference without JAX tracing)")
        self.output_shape = (output_shape,) if isinstance(output_shape, int) else tuple(output_shape)
        self.output_dtype = self.input_dtype if output_dtype is None else _np_dtype(output_dtype)
        self.shape = (self.output_shape, self.input_shape)
        self.input_size = _size(self.input_shape)
        self.output_size = _size(self.output_shape)
        self.matrix_shape = (self.output_size, self.input_size)
        if not hasattr(self, "_adj"):
            self._adj = None
        if callable(adj_fn):
            self._adj = adj_fn
        elif adj_fn is not None:
            raise TypeError(f"Argument 'adj_fn' must be either a Callable or None; got {adj_fn}.")
        self._gram = lambda x: self.adj(self(x))

    # -- evaluation ---------------------------------------------------------
    def __call__(self, x):
        if isinstance(x, LinearOperator):
            return ComposedLinearOperator(self, x)
        if _shape_of(x) != self.input_shape:
            raise ValueError(
                f"Cannot evaluate {type(self)} with input_shape={self.input_shape} "
                f"on array with shape={_shape_of(x)}."
            )
        return self._eval(x)

    def __matmul__(self, other):
        return self(other)

    def adj(self, y):
        if isinstance(y, LinearOperator):
            return ComposedLinearOperator(self.H, y)
        if self._adj is None:
            raise NotImplementedError(f"{type(self)} has no adjoint")
        if self.output_dtype != _dtype_of(y):
            raise ValueError(f"Dtype error: expected {self.output_dtype}, got {_dtype_of(y)}.")
        if self.output_shape != _shape_of(y):
            raise ValueError(
                f"Shapes do not conform: input array with shape {_shape_of(y)} does not match "
                f"LinearOperator output_shape {self.output_shape}."
            )
        return self._adj(y)

    @property
    def T(self) -> "LinearOperator":
        return LinearOperator(
            input_shape=self.output_shape,
            output_shape=self.input_shape,
            eval_fn=self.adj,
            adj_fn=self.__call__,
            input_dtype=self.output_dtype,
            output_dtype=self.input_dtype,
        )

    H = T  # real-valued operators only

    def gram(self, x):
        return self._gram(x)

    @property
    def gram_op(self) -> "LinearOperator":
        return LinearOperator(
            input_shape=self.input_shape,
            output_shape=self.input_shape,
            eval_fn=self.gram,
            adj_fn=self.gram,
            input_dtype=self.input_dtype,
            output_dtype=self.output_dtype,
        )

    # -- algebra (scico/linop/_linop.py:212-258) -----------------------------
    def _check_same(self, other):
        if not isinstance(other, LinearOperator):
            raise TypeError(f"Operation not defined between {type(self)} and {type(other)}.")
        if self.shape != other.shape:
            raise ValueError(f"Shapes {self.shape} and {other.shape} do not match.")

    def __add__(self, other):
        self._check_same(other)
        return LinearOperator(
            self.input_shape,
            self.output_shape,
            eval_fn=lambda x: _add(self(x), other(x)),
            adj_fn=lambda y: _add(self.adj(y), other.adj(y)),
            input_dtype=self.input_dtype,
            output_dtype=self.output_dtype,
        )

    def __sub__(self, other):
        self._check_same(other)
        return LinearOperator(
            self.input_shape,
            self.output_shape,
            eval_fn=lambda x: _add(self(x), _scale(other(x), -1.0)),
            adj_fn=lambda y: _add(self.adj(y), _scale(other.adj(y), -1.0)),
            input_dtype=self.input_dtype,
            output_dtype=self.output_dtype,
        )

    def __mul__(self, other):
        if not np.isscalar(other) and not (isinstance(other, np.ndarray) and other.ndim == 0):
            return NotImplemented
        c = float(other)
        if hasattr(self, "project") and hasattr(self, "back_project"):
            return ScaledProjector(self, c)
        return ScaledLinearOperator(self, c)

    __rmul__ = __mul__

    def __truediv__(self, other):
        if not np.isscalar(other):
            return NotImplemented
        return self.__mul__(1.0 / float(other))

    def __neg__(self):
        return self.__mul__(-1.0)

    def __repr__(self):
        return (
            f"{type(self).__module__}.{type(self).__qualname__}\n"
            f"  input_shape:  {self.input_shape}\n  output_shape: {self.output_shape}\n"
            f"  input_dtype:  {self.input_dtype}\n  output_dtype: {self.output_dtype}\n"
        )


def _size(shape) -> int:
    if len(shape) and isinstance(shape[0], tuple):
        return sum(_size(s) for s in shape)
    return int(np.prod(shape)) if len(shape) else 1


def _add(a, b):
    if isinstance(a, tuple):
        return tuple(_add(u, v) for u, v in zip(a, b))
    return a + b


def _scale(a, c: float):
    if isinstance(a, tuple):
        return tuple(_scale(u, c) for u in a)
    return a * c


class ScaledLinearOperator(LinearOperator):
    """``c * A`` (scico/linop/_linop.py:229-245), keeping ``base`` (A) and
    ``scale`` (c) so that solvers can recognise the operator."""

    def __init__(self, A: LinearOperator, c: float):
        self.base, self.scale = A, float(c)
        super().__init__(A.input_shape, A.output_shape, eval_fn=lambda x: _scale(A(x), self.scale),
                         adj_fn=lambda y: _scale(A.adj(y), self.scale), input_dtype=A.input_dtype,
                         output_dtype=A.output_dtype)

    def __mul__(self, other):
        if not np.isscalar(other) and not (isinstance(other, np.ndarray) and other.ndim == 0):
            return NotImplemented
        return type(self)(self.base, self.scale * float(other))

    __rmul__ = __mul__


class ScaledProjector(ScaledLinearOperator):
    """``c * A`` for a projector ``A``: also keeps A's batched ``project`` /
    ``back_project`` (scaled), so the scaled projector serves the
    differentiable networks as A does (the reference's training scripts
    normalise A by 1 / N)."""

    def project(self, x):
        return self.base.project(x) * self.scale

    def back_project(self, y):
        return self.base.back_project(y) * self.scale


class ComposedLinearOperator(LinearOperator):
    """A @ B (scico/linop/_linop.py:443-497)."""

    def __init__(self, A: LinearOperator, B: LinearOperator, jit: bool = False):
        if not isinstance(A, LinearOperator) or not isinstance(B, LinearOperator):
            raise TypeError("ComposedLinearOperator needs two LinearOperators")
        if A.input_shape != B.output_shape:
            raise ValueError(f"Incompatable LinearOperator shapes {A.shape}, {B.shape}.")
        if A.input_dtype != B.output_dtype:
            raise ValueError(f"Incompatable LinearOperator dtypes {A.input_dtype}, {B.output_dtype}.")
        self.A, self.B = A, B
        super().__init__(
            input_shape=B.input_shape,
            output_shape=A.output_shape,
            input_dtype=B.input_dtype,
            output_dtype=A.output_dtype,
            eval_fn=lambda x: A(B(x)),
            adj_fn=lambda z: B.adj(A.adj(z)),
        )


class Identity(LinearOperator):
    """Identity operator (scico/linop/_diag.py:271-305)."""

    def __init__(self, input_shape, input_dtype=np.float32, **kwargs):
        super().__init__(
            input_shape, input_shape, eval_fn=lambda x: x, adj_fn=lambda x: x, input_dtype=input_dtype
        )
        self.diagonal = 1.0

    @property
    def gram_op(self):
        return self


class VerticalStack(LinearOperator):
    """Operators stacked vertically (scico/linop/_stack.py:24-120,
    scico/operator/_stack.py:87-129): ``A x = (A_0 x, A_1 x, ...)``,
    ``A^T y = sum_k A_k^T y_k`` in block order.  The output is one stacked
    tensor when every block has the same shape and ``collapse_output`` is
    true, else a tuple of blocks (a BlockArray)."""

    def __init__(self, ops: Sequence[LinearOperator], collapse_output: bool = True, jit: bool = False):
        ops = list(ops)
        if not ops:
            raise ValueError("VerticalStack needs at least one operator")
        if any(op.input_shape != ops[0].input_shape for op in ops):
            raise ValueError("all operators must have the same input_shape")
        self.ops = ops
        shapes = [op.output_shape for op in ops]
        self.collapsed = collapse_output and all(sh == shapes[0] for sh in shapes) and not isinstance(
            shapes[0][0] if shapes[0] else None, tuple)
        out_shape = (len(ops),) + tuple(shapes[0]) if self.collapsed else tuple(shapes)

        def ev(x):
            blocks = [op(x) for op in ops]
            return torch.stack(blocks) if self.collapsed else tuple(blocks)

        def ad(y):
            acc = None
            for k, op in enumerate(ops):
                t = op.adj(y[k])
                acc = t if acc is None else _add(acc, t)
            return acc

        super().__init__(input_shape=ops[0].input_shape, output_shape=out_shape, eval_fn=ev, adj_fn=ad,
                         input_dtype=ops[0].input_dtype, output_dtype=ops[0].output_dtype)


def power_iteration(A: LinearOperator, maxiter: int = 100, seed: Optional[int] = None):
    """Largest eigenvalue of a diagonalizable operator by power iteration
    (scico/linop/_util.py:27-76): v normalized random start; per step
    ``Av = A v``, ``mu = <v, Av> / ||v||^2``, ``v = Av / ||Av||``.  Norms and
    inner products in float64.  Returns (mu, v)."""
    gen = torch.Generator().manual_seed(0 if seed is None else int(seed))
    v = _device.to_device(torch.randn(A.input_shape, generator=gen))
    v = v / torch.linalg.vector_norm(v.double()).float()
    mu = 0.0
    for _ in range(maxiter):
        Av = A(v)
        nAv = float(torch.linalg.vector_norm(Av.double()))
        if nAv == 0.0:  # a zero operator
            return 0.0, Av
        mu = float(torch.sum(v.double() * Av.double())) / float(torch.sum(v.double() ** 2))
        v = Av / nAv
    return mu, v


def operator_norm(A: LinearOperator, maxiter: int = 100, seed: Optional[int] = None) -> float:
    """||A||_2 = sqrt(largest eigenvalue of A^H A) by power iteration
    (scico/linop/_util.py:79-110)."""
    mu, _ = power_iteration(A.gram_op, maxiter=maxiter, seed=seed)
    return math.sqrt(max(mu, 0.0))


# ---------------------------------------------------------------------------
# 2D X-ray transform
# ---------------------------------------------------------------------------


class XRayTransform2D(LinearOperator):
    r"""Parallel ray, single axis, 2D X-ray projector.

    Same constructor, defaults and model as scico's XRayTransform2D
    (scico/linop/xray/_xray2d.py:52-136): each pixel projects as a boxcar
    of width ``(max+min)/2`` of its two projected diagonals and splits its
    value between the two detector bins it overlaps.  ``project`` runs
    ``ct_proj2d_fwd`` and ``back_project`` ``ct_proj2d_adj``; the adjoint
    uses the forward's exact weights.

    The per-view float32 geometry table is built once here, on the host,
    with the reference's float32 operation order, and kept on the device.
    """

    def __init__(
        self,
        input_shape: Shape,
        angles,
        x0=None,
        dx=None,
        y0: Optional[float] = None,
        det_count: Optional[int] = None,
        input_device=None,
        output_device=None,
    ):
        self.input_shape = tuple(input_shape)
        if len(self.input_shape) != 2:
            raise ValueError(f"XRayTransform2D needs a 2D input shape, got {self.input_shape}")
        self.angles = np.asarray(angles.cpu() if isinstance(angles, torch.Tensor) else angles)
        if self.angles.ndim != 1 or self.angles.size == 0:
            raise ValueError("angles must be a non-empty 1D array")
        self.nx = tuple(self.input_shape)
        if dx is None:
            dx = 2 * (np.sqrt(2) / 2,)
        if np.isscalar(dx) or np.ndim(dx) == 0:
            dx = 2 * (float(dx),)
        self.dx = tuple(float(v) for v in np.asarray(dx, dtype=np.float64).ravel()[:2])
        if x0 is None:
            x0 = -(np.array(self.nx) * np.array(self.dx)) / 2
        self.x0 = np.asarray(x0, dtype=np.float64)
        if det_count is None:
            det_count = int(np.ceil(np.linalg.norm(self.input_shape)))
        self.det_count = int(det_count)
        self.ny = self.det_count
        self.output_shape = (len(self.angles), self.det_count)
        if y0 is None:
            y0 = -self.ny / 2
        self.y0 = float(y0)
        self.dy = 1.0
        self.fbp_filter = None
        self.fbp_mask = None
        self.input_device = input_device
        self.output_device = output_device

        # per-view table: the float32 arithmetic of _calc_weights (:326-347)
        ang32 = np.ascontiguousarray(self.angles.astype(np.float32))
        nv = ang32.size
        table = np.zeros((nv, _lib.CT_VIEW2D_STRIDE), dtype=np.float32)
        maxw = _lib.c_float(0.0)
        _lib.call(
            "ct_proj2d_views",
            ang32.ctypes.data,
            nv,
            np.float32(self.x0[0]),
            np.float32(self.x0[1]),
            np.float32(self.dx[0]),
            np.float32(self.dx[1]),
            np.float32(self.y0),
            table.ctypes.data,
            _lib.ctypes.addressof(maxw),
        )
        self.view_table = table
        self.max_width = float(maxw.value)
        # XRayTransform2D.__init__ warns when a projected pixel is wider
        # than a detector bin (:96-106).
        if self.max_width > 1:
            warnings.warn(
                f"A projected pixel has width {self.max_width} > 1.0, "
                "which will reduce projector accuracy."
            )
        self._views_dev = None
        self._geom = None

        super().__init__(
            input_shape=self.input_shape,
            input_dtype=np.float32,
            output_shape=self.output_shape,
            output_dtype=np.float32,
            eval_fn=self.project,
            adj_fn=self.back_project,
        )

    # -- device geometry ----------------------------------------------------
    def geometry(self) -> _lib.Geom2D:
        """ct_geom2d for the C ABI (uploads the view table on first use)."""
        dev = _device.require_cuda()
        if self._views_dev is None or self._views_dev.device != dev:
            self._views_dev = torch.from_numpy(self.view_table).to(dev)
            self._geom = _lib.Geom2D(
                self.nx[0], self.nx[1], len(self.angles), self.det_count, self._views_dev.data_ptr(), self.max_width
            )
        return self._geom

    def workspace_bytes(self, batch: int = 1) -> Tuple[int, int]:
        fwd = _lib.c_size_t(0)
        adj = _lib.c_size_t(0)
        g = self.geometry()
        _lib.call("ct_proj2d_workspace", _lib.ctypes.addressof(g), batch,
                  _lib.ctypes.addressof(fwd), _lib.ctypes.addressof(adj))
        return int(fwd.value), int(adj.value)

    def autotune(self, batch: int = 1, reps: int = 10) -> dict:
        """Measure the projector's launch schedules for this geometry and
        ``batch`` (forward views per CTA, adjoint view splits) and record the
        fastest, which every later projection and fused solve on the same
        geometry uses (``ct_proj2d_autotune``).  Runs on the current stream
        and waits for it; not inside a stream capture.  No counterpart in the
        reference.  Returns the chosen schedule and its measured times."""
        g = self.geometry()
        fwd_bytes, adj_bytes = self.workspace_bytes(batch)
        ws = _device.workspace(max(fwd_bytes, adj_bytes, 256))
        img = _device.empty((batch,) + self.input_shape)
        sino = _device.empty((batch,) + self.output_shape)
        img.zero_()
        out = _lib.Proj2dSchedule()
        _lib.call("ct_proj2d_autotune", _lib.ctypes.addressof(g), batch, img.data_ptr(), sino.data_ptr(),
                  ws.data_ptr(), ws.numel(), reps, _device.stream(), _lib.ctypes.addressof(out))
        return self._schedule_dict(out)

    def schedule(self, batch: int = 1) -> dict:
        """The launch schedule projections of this geometry use now (recorded
        by :meth:`autotune`, else the planner's default)."""
        g = self.geometry()
        out = _lib.Proj2dSchedule()
        _lib.call("ct_proj2d_schedule_get", _lib.ctypes.addressof(g), batch, _lib.ctypes.addressof(out))
        return self._schedule_dict(out)

    @staticmethod
    def _schedule_dict(s) -> dict:
        return {"views_per_cta": int(s.views_per_cta), "adj_splits": int(s.adj_splits),
                "fwd_us": float(s.fwd_us), "adj_us": float(s.adj_us), "tuned": bool(s.tuned)}

    # -- operator -----------------------------------------------------------
    def _batched(self, x, core_shape, name):
        t = _device.to_device(x, name=name)
        if tuple(t.shape) == tuple(core_shape):
            return t, 1, False
        if t.ndim == len(core_shape) + 1 and tuple(t.shape[1:]) == tuple(core_shape):
            return t, t.shape[0], True
        raise ValueError(f"{name}: expected shape {tuple(core_shape)} or (batch, *{tuple(core_shape)}), got {tuple(t.shape)}")

    def project(self, im) -> torch.Tensor:
        """X-ray projection, ``H @ im`` (accepts a leading batch axis)."""
        t, batch, has_batch = self._batched(im, self.input_shape, "image")
        g = self.geometry()
        out = _device.empty(((batch,) if has_batch else ()) + self.output_shape)
        fwd_bytes, _ = self.workspace_bytes(batch)
        ws = _device.workspace(fwd_bytes)
        _lib.call("ct_proj2d_fwd", _lib.ctypes.addressof(g), t.data_ptr(), out.data_ptr(), batch,
                  ws.data_ptr(), ws.numel(), _device.stream())
        return out

    def back_project(self, y) -> torch.Tensor:
        """X-ray back projection, ``H.T @ y`` (accepts a leading batch axis)."""
        t, batch, has_batch = self._batched(y, self.output_shape, "sinogram")
        g = self.geometry()
        out = _device.empty(((batch,) if has_batch else ()) + self.input_shape)
        _, adj_bytes = self.workspace_bytes(batch)
        ws = _device.workspace(adj_bytes)
        _lib.call("ct_proj2d_adj", _lib.ctypes.addressof(g), t.data_ptr(), out.data_ptr(), batch,
                  ws.data_ptr(), ws.numel(), _device.stream())
        return out

    def fbp(self, y) -> torch.Tensor:
        r"""Filtered back projection (scico/linop/xray/_xray2d.py:158-197).

        Each sinogram row is ramp filtered (``ct_fbp_filter``, the filter of
        ``_ramp_filter``), the result back projected, multiplied by the mask of
        pixels whose back projection of ones reaches ``num_angles * (1 -
        1e-5)`` (computed once and kept, as the reference keeps
        ``fbp_mask``) and scaled by ``pi * dx[0] * dx[1] / num_angles``.
        Angles are assumed evenly spaced in [0, pi).  Accepts a leading batch
        axis.
        """
        t, batch, has_batch = self._batched(y, self.output_shape, "sinogram")
        nv = self.output_shape[0]
        hy = torch.empty_like(t)
        _lib.call("ct_fbp_filter", t.data_ptr(), hy.data_ptr(), batch * nv, self.det_count, _device.stream())
        if self.fbp_mask is None:
            ones = _device.to_device(torch.ones(self.output_shape))
            self.fbp_mask = self.back_project(ones) >= nv * (1.0 - 1e-5)
        scale = float(np.pi * self.dx[0] * self.dx[1] / nv)
        return scale * self.fbp_mask.to(torch.float32) * self.back_project(hy)


class XRayTransform3D(LinearOperator):
    r"""General-purpose, 3D, parallel ray X-ray projector.

    Same constructor and model as scico's XRayTransform3D
    (scico/linop/xray/_xray3d.py:54-93): one homogeneous (2, 4) projection
    matrix per view maps voxel centres onto the detector, and each voxel
    spreads over a 2x2 detector neighbourhood with the weights of
    ``_calc_weights`` (:206-266).  ``project`` runs ``ct_proj3d_fwd`` and
    ``back_project`` ``ct_proj3d_adj``.

    ``batch_size`` is accepted for signature compatibility; every view is
    computed in one launch.  Geometries that rotate about volume axis 0 with
    each slice on one detector row (``matrices_from_euler_angles(..., "X",
    ...)`` with equal slice and detector-row counts) run the AXIS0 kernels,
    which share each column weight across all slices; all others run the
    GENERAL kernels.  ``kind`` reports which.
    """

    def __init__(
        self,
        input_shape: Shape,
        matrices,
        det_shape: Shape,
        batch_size: int = 8,
        input_dtype=np.float32,
        input_device=None,
        output_device=None,
    ):
        self.input_shape = tuple(int(n) for n in input_shape)
        if len(self.input_shape) != 3:
            raise ValueError(f"XRayTransform3D needs a 3D input shape, got {self.input_shape}")
        m = matrices.cpu().numpy() if isinstance(matrices, torch.Tensor) else np.asarray(matrices)
        # the reference keeps the matrices as float32 (:80)
        self.matrices = np.ascontiguousarray(m, dtype=np.float32)
        if self.matrices.ndim != 3 or self.matrices.shape[1:] != (2, 4) or self.matrices.shape[0] == 0:
            raise ValueError(f"matrices must have shape (num_views, 2, 4), got {self.matrices.shape}")
        self.det_shape = tuple(int(n) for n in det_shape)
        if len(self.det_shape) != 2:
            raise ValueError(f"det_shape must have 2 entries, got {self.det_shape}")
        self.batch_size = batch_size
        self.output_shape = (len(self.matrices), *self.det_shape)
        self.input_device = input_device
        self.output_device = output_device
        nv = len(self.matrices)
        self.view_table = np.zeros((nv, _lib.CT_VIEW3D_STRIDE), dtype=np.float32)
        self.order_table = np.zeros((nv, _lib.CT_PROJ3D_ORDER), dtype=np.uint16)
        shape = np.asarray(self.input_shape, dtype=np.int32)
        det = np.asarray(self.det_shape, dtype=np.int32)
        kind = _lib.c_int32(0)
        row_offset = _lib.c_int32(0)
        _lib.call("ct_proj3d_views", self.matrices.ctypes.data, nv, shape.ctypes.data, det.ctypes.data,
                  self.view_table.ctypes.data, self.order_table.ctypes.data,
                  _lib.ctypes.addressof(kind), _lib.ctypes.addressof(row_offset))
        self.kind = "axis0" if kind.value == _lib.CT_PROJ3D_AXIS0 else "general"
        self._kind = int(kind.value)
        self._row_offset = int(row_offset.value)
        self._dev_tables = None
        self._geom = None
        super().__init__(
            input_shape=self.input_shape,
            input_dtype=np.float32,
            output_shape=self.output_shape,
            output_dtype=np.float32,
            eval_fn=self.project,
            adj_fn=self.back_project,
        )

    def geometry(self) -> _lib.Geom3D:
        """ct_geom3d for the C ABI (uploads the tables on first use)."""
        dev = _device.require_cuda()
        if self._dev_tables is None or self._dev_tables[0].device != dev:
            views = torch.from_numpy(self.view_table).to(dev)
            order = torch.from_numpy(self.order_table.view(np.int16)).to(dev)
            self._dev_tables = (views, order)
            g = _lib.Geom3D()
            g.shape[:] = list(self.input_shape)
            g.det_shape[:] = list(self.det_shape)
            g.n_views = len(self.matrices)
            g.kind = self._kind
            g.row_offset = self._row_offset
            g.views = views.data_ptr()
            g.order = order.data_ptr()
            self._geom = g
        return self._geom

    def workspace_bytes(self, batch: int = 1) -> Tuple[int, int]:
        fwd = _lib.c_size_t(0)
        adj = _lib.c_size_t(0)
        g = self.geometry()
        _lib.call("ct_proj3d_workspace", _lib.ctypes.addressof(g), batch,
                  _lib.ctypes.addressof(fwd), _lib.ctypes.addressof(adj))
        return int(fwd.value), int(adj.value)

    def autotune(self, reps: int = 5) -> dict:
        """Measure the 3D projector's launch schedules for this geometry
        (AXIS0 forward tile groups, adjoint view splits) and record the
        fastest, which every later projection and fused 3D solve on the same
        geometry uses (``ct_proj3d_autotune``).  Runs on the current stream
        and waits for it; not inside a stream capture.  No counterpart in the
        reference.  Returns the chosen schedule and its measured times."""
        g = self.geometry()
        fwd_bytes, adj_bytes = self.workspace_bytes()
        ws = _device.workspace(max(fwd_bytes, adj_bytes, 256))
        vol = _device.empty(self.input_shape)
        proj = _device.empty(self.output_shape)
        vol.zero_()
        out = _lib.Proj3dSchedule()
        _lib.call("ct_proj3d_autotune", _lib.ctypes.addressof(g), vol.data_ptr(), proj.data_ptr(), ws.data_ptr(),
                  ws.numel(), reps, _device.stream(), _lib.ctypes.addressof(out))
        return self._schedule_dict(out)

    def schedule(self) -> dict:
        """The launch schedule projections of this geometry use now (recorded
        by :meth:`autotune`, else the planner's default)."""
        g = self.geometry()
        out = _lib.Proj3dSchedule()
        _lib.call("ct_proj3d_schedule_get", _lib.ctypes.addressof(g), _lib.ctypes.addressof(out))
        return self._schedule_dict(out)

    @staticmethod
    def _schedule_dict(s) -> dict:
        return {"tile_groups": int(s.tile_groups), "adj_splits": int(s.adj_splits), "fwd_us": float(s.fwd_us),
                "adj_us": float(s.adj_us), "tuned": bool(s.tuned)}

    _batched = XRayTransform2D._batched

    def project(self, im) -> torch.Tensor:
        """Compute X-ray projection (accepts a leading batch axis)."""
        t, batch, has_batch = self._batched(im, self.input_shape, "volume")
        g = self.geometry()
        out = _device.empty(((batch,) if has_batch else ()) + self.output_shape)
        fwd_bytes, _ = self.workspace_bytes(batch)
        ws = _device.workspace(fwd_bytes)
        _lib.call("ct_proj3d_fwd", _lib.ctypes.addressof(g), t.data_ptr(), out.data_ptr(), batch,
                  ws.data_ptr(), ws.numel(), _device.stream())
        return out

    def back_project(self, proj) -> torch.Tensor:
        """Compute X-ray back projection (accepts a leading batch axis)."""
        t, batch, has_batch = self._batched(proj, self.output_shape, "projection")
        g = self.geometry()
        out = _device.empty(((batch,) if has_batch else ()) + self.input_shape)
        _, adj_bytes = self.workspace_bytes(batch)
        ws = _device.workspace(adj_bytes)
        _lib.call("ct_proj3d_adj", _lib.ctypes.addressof(g), t.data_ptr(), out.data_ptr(), batch,
                  ws.data_ptr(), ws.numel(), _device.stream())
        return out

    @staticmethod
    def matrices_from_euler_angles(
        input_shape: Shape,
        output_shape: Shape,
        seq: str,
        angles,
        degrees: bool = False,
        voxel_spacing=None,
        det_spacing=None,
    ) -> np.ndarray:
        """(num_views, 2, 4) projection matrices from Euler angles
        (scico/linop/xray/_xray3d.py:268-327): rotate the voxels by the
        given sequence, keep the first two rows, scale by the voxel and
        detector spacings and translate so that the centres line up.
        Computed in float64 like the reference's NumPy code."""
        from scipy.spatial.transform import Rotation

        vox = np.ones(3) if voxel_spacing is None else np.asarray(voxel_spacing, dtype=np.float64)
        inv_det = 1 / (np.ones(2) if det_spacing is None else np.asarray(det_spacing, dtype=np.float64))
        rows = Rotation.from_euler(seq, angles, degrees=degrees).as_matrix()[:, :2, :]
        # column scaling by the voxel spacing first, then row scaling by the
        # inverse detector spacing (the reference's rounding order)
        lin = (rows * vox[None, None, :]) * inv_det[None, :, None]
        centre_in = np.asarray(input_shape, dtype=np.float64) / 2
        centre_out = np.asarray(output_shape, dtype=np.float64) / 2
        proj_centre = lin[..., 0] * centre_in[0] + lin[..., 1] * centre_in[1] + lin[..., 2] * centre_in[2]
        shift = centre_out - proj_centre
        out = np.empty(lin.shape[:2] + (4,))
        out[..., :3] = lin
        out[..., 3] = shift
        return out


# ---------------------------------------------------------------------------
# Finite differences
# ---------------------------------------------------------------------------


def _norm_axes(axes, ndim):
    if axes is None:
        return tuple(range(ndim))
    if isinstance(axes, (int, np.integer)):
        return (int(axes),)
    return tuple(int(a) for a in axes)


class FiniteDifference(LinearOperator):
    """Finite differences along several axes, stacked (scico/linop/_diff.py:25-96).

    When every axis gives the same output shape the result is one
    ``(naxes, *shape)`` array (VerticalStack's collapsed output); otherwise a
    tuple of per-axis arrays (a BlockArray).
    """

    def __init__(
        self,
        input_shape: Shape,
        input_dtype=np.float32,
        axes=None,
        prepend=None,
        append=None,
        circular: bool = False,
        jit: bool = True,
        **kwargs,
    ):
        input_shape = tuple(input_shape)
        if _np_dtype(input_dtype) != np.float32:
            raise ValueError("only float32 finite differences are implemented on the device")
        ax = _norm_axes(axes, len(input_shape))
        for a in ax:
            if a >= len(input_shape) or a < -len(input_shape):
                raise ValueError(
                    f"Invalid axis {a} specified; axis must be less than len(input_shape)={len(input_shape)}."
                )
        ax = tuple(a % len(input_shape) for a in ax)
        self.axes = ax
        self.ops = [
            SingleAxisFiniteDifference(input_shape, input_dtype, axis=a, prepend=prepend, append=append,
                                       circular=circular)
            for a in ax
        ]
        self.prepend, self.append, self.circular = prepend, append, circular
        shapes = [op.output_shape for op in self.ops]
        self.collapsed = all(s == shapes[0] for s in shapes)
        out_shape = (len(ax),) + shapes[0] if self.collapsed else tuple(shapes)
        self._desc = _fd_desc(input_shape, ax, prepend, append, circular)
        super().__init__(input_shape=input_shape, output_shape=out_shape, input_dtype=input_dtype,
                         output_dtype=input_dtype, eval_fn=self._fwd, adj_fn=self._adjoint)
        self.block_shapes = shapes

    def _fwd(self, x):
        t, batch, has_batch = _batch_of(x, self.input_shape, "x")
        flat = _device.empty((batch, sum(_size(s) for s in self.block_shapes)))
        _lib.call("ct_fd_fwd", _lib.ctypes.addressof(self._desc), t.data_ptr(), flat.data_ptr(), batch,
                  _device.stream())
        if self.collapsed:
            out = flat.reshape(((batch,) if has_batch else ()) + self.output_shape)
            return out
        outs, off = [], 0
        for s in self.block_shapes:
            n = _size(s)
            blk = flat[:, off:off + n].reshape((batch,) + s)
            outs.append(blk if has_batch else blk[0])
            off += n
        return tuple(outs)

    def _adjoint(self, y):
        if isinstance(y, tuple):
            blocks = [_device.to_device(b) for b in y]
            has_batch = blocks[0].ndim == len(self.block_shapes[0]) + 1
            batch = blocks[0].shape[0] if has_batch else 1
            flat = torch.cat([b.reshape(batch, -1) for b in blocks], dim=1).contiguous()
        else:
            t = _device.to_device(y)
            has_batch = t.ndim == len(self.output_shape) + 1
            batch = t.shape[0] if has_batch else 1
            flat = t.reshape(batch, -1)
        out = _device.empty(((batch,) if has_batch else ()) + self.input_shape)
        _lib.call("ct_fd_adj", _lib.ctypes.addressof(self._desc), flat.data_ptr(), out.data_ptr(), batch,
                  _device.stream())
        return out


class SingleAxisFiniteDifference(LinearOperator):
    """Finite difference along one axis (scico/linop/_diff.py:99-272)."""

    def __init__(self, input_shape, input_dtype=np.float32, axis: int = -1, prepend=None, append=None,
                 circular: bool = False, jit: bool = True, **kwargs):
        if not isinstance(axis, (int, np.integer)) or isinstance(axis, bool):
            raise TypeError(f"Expected argument 'axis' to be of type int, got {type(axis)} instead.")
        input_shape = tuple(input_shape)
        if axis < 0:
            axis = len(input_shape) + axis
        if axis >= len(input_shape):
            raise ValueError(
                f"Invalid axis {axis} specified; axis must be less than len(input_shape)={len(input_shape)}."
            )
        self.axis = int(axis)
        if circular and (prepend is not None or append is not None):
            raise ValueError("Argument 'circular' must be False if either prepend or append is not None.")
        if prepend not in [None, 0, 1]:
            raise ValueError("Argument 'prepend' may only take values None, 0, or 1.")
        if append not in [None, 0, 1]:
            raise ValueError("Argument 'append' may only take values None, 0, or 1.")
        self.prepend, self.append, self.circular = prepend, append, circular
        if circular:
            out_shape = input_shape
        else:
            out_shape = tuple(
                n + ((i == self.axis) * ((prepend is not None) + (append is not None) - 1))
                for i, n in enumerate(input_shape)
            )
        self._desc = _fd_desc(input_shape, (self.axis,), prepend, append, circular)
        super().__init__(input_shape=input_shape, output_shape=out_shape, input_dtype=input_dtype,
                         output_dtype=input_dtype, eval_fn=self._fwd, adj_fn=self._adjoint)

    def _fwd(self, x):
        t, batch, has_batch = _batch_of(x, self.input_shape, "x")
        out = _device.empty(((batch,) if has_batch else ()) + self.output_shape)
        _lib.call("ct_fd_fwd", _lib.ctypes.addressof(self._desc), t.data_ptr(), out.data_ptr(), batch,
                  _device.stream())
        return out

    def _adjoint(self, y):
        t, batch, has_batch = _batch_of(y, self.output_shape, "y")
        out = _device.empty(((batch,) if has_batch else ()) + self.input_shape)
        _lib.call("ct_fd_adj", _lib.ctypes.addressof(self._desc), t.data_ptr(), out.data_ptr(), batch,
                  _device.stream())
        return out


def _fd_desc(input_shape, axes, prepend, append, circular) -> _lib.FdDesc:
    if len(input_shape) > 3:
        raise ValueError("finite differences are implemented for up to 3 axes")
    d = _lib.FdDesc()
    d.ndim = len(input_shape)
    for k, n in enumerate(input_shape):
        d.shape[k] = int(n)
    d.naxes = len(axes)
    for k, a in enumerate(axes):
        d.axes[k] = int(a)
    d.prepend = -1 if prepend is None else int(prepend)
    d.append = -1 if append is None else int(append)
    d.circular = 1 if circular else 0
    return d


def _batch_of(x, core_shape, name):
    t = _device.to_device(x, name=name)
    if tuple(t.shape) == tuple(core_shape):
        return t, 1, False
    if t.ndim == len(core_shape) + 1 and tuple(t.shape[1:]) == tuple(core_shape):
        return t, t.shape[0], True
    raise ValueError(f"{name}: expected shape {tuple(core_shape)}, got {tuple(t.shape)}")


# ---------------------------------------------------------------------------
# utilities (scico/linop/_util.py)
# ---------------------------------------------------------------------------


def valid_adjoint(A: LinearOperator, AT: LinearOperator, eps: Optional[float] = 1e-7, x=None, y=None,
                  seed: int = 0):
    """Dot test |y^T A x - (A^T y)^T x| / max(...) < eps (scico/linop/_util.py:113-183)."""
    gen = torch.Generator(device="cpu").manual_seed(seed)
    if x is None:
        x = torch.randn(A.input_shape, generator=gen, dtype=torch.float32)
    if y is None:
        y = torch.randn(AT.input_shape, generator=gen, dtype=torch.float32)
    x = _device.to_device(x)
    y = _device.to_device(y)
    u = A(x)
    v = AT(y)
    yTu = float((y.double() * u.double()).sum())
    vTx = float((v.double() * x.double()).sum())
    err = abs(yTu - vTx) / max(abs(yTu), abs(vTx))
    if eps is None:
        return err
    return err < eps
