"""Functionals of the CT ADMM-TV path, mirroring scico.functional.

* :class:`Functional`, :class:`ScaledFunctional` --
  scico/functional/_functional.py:24-198 (``lam * F`` scales the prox
  parameter, :198).
* :class:`L21Norm` -- scico/functional/_norm.py:208-296.
* :class:`L1Norm` -- scico/functional/_norm.py:65-117.
* :class:`ZeroFunctional`, :class:`SeparableFunctional` --
  scico/functional/_functional.py:201-290.
* :class:`AnisotropicTVNorm`, :class:`IsotropicTVNorm`, :func:`haar_transform`
  -- scico/functional/_tvnorm.py:33-538 (TV norm with the shift-invariant
  Haar approximation of its prox).

Values are returned as Python floats accumulated in float64 on the device;
proxes run in the ctgpu kernels.
"""

from __future__ import annotations

import ctypes
from typing import Tuple, Union

import numpy as np
import torch

from . import _device, _lib


class Functional:
    """Base class (scico/functional/_functional.py:24)."""

    has_eval = False
    has_prox = False

    def __call__(self, x) -> float:
        raise NotImplementedError(f"Functional {type(self)} cannot be evaluated")

    def prox(self, v, lam: float = 1.0, **kwargs):
        raise NotImplementedError(f"Functional {type(self)} has no prox")

    def __mul__(self, other):
        if np.isscalar(other) or (isinstance(other, np.ndarray) and other.ndim == 0):
            return ScaledFunctional(self, float(other))
        return NotImplemented

    __rmul__ = __mul__

    def __repr__(self):
        return f"{type(self).__module__}.{type(self).__qualname__}"


class ScaledFunctional(Functional):
    """``scale * functional`` (scico/functional/_functional.py:131-198)."""

    def __init__(self, functional: Functional, scale: float):
        self.functional = functional
        self.scale = float(scale)
        self.has_eval = functional.has_eval
        self.has_prox = functional.has_prox

    def __call__(self, x) -> float:
        return self.scale * self.functional(x)

    def __mul__(self, other):
        if np.isscalar(other):
            return ScaledFunctional(self.functional, float(other) * self.scale)
        return NotImplemented

    __rmul__ = __mul__

    def prox(self, v, lam: float = 1.0, **kwargs):
        return self.functional.prox(v, lam * self.scale, **kwargs)


class ZeroFunctional(Functional):
    """The zero functional (scico/functional/_functional.py:270-290): value 0,
    prox the identity."""

    has_eval = True
    has_prox = True

    def __call__(self, x) -> float:
        return 0.0

    def prox(self, v, lam: float = 1.0, **kwargs):
        return v


class SeparableFunctional(Functional):
    """Sum of functionals of the blocks of a block variable
    (scico/functional/_functional.py:201-267): value sum_k f_k(x_k), prox
    blockwise with the same parameter."""

    def __init__(self, functional_list):
        self.functional_list = list(functional_list)
        self.has_eval = all(f.has_eval for f in self.functional_list)
        self.has_prox = all(f.has_prox for f in self.functional_list)

    def __call__(self, x) -> float:
        if len(x) != len(self.functional_list):
            raise ValueError("the number of blocks does not match the number of functionals")
        return sum(f(xk) for f, xk in zip(self.functional_list, x))

    def prox(self, v, lam: float = 1.0, **kwargs):
        if len(v) != len(self.functional_list):
            raise ValueError("the number of blocks does not match the number of functionals")
        return tuple(f.prox(vk, lam) for f, vk in zip(self.functional_list, v))


def _l2_layout(x: torch.Tensor, l2_axis) -> Tuple[torch.Tensor, int, int, tuple]:
    """Move the l2 axes to the front; return (contiguous (ncomp, n) view, ncomp, n, perm)."""
    nd = x.ndim
    if l2_axis is None:
        ax = tuple(range(nd))
    elif isinstance(l2_axis, (int, np.integer)):
        ax = (int(l2_axis) % nd,)
    else:
        ax = tuple(int(a) % nd for a in l2_axis)
    rest = tuple(a for a in range(nd) if a not in ax)
    perm = ax + rest
    ncomp = int(np.prod([x.shape[a] for a in ax])) if ax else 1
    n = int(np.prod([x.shape[a] for a in rest])) if rest else 1
    xp = x if perm == tuple(range(nd)) else x.permute(perm)
    return xp.contiguous().reshape(ncomp, n), ncomp, n, perm


class L21Norm(Functional):
    r"""The :math:`\ell_{2,1}` norm: l2 over `l2_axis`, then sum (scico/functional/_norm.py:208)."""

    has_eval = True
    has_prox = True

    def __init__(self, l2_axis: Union[None, int, Tuple] = 0):
        self.l2_axis = l2_axis

    def __call__(self, x) -> float:
        if isinstance(x, tuple):
            if self.l2_axis is not None:
                raise ValueError("Initializer argument 'l2_axis' must be None for BlockArray input.")
            return float(sum(L21Norm(None)(b) for b in x))
        t = _device.to_device(x)
        v, ncomp, n, _ = _l2_layout(t, self.l2_axis)
        out = _device.zeros((1,), dtype=torch.float64)
        ws = _device.reduce_workspace()
        _lib.call("ct_l21_norm", v.data_ptr(), ncomp, n, out.data_ptr(), ws.data_ptr(), ws.numel(),
                  _device.stream())
        return float(out.item())

    def prox(self, v, lam: float = 1.0, **kwargs):
        if isinstance(v, tuple):
            if self.l2_axis is not None:
                raise ValueError("Initializer argument 'l2_axis' must be None for BlockArray input.")
            return tuple(L21Norm(None).prox(b, lam) for b in v)
        t = _device.to_device(v)
        vv, ncomp, n, perm = _l2_layout(t, self.l2_axis)
        out = torch.empty_like(vv)
        _lib.call("ct_l21_prox", vv.data_ptr(), out.data_ptr(), ncomp, n, float(np.float32(lam)),
                  _device.stream())
        if perm == tuple(range(t.ndim)):
            return out.reshape(t.shape)
        shp = tuple(t.shape[a] for a in perm)
        inv = tuple(np.argsort(perm))
        return out.reshape(shp).permute(inv).contiguous()


class L1Norm(Functional):
    r"""The :math:`\ell_1` norm (scico/functional/_norm.py:65-117)."""

    has_eval = True
    has_prox = True

    def __call__(self, x) -> float:
        if isinstance(x, tuple):
            return float(sum(self(b) for b in x))
        t = _device.to_device(x).reshape(-1)
        out = _device.zeros((1,), dtype=torch.float64)
        ws = _device.reduce_workspace()
        _lib.call("ct_l21_norm", t.data_ptr(), 0, t.numel(), out.data_ptr(), ws.data_ptr(), ws.numel(),
                  _device.stream())
        return float(out.item())

    def prox(self, v, lam: float = 1.0, **kwargs):
        if isinstance(v, tuple):
            return tuple(self.prox(b, lam) for b in v)
        t = _device.to_device(v)
        out = torch.empty_like(t)
        _lib.call("ct_l1_prox", t.data_ptr(), out.data_ptr(), t.numel(), float(np.float32(lam)),
                  _device.stream())
        return out


# ---------------------------------------------------------------------------
# TV norms (scico/functional/_tvnorm.py)
# ---------------------------------------------------------------------------

def _haar_desc(shape, axes):
    from .linop import _fd_desc

    return _fd_desc(tuple(shape), tuple(axes), None, None, True)


def _haar_fwd(x: torch.Tensor, axes) -> torch.Tensor:
    """Single-level shift-invariant Haar transform (HaarTransform,
    _tvnorm.py:458-538) by ct_haar_fwd: per axis a lowpass (x + x shifted by
    one, circular) and highpass (x shifted by one - x) component, each times
    float32(1/sqrt 2), stacked to (naxes, 2, *shape)."""
    x = x.contiguous()
    d = _haar_desc(x.shape, axes)
    w = _device.empty((len(axes), 2) + tuple(x.shape))
    _lib.call("ct_haar_fwd", ctypes.addressof(d), x.data_ptr(), w.data_ptr(), 1, _device.stream())
    return w


def _haar_adj(w: torch.Tensor, axes) -> torch.Tensor:
    """Adjoint of _haar_fwd (ct_haar_adj): the sum over axes of the adjoint
    of each component."""
    w = w.contiguous()
    shape = tuple(w.shape[2:])
    d = _haar_desc(shape, axes)
    x = _device.empty(shape)
    _lib.call("ct_haar_adj", ctypes.addressof(d), w.data_ptr(), x.data_ptr(), 1, _device.stream())
    return x


def haar_transform(x, axes=None, adjoint: bool = False) -> torch.Tensor:
    """HaarTransform (or its adjoint) of a device tensor over `axes` (all
    axes if None)."""
    x = _device.to_device(x)
    if adjoint:
        nd = x.ndim - 2
        axes = tuple(range(nd)) if axes is None else tuple(a % nd for a in ((axes,) if isinstance(axes, int) else axes))
        return _haar_adj(x, axes)
    nd = x.ndim
    axes = tuple(range(nd)) if axes is None else tuple(a % nd for a in ((axes,) if isinstance(axes, int) else axes))
    return _haar_fwd(x, axes)


class TVNorm(Functional):
    """Total variation norm ``norm(D x)`` with the approximate prox of
    Kamilov (2016) / Chandler (2024) (scico/functional/_tvnorm.py:33-237):
    D = FiniteDifference over `axes` (circular, or append=0 otherwise); the
    prox applies the base norm's prox with parameter sqrt(2) K lam (K = 2
    naxes) to the highpass part of the single-level shift-invariant Haar
    transform of v -- edge-padded by one on the differenced axes when not
    circular, only the non-boundary region shrunk -- and returns 1/K times
    the adjoint transform, cropped back."""

    has_eval = True
    has_prox = True

    def __init__(self, norm: Functional, circular: bool = True, axes=None, input_shape=None,
                 input_dtype=np.float32):
        self.norm = norm
        self.circular = bool(circular)
        self.axes = axes
        self._G = None

    def _axes_of(self, nd):
        if self.axes is None:
            return tuple(range(nd))
        ax = (self.axes,) if isinstance(self.axes, (int, np.integer)) else tuple(self.axes)
        return tuple(int(a) % nd for a in ax)

    def __call__(self, x) -> float:
        from . import linop

        x = _device.to_device(x)
        shape = tuple(x.shape)
        if self._G is None or self._G.input_shape != shape:
            self._G = linop.FiniteDifference(shape, axes=self._axes_of(len(shape)), circular=self.circular,
                                             append=None if self.circular else 0)
        return self.norm(self._G(x))

    def prox(self, v, lam: float = 1.0, **kwargs):
        v = _device.to_device(v)
        nd = v.ndim
        axes = self._axes_of(nd)
        K = 2 * len(axes)
        # the base norm's prox parameter snp.sqrt(2) * K * lam (_tvnorm.py:203),
        # evaluated in float32 as jax evaluates it
        f = np.float32
        thr = float(f(f(np.sqrt(f(2.0))) * f(K)) * f(lam))
        if self.circular:
            w = _haar_fwd(v, axes)
            hi = w[:, 1].contiguous()
            w[:, 1] = self.norm.prox(hi, thr)
            return (1.0 / K) * _haar_adj(w, axes)
        # replicate-pad by one at the end of each differenced axis
        vp = v
        for a in axes:
            last = vp.narrow(a, vp.shape[a] - 1, 1)
            vp = torch.cat((vp, last), dim=a)
        w = _haar_fwd(vp, axes)
        region = [slice(None)] * (nd + 2)
        region[1] = 1
        for a in axes:
            region[2 + a] = slice(0, vp.shape[a] - 1)
        region = tuple(region)
        hi = w[region].contiguous()
        w[region] = self.norm.prox(hi, thr)
        u = _haar_adj(w, axes)
        crop = tuple(slice(0, v.shape[a]) for a in range(nd))
        return (1.0 / K) * u[crop]


class AnisotropicTVNorm(TVNorm):
    """Anisotropic TV: ``L1Norm(D x)`` (scico/functional/_tvnorm.py:239-294)."""

    def __init__(self, circular: bool = False, axes=None, input_shape=None, input_dtype=np.float32):
        super().__init__(L1Norm(), circular=circular, axes=axes, input_shape=input_shape, input_dtype=input_dtype)


class IsotropicTVNorm(TVNorm):
    """Isotropic TV: ``L21Norm(D x)`` (scico/functional/_tvnorm.py:297-352)."""

    def __init__(self, circular: bool = False, axes=None, input_shape=None, input_dtype=np.float32):
        super().__init__(L21Norm(), circular=circular, axes=axes, input_shape=input_shape, input_dtype=input_dtype)
