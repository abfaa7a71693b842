"""CPU oracle for the CT ADMM-TV hot path -- TEST INFRASTRUCTURE ONLY.

A NumPy restatement of scico's CT reconstruction path, used as the checker
of the GPU library.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import it; the product path never
calls it.

Every function cites the scico source lines it restates (paths within the
scico source tree).  ``dtype=np.float32`` follows the reference's float32
arithmetic (JAX with x64 disabled, the default) operation by operation;
``dtype=np.float64`` is the float64 restatement used to state errors
against exact arithmetic.

Pinning.  scico runs on JAX, which cannot be installed in this build
environment, so outputs of scico itself cannot be generated here.  The
restatement is pinned against the known-answer tests the reference's own
test suite holds for this path (tests/golden/reference_kat.json, values
transcribed from scico/test/linop/xray/test_xray_3d.py:29-60,
scico/test/linop/test_diff.py:11-65 and scico/test/functional/
test_norm.py:9-28) and against the analytic properties those tests check
(dot tests test_xray_2d.py:52-85 and test_xray_3d.py:9-26, the FD adjoint
test test_diff.py:68-78).  The 2D projector has no known-answer test in the
reference: its parity is pinned through the documented geometry (angle 0
sums image rows, pi/2 sums columns, _xray2d.py:66-70), mass conservation
and the dot test -- parity of the 2D projector to scico's exact XLA output
is therefore only partially pinned.
"""

from __future__ import annotations

import math
from typing import Callable, List, Optional, Sequence, Tuple

import numpy as np

# ---------------------------------------------------------------------------
# 2D parallel-beam projector -- scico/linop/xray/_xray2d.py
# ---------------------------------------------------------------------------


def xray2d_defaults(input_shape, angles, x0=None, dx=None, y0=None, det_count=None):
    """Constructor defaults of XRayTransform2D.__init__ (_xray2d.py:86-121)."""
    nx = tuple(input_shape)
    if dx is None:
        dx = 2 * (np.sqrt(2) / 2,)
    if np.isscalar(dx) or np.ndim(dx) == 0:
        dx = 2 * (float(dx),)
    dx = tuple(float(v) for v in dx)
    if x0 is None:
        x0 = -(np.array(nx) * np.array(dx)) / 2
    if det_count is None:
        det_count = int(np.ceil(np.linalg.norm(input_shape)))
    if y0 is None:
        y0 = -det_count / 2
    return dict(nx=nx, angles=np.asarray(angles), x0=np.asarray(x0, dtype=np.float64), dx=dx,
                y0=float(y0), ny=int(det_count))


def xray2d_view_params(g: dict, dtype=np.float32):
    """Per-view scalars of _calc_weights (_xray2d.py:326-347).

    Returns (Pxmin, Pdx0, Pdx1, width), each (n_views,).  float32: the
    angles are cast to float32 (as jit does with x64 disabled) and cos/sin
    are the correctly rounded float32 values; every later operation is one
    float32 rounding, in the reference's order.
    """
    f = np.dtype(dtype).type
    if dtype == np.float32:
        ang = np.asarray(g["angles"], dtype=np.float32).astype(np.float64)
        u0 = np.cos(ang).astype(np.float32)
        u1 = np.sin(ang).astype(np.float32)
    else:
        ang = np.asarray(g["angles"], dtype=np.float64)
        u0, u1 = np.cos(ang), np.sin(ang)
    x00, x01 = f(g["x0"][0]), f(g["x0"][1])
    dx0, dx1 = f(g["dx"][0]), f(g["dx"][1])
    y0 = f(g["y0"])
    Px0 = (x00 * u0 + x01 * u1) - y0  # :327
    Pd0 = dx0 * u0  # :328
    Pd1 = dx1 * u1
    Pxmin = np.min(np.stack([Px0, Px0 + Pd0, Px0 + Pd1, (Px0 + Pd0) + Pd1]), axis=0)  # :329
    diag1 = np.abs(Pd0 + Pd1)  # :342
    diag2 = np.abs(Pd0 - Pd1)
    w = np.maximum(diag1, diag2)  # :344
    fmin = np.minimum(diag1, diag2)
    width = (w + fmin) / f(2)  # :347
    return Pxmin.astype(dtype), Pd0.astype(dtype), Pd1.astype(dtype), width.astype(dtype)


def xray2d_calc_weights(g: dict, views: slice = slice(None), dtype=np.float32):
    """inds, weights of _calc_weights (_xray2d.py:331-349) for a range of views."""
    f = np.dtype(dtype).type
    Pxmin, Pd0, Pd1, width = (a[views] for a in xray2d_view_params(g, dtype))
    i = np.arange(g["nx"][0], dtype=dtype).reshape(1, -1, 1)
    j = np.arange(g["nx"][1], dtype=dtype).reshape(1, 1, -1)
    Px = (Pxmin.reshape(-1, 1, 1) + Pd0.reshape(-1, 1, 1) * i) + Pd1.reshape(-1, 1, 1) * j  # :331-335
    fl = np.floor(Px)
    inds = fl.astype(np.int64)  # :338
    dist = f(1) - (Px - fl)  # :348
    wd = width.reshape(-1, 1, 1)
    weights = np.minimum(dist, wd) / wd  # :349
    return inds, weights.astype(dtype)


def xray2d_project(im: np.ndarray, g: dict, dtype=np.float32, chunk: int = 32) -> np.ndarray:
    """y = H im (_xray2d.py:223-265): two scatter-adds, out-of-range bins dropped.

    float32: sequential scatter order (np.add.at over the (view, i, j)
    updates, first the w terms then the 1-w terms).  float64: exact-ish
    accumulation with np.bincount.
    """
    nv, ny = len(g["angles"]), g["ny"]
    im = np.asarray(im, dtype=dtype)
    y = np.zeros(nv * ny, dtype=dtype)
    # first scatter (:254-260) over all updates, then the second (:262-263)
    # into its result
    for shift in (0, 1):
        for a0 in range(0, nv, chunk):
            sl = slice(a0, min(nv, a0 + chunk))
            inds, w = xray2d_calc_weights(g, sl, dtype)
            wt = w if shift == 0 else np.asarray(1, dtype) - w
            a = np.arange(sl.start, sl.stop).reshape(-1, 1, 1)
            k = inds + shift
            valid = (k >= 0) & (k < ny)  # :255, :262
            idx = (a * ny + k)[valid]
            val = (im[None] * wt)[valid]
            if dtype == np.float32:
                np.add.at(y, idx, val)
            else:
                y += np.bincount(idx, weights=val, minlength=nv * ny)
    return y.reshape(nv, ny)


def xray2d_back_project(y: np.ndarray, g: dict, dtype=np.float32, chunk: int = 32) -> np.ndarray:
    """H^T y (_xray2d.py:267-306): two masked gathers summed over the views."""
    nv, ny = len(g["angles"]), g["ny"]
    y = np.asarray(y, dtype=dtype).reshape(nv, ny)
    s1 = np.zeros(g["nx"], dtype=dtype)
    s2 = np.zeros(g["nx"], dtype=dtype)
    for a0 in range(0, nv, chunk):
        sl = slice(a0, min(nv, a0 + chunk))
        inds, w = xray2d_calc_weights(g, sl, dtype)
        a = np.arange(sl.start, sl.stop).reshape(-1, 1, 1)
        for shift, wt, acc in ((0, w, s1), (1, np.asarray(1, dtype) - w, s2)):
            k = inds + shift
            valid = (k >= 0) & (k < ny)  # :295, :301
            vals = y[a, np.clip(k, 0, ny - 1)] * np.where(valid, wt, np.asarray(0, dtype))
            for r in range(vals.shape[0]):  # sum over the view axis in view order
                acc += vals[r]
    return ((np.zeros(g["nx"], dtype=dtype) + s1) + s2).astype(dtype)  # :298-306


def xray2d_fbp_filter(N: int) -> np.ndarray:
    """Ramp filter taps of XRayTransform2D._ramp_filter (_xray2d.py:199-221), tau = 1."""
    x = np.arange(N) - (N - 1) // 2
    out = np.zeros(N, dtype=np.float64)
    out[x == 0] = 0.25
    odd = (x % 2) != 0
    out[odd] = -1.0 / (x[odd].astype(np.float64) ** 2 * np.pi**2)
    return out


def xray2d_fbp_rows(y: np.ndarray, dtype=np.float64) -> np.ndarray:
    """Ramp-filtered sinogram rows of XRayTransform2D.fbp (_xray2d.py:191-195):
    FFT product of each row and the filter, both zero-padded to 2N-1, inverse
    FFT, real part of samples (N-1)//2 .. (N-1)//2 + N - 1."""
    y = np.asarray(y, dtype=dtype)
    N = y.shape[-1]
    L = 2 * N - 1
    h = xray2d_fbp_filter(N).astype(dtype)
    c = np.fft.ifft(np.fft.fft(h, n=L)[None, :] * np.fft.fft(y, n=L, axis=-1), n=L, axis=-1).real
    off = (N - 1) // 2
    return c[..., off:off + N].astype(dtype)


def xray2d_fbp(y: np.ndarray, g: dict, dtype=np.float64) -> np.ndarray:
    """XRayTransform2D.fbp (_xray2d.py:158-197): filtered rows back projected,
    masked to pixels whose footprint stays on the detector in every view
    (back projection of ones >= views * (1 - 1e-5)) and scaled by
    pi * dx0 * dx1 / views."""
    nv = y.shape[0]
    ones = np.ones(y.shape, dtype=dtype)
    mask = xray2d_back_project(ones, g, dtype) >= nv * (1.0 - 1e-5)
    hy = xray2d_fbp_rows(y, dtype)
    return (np.pi * g["dx"][0] * g["dx"][1] / nv) * mask * xray2d_back_project(hy, g, dtype)


# ---------------------------------------------------------------------------
# 3D parallel-beam projector -- scico/linop/xray/_xray3d.py
# ---------------------------------------------------------------------------


def xray3d_matrices_from_euler_angles(input_shape, output_shape, seq, angles, degrees=False,
                                      voxel_spacing=None, det_spacing=None) -> np.ndarray:
    """(views, 2, 4) projection matrices (_xray3d.py:268-327)."""
    from scipy.spatial.transform import Rotation

    if voxel_spacing is None:
        voxel_spacing = np.ones(3)
    if det_spacing is None:
        det_spacing = np.ones(2)
    M = Rotation.from_euler(seq, angles, degrees=degrees).as_matrix()[:, :2, :]  # :311-312
    M = np.einsum("vmn,nn->vmn", M, np.diag(voxel_spacing))  # :315-319
    M = np.einsum("mm,vmn->vmn", np.diag(1 / np.array(det_spacing)), M)  # :316,320
    x0 = np.array(input_shape) / 2  # :323
    t = -np.einsum("vmn,n->vm", M, x0) + np.array(output_shape) / 2  # :324
    return np.concatenate((M, t[..., None]), axis=2)  # :325


def xray3d_calc_weights(input_shape, matrix, det_shape, dtype=np.float32):
    """ul index and the four weights (_xray3d.py:206-266) for one view."""
    f = np.dtype(dtype).type
    m = np.asarray(matrix, dtype=dtype)
    x = np.mgrid[: input_shape[0], : input_shape[1], : input_shape[2]].astype(dtype) + f(0.5)  # :211
    Px = np.stack(
        (
            ((m[0, 0] * x[0] + m[0, 1] * x[1]) + m[0, 2] * x[2]) + m[0, 3],  # :216
            ((m[1, 0] * x[0] + m[1, 1] * x[1]) + m[1, 2] * x[2]) + m[1, 3],  # :217
        )
    )
    w = f(0.5)  # :222
    left = Px - w / f(2)  # :223
    to_next = np.minimum(np.ceil(left) - left, w)  # :224
    ul = np.floor(left).astype(np.int64)  # :225
    inv = f(1) / (w * w)
    ul_w = to_next[0] * to_next[1] * inv  # :227
    ur_w = (w - to_next[0]) * to_next[1] * inv  # :228
    ll_w = to_next[0] * (w - to_next[1]) * inv  # :229
    lr_w = (w - to_next[0]) * (w - to_next[1]) * inv  # :230

    def inb(a, b):
        return (a >= 0) & (a < det_shape[0]) & (b >= 0) & (b < det_shape[1])

    z = f(0)
    ul_w = np.where(inb(ul[0], ul[1]), ul_w, z)  # :233-240
    ur_w = np.where(inb(ul[0] + 1, ul[1]), ur_w, z)  # :241-248
    ll_w = np.where(inb(ul[0], ul[1] + 1), ll_w, z)  # :249-256
    lr_w = np.where(inb(ul[0] + 1, ul[1] + 1), lr_w, z)  # :257-264
    return ul, ul_w, ur_w, ll_w, lr_w


def xray3d_project(im: np.ndarray, matrices: np.ndarray, det_shape, dtype=np.float32, acc_dtype=None) -> np.ndarray:
    """(views, *det_shape) projections (_xray3d.py:110-159), 4 scatter-adds per view.

    Weights are computed in `dtype`; acc_dtype (default `dtype`) is the
    precision of the voxel values and the sums.  The weight model is
    discontinuous where left is an exact integer, so float64 weights move
    different voxels than the reference's float32 ones: use dtype=float32,
    acc_dtype=float64 for a float32-model reference with exact sums."""
    acc = np.dtype(dtype if acc_dtype is None else acc_dtype).type
    im = np.asarray(im, dtype=acc)
    nv = len(matrices)
    out = np.zeros((nv,) + tuple(det_shape), dtype=acc)
    for v in range(nv):
        ul, w00, w10, w01, w11 = xray3d_calc_weights(im.shape, matrices[v], det_shape, dtype)
        proj = np.zeros(det_shape, dtype=acc)
        for (d0, d1), w in (((0, 0), w00), ((1, 0), w10), ((0, 1), w01), ((1, 1), w11)):
            a, b = ul[0] + d0, ul[1] + d1
            ok = (a >= 0) & (a < det_shape[0]) & (b >= 0) & (b < det_shape[1])  # mode="drop"
            np.add.at(proj, (a[ok], b[ok]), (w.astype(acc) * im)[ok])
        out[v] = proj
    return out


def xray3d_back_project(proj: np.ndarray, matrices: np.ndarray, input_shape, dtype=np.float32,
                        acc_dtype=None) -> np.ndarray:
    """Back projection (_xray3d.py:161-204): view-sequential scan of 4 gathers
    (weights in `dtype`, values and sums in acc_dtype, as xray3d_project)."""
    acc = np.dtype(dtype if acc_dtype is None else acc_dtype).type
    proj = np.asarray(proj, dtype=acc)
    det_shape = proj.shape[1:]
    HTy = np.zeros(input_shape, dtype=acc)
    for v in range(len(matrices)):
        ul, w00, w10, w01, w11 = xray3d_calc_weights(input_shape, matrices[v], det_shape, dtype)
        y = proj[v]
        for (d0, d1), w in (((0, 0), w00), ((1, 0), w10), ((0, 1), w01), ((1, 1), w11)):
            a = np.clip(ul[0] + d0, 0, det_shape[0] - 1)
            b = np.clip(ul[1] + d1, 0, det_shape[1] - 1)
            HTy = HTy + y[a, b] * w.astype(acc)  # :200-203 (weights are 0 out of range)
    return HTy


# ---------------------------------------------------------------------------
# Finite differences -- scico/linop/_diff.py
# ---------------------------------------------------------------------------


def fd_single(x: np.ndarray, axis: int, prepend=None, append=None, circular=False) -> np.ndarray:
    """SingleAxisFiniteDifference._eval (_diff.py:236-272): np.diff with extension."""
    kw = {}
    if circular:
        kw["append"] = np.take(x, [0], axis=axis)  # :239-245
    else:
        if prepend == 0:
            kw["prepend"] = np.take(x, [0], axis=axis)  # :247-254
        elif prepend == 1:
            kw["prepend"] = 0  # :255-258
        if append == 0:
            kw["append"] = np.take(x, [x.shape[axis] - 1], axis=axis)  # :259-266
        elif append == 1:
            kw["append"] = 0  # :267-270
    return np.diff(x, axis=axis, **kw).astype(x.dtype)


def fd_eval(x: np.ndarray, axes=None, prepend=None, append=None, circular=False):
    """FiniteDifference: blocks in axis order, stacked when their shapes agree
    (VerticalStack collapse, scico/operator/_stack.py:87-88,126-129)."""
    axes = tuple(range(x.ndim)) if axes is None else ((axes,) if np.isscalar(axes) else tuple(axes))
    blocks = [fd_single(x, a, prepend, append, circular) for a in axes]
    if all(b.shape == blocks[0].shape for b in blocks):
        return np.stack(blocks)
    return blocks


def fd_single_adj(d: np.ndarray, n: int, axis: int, prepend=None, append=None, circular=False) -> np.ndarray:
    """Adjoint of fd_single as jax.linear_transpose builds it from _eval
    (scico/linop/_diff.py:236-272, scico/_core.py:140-153).  jnp.diff forms
    the extended line e (prepend / append copies concatenated to x) and
    d = e[1:] - e[:-1]; its transpose gives e the cotangent
    ce[q] = pad(d, (1, 0))[q] + pad(-d, (0, 1))[q] = d[q-1] - d[q] (a missing
    term is 0), and x[t] receives ce[q] of every position q holding x[t],
    summed in float32: one position for interior samples, two at a copied
    end (prepend=0 at t=0, append=0 at t=n-1), three for a single-sample
    axis with both (summed in position order)."""
    d = np.moveaxis(np.asarray(d), axis, 0)
    M = d.shape[0]
    out = np.zeros((n,) + d.shape[1:], dtype=d.dtype)
    if circular:
        for t in range(n):
            out[t] = d[(t - 1) % n] - d[t]
        return np.moveaxis(out, 0, axis)
    P = 1 if prepend is not None else 0
    z = np.zeros(d.shape[1:], dtype=d.dtype)

    def ce(q):
        return (d[q - 1] if 0 <= q - 1 < M else z) - (d[q] if 0 <= q < M else z)

    for t in range(n):
        qa = 0 if (prepend == 0 and t == 0) else t + P
        qb = n + P if (append == 0 and t == n - 1) else t + P
        v = ce(qa)
        for q in range(qa + 1, qb + 1):
            v = v + ce(q)
        out[t] = v
    return np.moveaxis(out, 0, axis)


def fd_adj(d, shape, axes=None, prepend=None, append=None, circular=False) -> np.ndarray:
    """sum over blocks of the single-axis adjoints (scico/linop/_stack.py:71-72)."""
    axes = tuple(range(len(shape))) if axes is None else ((axes,) if np.isscalar(axes) else tuple(axes))
    out = None
    for k, a in enumerate(axes):
        r = fd_single_adj(d[k], shape[a], a, prepend, append, circular)
        out = r if out is None else out + r
    return out


# ---------------------------------------------------------------------------
# Norms and proximal operators -- scico/functional/_norm.py
# ---------------------------------------------------------------------------


def no_nan_divide(x, y):
    """scico/numpy/util.py:302-315."""
    one = np.asarray(1, dtype=y.dtype)
    return np.where(y != 0, x / np.where(y != 0, y, one), np.asarray(0, dtype=x.dtype))


def l21_norm(x: np.ndarray, l2_axis=0) -> float:
    """L21Norm.__call__ (_norm.py:240-250)."""
    l2 = np.sqrt((np.abs(x) ** 2).sum(axis=l2_axis))
    return float(np.sum(np.abs(l2), dtype=np.float64))


def l21_prox(v: np.ndarray, lam: float, l2_axis=0) -> np.ndarray:
    """L21Norm._prox (_norm.py:254-263)."""
    f = v.dtype.type
    length = np.sqrt((np.abs(v) ** 2).sum(axis=l2_axis, keepdims=True))
    direction = no_nan_divide(v, length)
    new_length = length - f(lam)
    new_length = f(0.5) * (new_length + np.abs(new_length))
    return (new_length * direction).astype(v.dtype)


def l1_norm(x: np.ndarray) -> float:
    """L1Norm.__call__ (_norm.py:79-80)."""
    return float(np.sum(np.abs(x), dtype=np.float64))


def l1_prox(v: np.ndarray, lam: float) -> np.ndarray:
    """L1Norm.prox (_norm.py:110-116), real input."""
    f = v.dtype.type
    tmp = np.abs(v) - f(lam)
    tmp = f(0.5) * (tmp + np.abs(tmp))
    return (np.sign(v) * tmp).astype(v.dtype)


# ---------------------------------------------------------------------------
# CG -- scico/solver.py:326-405
# ---------------------------------------------------------------------------


def cg(A: Callable, b: np.ndarray, x0: np.ndarray, tol=1e-5, atol=0.0, maxiter=1000, dot_dtype=None):
    """scico.solver.cg with M = identity, vectors in the dtype of b.

    dot_dtype=None keeps the dot products in that dtype (the reference);
    dot_dtype=np.float64 gives float64 products and sums with float32
    vectors -- the precision policy of the GPU solver.
    """
    f = b.dtype.type

    def dot(u, v):
        if dot_dtype is None:
            return np.sum(u * v)
        return np.sum(u.astype(dot_dtype) * v.astype(dot_dtype))

    x = x0.copy()
    Ax = A(x0)  # :379
    bn = np.sqrt(dot(b, b))  # :380
    r = b - Ax  # :381
    p = r.copy()  # :382-383
    num = dot(r, r)  # :384
    ii = 0
    tol_sq = max(tol * bn, atol) ** 2  # :388
    while ii < maxiter and num > tol_sq:  # :390
        Ap = A(p)
        alpha = num / dot(p, Ap)  # :392
        x = x + f(alpha) * p
        r = r - f(alpha) * Ap
        num_old = num
        num = dot(r, r)
        beta = num / num_old
        p = r + f(beta) * p
        ii += 1
    return x, {"num_iter": ii, "rel_res": float(np.sqrt(num) / bn)}


# ---------------------------------------------------------------------------
# ADMM-TV -- scico/optimize/_admm.py, _admmaux.py
# ---------------------------------------------------------------------------


def cg_fixed(A: Callable, b: np.ndarray, x0=None, maxiter: int = 50, dot_dtype=None) -> np.ndarray:
    """Fixed-iteration CG of scico.flax.inverse.cg_solver (flax/inverse.py:
    113-158): r0 = b - A(x0), p0 = r0, then exactly maxiter steps of
    alpha = num / <p, Ap>, x += alpha p, r -= alpha Ap, beta = num' / num,
    p = r + beta p (no stopping test)."""
    dt = b.dtype
    dd = np.dtype(dot_dtype if dot_dtype is not None else dt).type

    def dot(u, v):
        return dd(np.sum(u.astype(dd) * v.astype(dd)))

    x = np.zeros_like(b) if x0 is None else np.asarray(x0, dtype=dt).copy()
    r = b - A(x)
    num = dot(r, r)
    p = r
    for _ in range(maxiter):
        Ap = A(p)
        alpha = num / dot(p, Ap)
        x = x + dt.type(alpha) * p
        r = r - dt.type(alpha) * Ap
        num_old, num = num, dot(r, r)
        p = r + dt.type(num / num_old) * p
    return x


def admm_tv(fwd: Callable, adj: Callable, y: np.ndarray, shape, lam_l21: float = 0.0, lam_l1: float = 0.0,
            rho: float = 1.0, maxiter: int = 10, cg_tol: float = 1e-4, cg_maxiter: int = 10, x0=None,
            scale: float = 0.5, alpha: float = 1.0, dtype=np.float32, dot_dtype=None):
    """ADMM with LinearSubproblemSolver for scale||Ax-y||^2 + sum_i lam_i g_i(Dx).

    D = FiniteDifference(append=0) over all axes; g = L21 (if lam_l21) then
    L1 (if lam_l1), each with its own z_i/u_i.  Follows ADMM.__init__/step
    (_admm.py:96-148, 297-378), LinearSubproblemSolver.internal_init /
    compute_rhs / solve (_admmaux.py:205-269) and the itstat quantities
    objective / norm_primal_residual / norm_dual_residual (:210-295).
    dot_dtype: see cg (np.float64 with dtype=np.float32 is the GPU solver's
    precision policy).  Returns (x, itstat list of dicts, z_list, u_list).
    """
    f = np.dtype(dtype).type
    shape = tuple(shape)
    y = np.asarray(y, dtype=dtype)
    x = np.zeros(shape, dtype=dtype) if x0 is None else np.asarray(x0, dtype=dtype).copy()
    terms = []
    if lam_l21:
        terms.append(("l21", lam_l21))
    if lam_l1:
        terms.append(("l1", lam_l1))
    D = lambda v: fd_eval(v, append=0)
    DT = lambda d: fd_adj(d, shape, append=0)
    c = f(2.0 * scale)
    rho_f = f(rho)

    def lhs(v):  # (_admmaux.py:222-229): sum rho_i C_i^T C_i + hessian
        g = DT(D(v))
        acc = None
        for _ in terms:
            t = rho_f * g
            acc = t if acc is None else acc + t
        return acc + c * adj(fwd(v))

    ATy = adj(y)
    z = [D(x) for _ in terms]  # z_init (:297-315)
    u = [np.zeros_like(zi) for zi in z]  # u_init (:317-332)
    hist = []
    for it in range(maxiter):
        rhs = np.zeros(shape, dtype=dtype) + c * ATy  # compute_rhs (:245-256)
        for zi, ui in zip(z, u):
            rhs = rhs + rho_f * DT(zi - ui)
        x, info = cg(lhs, rhs, x, tol=cg_tol, maxiter=cg_maxiter, dot_dtype=dot_dtype)
        z_old = [zi.copy() for zi in z]
        Cx = D(x)
        for k, (kind, lam) in enumerate(terms):  # step (:368-378)
            Cix = Cx if alpha == 1.0 else f(alpha) * Cx + f(1.0 - alpha) * z[k]
            thr = f((1.0 / rho) * lam)  # ScaledFunctional.prox (_functional.py:198)
            v = Cix + u[k]
            z[k] = l21_prox(v, thr) if kind == "l21" else l1_prox(v, thr)
            u[k] = u[k] + Cix - z[k]
        r = y - fwd(x)
        obj = scale * float(np.sum(r.astype(np.float64) ** 2))
        for (kind, lam), zk in zip(terms, z):
            obj += lam * (l21_norm(zk) if kind == "l21" else l1_norm(zk))
        prim = math.sqrt(sum(rho * float(np.sum((Cx - zk).astype(np.float64) ** 2)) for zk in z))
        dsum = None
        for zk, zo in zip(z, z_old):
            t = rho_f * DT(zk - zo)
            dsum = t if dsum is None else dsum + t
        dual = float(np.sqrt(np.sum(dsum.astype(np.float64) ** 2)))
        hist.append(dict(Iter=it, Objective=obj, Prml_Rsdl=prim, Dual_Rsdl=dual, CG_It=info["num_iter"],
                         CG_Res=info["rel_res"]))
    return x, hist, z, u


def padmm_tv(fwd: Callable, adj: Callable, y: np.ndarray, shape, lam: float, alpha: float, rho: float, mu: float,
             nu: float, maxiter: int, dtype=np.float64):
    """ProximalADMM (_padmm.py:349-363) on the split of the reference's
    ct_3d_tv_padmm example: f = 0, A = (C, alpha D) stacked, B = -I, c = 0,
    g = (1/2 ||y - z0||^2, (lam / alpha) ||z1||_{2,1}).  D = FiniteDifference
    (append=0) over all axes.  Returns (x, list of (primal, dual) residual
    norms, fast dual residual)."""
    f = np.dtype(dtype).type
    shape = tuple(shape)
    y = np.asarray(y, dtype=dtype)
    D = lambda v: fd_eval(v, append=0)
    DT = lambda d: fd_adj(d, shape, append=0)
    A = lambda v: (fwd(v), f(alpha) * D(v))
    AT = lambda w: adj(w[0]) + f(alpha) * DT(w[1])
    x = np.zeros(shape, dtype=dtype)
    z = (np.zeros(y.shape, dtype=dtype), np.zeros((len(shape),) + shape, dtype=dtype))
    u = (np.zeros_like(z[0]), np.zeros_like(z[1]))
    u_old = u
    lam_p = 1.0 / (rho * nu)
    c0 = f(2.0 * 0.5 * lam_p)  # SquaredL2Loss.prox, A = I (loss.py:220-226)
    hist = []
    for _ in range(maxiter):
        x = x - f(1.0 / mu) * AT(tuple(f(2.0) * a - b for a, b in zip(u, u_old)))  # f = 0: prox is identity
        Ax = A(x)
        pz = tuple(zk + f(1.0 / nu) * (a - zk + uk) for zk, a, uk in zip(z, Ax, u))  # B^T = -I, B z = -z
        z_old = z
        z = ((c0 * y + pz[0]) / (c0 + f(1.0)), l21_prox(pz[1], f((lam / alpha) * lam_p)))
        u_old = u
        u = tuple(uk + a - zk for uk, a, zk in zip(u, Ax, z))
        prim = math.sqrt(sum(float(np.sum((a - zk).astype(np.float64) ** 2)) for a, zk in zip(Ax, z)))
        dual = math.sqrt(sum(float(np.sum((zk - zo).astype(np.float64) ** 2)) for zk, zo in zip(z, z_old)))
        hist.append((prim, dual))
    return x, hist


def haar_fwd(x: np.ndarray, axes) -> np.ndarray:
    """Single-level shift-invariant Haar transform (_tvnorm.py:458-538):
    per axis (x + roll(x, -1)) / sqrt2 and (roll(x, -1) - x) / sqrt2."""
    r = 1.0 / math.sqrt(2.0)
    return np.stack([np.stack((r * (x + np.roll(x, -1, a)), r * (np.roll(x, -1, a) - x))) for a in axes])


def haar_adj(w: np.ndarray, axes) -> np.ndarray:
    r = 1.0 / math.sqrt(2.0)
    return sum(r * (w[k, 0] + np.roll(w[k, 0], 1, a)) + r * (np.roll(w[k, 1], 1, a) - w[k, 1])
               for k, a in enumerate(axes))


def tv_prox(v: np.ndarray, lam: float, isotropic: bool, circular: bool, axes=None, dtype=np.float64) -> np.ndarray:
    """TVNorm.prox (_tvnorm.py:183-237): the base norm's prox, parameter
    sqrt2 K lam (K = 2 naxes), on the highpass Haar components of v --
    replicate-padded by one on the differenced axes and restricted to the
    non-boundary region when not circular -- then 1/K times the adjoint
    transform, cropped."""
    v = np.asarray(v, dtype=dtype)
    nd = v.ndim
    axes = tuple(range(nd)) if axes is None else tuple(axes)
    K = 2 * len(axes)
    # snp.sqrt(2) * K * lam and (1.0 / K) * ... (_tvnorm.py:203, 206) in the
    # array dtype, as jax evaluates them on float32 arrays
    f = np.dtype(dtype).type
    thr = f(f(np.sqrt(f(2.0))) * f(K)) * f(lam)
    inv_k = f(1.0 / K)
    prox = (lambda t: l21_prox(t, thr)) if isotropic else (lambda t: l1_prox(t, thr))
    if circular:
        w = haar_fwd(v, axes)
        w[:, 1] = prox(w[:, 1])
        return inv_k * haar_adj(w, axes)
    vp = np.pad(v, [(0, 1) if a in axes else (0, 0) for a in range(nd)], mode="edge")
    w = haar_fwd(vp, axes)
    region = (slice(None), 1) + tuple(slice(0, vp.shape[a] - 1) if a in axes else slice(None) for a in range(nd))
    w[region] = prox(w[region])
    return (inv_k * haar_adj(w, axes))[tuple(slice(0, n) for n in v.shape)]


def snr(reference: np.ndarray, comparison: np.ndarray) -> float:
    """scico.metric.snr (scico/metric.py:48-62)."""
    reference = np.asarray(reference, dtype=np.float64)
    comparison = np.asarray(comparison, dtype=np.float64)
    return float(10 * np.log10(np.var(reference) / np.mean((reference - comparison) ** 2)))


def psnr(reference: np.ndarray, comparison: np.ndarray) -> float:
    """scico.metric.psnr with the reference's own range (scico/metric.py:65-100)."""
    reference = np.asarray(reference, dtype=np.float64)
    comparison = np.asarray(comparison, dtype=np.float64)
    rng = abs(reference.max() - reference.min())
    return float(20 * np.log10(rng) - 10 * np.log10(np.mean((reference - comparison) ** 2)))


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
