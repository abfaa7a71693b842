"""Golden vectors of the 2D projector from the reference's own code.

JAX cannot be installed here, so scico itself cannot be imported.  This
script reads scico/linop/xray/_xray2d.py as text, takes the source of the
three functions that define the 2D projector -- ``_calc_weights``,
``_project`` and ``_back_project`` (the static methods of
XRayTransform2D) -- and executes those function bodies unchanged with a
small stand-in for the jax.numpy operations they use, with jax.numpy's
float32 semantics:

* integer arrays meeting float32 arrays give float32 (jax's promotion; NumPy
  would give float64), ``astype(int)`` gives int32 (x64 disabled);
* ``x.at[idx].add(v)`` is a sequential scatter-add (NumPy's ``add.at``);
* ``jax.vmap`` over the angles is a loop, ``jax.jit`` the identity;
* cos and sin of the float32 angles are the correctly rounded float32
  values.  XLA's float32 cos/sin may differ from these by an ulp; that is
  the one part of a scico run this cannot reproduce.

It writes xray2d_reference_code.npz: for a few seeded geometries and
images, the reference code's inds and weights, projection and back
projection.  tests/test_oracle.py checks the oracle against them and
tests/test_gpu_proj2d.py the GPU projector.

Usage: python tests/golden/make_xray2d_reference.py [/path/to/scico/checkout]
"""

from __future__ import annotations

import ast
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
DEFAULT_CHECKOUT = Path("/root/reference")  # the reference checkout read as text
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))

from oracle import ctref  # noqa: E402  (the constructor defaults)


class JArr(np.ndarray):
    """NumPy array with jax.numpy's float32 promotion and int32 ``astype(int)``."""

    def __array_ufunc__(self, ufunc, method, *inputs, **kwargs):
        args = [np.asarray(a) if isinstance(a, np.ndarray) else a for a in inputs]
        floats = [a.dtype for a in args if isinstance(a, np.ndarray) and a.dtype.kind == "f"]
        if not floats and any(isinstance(a, float) for a in args):
            floats = [np.dtype(np.float32)]  # a weak python float meets integers: float32
        if floats:
            ft = np.result_type(*floats)
            args = [a.astype(ft) if isinstance(a, np.ndarray) and a.dtype.kind in "iub" and ufunc.nin == 2 else a
                    for a in args]
        if "out" in kwargs:
            kwargs["out"] = tuple(np.asarray(o) for o in kwargs["out"])
        out = getattr(ufunc, method)(*args, **kwargs)
        return _wrap(out)

    def astype(self, dtype, *a, **k):
        if dtype is int:
            dtype = np.int32
        return _wrap(np.asarray(self).astype(dtype, *a, **k))

    @property
    def at(self):
        return _At(self)

    def __getitem__(self, idx):
        a = np.asarray(self)
        return _wrap(a[_clamped(_unwrap(idx), a.shape)])


def _unwrap(idx):
    if isinstance(idx, tuple):
        return tuple(np.asarray(i) if isinstance(i, np.ndarray) else i for i in idx)
    return np.asarray(idx) if isinstance(idx, np.ndarray) else idx


def _clamped(idx, shape):
    """jax.numpy gather indexing: negative integer indices count from the end,
    out-of-range ones are clamped (the reference multiplies such values by a
    zero weight)."""
    if not isinstance(idx, tuple):
        idx = (idx,)
    out = []
    for k, i in enumerate(idx):
        if isinstance(i, np.ndarray) and i.dtype.kind in "iu":
            i = np.where(i < 0, i + shape[k], i)
            i = np.clip(i, 0, shape[k] - 1)
        out.append(i)
    return tuple(out)


def _wrap(x):
    if isinstance(x, tuple):
        return tuple(_wrap(v) for v in x)
    if isinstance(x, np.ndarray):
        return x.view(JArr)
    if isinstance(x, (np.floating, np.integer, np.bool_)):
        return np.asarray(x).view(JArr)
    return x


class _At:
    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        arr = self.arr

        class _Upd:
            @staticmethod
            def add(v, mode=None):
                # jax.numpy scatter: negative indices count from the end,
                # updates at out-of-range indices are dropped; the others are
                # added one after another in index order
                out = np.array(arr, copy=True)
                ix = _unwrap(idx) if isinstance(idx, tuple) else (_unwrap(idx),)
                ix = np.broadcast_arrays(*[np.asarray(i) for i in ix])
                vals = np.broadcast_to(np.asarray(v), ix[0].shape).astype(out.dtype)
                keep = np.ones(ix[0].shape, dtype=bool)
                norm = []
                for k, i in enumerate(ix):
                    i = np.where(i < 0, i + out.shape[k], i)
                    keep &= (i >= 0) & (i < out.shape[k])
                    norm.append(i)
                np.add.at(out, tuple(i[keep] for i in norm), vals[keep])
                return _wrap(out)

        return _Upd


class _JNP:
    """The jax.numpy functions the three reference functions call."""

    float32 = np.float32

    @staticmethod
    def _f32round(fn, a):
        a = np.asarray(a)
        return _wrap(fn(a.astype(np.float64)).astype(a.dtype))

    def cos(self, a):
        return self._f32round(np.cos, a)

    def sin(self, a):
        return self._f32round(np.sin, a)

    @staticmethod
    def array(v, dtype=None):
        if isinstance(v, (list, tuple)):
            v = [np.asarray(x) for x in v]
        return _wrap(np.asarray(v, dtype=dtype) if dtype is not None else np.asarray(v))

    @staticmethod
    def zeros(shape, dtype=None, device=None):
        return _wrap(np.zeros(shape, dtype=dtype or np.float32))

    @staticmethod
    def arange(n):
        return _wrap(np.arange(n, dtype=np.int32))

    class _MGrid:
        def __getitem__(self, idx):
            return _wrap(np.mgrid[idx].astype(np.int32))

    mgrid = _MGrid()

    def __getattr__(self, name):  # min, max, abs, floor, minimum, where, sum
        fn = getattr(np, name)
        return lambda *a, **k: _wrap(fn(*[np.asarray(x) if isinstance(x, np.ndarray) else x for x in a], **k))


class _LAX:
    @staticmethod
    def map(f, xs, batch_size=None):
        return _wrap(np.stack([np.asarray(f(_wrap(np.asarray(x)))) for x in np.asarray(xs)]))

    @staticmethod
    def scan(f, init, xs):
        carry = init
        for k in range(len(np.asarray(xs[0]))):
            carry, _ = f(carry, tuple(_wrap(np.asarray(a)[k]) for a in xs))
        return carry, None


class _JAX:
    lax = _LAX

    @staticmethod
    def jit(f=None, **_):
        return f if f is not None else (lambda g: g)

    @staticmethod
    def vmap(f, in_axes):
        def mapped(*args):
            ax = [i for i, a in enumerate(in_axes) if a == 0][0]
            outs = [f(*(args[:ax] + (_wrap(np.asarray(v)),) + args[ax + 1:])) for v in np.asarray(args[ax])]
            return tuple(_wrap(np.stack([np.asarray(o[k]) for o in outs])) for k in range(len(outs[0])))

        return mapped


def reference_functions(checkout: Path):
    """The three static methods, their decorators replaced by the stand-ins."""
    src = (checkout / "scico/linop/xray/_xray2d.py").read_text()
    tree = ast.parse(src)
    cls = next(n for n in tree.body if isinstance(n, ast.ClassDef) and n.name == "XRayTransform2D")
    funcs = {n.name: n for n in cls.body if isinstance(n, ast.FunctionDef)
             and n.name in ("_calc_weights", "_project", "_back_project")}
    ns = {"jnp": _JNP(), "jax": _JAX, "np": np}
    holder = type("XRayTransform2D", (), {})
    ns["XRayTransform2D"] = holder
    for name in ("_calc_weights", "_project", "_back_project"):
        node = funcs[name]
        node.decorator_list = []
        for a in node.args.args:
            a.annotation = None
        node.returns = None
        code = ast.unparse(node)
        exec(compile(code, f"_xray2d.py:{name}", "exec"), ns)
        fn = ns[name]
        if name == "_calc_weights":
            fn = _JAX.vmap(fn, in_axes=(None, None, None, 0, None))
        setattr(holder, name, staticmethod(fn))
    return holder


CASES = [
    dict(shape=(24, 20), nv=7, seed=1),
    dict(shape=(33, 47), nv=17, dx=0.5, det=40, seed=2),
    dict(shape=(40, 40), nv=12, dx=1.0, det=60, seed=3),
    dict(shape=(64, 64), nv=45, seed=4),
    dict(shape=(70, 31), nv=29, det=30, seed=5),
]


def main():
    checkout = Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_CHECKOUT
    X = reference_functions(checkout)
    out = {}
    for k, c in enumerate(CASES):
        ang = np.linspace(0, np.pi, c["nv"], endpoint=False).astype(np.float32)
        g = ctref.xray2d_defaults(c["shape"], ang, dx=c.get("dx"), det_count=c.get("det"))
        x0 = _wrap(np.asarray(g["x0"], np.float32))
        dx = _wrap(np.asarray(g["dx"], np.float32))
        y0 = float(g["y0"])
        rng = np.random.default_rng(c["seed"])
        im = rng.random(c["shape"]).astype(np.float32)
        sino = rng.random((c["nv"], g["ny"])).astype(np.float32)
        inds, w = X._calc_weights(x0, dx, tuple(c["shape"]), _wrap(ang), y0)
        y = X._project(_wrap(im), x0, dx, y0, g["ny"], _wrap(ang))
        b = X._back_project(_wrap(sino), x0, dx, tuple(c["shape"]), y0, _wrap(ang))
        p = f"c{k}_"
        out.update({p + "shape": np.array(c["shape"]), p + "angles": ang, p + "dx": np.array(g["dx"]),
                    p + "det": np.array(g["ny"]), p + "image": im, p + "sino_in": sino,
                    p + "project": np.asarray(y).astype(np.float32),
                    p + "back_project": np.asarray(b).astype(np.float32)})
        if k < 2:  # the weight tables of the two smallest cases (the projections pin the rest)
            out.update({p + "inds": np.asarray(inds).astype(np.int32), p + "weights": np.asarray(w).astype(np.float32)})
    np.savez_compressed(HERE / "xray2d_reference_code.npz", **out)
    print("wrote", HERE / "xray2d_reference_code.npz", sum(v.nbytes for v in out.values()), "bytes")


if __name__ == "__main__":
    main()
