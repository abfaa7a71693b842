"""Golden vectors of the MoDL unrolled CG from the reference's own code.

Reads scico/flax/inverse.py as text and runs the source of ``cg_solver``
(:113-158) unchanged under the float32 jax.numpy stand-in of
make_xray2d_reference.py, with ``lax.scan`` as a loop, on the MoDL system
(A^T A + lambda I) x = b of a small CT problem, A the reference's own
``_project`` / ``_back_project`` (run the same way) and the operator formed
as MoDLNet forms it (``ahaI_f``, :100).  jnp's float32 vector dot
(``p.ravel().conj().T @ Ap.ravel()``) is an XLA reduction whose summation
order cannot be reproduced here; the stand-in sums the float32 products
with NumPy's pairwise float32 sum, as the oracle's dot does.  Everything
else -- the recurrence, the order of the operations, the scalar types -- is
the reference's code.  Writes modl_cg_reference_code.npz.

Usage: python tests/golden/make_modl_cg_reference.py [/path/to/scico/checkout]
"""

from __future__ import annotations

import ast
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
DEFAULT_CHECKOUT = Path("/root/reference")  # the reference checkout read as text
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent.parent))

import make_xray2d_reference as mx  # noqa: E402
from oracle import ctref  # noqa: E402


class _JArrDot(mx.JArr):
    """JArr whose 1-D float32 ``@`` is the float32 pairwise sum of the products."""

    def __array_ufunc__(self, ufunc, method, *inputs, **kwargs):
        if ufunc is np.matmul and method == "__call__":
            a, b = (np.asarray(v) for v in inputs)
            if a.ndim == 1 and b.ndim == 1:
                return _wrapd(np.sum(a * b, dtype=a.dtype))
        out = super().__array_ufunc__(ufunc, method, *inputs, **kwargs)
        return _wrapd(out)


def _wrapd(x):
    if isinstance(x, tuple):
        return tuple(_wrapd(v) for v in x)
    if isinstance(x, np.ndarray):
        return np.asarray(x).view(_JArrDot)
    if isinstance(x, (np.floating, np.integer, np.bool_)):
        return np.asarray(x).view(_JArrDot)
    return x


class _JNPm(mx._JNP):
    @staticmethod
    def zeros_like(a):
        return _wrapd(np.zeros_like(np.asarray(a)))


class _LAXm:
    @staticmethod
    def scan(f, init, xs=None, length=None):
        carry = init
        for _ in range(length):
            carry, _ = f(carry, None)
        return carry, None


def reference_cg_solver(checkout: Path):
    src = (checkout / "scico/flax/inverse.py").read_text()
    node = next(n for n in ast.parse(src).body if isinstance(n, ast.FunctionDef) and n.name == "cg_solver")
    node.decorator_list = []
    for a in node.args.args + node.args.kwonlyargs:
        a.annotation = None
    node.returns = None
    ns = {"jnp": _JNPm(), "lax": _LAXm, "np": np}
    exec(compile(ast.unparse(node), "flax/inverse.py:cg_solver", "exec"), ns)
    return ns["cg_solver"]


CASES = [dict(n=24, nv=18, lmbda=0.1, maxiter=10, seed=1), dict(n=32, nv=30, lmbda=0.5, maxiter=6, seed=2)]


def main():
    checkout = Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_CHECKOUT
    X = mx.reference_functions(checkout)
    cg_solver = reference_cg_solver(checkout)
    out = {}
    for k, c in enumerate(CASES):
        n, nv = c["n"], c["nv"]
        ang = np.linspace(0, np.pi, nv, endpoint=False).astype(np.float32)
        g = ctref.xray2d_defaults((n, n), ang)
        x0, dx, y0, ny = (_wrapd(np.asarray(g["x0"], np.float32)), _wrapd(np.asarray(g["dx"], np.float32)),
                          float(g["y0"]), g["ny"])
        lmbda = _wrapd(np.ones((1,), np.float32) * np.float32(c["lmbda"]))  # MoDLNet's lmbda parameter

        def ahaI_f(v):  # MoDLNet (flax/inverse.py:100): A.adj(A(v)) + lmbda * v
            v = np.asarray(v, np.float32)
            av = X._project(mx._wrap(v), x0, dx, y0, ny, mx._wrap(ang))
            ata = np.asarray(X._back_project(mx._wrap(np.asarray(av)), x0, dx, (n, n), y0, mx._wrap(ang)))
            return _wrapd(ata) + lmbda * _wrapd(v)

        rng = np.random.default_rng(c["seed"])
        b = rng.random((n, n)).astype(np.float32)
        x = cg_solver(ahaI_f, _wrapd(b), maxiter=c["maxiter"])
        p = f"c{k}_"
        out.update({p + "n": np.array(n), p + "nv": np.array(nv), p + "lmbda": np.array(c["lmbda"]),
                    p + "maxiter": np.array(c["maxiter"]), p + "b": b, p + "x": np.asarray(x).astype(np.float32)})
        print(k, "x norm", float(np.linalg.norm(np.asarray(x))))
    np.savez_compressed(HERE / "modl_cg_reference_code.npz", **out)


if __name__ == "__main__":
    main()
