"""Golden vectors of the CG x-update from the reference's own code.

Reads scico/solver.py as text and runs the source of ``cg`` (:326-405)
unchanged under the float32 jax.numpy stand-in of make_xray2d_reference.py
(scico.numpy's sum, maximum, sqrt, zeros and linalg.norm as jax.numpy
computes them on float32 arrays: norm = sqrt(sum(x * x)) in float32), on the
ADMM-TV x-update's system (rho D^T D + c A^T A) x = b of a small CT problem,
with A the reference's own _project / _back_project (run the same way) and
D the forward difference with append=0.  Two cases: CG stopped by its
tolerance and CG stopped by maxiter.  Writes cg_reference_code.npz.

Usage: python tests/golden/make_cg_reference.py [/path/to/scico/checkout]
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

from make_xray2d_reference import _JNP, _wrap, reference_functions  # noqa: E402
from oracle import ctref  # noqa: E402


class _SNP(_JNP):
    """scico.numpy as the CG uses it, on float32 arrays."""

    class linalg:
        @staticmethod
        def norm(x):
            x = np.asarray(x)
            return _wrap(np.sqrt(np.sum(x * x)))


def reference_cg(checkout: Path):
    src = (checkout / "scico/solver.py").read_text()
    node = next(n for n in ast.parse(src).body if isinstance(n, ast.FunctionDef) and n.name == "cg")
    node.decorator_list = []
    for a in node.args.args + node.args.kwonlyargs:
        a.annotation = None
    node.returns = None
    ns = {"snp": _SNP(), "LinearOperator": type("LinearOperator", (), {}), "np": np}
    exec(compile(ast.unparse(node), "solver.py:cg", "exec"), ns)
    return ns["cg"]


def dtd(q):
    """D^T D q, D = forward differences with append=0 over both axes, float32
    (the oracle's fd operators)."""
    d = ctref.fd_eval(q, axes=None, append=0)
    return ctref.fd_adj(d, q.shape, axes=None, append=0)


CASES = [dict(n=24, nv=18, tol=1e-4, maxiter=100, seed=1), dict(n=32, nv=24, tol=1e-6, maxiter=6, seed=2)]


def main():
    checkout = Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_CHECKOUT
    X = reference_functions(checkout)
    cg = reference_cg(checkout)
    out = {}
    for k, c in enumerate(CASES):
        n, nv = c["n"], c["nv"]
        ang = np.linspace(0, np.pi, nv, endpoint=False).astype(np.float32)
        g = ctref.xray2d_defaults((n, n), ang)
        x0, dx, y0, ny = _wrap(np.asarray(g["x0"], np.float32)), _wrap(np.asarray(g["dx"], np.float32)), float(g["y0"]), g["ny"]
        rho, scale = np.float32(2.0), np.float32(1.0)  # c = 2 * scale of 0.5 ||Ax - y||^2

        def A(v):
            v = np.asarray(v, np.float32)
            ata = np.asarray(X._back_project(X._project(_wrap(v), x0, dx, y0, ny, _wrap(ang)), x0, dx, (n, n), y0,
                                             _wrap(ang)))
            return _wrap(rho * dtd(v) + scale * ata)

        rng = np.random.default_rng(c["seed"])
        b = rng.random((n, n)).astype(np.float32)
        xs = (rng.random((n, n)) * 0.1).astype(np.float32)
        x, info = cg(A, _wrap(b), _wrap(xs), tol=c["tol"], maxiter=c["maxiter"])
        p = f"c{k}_"
        out.update({p + "n": np.array(n), p + "nv": np.array(nv), p + "tol": np.array(c["tol"]),
                    p + "maxiter": np.array(c["maxiter"]), p + "b": b, p + "x0": xs,
                    p + "x": np.asarray(x).astype(np.float32), p + "num_iter": np.array(info["num_iter"]),
                    p + "rel_res": np.array(float(np.asarray(info["rel_res"])))})
        print(k, "iterations", info["num_iter"], "rel_res", float(np.asarray(info["rel_res"])))
    np.savez_compressed(HERE / "cg_reference_code.npz", **out)


if __name__ == "__main__":
    main()
