"""Golden vectors of ADMM-TV iterations from the reference's own code.

JAX cannot be installed here, so scico itself cannot be imported.  This
script reads the reference's source files as text and executes, unchanged,
under the float32 jax.numpy stand-in of make_xray2d_reference.py:

* ``ADMM.step`` (scico/optimize/_admm.py:334-378) and the itstat quantities
  ``objective``, ``norm_primal_residual``, ``norm_dual_residual``
  (:210-295);
* ``LinearSubproblemSolver.compute_rhs`` and ``.solve``
  (scico/optimize/_admmaux.py:231-269);
* ``scico.solver.cg`` (scico/solver.py:326-405);
* ``L21Norm._l2norm``, ``._prox``, ``.prox``, ``.__call__``, ``L1Norm.prox``,
  ``.__call__``
  (scico/functional/_norm.py:238-296), ``ScaledFunctional.prox`` and
  ``__call__`` (scico/functional/_functional.py:159-198) and
  ``no_nan_divide`` (scico/numpy/util.py:302-315);
* ``SingleAxisFiniteDifference._eval`` (scico/linop/_diff.py:236-272) and
  ``VerticalStack._adj`` (scico/linop/_stack.py:71-72);
* ``SquaredL2Loss.__call__`` (scico/loss.py:208-209);
* the 2D projector's ``_project`` / ``_back_project``.

Two pieces are restated because they are built by JAX rather than written
in scico: the adjoint of a single-axis difference, which scico obtains with
jax.linear_transpose of ``_eval`` (written out below as the transpose rules
of jnp.diff's concatenate / slice / subtract), and the operator algebra of
``internal_init`` (``rho * C.gram_op + f.hessian`` evaluates
``rho * C.adj(C(x)) + 2 * scale * A.adj(W(A(x)))``, scico/loss.py:259).

It writes admm_reference_code.npz: per case the problem, the iterate x after
every iteration, the final z and u of every term, the CG step count of each
x-update and the float32 itstat values; the cases include L2,1 + L1 on the
same differences in 2D and on a volume with the reference's 3D projector
(make_xray3d_reference.py).  tests/test_oracle.py checks the oracle's
admm_tv against it bit for bit (iterates and step counts; itstat within
float32 summation rounding) and tests/test_gpu_admm.py the GPU solver.

Usage: python tests/golden/make_admm_reference.py [/path/to/scico/checkout]
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

from make_cg_reference import _SNP, reference_cg  # noqa: E402
from make_xray2d_reference import _wrap, reference_functions  # noqa: E402
from oracle import ctref  # noqa: E402


class _SNP2(_SNP):
    BlockArray = type("BlockArray", (), {})

    @staticmethod
    def diff(x, axis=-1, prepend=None, append=None):
        # jnp.diff: concatenate the prepended/appended values, then ext[1:] - ext[:-1]
        x = np.asarray(x)

        def edge(v):
            v = np.asarray(v, dtype=x.dtype)
            if v.ndim == 0:
                shp = list(x.shape)
                shp[axis] = 1
                v = np.broadcast_to(v, shp)
            return v

        parts = ([edge(prepend)] if prepend is not None else []) + [x] + \
            ([edge(append)] if append is not None else [])
        ext = np.concatenate(parts, axis=axis)
        hi = [slice(None)] * ext.ndim
        lo = [slice(None)] * ext.ndim
        hi[axis], lo[axis] = slice(1, None), slice(None, -1)
        return _wrap(ext[tuple(hi)] - ext[tuple(lo)])

    @staticmethod
    def stack(xs, axis=0):
        return _wrap(np.stack([np.asarray(x) for x in xs], axis=axis))

    class util:
        @staticmethod
        def is_complex_dtype(dtype):
            return np.dtype(dtype).kind == "c"


def _source(checkout: Path, rel: str, cls: str | None, names):
    """The named functions (methods of ``cls`` if given) of a reference file,
    with decorators and annotations removed."""
    tree = ast.parse((checkout / rel).read_text())
    body = tree.body
    if cls is not None:
        body = next(n for n in body if isinstance(n, ast.ClassDef) and n.name == cls).body
    out = {}
    for n in body:
        if isinstance(n, ast.FunctionDef) and n.name in names:
            n.decorator_list = []
            for a in n.args.args + n.args.kwonlyargs:
                a.annotation = None
            if n.args.vararg is not None:
                n.args.vararg.annotation = None
            if n.args.kwarg is not None:
                n.args.kwarg.annotation = None
            n.returns = None
            out[n.name] = ast.unparse(n)
    assert set(out) == set(names), (rel, cls, set(names) - set(out))
    return out


def _exec(src: str, ns: dict, label: str):
    exec(compile(src, label, "exec"), ns)


def build(checkout: Path):
    """The reference objects, assembled from the executed sources."""
    snp = _SNP2()
    ns = {"snp": snp, "np": np, "norm": snp.linalg.norm}

    fns = _source(checkout, "scico/numpy/util.py", None, ["no_nan_divide"])
    _exec(fns["no_nan_divide"], ns, "util.py:no_nan_divide")

    class L21Norm:
        def __init__(self, l2_axis=0):
            self.l2_axis = l2_axis

    ns["L21Norm"] = L21Norm
    src = _source(checkout, "scico/functional/_norm.py", "L21Norm", ["_l2norm", "_prox", "prox", "__call__"])
    for name in ("_l2norm", "_prox"):
        _exec(src[name], ns, f"_norm.py:{name}")
        setattr(L21Norm, name, staticmethod(ns[name]))
    for name in ("prox", "__call__"):
        _exec(src[name], ns, f"_norm.py:{name}")
        setattr(L21Norm, name, ns[name])

    class L1Norm:
        pass

    src = _source(checkout, "scico/functional/_norm.py", "L1Norm", ["prox", "__call__"])
    for name in ("prox", "__call__"):
        _exec(src[name], ns, f"_norm.py:L1Norm.{name}")
        setattr(L1Norm, name, staticmethod(ns[name]))

    class ScaledFunctional:
        def __init__(self, functional, scale):
            self.functional, self.scale = functional, scale

    src = _source(checkout, "scico/functional/_functional.py", "ScaledFunctional", ["prox", "__call__"])
    for name in ("prox", "__call__"):
        _exec(src[name], ns, f"_functional.py:{name}")
        setattr(ScaledFunctional, name, ns[name])

    class SingleAxisFiniteDifference:
        def __init__(self, shape, axis, append):
            self.input_shape, self.axis, self.append = shape, axis, append
            self.prepend, self.circular = None, False

        def __call__(self, x):
            return self._eval(x)

        def adj(self, ct):
            """jax.linear_transpose of _eval for append=0: with ext = concat(x,
            x[-1:]) and d = ext[1:] - ext[:-1], the cotangent of ext is
            pad(ct, (1, 0)) + pad(-ct, (0, 1)) and x[n-1] adds that of the
            appended copy."""
            assert self.append == 0 and self.prepend is None and not self.circular
            ct = np.moveaxis(np.asarray(ct), self.axis, 0)
            z = np.zeros_like(ct[:1])
            ext = np.concatenate([z, ct]) + np.concatenate([-ct, z])
            n = self.input_shape[self.axis]
            out = ext[:n].copy()
            out[n - 1] = out[n - 1] + ext[n]
            return _wrap(np.moveaxis(out, 0, self.axis))

    src = _source(checkout, "scico/linop/_diff.py", "SingleAxisFiniteDifference", ["_eval"])
    _exec(src["_eval"], ns, "_diff.py:_eval")
    SingleAxisFiniteDifference._eval = ns["_eval"]

    class FiniteDifference:  # a VerticalStack of single-axis differences, collapse_output
        def __init__(self, shape, append=0):
            self.input_shape, self.input_dtype = shape, np.float32
            self.ops = [SingleAxisFiniteDifference(shape, a, append) for a in range(len(shape))]

        def __call__(self, x):
            return snp.stack([op(x) for op in self.ops])

        def adj(self, y):
            return self._adj(y)

    src = _source(checkout, "scico/linop/_stack.py", "VerticalStack", ["_adj"])
    _exec(src["_adj"], ns, "_stack.py:_adj")
    FiniteDifference._adj = ns["_adj"]

    class SquaredL2Loss:
        def __init__(self, y, A, scale=0.5):
            self.y, self.A, self.scale = y, A, scale

            class W:
                diagonal = _wrap(np.ones(np.asarray(y).shape, np.float32))

                def __call__(self, v):
                    return v

            self.W = W()

    src = _source(checkout, "scico/loss.py", "SquaredL2Loss", ["__call__"])
    _exec(src["__call__"], ns, "loss.py:__call__")
    SquaredL2Loss.__call__ = ns["__call__"]

    class LinearSubproblemSolver:
        def __init__(self, cg, cg_kwargs):
            self.cg, self.cg_kwargs, self.device, self.info = cg, cg_kwargs, None, None

        def internal_init(self, admm):
            self.admm = admm
            f = admm.f

            # reduce(+, [rho_i * C_i.gram_op]) + f.hessian (operator sums and
            # scalar multiples, _admmaux.py:222-227)
            def lhs(x):
                acc = None
                for rho, C in zip(admm.rho_list, admm.C_list):
                    t = rho * C.adj(C(x))
                    acc = t if acc is None else acc + t
                return acc + 2 * f.scale * f.A.adj(f.W(f.A(x)))

            self.lhs_op = lhs

    src = _source(checkout, "scico/optimize/_admmaux.py", "LinearSubproblemSolver", ["compute_rhs", "solve"])
    for name in ("compute_rhs", "solve"):
        _exec(src[name], ns, f"_admmaux.py:{name}")
        setattr(LinearSubproblemSolver, name, ns[name])

    class ADMM:
        def __init__(self, f, g_list, C_list, rho_list, subproblem_solver, x0):
            self.f, self.g_list, self.C_list, self.rho_list = f, g_list, C_list, rho_list
            self.alpha = 1.0
            self.x = x0
            self.z_list = [C(x0) for C in C_list]  # z_init (_admm.py:297-315)
            self.z_list_old = self.z_list.copy()
            self.u_list = [_wrap(np.zeros(np.asarray(z).shape, np.float32)) for z in self.z_list]
            self.subproblem_solver = subproblem_solver
            subproblem_solver.internal_init(self)

    src = _source(checkout, "scico/optimize/_admm.py", "ADMM",
                  ["step", "objective", "norm_primal_residual", "norm_dual_residual"])
    for name in ("step", "objective", "norm_primal_residual", "norm_dual_residual"):
        _exec(src[name], ns, f"_admm.py:{name}")
        setattr(ADMM, name, ns[name])

    return dict(L21Norm=L21Norm, L1Norm=L1Norm, ScaledFunctional=ScaledFunctional, FiniteDifference=FiniteDifference,
                SquaredL2Loss=SquaredL2Loss, LinearSubproblemSolver=LinearSubproblemSolver, ADMM=ADMM,
                cg=reference_cg(checkout), X=reference_functions(checkout))


# Two regimes with one L2,1 term: CG stopped by its tolerance in every
# x-update (rho = 50), and the benchmark-like split (rho = 2, lambda 0.005,
# CG capped at 10 steps); then L2,1 and L1 on the same differences, in 2D and
# on a volume (the 3D workload's two-term pattern, rho 1, CG capped at 8).
CASES = [
    dict(kind=2, n=24, nv=18, lam=0.05, lam1=0.0, rho=50.0, cg_tol=1e-4, cg_maxiter=100, iters=6, seed=1),
    dict(kind=2, n=32, nv=24, lam=0.005, lam1=0.0, rho=2.0, cg_tol=1e-4, cg_maxiter=10, iters=8, seed=2),
    dict(kind=2, n=28, nv=20, lam=0.01, lam1=0.005, rho=1.0, cg_tol=1e-4, cg_maxiter=10, iters=6, seed=3),
    dict(kind=3, shape=(10, 12, 12), det=(10, 18), nv=12, lam=0.01, lam1=0.01, rho=1.0, cg_tol=1e-4,
         cg_maxiter=8, iters=4, seed=4),
]


def main():
    checkout = Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_CHECKOUT
    R = build(checkout)
    X = R["X"]
    X3 = None
    out = {}
    for k, c in enumerate(CASES):
        rng = np.random.default_rng(c["seed"])
        extra = {}
        if c["kind"] == 2:
            n, nv = c["n"], c["nv"]
            shape = (n, n)
            ang = np.linspace(0, np.pi, nv, endpoint=False).astype(np.float32)
            g = ctref.xray2d_defaults(shape, ang)
            x0g, dx, y0, ny = _wrap(np.asarray(g["x0"], np.float32)), _wrap(np.asarray(g["dx"], np.float32)), \
                float(g["y0"]), g["ny"]

            class A:  # the 2D projector as a LinearOperator
                def __call__(self, v):
                    return X._project(_wrap(np.asarray(v, np.float32)), x0g, dx, y0, ny, _wrap(ang))

                def adj(self, s):
                    return X._back_project(_wrap(np.asarray(s, np.float32)), x0g, dx, shape, y0, _wrap(ang))

            extra = {"n": np.array(n), "nv": np.array(nv)}
        else:
            if X3 is None:
                import make_xray3d_reference as m3

                X3 = m3.reference_functions(checkout)
            shape, det, nv = tuple(c["shape"]), tuple(c["det"]), c["nv"]
            ang = np.linspace(0, np.pi, nv, endpoint=False)
            M = np.asarray(X3.matrices_from_euler_angles(shape, det, "X", ang[:, None]), np.float32)

            class A:  # the 3D projector (rotation about axis 0) as a LinearOperator
                def __call__(self, v):
                    return X3._project(_wrap(np.asarray(v, np.float32)), _wrap(M), det)

                def adj(self, s):
                    return X3._back_project(_wrap(np.asarray(s, np.float32)), _wrap(M), shape)

            extra = {"shape": np.array(shape), "det": np.array(det), "M": M}
        im = rng.random(shape).astype(np.float32)
        y = np.asarray(A()(im)).astype(np.float32)
        y = (y + rng.normal(0, 0.01 * float(np.abs(y).max()), y.shape)).astype(np.float32)

        f = R["SquaredL2Loss"](_wrap(y), A())
        C = R["FiniteDifference"](shape, append=0)
        gl, cl = [R["ScaledFunctional"](R["L21Norm"](), c["lam"])], [C]
        if c["lam1"]:
            gl.append(R["ScaledFunctional"](R["L1Norm"](), c["lam1"]))
            cl.append(C)
        sp = R["LinearSubproblemSolver"](R["cg"], {"tol": c["cg_tol"], "maxiter": c["cg_maxiter"]})
        admm = R["ADMM"](f, gl, cl, [c["rho"]] * len(gl), sp, _wrap(np.zeros(shape, np.float32)))
        xs, its, stats = [], [], []
        for _ in range(c["iters"]):
            admm.step()
            xs.append(np.asarray(admm.x).astype(np.float32))
            its.append(int(sp.info["num_iter"]))
            stats.append([float(np.asarray(admm.objective())), float(np.asarray(admm.norm_primal_residual())),
                          float(np.asarray(admm.norm_dual_residual()))])
        p = f"c{k}_"
        out.update({p + key: v for key, v in extra.items()})
        out.update({p + "kind": np.array(c["kind"]), p + "lam": np.array(c["lam"]), p + "lam1": np.array(c["lam1"]),
                    p + "rho": np.array(c["rho"]), p + "cg_tol": np.array(c["cg_tol"]),
                    p + "cg_maxiter": np.array(c["cg_maxiter"]), p + "y": y, p + "x": np.stack(xs),
                    p + "z": np.stack([np.asarray(z).astype(np.float32) for z in admm.z_list]),
                    p + "u": np.stack([np.asarray(u).astype(np.float32) for u in admm.u_list]),
                    p + "cg_iters": np.array(its), p + "itstat": np.array(stats)})
        print(k, "CG steps", its, "objective", [s[0] for s in stats])
    np.savez_compressed(HERE / "admm_reference_code.npz", **out)
    print("wrote", HERE / "admm_reference_code.npz", sum(v.nbytes for v in out.values()), "bytes")


if __name__ == "__main__":
    main()
