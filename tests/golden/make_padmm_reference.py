"""Golden vectors of proximal ADMM (CG-free CT-TV split) from the reference's own code.

Reads the reference's sources as text and runs, unchanged, under the float32
jax.numpy stand-in of make_xray2d_reference.py:

* ``ProximalADMM.step`` (scico/optimize/_padmm.py:349-362);
* ``SeparableFunctional.prox`` and ``ZeroFunctional.prox``
  (scico/functional/_functional.py:248-271, 376-379);
* ``SquaredL2Loss.prox`` (scico/loss.py:211-226; its Diagonal branch, taken
  for A = Identity);
* ``L21Norm`` / ``ScaledFunctional`` prox, ``SingleAxisFiniteDifference._eval``,
  ``VerticalStack._adj`` and the 2D projector (make_admm_reference.py);

on the split of the reference's ct_3d_tv_padmm example
(examples/scripts/ct_3d_tv_padmm.py:96-120): f = 0, g = (1/2 ||y - z0||^2,
(lambda / alpha) ||z1||_{2,1}), A = (C, alpha D) stacked, B = -I, c = 0,
with a 2D projector C.  Restated because JAX builds them rather than
scico's source: the operator algebra (``alpha * D`` evaluates
``alpha * D(x)`` with adjoint ``conj(alpha) * D.adj(y)``,
scico/linop/_linop.py:234-243; ``-Identity`` multiplies by the float32
diagonal -1, scico/linop/_diag.py:158-184), a BlockArray (blockwise
arithmetic) and the FD adjoint (jax's transpose rules).  mu and nu are
fixed numbers above ||A||^2 (the example estimates them by power
iteration).  Writes padmm_reference_code.npz: x, z and u after every
iteration.

Usage: python tests/golden/make_padmm_reference.py [/path/to/scico/checkout]
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
DEFAULT_CHECKOUT = Path("/root/reference")  # the reference checkout read as text
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent.parent))

from make_admm_reference import _exec, _source, build  # noqa: E402
from make_xray2d_reference import _wrap  # noqa: E402
from oracle import ctref  # noqa: E402


class BA:
    """BlockArray: a list of float32 arrays with blockwise arithmetic."""

    def __init__(self, blocks):
        self.blocks = [_wrap(np.asarray(b)) for b in blocks]

    @property
    def shape(self):
        return tuple(b.shape for b in self.blocks)

    def __iter__(self):
        return iter(self.blocks)

    def __len__(self):
        return len(self.blocks)

    def _op(self, other, f):
        if isinstance(other, BA):
            return BA([f(a, b) for a, b in zip(self.blocks, other.blocks)])
        return BA([f(a, other) for a in self.blocks])

    def __add__(self, o):
        return self._op(o, lambda a, b: a + b)

    def __radd__(self, o):
        return self._op(o, lambda a, b: b + a)

    def __sub__(self, o):
        return self._op(o, lambda a, b: a - b)

    def __rsub__(self, o):
        return self._op(o, lambda a, b: b - a)

    def __mul__(self, o):
        return self._op(o, lambda a, b: a * b)

    def __rmul__(self, o):
        return self._op(o, lambda a, b: b * a)


def main():
    checkout = Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_CHECKOUT
    R = build(checkout)
    X = R["X"]
    ns = {"snp": type("snp", (), {"blockarray": staticmethod(lambda bl: BA(bl))}), "np": np}

    class Diagonal:  # stands for scico.linop.Diagonal in SquaredL2Loss.prox's isinstance test
        pass

    ns["linop"] = type("linop", (), {"Diagonal": Diagonal, "LinearOperator": object})

    class Identity(Diagonal):
        diagonal = _wrap(np.ones((), np.float32))  # 1.0 * snp.ones((), float32)

        def conj(self):
            return self

        def __call__(self, v):
            return v

    class SquaredL2Loss:
        def __init__(self, y):
            self.y, self.A, self.W, self.scale = y, Identity(), Identity(), 0.5

    src = _source(checkout, "scico/loss.py", "SquaredL2Loss", ["prox"])
    _exec(src["prox"], ns, "loss.py:prox")
    SquaredL2Loss.prox = ns["prox"]

    class SeparableFunctional:
        def __init__(self, fl):
            self.functional_list = fl

    src = _source(checkout, "scico/functional/_functional.py", "SeparableFunctional", ["prox"])
    _exec(src["prox"], ns, "_functional.py:SeparableFunctional.prox")
    SeparableFunctional.prox = ns["prox"]

    class ZeroFunctional:
        pass

    src = _source(checkout, "scico/functional/_functional.py", "ZeroFunctional", ["prox"])
    _exec(src["prox"], ns, "_functional.py:ZeroFunctional.prox")
    ZeroFunctional.prox = ns["prox"]

    class ProximalADMM:
        pass

    src = _source(checkout, "scico/optimize/_padmm.py", "ProximalADMM", ["step"])
    _exec(src["step"], ns, "_padmm.py:step")
    ProximalADMM.step = ns["step"]

    out = {}
    cases = [dict(n=32, nv=24, lam=2.0, alpha=10.0, rho=0.05, iters=6, seed=1),
             dict(n=24, nv=30, lam=0.5, alpha=100.0, rho=5e-3, iters=5, seed=2)]
    for k, c in enumerate(cases):
        n, nv = c["n"], c["nv"]
        ang = np.linspace(0, np.pi, nv, endpoint=False).astype(np.float32)
        g = ctref.xray2d_defaults((n, n), ang)
        x0g, dx, y0, ny = _wrap(np.asarray(g["x0"], np.float32)), _wrap(np.asarray(g["dx"], np.float32)), \
            float(g["y0"]), g["ny"]
        alpha = c["alpha"]
        D = R["FiniteDifference"]((n, n), append=0)

        class Cop:
            def __call__(self, v):
                return X._project(_wrap(np.asarray(v, np.float32)), x0g, dx, y0, ny, _wrap(ang))

            def adj(self, s):
                return X._back_project(_wrap(np.asarray(s, np.float32)), x0g, dx, (n, n), y0, _wrap(ang))

        class AlphaD:  # alpha * D (LinearOperator.__mul__)
            def __call__(self, v):
                return alpha * D(v)

            def adj(self, w):
                return alpha * D.adj(w)  # snp.conj(alpha) of a real scalar is alpha

        class Stack:  # VerticalStack((C, alpha D)), BlockArray output
            def __init__(self):
                self.ops = [Cop(), AlphaD()]

            def __call__(self, v):
                return BA([op(v) for op in self.ops])

            def adj(self, w):
                return self._adj(w)

            @property
            def H(self):
                return type("H", (), {"__call__": lambda _s, w: self.adj(w)})()

        Stack._adj = R["FiniteDifference"]._adj

        class NegIdentity:  # -Identity: the float32 diagonal -1
            d = _wrap(np.asarray(-1.0, np.float32))

            def __call__(self, v):
                return self.d * v if not isinstance(v, BA) else v._op(self.d, lambda a, b: b * a)

            @property
            def H(self):
                return self

        rng = np.random.default_rng(c["seed"])
        im = rng.random((n, n)).astype(np.float32)
        y = np.asarray(Cop()(im)).astype(np.float32)
        y = (y + rng.normal(0, 0.01 * float(np.abs(y).max()), y.shape)).astype(np.float32)
        # ||A||^2 <= ||C||^2 + alpha^2 ||D||^2; power iteration on the oracle's float64 operators
        v = rng.standard_normal((n, n))
        for _ in range(60):
            w = ctref.xray2d_back_project(ctref.xray2d_project(v, g, np.float64), g, np.float64) + \
                alpha ** 2 * ctref.fd_adj(ctref.fd_eval(v, append=0), (n, n), append=0)
            v = w / np.linalg.norm(w)
        normsq = float(np.linalg.norm(ctref.xray2d_back_project(ctref.xray2d_project(v, g, np.float64), g,
                                                                np.float64)
                                      + alpha ** 2 * ctref.fd_adj(ctref.fd_eval(v, append=0), (n, n), append=0)))
        mu, nu = 1.01 * normsq, 1.01

        s = ProximalADMM()
        s.A, s.B, s.c = Stack(), NegIdentity(), 0.0
        s.f = ZeroFunctional()
        s.g = SeparableFunctional([SquaredL2Loss(_wrap(y)), R["ScaledFunctional"](R["L21Norm"](), c["lam"] / alpha)])
        s.rho, s.mu, s.nu = c["rho"], mu, nu
        s.x = _wrap(np.zeros((n, n), np.float32))
        s.z = BA([np.zeros(y.shape, np.float32), np.zeros((2, n, n), np.float32)])
        s.z_old = s.z
        s.u = BA([np.zeros(y.shape, np.float32), np.zeros((2, n, n), np.float32)])
        s.u_old = s.u
        xs = []
        for _ in range(c["iters"]):
            s.step()
            xs.append(np.asarray(s.x).astype(np.float32))
        p = f"c{k}_"
        out.update({p + "n": np.array(n), p + "nv": np.array(nv), p + "lam": np.array(c["lam"]),
                    p + "alpha": np.array(alpha), p + "rho": np.array(c["rho"]), p + "mu": np.array(mu),
                    p + "nu": np.array(nu), p + "y": y, p + "x": np.stack(xs),
                    p + "z0": np.asarray(s.z.blocks[0]), p + "z1": np.asarray(s.z.blocks[1]),
                    p + "u0": np.asarray(s.u.blocks[0]), p + "u1": np.asarray(s.u.blocks[1])})
        print(k, "mu", mu, "x norm", float(np.linalg.norm(xs[-1])))
    np.savez_compressed(HERE / "padmm_reference_code.npz", **out)


if __name__ == "__main__":
    main()
