"""Golden vectors of the 3D projector from the reference's own code.

As make_xray2d_reference.py does for the 2D projector: reads
scico/linop/xray/_xray3d.py as text, takes the source of ``_project``,
``_project_single``, ``_back_project``, ``_back_project_single`` and
``_calc_weights`` (the static methods of XRayTransform3D, :110-266) and
``matrices_from_euler_angles`` (:268-327, with scipy's Rotation as the
reference imports it and scico.numpy.concatenate's float32 result) and runs
those function bodies unchanged under the same float32 jax.numpy stand-in
(``lax.map`` and ``lax.scan`` as loops, ``mgrid`` int32, scatter-adds with
``mode="drop"`` dropping out-of-range indices, gathers clamping).  The
geometries: rotation about axis 0 (the AXIS0 kernels), the reference's own
tilted "XY" example geometry (examples/scripts/ct_projector_comparison_3d.py:
44-50, the GENERAL kernels) and random matrices.  Writes
xray3d_reference_code.npz.

Usage: python tests/golden/make_xray3d_reference.py [/path/to/scico/checkout]
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

from make_xray2d_reference import _JAX, _JNP, _wrap  # noqa: E402
from oracle import ctref  # noqa: E402

NAMES = ("_calc_weights", "_project_single", "_back_project_single", "_project", "_back_project",
         "matrices_from_euler_angles")


class _SNP:
    """scico.numpy.concatenate as jax.numpy computes it with x64 disabled
    (float64 inputs become float32)."""

    @staticmethod
    def concatenate(arrs, axis=0):
        return np.concatenate([np.asarray(a) for a in arrs], axis=axis).astype(np.float32)


def reference_functions(checkout: Path):
    src = (checkout / "scico/linop/xray/_xray3d.py").read_text()
    tree = ast.parse(src)
    cls = next(n for n in tree.body if isinstance(n, ast.ClassDef) and n.name == "XRayTransform3D")
    funcs = {n.name: n for n in cls.body if isinstance(n, ast.FunctionDef) and n.name in NAMES}
    from scipy.spatial.transform import Rotation

    ns = {"jnp": _JNP(), "jax": _JAX, "np": np, "snp": _SNP, "Rotation": Rotation}
    holder = type("XRayTransform3D", (), {})
    ns["XRayTransform3D"] = holder
    for name in NAMES:
        node = funcs[name]
        node.decorator_list = []
        for a in node.args.args:
            a.annotation = None
        node.returns = None
        exec(compile(ast.unparse(node), f"_xray3d.py:{name}", "exec"), ns)
        setattr(holder, name, staticmethod(ns[name]))
    return holder


def cases(X):
    """(name, volume shape, detector shape, matrices, how the matrices were
    made); the Euler-angle matrices come from the reference's own
    matrices_from_euler_angles."""
    rng = np.random.default_rng(7)
    out = []
    shape = (12, 14, 10)
    det = (12, 20)
    ang = np.linspace(0, np.pi, 9, endpoint=False)
    out.append(("axis0", shape, det, X.matrices_from_euler_angles(shape, det, "X", ang[:, None]),
                ("X", ang[:, None], False)))
    # the reference's tilted geometry (rot_X 74 degrees, rot_Y over [0, 180))
    rot = np.stack(np.broadcast_arrays(90.0 - 16.0, np.linspace(0, 180, 5, endpoint=False)), axis=-1)
    out.append(("xy_tilted", shape, (22, 22), X.matrices_from_euler_angles(shape, (22, 22), "XY", rot, degrees=True),
                ("XY", rot, True)))
    m = rng.normal(size=(4, 2, 4)) * np.array([1.0, 1.0, 1.0, 3.0]) + np.array([0, 0, 0, 8.0])
    out.append(("random", (9, 11, 13), (18, 18), m.astype(np.float32), None))
    return out


def main():
    checkout = Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_CHECKOUT
    X = reference_functions(checkout)
    out = {}
    for k, (name, shape, det, M, euler) in enumerate(cases(X)):
        M = np.asarray(M, np.float32)
        rng = np.random.default_rng(100 + k)
        vol = rng.random(shape).astype(np.float32)
        proj = rng.random((len(M),) + tuple(det)).astype(np.float32)
        y = X._project(_wrap(vol), _wrap(M), tuple(det))
        b = X._back_project(_wrap(proj), _wrap(M), tuple(shape))
        p = f"c{k}_"
        out.update({p + "name": np.array(name), p + "shape": np.array(shape), p + "det": np.array(det),
                    p + "matrices": M, p + "volume": vol, p + "proj_in": proj,
                    p + "project": np.asarray(y).astype(np.float32),
                    p + "back_project": np.asarray(b).astype(np.float32)})
        if euler is not None:
            out.update({p + "euler_seq": np.array(euler[0]), p + "euler_angles": np.asarray(euler[1], np.float64),
                        p + "euler_degrees": np.array(euler[2])})
    np.savez_compressed(HERE / "xray3d_reference_code.npz", **out)
    print("wrote", HERE / "xray3d_reference_code.npz")


if __name__ == "__main__":
    main()
