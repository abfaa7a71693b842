"""Regenerate the golden fixtures of the parity tests.

1. ``reference_kat.json`` -- the known-answer tests of scico's own test
   suite for this path, extracted (with ``ast``, no code execution) from the
   reference checkout:
     scico/test/linop/xray/test_xray_3d.py  test_scaling   (3D projector)
     scico/test/linop/test_diff.py          test_eval, test_eval_prepend,
                                            test_eval_append (FiniteDifference)
   Each entry records the source file and line of the literal.
2. ``oracle_small.npz`` -- float64 oracle outputs on small seeded cases
   (2D/3D projector, FD, prox, a short ADMM-TV solve), used as regression
   fixtures for the GPU parity tests so that those tests need no oracle
   run for their smallest cases.

Usage: python tests/golden/make_golden.py [/path/to/scico/checkout]
(the KAT extraction needs the checkout; the npz part does not).
"""

from __future__ import annotations

import ast
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))


def _array_literals(path: Path):
    """(lineno, value) of every literal first argument of a call to `array`."""
    tree = ast.parse(path.read_text())
    out = []
    for node in ast.walk(tree):
        if isinstance(node, ast.Call) and getattr(node.func, "attr", None) == "array" and node.args:
            try:
                out.append((node.lineno, ast.literal_eval(node.args[0])))
            except ValueError:
                pass
    return sorted(out, key=lambda t: t[0])


def extract_kats(ref_root: Path) -> dict:
    kat = {"source": "scico test suite (known-answer tests), extracted by tests/golden/make_golden.py"}
    p3 = ref_root / "scico/test/linop/xray/test_xray_3d.py"
    lits = [v for v in _array_literals(p3) if isinstance(v[1], list) and np.ndim(v[1]) == 3]
    # test_scaling: default spacing, then voxel_spacing=[2, 1, 1]
    kat["xray3d_scaling"] = {
        "file": "scico/test/linop/xray/test_xray_3d.py",
        "input": "x = zeros((4,4,1)); x[1:3,1:3,0] = 1; M = matrices_from_euler_angles(x.shape, x.shape[:2], 'X', [[0.0]])",
        "cases": [
            {"voxel_spacing": [1.0, 1.0, 1.0], "line": lits[0][0], "truth": lits[0][1]},
            {"voxel_spacing": [2.0, 1.0, 1.0], "line": lits[1][0], "truth": lits[1][1]},
        ],
    }
    pd = ref_root / "scico/test/linop/test_diff.py"
    lits = _array_literals(pd)
    byline = {ln: v for ln, v in lits}
    ev = [v for v in lits if isinstance(v[1], list)]
    # test_eval: x, Ax[0], Ax[1] (append=1), then the scaled repeats
    x2 = ev[0]
    kat["fd_eval_append1"] = {
        "file": "scico/test/linop/test_diff.py",
        "line": x2[0],
        "x": x2[1],
        "axis0": ev[1][1],
        "axis1": ev[2][1],
        "append": 1,
    }
    one_d = [v for v in ev if np.ndim(v[1]) == 1]
    kat["fd_1d"] = {
        "file": "scico/test/linop/test_diff.py",
        "x": [1, 2, 3, 4, 5],
        "cases": [
            {"prepend": 0, "append": None, "line": one_d[0][0], "truth": one_d[0][1]},
            {"prepend": 1, "append": None, "line": one_d[1][0], "truth": one_d[1][1]},
            {"prepend": None, "append": 0, "line": one_d[2][0], "truth": one_d[2][1]},
            {"prepend": None, "append": 1, "line": one_d[3][0], "truth": one_d[3][1]},
        ],
    }
    kat["l21_analytic"] = {
        "file": "scico/test/functional/test_norm.py",
        "line": 9,
        "x": "ones((3, 4, 5))",
        "axes": [[0], [1], [0, 2]],
        "value": "sqrt(prod(l2 shape)) * prod(l1 shape)",
        "prox_lam1": "(l2 - 1) / l2 * x with l2 = sqrt(prod(l2 shape))",
    }
    return kat


def oracle_fixtures() -> dict:
    from oracle import ctref
    from scico_gb300 import workloads

    out = {}
    # 2D: 24x20 image, 7 views, det 33 (default geometry) and a narrow detector
    rng = np.random.default_rng(7)
    im = rng.random((24, 20)).astype(np.float32)
    ang = np.linspace(0, np.pi, 7, endpoint=False)
    g = ctref.xray2d_defaults(im.shape, ang)
    out["p2_img"] = im
    out["p2_angles"] = ang
    out["p2_sino64"] = ctref.xray2d_project(im, g, np.float64)
    ys = rng.standard_normal((7, g["ny"])).astype(np.float32)
    out["p2_sino_in"] = ys
    out["p2_back64"] = ctref.xray2d_back_project(ys, g, np.float64)
    # 3D: 10x9x8 volume, 5 views about axis 0, det 12x14
    vol = rng.random((10, 9, 8)).astype(np.float32)
    M = ctref.xray3d_matrices_from_euler_angles(vol.shape, (12, 14), "X",
                                                np.linspace(0, np.pi, 5, endpoint=False)[:, None])
    out["p3_vol"] = vol
    out["p3_mats"] = M.astype(np.float32)
    out["p3_proj64"] = ctref.xray3d_project(vol, M.astype(np.float32), (12, 14), np.float64)
    # ADMM-TV: 32x32 phantom, 64 views, rho 50, CG converged each step
    # (tol 1e-5, <= 30 steps), 5 iterations
    x_gt = workloads.random_ellipses(32, 4, 11)
    ang2 = np.linspace(0, np.pi, 64, endpoint=False)
    g2 = ctref.xray2d_defaults(x_gt.shape, ang2)
    y = ctref.xray2d_project(x_gt, g2, np.float64).astype(np.float32)
    y = workloads.noisy(y, 0.01, 12)
    fwd = lambda v: ctref.xray2d_project(v, g2, np.float64)
    adj = lambda v: ctref.xray2d_back_project(v, g2, np.float64)
    x64, hist, _, _ = ctref.admm_tv(fwd, adj, y.astype(np.float64), x_gt.shape, lam_l21=0.02, rho=50.0,
                                     maxiter=5, cg_maxiter=30, cg_tol=1e-5, dtype=np.float64)
    out["admm_y"] = y
    out["admm_angles"] = ang2
    out["admm_x64"] = x64
    out["admm_obj64"] = np.array([h["Objective"] for h in hist])
    return out


def main():
    ref = Path(sys.argv[1]) if len(sys.argv) > 1 else Path("/root/reference")
    if (ref / "scico").is_dir():
        kat = extract_kats(ref)
        (HERE / "reference_kat.json").write_text(json.dumps(kat, indent=1) + "\n")
        print("wrote reference_kat.json")
    else:
        print(f"no scico checkout at {ref}; reference_kat.json left as committed")
    np.savez_compressed(HERE / "oracle_small.npz", **oracle_fixtures())
    print("wrote oracle_small.npz")


if __name__ == "__main__":
    main()
