"""The CPU oracle against the reference's own known-answer tests and the
analytic properties its tests check (no GPU)."""

import json
from pathlib import Path

import numpy as np
import pytest

from oracle import ctref

GOLDEN = Path(__file__).resolve().parent / "golden"
KAT = json.loads((GOLDEN / "reference_kat.json").read_text())


@pytest.mark.parametrize("case", range(2))
def test_xray3d_scaling_kat(case):
    """scico/test/linop/xray/test_xray_3d.py:29-60 (test_scaling)."""
    c = KAT["xray3d_scaling"]["cases"][case]
    x = np.zeros((4, 4, 1), dtype=np.float32)
    x[1:3, 1:3, 0] = 1.0
    M = ctref.xray3d_matrices_from_euler_angles(x.shape, x.shape[:2], "X", [[0.0]],
                                                voxel_spacing=c["voxel_spacing"])
    for dt in (np.float32, np.float64):
        y = ctref.xray3d_project(x, M.astype(dt), x.shape[:2], dt)
        np.testing.assert_allclose(y, np.array(c["truth"]), rtol=1e-7, atol=0)


def test_fd_eval_kat():
    """scico/test/linop/test_diff.py:11-31 (test_eval, append=1)."""
    k = KAT["fd_eval_append1"]
    x = np.array(k["x"], dtype=np.float32)
    blocks = ctref.fd_eval(x, append=1)
    np.testing.assert_array_equal(blocks[0], np.array(k["axis0"]))
    np.testing.assert_array_equal(blocks[1], np.array(k["axis1"]))
    np.testing.assert_array_equal(2.0 * blocks[0], 2.0 * np.array(k["axis0"]))


@pytest.mark.parametrize("case", range(4))
def test_fd_1d_kat(case):
    """scico/test/linop/test_diff.py:50-65 (prepend / append values)."""
    c = KAT["fd_1d"]["cases"][case]
    x = np.array(KAT["fd_1d"]["x"], dtype=np.float32)
    y = ctref.fd_single(x, 0, c["prepend"], c["append"])
    np.testing.assert_array_equal(y, np.array(c["truth"]))


@pytest.mark.parametrize("axis", [0, 1, (0, 2)])
def test_l21_analytic(axis):
    """scico/test/functional/test_norm.py:9-28."""
    x = np.ones((3, 4, 5), dtype=np.float32)
    l2axis = (axis,) if isinstance(axis, int) else axis
    l2shape = [x.shape[k] for k in l2axis]
    l1shape = [x.shape[k] for k in set(range(3)) - set(l2axis)]
    ana = np.sqrt(np.prod(l2shape)) * np.prod(l1shape)
    np.testing.assert_allclose(ctref.l21_norm(x, l2axis), ana, rtol=1e-5)
    l2 = np.sqrt(np.prod(l2shape))
    np.testing.assert_allclose(ctref.l21_prox(x, 1.0, l2axis), (l2 - 1.0) / l2 * x, rtol=1e-5)


@pytest.mark.parametrize("shape", [(16,), (16, 24), (5, 6, 7)])
@pytest.mark.parametrize("mode", ["none", "pre0", "pre1", "app0", "app1", "both01", "circ"])
def test_fd_adjoint_dot(shape, mode):
    """Dot test of the FD adjoint (test_diff.py:68-78), float64."""
    kw = dict(none={}, pre0=dict(prepend=0), pre1=dict(prepend=1), app0=dict(append=0),
              app1=dict(append=1), both01=dict(prepend=0, append=1), circ=dict(circular=True))[mode]
    rng = np.random.default_rng(0)
    x = rng.standard_normal(shape)
    for ax in range(len(shape)):
        d = ctref.fd_single(x, ax, kw.get("prepend"), kw.get("append"), kw.get("circular", False))
        r = rng.standard_normal(d.shape)
        back = ctref.fd_single_adj(r, shape[ax], ax, kw.get("prepend"), kw.get("append"), kw.get("circular", False))
        np.testing.assert_allclose(np.sum(d * r), np.sum(x * back), rtol=1e-12)


@pytest.mark.parametrize("shape", [(1,), (2,), (16,), (5, 6, 7)])
@pytest.mark.parametrize("mode", ["none", "pre0", "pre1", "app0", "app1", "both00", "both01", "circ"])
def test_fd_adjoint_is_the_jax_transpose(shape, mode):
    """The oracle's single-axis adjoint against the transpose jax builds for
    jnp.diff (scico obtains FiniteDifference.adj by jax.linear_transpose of
    _eval, scico/linop/_diff.py:236-272): the extended line's cotangent
    pad(d, (1, 0)) + pad(-d, (0, 1)), its x part, plus the cotangents of the
    copied end samples; float32, bit for bit, on arbitrary d (not only on
    the range of D, where the copied ends hold 0)."""
    kw = dict(none={}, pre0=dict(prepend=0), pre1=dict(prepend=1), app0=dict(append=0),
              app1=dict(append=1), both00=dict(prepend=0, append=0), both01=dict(prepend=0, append=1),
              circ=dict(circular=True))[mode]
    pre, app, circ = kw.get("prepend"), kw.get("append"), kw.get("circular", False)
    rng = np.random.default_rng(3)
    x = rng.standard_normal(shape).astype(np.float32)
    for ax in range(len(shape)):
        n = shape[ax]
        d = ctref.fd_single(x, ax, pre, app, circ)
        r = rng.standard_normal(d.shape).astype(np.float32)
        ct = np.moveaxis(r, ax, 0)
        zero = np.zeros((1,) + ct.shape[1:], np.float32)
        ce = np.concatenate([zero, ct]) + np.concatenate([-ct, zero])
        P = 1 if pre is not None else 0
        want = ce[P:P + n].copy()
        if pre == 0:
            want[0] = ce[0] + want[0]
        if app == 0:
            want[n - 1] = want[n - 1] + ce[n + P]
        if circ:
            want[0] = want[0] + ce[n]
        got = ctref.fd_single_adj(r, n, ax, pre, app, circ)
        assert np.array_equal(got, np.moveaxis(want, 0, ax)), (ax, mode)


def test_xray2d_angle0_sums_rows():
    """Angle 0 sums image rows (_xray2d.py:66-70): exact with unit pixels."""
    rng = np.random.default_rng(1)
    im = rng.integers(0, 9, size=(12, 12)).astype(np.float32)
    g = ctref.xray2d_defaults(im.shape, np.array([0.0]), dx=1.0, det_count=12)
    y = ctref.xray2d_project(im, g, np.float32)
    np.testing.assert_array_equal(y[0], im.sum(axis=1))


def test_xray2d_angle90_sums_columns():
    rng = np.random.default_rng(2)
    im = rng.random((10, 10)).astype(np.float32)
    g = ctref.xray2d_defaults(im.shape, np.array([np.pi / 2]), dx=1.0, det_count=10)
    y = ctref.xray2d_project(im, g, np.float64)
    np.testing.assert_allclose(y[0], im.sum(axis=0), rtol=1e-5, atol=1e-5)


def test_xray2d_mass_and_adjoint():
    """Every pixel splits w + (1-w) = 1 over two bins; matched adjoint
    (test_xray_2d.py:52-85)."""
    rng = np.random.default_rng(3)
    im = rng.random((12, 13)).astype(np.float32)
    ang = np.linspace(0, np.pi, 10, endpoint=False)
    g = ctref.xray2d_defaults(im.shape, ang)
    y = ctref.xray2d_project(im, g, np.float64)
    np.testing.assert_allclose(y.sum(axis=1), np.full(10, im.astype(np.float64).sum()), rtol=1e-12)
    yr = rng.standard_normal(y.shape)
    bp = ctref.xray2d_back_project(yr, g, np.float64)
    np.testing.assert_allclose(np.sum(y * yr), np.sum(im * bp), rtol=1e-12)
    # narrow detector, N=16, det=int(16*1.05/sqrt2), dx=1/sqrt2 (:77-85)
    g2 = ctref.xray2d_defaults((16, 16), np.linspace(0, np.pi, 3, endpoint=False), dx=1 / np.sqrt(2),
                               det_count=int(16 * 1.05 / np.sqrt(2.0)))
    x = rng.standard_normal((16, 16)).astype(np.float32)
    y2 = ctref.xray2d_project(x, g2, np.float32)
    yr2 = rng.standard_normal(y2.shape).astype(np.float32)
    bp2 = ctref.xray2d_back_project(yr2, g2, np.float32)
    a, b = float(np.sum(y2.astype(np.float64) * yr2)), float(np.sum(x.astype(np.float64) * bp2))
    assert abs(a - b) / max(abs(a), abs(b)) < 1e-5


def _reference_code_cases():
    z = np.load(GOLDEN / "xray2d_reference_code.npz")
    for k in range(len([n for n in z.files if n.endswith("_image")])):
        p = f"c{k}_"
        g = ctref.xray2d_defaults(tuple(int(v) for v in z[p + "shape"]), z[p + "angles"],
                                  dx=tuple(float(v) for v in z[p + "dx"]), det_count=int(z[p + "det"]))
        yield k, z, p, g


def test_xray2d_oracle_is_the_reference_code():
    """The float32 2D projector oracle against the reference's own
    _calc_weights / _project / _back_project (scico/linop/xray/_xray2d.py:
    223-351) executed under a float32 jax.numpy stand-in
    (tests/golden/make_xray2d_reference.py): bit-identical weights, detector
    indices, projections and back projections on five geometries."""
    n = 0
    for k, z, p, g in _reference_code_cases():
        if p + "inds" in z.files:
            inds, w = ctref.xray2d_calc_weights(g)
            assert np.array_equal(inds, z[p + "inds"]) and np.array_equal(w, z[p + "weights"]), k
        assert np.array_equal(ctref.xray2d_project(z[p + "image"], g, np.float32), z[p + "project"]), k
        assert np.array_equal(ctref.xray2d_back_project(z[p + "sino_in"], g, np.float32), z[p + "back_project"]), k
        n += 1
    assert n == 5


def test_xray3d_oracle_is_the_reference_code():
    """The float32 3D projector oracle and its matrices_from_euler_angles
    against the reference's own code (scico/linop/xray/_xray3d.py:110-327)
    executed under a float32 jax.numpy stand-in
    (tests/golden/make_xray3d_reference.py): bit-identical matrices,
    projections and back projections for rotation about axis 0, the
    reference's tilted "XY" example geometry and random matrices."""
    z = np.load(GOLDEN / "xray3d_reference_code.npz")
    for k in range(3):
        p = f"c{k}_"
        shape = tuple(int(v) for v in z[p + "shape"])
        det = tuple(int(v) for v in z[p + "det"])
        if p + "euler_seq" in z.files:
            M = ctref.xray3d_matrices_from_euler_angles(shape, det, str(z[p + "euler_seq"]), z[p + "euler_angles"],
                                                        degrees=bool(z[p + "euler_degrees"]))
            assert np.array_equal(np.asarray(M, np.float32), z[p + "matrices"]), k
        M = z[p + "matrices"]
        assert np.array_equal(ctref.xray3d_project(z[p + "volume"], M, det, np.float32), z[p + "project"]), k
        assert np.array_equal(ctref.xray3d_back_project(z[p + "proj_in"], M, shape, np.float32),
                              z[p + "back_project"]), k


def test_cg_oracle_is_the_reference_code():
    """The oracle's CG (scico.solver.cg restated) against scico's own cg
    (scico/solver.py:326-405) executed under the float32 jax.numpy stand-in
    on the ADMM-TV x-update system rho D^T D + A^T A with the reference's
    own projector code (tests/golden/make_cg_reference.py): bit-identical
    iterates, step counts and relative residuals, stopped by the tolerance
    (32 steps) and by maxiter (6)."""
    z = np.load(GOLDEN / "cg_reference_code.npz")
    for k in range(2):
        p = f"c{k}_"
        n, nv = int(z[p + "n"]), int(z[p + "nv"])
        g = ctref.xray2d_defaults((n, n), np.linspace(0, np.pi, nv, endpoint=False).astype(np.float32))

        def A(v):
            dtd = ctref.fd_adj(ctref.fd_eval(v, axes=None, append=0), v.shape, axes=None, append=0)
            ata = ctref.xray2d_back_project(ctref.xray2d_project(v, g, np.float32), g, np.float32)
            return np.float32(2.0) * dtd + np.float32(1.0) * ata

        x, info = ctref.cg(A, z[p + "b"], z[p + "x0"], tol=float(z[p + "tol"]), maxiter=int(z[p + "maxiter"]))
        assert np.array_equal(x, z[p + "x"]), k
        assert info["num_iter"] == int(z[p + "num_iter"]) and info["rel_res"] == float(z[p + "rel_res"]), k


def _admm_operators(z, p):
    """The case's projector pair (the oracle's float32 2D or 3D projector)
    and image shape."""
    if int(z[p + "kind"]) == 2:
        n, nv = int(z[p + "n"]), int(z[p + "nv"])
        g = ctref.xray2d_defaults((n, n), np.linspace(0, np.pi, nv, endpoint=False).astype(np.float32))
        return (lambda v: ctref.xray2d_project(v, g, np.float32),
                lambda s: ctref.xray2d_back_project(s, g, np.float32), (n, n))
    shape, det, M = tuple(int(v) for v in z[p + "shape"]), tuple(int(v) for v in z[p + "det"]), z[p + "M"]
    return (lambda v: ctref.xray3d_project(v, M, det, np.float32),
            lambda s: ctref.xray3d_back_project(s, M, shape, np.float32), shape)


def test_admm_oracle_is_the_reference_code():
    """The oracle's ADMM-TV against scico's own ADMM.step, LinearSubproblemSolver
    .compute_rhs/.solve, cg, L21Norm / L1Norm prox, FiniteDifference and
    projector code executed under the float32 jax.numpy stand-in
    (tests/golden/make_admm_reference.py): the iterate x after every
    iteration, the final z and u of every term and every x-update's CG step
    count are bit-identical -- CG stopped by its tolerance (rho 50), capped at
    10 steps (rho 2, lambda 0.005), and L2,1 + L1 on the same differences in
    2D and on a volume with the 3D projector.  The itstat values, which the
    reference sums in float32 and the oracle in float64, agree to 1e-6."""
    z = np.load(GOLDEN / "admm_reference_code.npz")
    for k in range(4):
        p = f"c{k}_"
        fwd, adj, shape = _admm_operators(z, p)
        kw = dict(lam_l21=float(z[p + "lam"]), lam_l1=float(z[p + "lam1"]), rho=float(z[p + "rho"]),
                  cg_tol=float(z[p + "cg_tol"]), cg_maxiter=int(z[p + "cg_maxiter"]))
        X = z[p + "x"]
        for it in (1, len(X)):
            x, hist, zl, ul = ctref.admm_tv(fwd, adj, z[p + "y"], shape, maxiter=it, dtype=np.float32, **kw)
            assert np.array_equal(x, X[it - 1]), (k, it)
        assert all(np.array_equal(a, b) for a, b in zip(zl, z[p + "z"])), k
        assert all(np.array_equal(a, b) for a, b in zip(ul, z[p + "u"])), k
        assert [h["CG_It"] for h in hist] == list(z[p + "cg_iters"]), k
        ours = np.array([[h["Objective"], h["Prml_Rsdl"], h["Dual_Rsdl"]] for h in hist])
        np.testing.assert_allclose(ours, z[p + "itstat"], rtol=1e-6)


def test_modl_cg_oracle_is_the_reference_code():
    """The oracle's fixed-iteration CG (cg_fixed) against scico.flax's own
    cg_solver (flax/inverse.py:113-158) executed under the float32
    jax.numpy stand-in on MoDLNet's system A^T A + lambda I with the
    reference projector (tests/golden/make_modl_cg_reference.py): the same
    iterate bit for bit, at lambda 0.1 / 10 steps and 0.5 / 6 steps."""
    z = np.load(GOLDEN / "modl_cg_reference_code.npz")
    for k in range(2):
        p = f"c{k}_"
        n, nv = int(z[p + "n"]), int(z[p + "nv"])
        g = ctref.xray2d_defaults((n, n), np.linspace(0, np.pi, nv, endpoint=False).astype(np.float32))
        lm = np.float32(float(z[p + "lmbda"]))

        def A(v):
            return ctref.xray2d_back_project(ctref.xray2d_project(v, g, np.float32), g, np.float32) + lm * v

        x = ctref.cg_fixed(A, z[p + "b"], maxiter=int(z[p + "maxiter"]))
        assert np.array_equal(x, z[p + "x"]), k


def test_padmm_oracle_is_the_reference_code():
    """The oracle's proximal ADMM (padmm_tv, float32) against scico's own
    ProximalADMM.step, SeparableFunctional / ZeroFunctional / SquaredL2Loss /
    L21Norm prox, FiniteDifference and projector code executed under the
    float32 jax.numpy stand-in on the ct_3d_tv_padmm split with a 2D
    projector (tests/golden/make_padmm_reference.py): x after every
    iteration bit for bit."""
    z = np.load(GOLDEN / "padmm_reference_code.npz")
    for k in range(2):
        p = f"c{k}_"
        n, nv = int(z[p + "n"]), int(z[p + "nv"])
        g = ctref.xray2d_defaults((n, n), np.linspace(0, np.pi, nv, endpoint=False).astype(np.float32))
        fwd = lambda v: ctref.xray2d_project(v, g, np.float32)
        adj = lambda s: ctref.xray2d_back_project(s, g, np.float32)
        X = z[p + "x"]
        for it in (1, len(X)):
            x, _ = ctref.padmm_tv(fwd, adj, z[p + "y"], (n, n), lam=float(z[p + "lam"]), alpha=float(z[p + "alpha"]),
                                  rho=float(z[p + "rho"]), mu=float(z[p + "mu"]), nu=float(z[p + "nu"]), maxiter=it,
                                  dtype=np.float32)
            assert np.array_equal(x, X[it - 1]), (k, it)


def test_xray2d_f32_vs_f64():
    rng = np.random.default_rng(4)
    im = rng.random((20, 20)).astype(np.float32)
    g = ctref.xray2d_defaults(im.shape, np.linspace(0, np.pi, 9, endpoint=False))
    y32 = ctref.xray2d_project(im, g, np.float32)
    y64 = ctref.xray2d_project(im, g, np.float64)
    assert ctref.rel_l2(y32, y64) < 1e-6


def test_xray3d_adjoint_dot():
    """test_xray_3d.py:9-26 (matched adjoint, 3 views about 'X')."""
    N = 16
    det = int(N * 1.05 / np.sqrt(2.0))
    M = ctref.xray3d_matrices_from_euler_angles((N, N, N), (det, det), "X",
                                                np.linspace(0, np.pi, 3, endpoint=False)[:, None])
    rng = np.random.default_rng(5)
    x = rng.standard_normal((N, N, N))
    y = ctref.xray3d_project(x, M, (det, det), np.float64)
    r = rng.standard_normal(y.shape)
    bp = ctref.xray3d_back_project(r, M, (N, N, N), np.float64)
    np.testing.assert_allclose(np.sum(y * r), np.sum(x * bp), rtol=1e-12)


def test_cg_spd():
    """scico/test/test_solver.py:28-60: CG on an SPD system."""
    rng = np.random.default_rng(6)
    n = 64
    A = rng.standard_normal((n, n))
    A = A.T @ A + n * np.eye(n)
    b = rng.standard_normal(n)
    x, info = ctref.cg(lambda v: A @ v, b, np.zeros(n), tol=1e-12, maxiter=200)
    assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) < 1e-6
    assert info["num_iter"] <= 200


def test_admm_tv_oracle_decreases():
    from scico_gb300 import workloads

    x_gt = workloads.random_ellipses(24, 3, 5)
    ang = np.linspace(0, np.pi, 20, endpoint=False)
    g = ctref.xray2d_defaults(x_gt.shape, ang)
    y = ctref.xray2d_project(x_gt, g, np.float64)
    fwd = lambda v: ctref.xray2d_project(v, g, np.float64)
    adj = lambda v: ctref.xray2d_back_project(v, g, np.float64)
    x, hist, _, _ = ctref.admm_tv(fwd, adj, y, x_gt.shape, lam_l21=0.01, rho=1.0, maxiter=8, dtype=np.float64)
    obj = [h["Objective"] for h in hist]
    assert obj[-1] < obj[0]
    assert ctref.snr(x_gt, x) > 10


def test_fbp_oracle_reference_quality():
    """The oracle's FBP meets the reference's own criterion
    (test_xray_2d.py:88-102, one of its four cases): PSNR > 28 dB."""
    N = 256
    x_gt = np.zeros((N, N), dtype=np.float32)
    x_gt[N // 4:-N // 4, N // 4:-N // 4] = 1.0
    angles = np.linspace(0, np.pi, 360, endpoint=False)
    g = ctref.xray2d_defaults((N, N), angles, det_count=N, dx=1.0 / np.sqrt(2))
    y = ctref.xray2d_project(x_gt, g, np.float64)
    assert ctref.psnr(x_gt, ctref.xray2d_fbp(y, g)) > 28


def test_haar_oracle_identities():
    """test_tvnorm.py:13-25: H^T H x = 2 x per axis, 4 x over two axes."""
    x = np.random.default_rng(1234).standard_normal((3, 4))
    for axes, k in (((0,), 2), ((1,), 2), ((0, 1), 4)):
        np.testing.assert_allclose(ctref.haar_adj(ctref.haar_fwd(x, axes), axes), k * x, rtol=1e-12, atol=1e-12)


def test_c_proj3d_matches_numpy_oracle():
    """The C/OpenMP 3D projector (CPU baseline of the 3D workload) against
    the NumPy restatement, AXIS0 and general geometries."""
    from oracle import ctref_c

    for shape, det, seq, ang in [((6, 10, 12), (6, 17), "X", np.linspace(0, np.pi, 5, endpoint=False)[:, None]),
                                 ((7, 8, 9), (12, 13), "XYZ", np.random.default_rng(2).uniform(0, 3, (4, 3)))]:
        M = ctref.xray3d_matrices_from_euler_angles(shape, det, seq, ang).astype(np.float32)
        G = ctref_c.Geometry3D(shape, M, det)
        x = np.random.default_rng(1).random(shape).astype(np.float32)
        assert ctref.rel_l2(G.project(x), ctref.xray3d_project(x, M, det, np.float32, np.float64)) <= 1e-6
        y = np.random.default_rng(3).standard_normal((len(M),) + det).astype(np.float32)
        assert ctref.rel_l2(G.back_project(y), ctref.xray3d_back_project(y, M, shape, np.float32, np.float64)) <= 1e-6


@pytest.mark.parametrize("dot64", [False, True])
def test_c_admm_matches_numpy_oracle(dot64):
    """The C/OpenMP 2D ADMM-TV against the NumPy restatement, converged
    regime (each CG solve meets its tolerance), both precision policies:
    the reference's float32 CG scalars and float64 dot products.  The
    iterates, CG step counts and statistics agree to float32 rounding."""
    from oracle import ctref_c
    from scico_gb300 import workloads

    x_gt = workloads.random_ellipses(24, 3, 5)
    ang = np.linspace(0, np.pi, 30, endpoint=False)
    G = ctref_c.Geometry(x_gt.shape, ang)
    y = workloads.noisy(G.project(x_gt), 0.01, 6)
    kw = dict(rho=20.0, maxiter=6, cg_maxiter=40, cg_tol=1e-5)
    x, _, _, it = G.admm_tv(y, 0.02, dot64=dot64, **kw)
    fwd = lambda v: ctref.xray2d_project(v, G.g, np.float32)
    adj = lambda v: ctref.xray2d_back_project(v, G.g, np.float32)
    xn, hist, _, _ = ctref.admm_tv(fwd, adj, y, x_gt.shape, lam_l21=0.02, dtype=np.float32,
                                   dot_dtype=np.float64 if dot64 else None, **kw)
    assert ctref.rel_l2(x, xn) <= 2e-5
    np.testing.assert_allclose(it[:, 0], [h["Objective"] for h in hist], rtol=1e-5)
    assert all(abs(a - h["CG_It"]) <= 1 for a, h in zip(it[:, 3], hist))
    assert np.all(it[:, 4] <= 1e-5 * 1.01)  # relres below the tolerance: a true relative residual


def test_c_admm3d_matches_numpy_oracle():
    """The C/OpenMP 3D ADMM-TV (L2,1 + L1 on one FiniteDifference, the 3D
    benchmark's split) against the NumPy restatement, converged regime."""
    from oracle import ctref_c

    shape, det = (6, 10, 12), (6, 17)
    M = ctref.xray3d_matrices_from_euler_angles(shape, det, "X", np.linspace(0, np.pi, 9, endpoint=False)[:, None])
    M = M.astype(np.float32)
    G = ctref_c.Geometry3D(shape, M, det)
    x_gt = np.clip(np.random.default_rng(4).random(shape), 0.3, 0.7).astype(np.float32)
    y = G.project(x_gt)
    kw = dict(rho=20.0, maxiter=5, cg_maxiter=40, cg_tol=1e-5)
    x, z, u, it = G.admm_tv(y, 0.02, 0.01, dot64=True, **kw)
    assert z.shape == (2, 3) + shape
    fwd = lambda v: ctref.xray3d_project(v, M, det, np.float32, np.float32)
    adj = lambda v: ctref.xray3d_back_project(v, M, shape, np.float32, np.float32)
    xn, hist, zn, un = ctref.admm_tv(fwd, adj, y, shape, lam_l21=0.02, lam_l1=0.01, dtype=np.float32,
                                     dot_dtype=np.float64, **kw)
    assert ctref.rel_l2(x, xn) <= 2e-5
    np.testing.assert_allclose(it[:, 0], [h["Objective"] for h in hist], rtol=1e-5)
    np.testing.assert_allclose(it[:, 1], [h["Prml_Rsdl"] for h in hist], rtol=1e-3, atol=1e-6)
    for k in range(2):
        assert ctref.rel_l2(z[k], zn[k]) <= 1e-4


def test_c_f64_build_matches_numpy_f64():
    """The float64 build of the C restatement (an x64 run of the reference:
    float64 view parameters, weights, sums and solver) against the NumPy
    restatement in float64: projector, adjoint and a short ADMM-TV solve."""
    from oracle import ctref_c
    from scico_gb300 import workloads

    x_gt = workloads.random_ellipses(20, 3, 8).astype(np.float64)
    ang = np.linspace(0, np.pi, 24, endpoint=False)
    G = ctref_c.Geometry(x_gt.shape, ang, f64=True)
    y = G.project(x_gt)
    assert y.dtype == np.float64
    assert ctref.rel_l2(y, ctref.xray2d_project(x_gt, G.g, np.float64)) <= 1e-13
    assert ctref.rel_l2(G.back_project(y), ctref.xray2d_back_project(y, G.g, np.float64)) <= 1e-13
    kw = dict(rho=1.0, maxiter=4, cg_maxiter=10, cg_tol=1e-4)
    x, _, _, it = G.admm_tv(y, 0.01, dot64=True, **kw)
    fwd = lambda v: ctref.xray2d_project(v, G.g, np.float64)
    adj = lambda v: ctref.xray2d_back_project(v, G.g, np.float64)
    xn, hist, _, _ = ctref.admm_tv(fwd, adj, y, x_gt.shape, lam_l21=0.01, dtype=np.float64, **kw)
    assert ctref.rel_l2(x, xn) <= 1e-10
    # noise-free data: the data term is a small difference of large sums
    np.testing.assert_allclose(it[:, 0], [h["Objective"] for h in hist], rtol=1e-7)


@pytest.mark.parametrize("script", ["make_xray2d_reference", "make_xray3d_reference", "make_cg_reference",
                                    "make_admm_reference", "make_modl_cg_reference", "make_padmm_reference"])
def test_reference_code_fixtures_reproduce(script, tmp_path, monkeypatch, capsys):
    """Each committed reference-code fixture is exactly what its committed
    script writes from the reference's sources (skipped where the reference
    checkout is not present)."""
    import importlib
    import sys

    monkeypatch.syspath_prepend(str(GOLDEN))
    m = importlib.import_module(script)
    if not (m.DEFAULT_CHECKOUT / "scico").is_dir():
        pytest.skip("the reference checkout is not present here")
    monkeypatch.setattr(m, "HERE", tmp_path)
    monkeypatch.setattr(sys, "argv", [script])
    m.main()
    outs = sorted(tmp_path.glob("*.npz"))
    assert outs
    for o in outs:
        a, b = np.load(o), np.load(GOLDEN / o.name)
        assert set(a.files) == set(b.files), o.name
        for k in a.files:
            assert np.array_equal(a[k], b[k]), (o.name, k)
