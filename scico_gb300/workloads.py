"""Seeded synthetic CT workloads (the five benchmark configurations).

scico's CT examples build phantoms with xdesign (not a dependency here);
these configurations instead use seeded random-ellipse phantoms of the
stated sizes and value ranges.  Generation order per ellipse: centre,
semi-axes, rotation angle, intensity, all from
``numpy.random.default_rng(seed)``; pixel centres lie on [-1, 1]^2
(axis 0 = y, axis 1 = x); ellipses add and the image is clipped to [0, 1].
"""

from __future__ import annotations

import dataclasses
import math
from typing import List, Tuple, Optional

import numpy as np


def random_ellipses(n: int, count: int, seed: int, semi=(0.05, 0.4), rng=None) -> np.ndarray:
    """(n, n) float32 phantom of `count` random ellipses."""
    rng = np.random.default_rng(seed) if rng is None else rng
    c = ((np.arange(n) + 0.5) / n * 2.0 - 1.0).astype(np.float64)
    Y, X = np.meshgrid(c, c, indexing="ij")
    img = np.zeros((n, n), dtype=np.float64)
    for _ in range(count):
        cx, cy = rng.uniform(-0.6, 0.6, size=2)
        a, b = rng.uniform(semi[0], semi[1], size=2)
        th = rng.uniform(0.0, math.pi)
        val = rng.uniform(-0.5, 1.0)
        ct, st = math.cos(th), math.sin(th)
        xr = (X - cx) * ct + (Y - cy) * st
        yr = -(X - cx) * st + (Y - cy) * ct
        img[(xr / a) ** 2 + (yr / b) ** 2 <= 1.0] += val
    return np.clip(img, 0.0, 1.0).astype(np.float32)


def random_ellipsoids(n: int, count: int, seed: int, semi=(0.05, 0.35)) -> np.ndarray:
    """(n, n, n) float32 phantom of `count` randomly rotated ellipsoids."""
    rng = np.random.default_rng(seed)
    c = ((np.arange(n) + 0.5) / n * 2.0 - 1.0).astype(np.float32)
    vol = np.zeros((n, n, n), dtype=np.float32)
    Z, Y, X = np.meshgrid(c, c, c, indexing="ij")
    P = np.stack([X.ravel(), Y.ravel(), Z.ravel()])
    del X, Y, Z
    for _ in range(count):
        ctr = rng.uniform(-0.6, 0.6, size=3).astype(np.float32)
        ax = rng.uniform(semi[0], semi[1], size=3).astype(np.float32)
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        w, x, y, z = q
        Rm = np.array(
            [
                [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
            ],
            dtype=np.float32,
        )
        val = np.float32(rng.uniform(-0.5, 1.0))
        L = Rm.T @ (P - ctr[:, None])
        inside = ((L / ax[:, None]) ** 2).sum(axis=0) <= 1.0
        vol.reshape(-1)[inside] += val
    return np.clip(vol, 0.0, 1.0)


def circular_phantom(shape, radii, values) -> np.ndarray:
    """Concentric discs (or balls) about the array centre: each radius in
    turn sets the points closer than it to its value (later ones on top)."""
    grids = np.meshgrid(*[np.arange(n) - (n - 1) / 2 for n in shape], indexing="ij", sparse=True)
    dist = np.sqrt(sum(g.astype(np.float64) ** 2 for g in grids))
    out = np.zeros(shape)
    for r, v in zip(radii, values):
        out[dist < r] = v
    return out


def noisy(y: np.ndarray, rel_sigma: float, seed: int) -> np.ndarray:
    """y + N(0, (rel_sigma * max|y|)^2), float32."""
    rng = np.random.default_rng(seed)
    sigma = rel_sigma * float(np.max(np.abs(y)))
    return (y + rng.normal(0.0, sigma, size=y.shape)).astype(np.float32)


@dataclasses.dataclass
class Slice2D:
    """One 2D parallel-beam ADMM-TV problem."""

    n: int
    n_views: int
    det_count: int
    lam: float
    rho: float
    maxiter: int
    cg_maxiter: int
    cg_tol: float
    phantom_seed: int
    n_ellipses: int
    noise: float
    noise_seed: int

    @property
    def angles(self) -> np.ndarray:
        return np.linspace(0, np.pi, self.n_views, endpoint=False)

    @property
    def interactions(self) -> int:
        return self.n * self.n * self.n_views

    def phantom(self) -> np.ndarray:
        return random_ellipses(self.n, self.n_ellipses, self.phantom_seed)


# C1: 256x256, 180 views, 363 bins (default det_count), lambda 0.01, rho 1, 50 it, CG <= 10
C1 = Slice2D(256, 180, 363, 0.01, 1.0, 50, 10, 1e-4, 0, 10, 0.01, 1)
# C2: 512x512, 360 views, 725 bins, lambda 0.005, rho 2, 100 it, CG <= 10
C2 = Slice2D(512, 360, 725, 0.005, 2.0, 100, 10, 1e-4, 2, 20, 0.005, 3)


@dataclasses.dataclass
class Volume3D:
    """One 3D parallel-beam ADMM-TV problem: rotation about volume axis 0
    (``matrices_from_euler_angles(shape, det, "X", angles[:, None])``),
    g = lam_l1 ||Dx||_1 + lam_l21 ||Dx||_2,1 on one finite difference."""

    n: int
    n_views: int
    det_shape: Tuple[int, int]
    lam_l1: float
    lam_l21: float
    rho: float
    maxiter: int
    cg_maxiter: int
    cg_tol: float
    phantom_seed: int
    n_ellipsoids: int
    noise: float
    noise_seed: int

    @property
    def shape(self) -> Tuple[int, int, int]:
        return (self.n, self.n, self.n)

    @property
    def angles(self) -> np.ndarray:
        return np.linspace(0, np.pi, self.n_views, endpoint=False)

    @property
    def interactions(self) -> int:
        return self.n**3 * self.n_views

    def matrices(self) -> np.ndarray:
        from .linop import XRayTransform3D

        return XRayTransform3D.matrices_from_euler_angles(self.shape, self.det_shape, "X", self.angles[:, None])

    def phantom(self) -> np.ndarray:
        return random_ellipsoids(self.n, self.n_ellipsoids, self.phantom_seed)


# C5: 256^3, 360 views about axis 0, 256 x 363 detector, lambda 0.005 (L1 and
# L21 on the same FD), rho 1, 30 it, CG <= 8
C5 = Volume3D(256, 360, (256, 363), 0.005, 0.005, 1.0, 30, 8, 1e-4, 6, 30, 0.01, 7)


@dataclasses.dataclass
class MoDLWorkload:
    """Unrolled MoDL reconstruction of a batch of 2D slices: MoDLNet(depth,
    ResNet(block_depth, num_filters)) with cg_iter CG steps on A^T A + lmbda I
    per block, trained with an MSE loss."""

    batch: int
    n: int
    n_views: int
    det_count: int
    depth: int
    block_depth: int
    num_filters: int
    cg_iter: int
    lmbda_ini: float
    phantom_seed: int
    n_ellipses: int
    noise: float
    weight_seed: int

    @property
    def angles(self) -> np.ndarray:
        return np.linspace(0, np.pi, self.n_views, endpoint=False)

    def phantoms(self) -> np.ndarray:
        return np.stack([random_ellipses(self.n, self.n_ellipses, self.phantom_seed * 1000 + k)
                         for k in range(self.batch)])


# C4: 16 x 256^2 slices, 180 views, 363 bins, 5 blocks of CG(10) on
# A^T A + 0.1 I with a 3-layer, 32-filter ResNet denoiser
C4 = MoDLWorkload(16, 256, 180, 363, 5, 3, 32, 10, 0.1, 4, 10, 0.01, 5)


def batched_configs(count: int = 64, seed: int = 3) -> List[Slice2D]:
    """C3: `count` scans with N from {128..768}, views from {90..720}, det = ceil(sqrt2 N)+1."""
    rng = np.random.default_rng(seed)
    out = []
    sizes = [128, 192, 256, 384, 512, 768]
    views = [90, 180, 360, 720]
    for k in range(count):
        n = int(rng.choice(sizes))
        v = int(rng.choice(views))
        lam = float(rng.uniform(0.002, 0.02))
        out.append(Slice2D(n, v, int(math.ceil(math.sqrt(2.0) * n)) + 1, lam, 1.0, 50, 10, 1e-4,
                           1000 + k, 10, 0.01, 2000 + k))
    return out
