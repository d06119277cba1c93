"""Seeded ellipsoid phantoms and noisy projection data.

PRNG: splitmix64 (G. Steele, D. Lea, C. Flood, "Fast splittable
pseudorandom number generators", OOPSLA 2014).  A phantom is a background
ellipsoid plus N rotated ellipsoids with additive attenuation, sampled at
voxel centres; the parameters are drawn here and rasterised by the engine
(kv_phantom_ellipsoids).  Seed convention: 20261203 + 1000*config + case.
"""
from __future__ import annotations

import math

import numpy as np

MASK64 = (1 << 64) - 1


class SplitMix64:
    def __init__(self, seed: int):
        self.state = seed & MASK64

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def uniform(self, lo=0.0, hi=1.0) -> float:
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / 9007199254740992.0))


def seed_for(config: int, case: int = 0) -> int:
    return 20261203 + 1000 * config + case


def _rotation_zyz(phi, theta, psi):
    """R = Rz(phi) Ry(theta) Rz(psi); a world offset r maps to local R^T r."""
    def rz(a):
        c, s = math.cos(a), math.sin(a)
        return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]])

    def ry(a):
        c, s = math.cos(a), math.sin(a)
        return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])
    return rz(phi) @ ry(theta) @ rz(psi)


def ellipsoid_params(nx, ny, nz, dx, dy, dz, n_ellipsoids, seed, background=0.02,
                     mu_max=0.05) -> np.ndarray:
    """[n+1, 16] float32 rows: centre(3), semi-axes(3), M(9, row-major, local =
    M (q - c)), density.  Row 0 is the background ellipsoid (semi-axes 0.45 x
    extent, density `background`); the others have centres uniform in 0.8 x
    the background's box, semi-axes uniform in [0.02, 0.15] x extent, ZYZ
    Euler angles uniform in [0, 2 pi), density uniform in [0, mu_max]."""
    ext = np.array([nx * dx, ny * dy, nz * dz], np.float64)
    rng = SplitMix64(seed)
    rows = []
    rows.append(np.concatenate([[0, 0, 0], 0.45 * ext, np.eye(3).ravel(), [background]]))
    for _ in range(n_ellipsoids):
        c = [rng.uniform(-0.8 * 0.45 * e, 0.8 * 0.45 * e) for e in ext]
        a = [rng.uniform(0.02, 0.15) * e for e in ext]
        ang = [rng.uniform(0.0, 2 * math.pi) for _ in range(3)]
        mu = rng.uniform(0.0, mu_max)
        m = _rotation_zyz(*ang).T
        rows.append(np.concatenate([c, a, m.ravel(), [mu]]))
    return np.asarray(rows, np.float32)


def poisson_log_data(line_integrals: np.ndarray, i0: float, seed: int) -> np.ndarray:
    """Noisy log data p = ln(I0 / max(counts, 1)), counts ~ Poisson(I0 e^-p),
    from a seeded host sampler (numpy PCG64).  Values are clipped at 0: a
    count above I0 (a ray through little or no material) would otherwise give
    a negative datum, which MLEM cannot fit."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lam = i0 * np.exp(-line_integrals.astype(np.float64))
    counts = rng.poisson(lam)
    return np.maximum(np.log(i0 / np.maximum(counts, 1)), 0.0).astype(np.float32)
