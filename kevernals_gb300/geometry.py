"""Geometry description of a linear-sweep tomosynthesis acquisition.

Mirrors what the reference's TomoGeometry hands to its projector
(source/modules/geometry/TomoGeometry.h:34-89 and the flattening in
source/modules/reconstruction/Projector.cu:917-940): volume size and voxel
spacing, a volume-centred frame (TomoGeometry.cpp:127,162,330), per-view
source positions, per-view detector-ROI bottom-left corners on a common
detector plane, ROI size and pixel spacing, and the fulcrum height used by
shift-and-add.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np


@dataclasses.dataclass
class Geometry:
    nx: int
    ny: int
    nz: int
    dx: float
    dy: float
    dz: float
    nu: int
    nv: int
    du: float
    dv: float
    src: np.ndarray          # [n_views, 3] float32, volume-centred frame
    det_origin: np.ndarray   # [n_views, 3] float32, bottom-left corner of pixel (0,0)
    fulcrum_z: float = 0.0   # shift-and-add focal height (see kv_geometry)

    def __post_init__(self):
        # the C ABI carries spacings as float32: keep exactly those values here
        for f in ("dx", "dy", "dz", "du", "dv", "fulcrum_z"):
            setattr(self, f, float(np.float32(getattr(self, f))))
        self.src = np.ascontiguousarray(self.src, dtype=np.float32).reshape(-1, 3)
        self.det_origin = np.ascontiguousarray(self.det_origin, dtype=np.float32).reshape(-1, 3)
        if self.src.shape != self.det_origin.shape:
            raise ValueError("src and det_origin must both be [n_views, 3]")

    @property
    def n_views(self) -> int:
        return int(self.src.shape[0])

    @property
    def volume_shape(self):
        """numpy shape of a volume: (nz, ny, nx)."""
        return (self.nz, self.ny, self.nx)

    @property
    def proj_shape(self):
        """numpy shape of a projection stack: (n_views, nv, nu)."""
        return (self.n_views, self.nv, self.nu)

    @property
    def n_voxels(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def n_rays(self) -> int:
        return self.n_views * self.nu * self.nv

    def subset_views(self, views) -> "Geometry":
        views = np.asarray(views)
        return dataclasses.replace(self, src=self.src[views].copy(),
                                   det_origin=self.det_origin[views].copy())


def linear_sweep(nx, ny, nz, dx, dy, dz, n_views, nu, nv, du, dv, half_angle_deg,
                 sid=1000.0, sod=850.0, gap=10.0) -> Geometry:
    """Linear-sweep geometry in the volume-centred frame.

    World frame: detector plane z = 0, centred on x = y = 0; the volume sits
    laterally centred with its bottom face `gap` mm above the detector.  The
    tube moves along y at height `sid`; its central ray through the isocentre
    (height sid - sod above the detector) makes the angle theta_i, equally
    spaced over [-half_angle, +half_angle], so y_i = sod * tan(theta_i).  All
    positions are then translated so that the volume centre is the origin.
    The fulcrum height is the isocentre, in the same frame.
    """
    zc = gap + 0.5 * nz * dz                      # volume centre height (world)
    theta = np.deg2rad(np.linspace(-half_angle_deg, half_angle_deg, n_views)) \
        if n_views > 1 else np.zeros(1)
    ys = sod * np.tan(theta)
    src = np.zeros((n_views, 3), np.float64)
    src[:, 1] = ys
    src[:, 2] = sid - zc
    det = np.zeros((n_views, 3), np.float64)
    det[:, 0] = -0.5 * nu * du
    det[:, 1] = -0.5 * nv * dv
    det[:, 2] = -zc
    return Geometry(nx, ny, nz, float(dx), float(dy), float(dz), nu, nv, float(du), float(dv),
                    src.astype(np.float32), det.astype(np.float32),
                    fulcrum_z=float((sid - sod) - zc))


# ---- the workloads of the benchmark configurations -----------------------

def config_small() -> Geometry:
    """256x256x64 at 0.5x0.5x1.0 mm, 15 views over +-15 deg, 512^2 at 0.4 mm."""
    return linear_sweep(256, 256, 64, 0.5, 0.5, 1.0, 15, 512, 512, 0.4, 0.4, 15.0)


def config_chest() -> Geometry:
    """Chest-DT size: 1024x1024x128 at 0.4x0.4x2.5 mm, 60 views over +-17.5 deg,
    2048^2 detector at 0.2 mm."""
    return linear_sweep(1024, 1024, 128, 0.4, 0.4, 2.5, 60, 2048, 2048, 0.2, 0.2, 17.5)


def uneven_cases(n: int, seed: int, scale: int = 1):
    """Seeded uneven reconstruction problems (the batched-solve workload):
    in-plane 128-512 voxels (multiples of 32), 32-96 slices, detector
    256-1024 square, 9-49 views over +-10..+-25 deg; 0.5x0.5x1.0 mm voxels,
    0.4 mm pixels.  `scale` > 1 shrinks every size by that factor (many
    small problems)."""
    from .phantom import SplitMix64
    rng = SplitMix64(seed)
    out = []
    for _ in range(n):
        nxy = 32 * int(rng.uniform(4, 17))
        nz = int(rng.uniform(32, 97))
        nd = int(rng.uniform(256, 1025))
        views = int(rng.uniform(9, 50))
        ang = rng.uniform(10.0, 25.0)
        out.append(linear_sweep(nxy // scale, nxy // scale, max(2, nz // scale), 0.5 * scale, 0.5 * scale,
                                1.0 * scale, views, nd // scale, nd // scale, 0.4 * scale, 0.4 * scale, ang))
    return out


def scaled(g: Geometry, factor: int) -> Geometry:
    """Same physical acquisition with volume and detector sampled `factor`
    times coarser (used for quick checks of a large workload)."""
    return linear_sweep(g.nx // factor, g.ny // factor, g.nz, g.dx * factor, g.dy * factor, g.dz,
                        g.n_views, g.nu // factor, g.nv // factor, g.du * factor, g.dv * factor,
                        _half_angle(g))


def _half_angle(g: Geometry) -> float:
    zc = -float(g.det_origin[0, 2])
    sid = float(g.src[0, 2]) + zc
    sod = sid - (float(g.fulcrum_z) + zc)
    return math.degrees(math.atan(abs(float(g.src[:, 1].max())) / sod))


# ---- Siddon segment counts (the gather work of one projector pass) -------

def segments_per_ray(g: Geometry, view: int, uc, vc) -> np.ndarray:
    """Voxels with a positive intersection length along the rays of `view`
    through detector positions (uc, vc) in pixels (pixel centres are
    u + 0.5, v + 0.5; the arrays broadcast).  Between the box entry and exit
    a ray visits 1 + the x, y and z planes it crosses; a ray through an edge
    or a corner of the grid (a set of measure zero) is counted one voxel
    high.  Rays that miss the box count 0."""
    s = g.src[view].astype(np.float64)
    o = g.det_origin[view].astype(np.float64)
    uc, vc = np.broadcast_arrays(np.asarray(uc, np.float64), np.asarray(vc, np.float64))
    d = (o[0] + uc * g.du - s[0], o[1] + vc * g.dv - s[1], np.full(uc.shape, o[2] - s[2]))
    n = (g.nx, g.ny, g.nz)
    sp = (g.dx, g.dy, g.dz)
    tin = np.zeros(uc.shape)
    tout = np.ones(uc.shape)
    for a in range(3):
        h = 0.5 * n[a] * sp[a]
        da = d[a]
        moving = da != 0.0
        safe = np.where(moving, da, 1.0)
        t_lo, t_hi = (-h - s[a]) / safe, (h - s[a]) / safe
        lo = np.where(moving, np.minimum(t_lo, t_hi), np.where(abs(s[a]) < h, -np.inf, np.inf))
        hi = np.where(moving, np.maximum(t_lo, t_hi), np.where(abs(s[a]) < h, np.inf, -np.inf))
        tin = np.maximum(tin, lo)
        tout = np.minimum(tout, hi)
    hit = tout > tin
    eps = 1e-9 * np.where(hit, tout - tin, 0.0)
    te, tx = tin + eps, tout - eps
    count = np.ones(uc.shape)
    for a in range(3):
        h = 0.5 * n[a] * sp[a]
        ie = np.floor((s[a] + te * d[a] + h) / sp[a])
        ix = np.floor((s[a] + tx * d[a] + h) / sp[a])
        count += np.abs(ix - ie)
    return np.where(hit, count, 0.0)


def siddon_segments(g: Geometry, stride: int = 1) -> float:
    """Siddon segments -- (ray, voxel) pairs with a positive intersection
    length -- of one forward projection (equally, of its transpose), from the
    rays of every `stride`-th detector column and row of every view, scaled
    to all rays when stride > 1."""
    us = np.arange(stride // 2, g.nu, stride) + 0.5     # the middle column of each block
    vs = np.arange(stride // 2, g.nv, stride) + 0.5
    total = 0.0
    for p in range(g.n_views):
        total += float(segments_per_ray(g, p, us[None, :], vs[:, None]).sum())
    return total * (g.nu * g.nv) / (len(us) * len(vs))
