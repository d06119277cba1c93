"""CPU model of the TMA-staged EXACT backprojector's patch placement
(kv_back_stage.cu).

The kernel stages, per view, the detector patch that a CTA's voxel tile (32
voxel columns x 8R voxel rows of one slice) can see: origin = the first
candidate column of the tile's first voxel column (rounded down to 4
columns, TMA's 16-byte grid) and the first candidate row of its first voxel
row; extent BU x BV sized on the host as the maximum over every view, slice
and tile.  This model replays in numpy float32 the candidate ranges of the
backprojector (the per-view plane coefficients `rng`, restated from
exact_build_tables in kv_exact.cu) and checks that every voxel's candidate
detector columns and rows lie inside its tile's patch, i.e. that every
shared-memory read the kernel makes stays inside the staged box, on the test
geometries in full and on sampled slices of the chest-DT geometry.
"""
import numpy as np
import pytest

from kevernals_gb300.geometry import config_chest, linear_sweep

f32 = np.float32


def rng_table(g):
    """rng[p][k] = (Ax, 1/Bx, Ay, 1/By), double precision stored as float32."""
    X0, Y0 = -0.5 * g.nx * float(g.dx), -0.5 * g.ny * float(g.dy)
    Zbot = -0.5 * g.nz * float(g.dz)
    out = np.zeros((g.n_views, g.nz + 1, 4), f32)
    for p in range(g.n_views):
        sx, sy, sz = (float(v) for v in g.src[p])
        ox, oy, zd = (float(v) for v in g.det_origin[p])
        H = sz - zd
        for k in range(g.nz + 1):
            h = (Zbot + k * float(g.dz) - zd) / H
            Bx = float(g.du) * (1.0 - h) / float(g.dx)
            By = float(g.dv) * (1.0 - h) / float(g.dy)
            Ax = ((ox - X0) + (sx - ox) * h + 0.5 * float(g.du) * (1.0 - h)) / float(g.dx)
            Ay = ((oy - Y0) + (sy - oy) * h + 0.5 * float(g.dv) * (1.0 - h)) / float(g.dy)
            out[p, k] = (Ax, 1.0 / Bx, Ay, 1.0 / By)
    return out


def cand(idx, a0, b0, a1, b1, n):
    """First and last candidate detector index of each voxel index (float32,
    the backprojector's expressions)."""
    i = idx.astype(f32)
    lo = np.minimum((i - a0) * b0, (i - a1) * b1)
    hi = np.maximum(((i + f32(1)) - a0) * b0, ((i + f32(1)) - a1) * b1)
    c0 = np.maximum(0, np.ceil(np.minimum(lo, hi) - f32(0.01)).astype(np.int64))
    c1 = np.minimum(n - 1, np.floor(np.maximum(lo, hi) + f32(0.01)).astype(np.int64))
    return c0, c1


def patch_extent(g, R, slices=None):
    """(BU, BV) as back_stage_fit sizes them, over the given slices."""
    T = rng_table(g)
    TV = 8 * R
    bu = bv = 0
    ks = range(g.nz) if slices is None else slices
    i0 = np.arange(0, g.nx, 32)
    i1 = np.minimum(i0 + 31, g.nx - 1)
    j0 = np.arange(0, g.ny, TV)
    j1 = np.minimum(j0 + TV - 1, g.ny - 1)
    for p in range(g.n_views):
        for k in ks:
            a0, b0, c0_, d0 = T[p, k]
            a1, b1, c1_, d1 = T[p, k + 1]
            ua, _ = cand(i0, a0, b0, a1, b1, g.nu)
            _, ub = cand(i1, a0, b0, a1, b1, g.nu)
            va, _ = cand(j0, c0_, d0, c1_, d1, g.nv)
            _, vb = cand(j1, c0_, d0, c1_, d1, g.nv)
            bu = max(bu, int((ub - (ua & ~3) + 1).max()))
            bv = max(bv, int((vb - va + 1).max()))
    return (bu + 3) // 4 * 4, bv


def check_reads_inside(g, R, slices=None):
    """Every voxel's candidates lie in its tile's patch; returns (BU, BV)."""
    BU, BV = patch_extent(g, R, slices)
    T = rng_table(g)
    TV = 8 * R
    ks = range(g.nz) if slices is None else slices
    ii = np.arange(g.nx)
    jj = np.arange(g.ny)
    for p in range(g.n_views):
        for k in ks:
            a0, b0, c0_, d0 = T[p, k]
            a1, b1, c1_, d1 = T[p, k + 1]
            u0, u1 = cand(ii, a0, b0, a1, b1, g.nu)
            v0, v1 = cand(jj, c0_, d0, c1_, d1, g.nv)
            # candidates grow with the voxel index: the tile's first voxel
            # has the first, its last voxel the last
            assert np.all(np.diff(u0) >= 0) and np.all(np.diff(u1) >= 0)
            assert np.all(np.diff(v0) >= 0) and np.all(np.diff(v1) >= 0)
            x0 = (u0[(ii // 32) * 32]) & ~3
            y0 = v0[(jj // TV) * TV]
            live_u = u1 >= u0
            live_v = v1 >= v0
            assert np.all(~live_u | ((u0 >= x0) & (u1 < x0 + BU))), f"view {p} slice {k}: columns outside"
            assert np.all(~live_v | ((v0 >= y0) & (v1 < y0 + BV))), f"view {p} slice {k}: rows outside"
            assert np.all(x0 % 4 == 0) and np.all(x0 >= 0) and np.all(y0 >= 0)
    return BU, BV


@pytest.mark.parametrize("R", [4, 8])
def test_staged_patch_holds_every_candidate_small_geometries(R):
    for g in [linear_sweep(40, 36, 12, 0.5, 0.5, 1.0, 5, 48, 44, 0.4, 0.4, 15.0),
              linear_sweep(64, 64, 16, 0.4, 0.4, 2.5, 9, 96, 96, 0.2, 0.2, 17.5),
              linear_sweep(24, 12, 6, 1.0, 1.0, 1.0, 5, 96, 256, 0.3, 0.05, 15.0)]:
        BU, BV = check_reads_inside(g, R)
        assert BU <= 256 and BV <= 256 and BU % 4 == 0


def test_staged_patch_chest_dt_sampled_slices():
    """Chest-DT: the patch of a 64-row tile (104 x 199 pixels on these
    slices) holds every candidate on the first, middle and last slices."""
    g = config_chest()
    BU, BV = check_reads_inside(g, 8, slices=[0, g.nz // 2, g.nz - 1])
    assert (BU, BV) == (104, 199)
