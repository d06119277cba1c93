"""CPU model of the slab-staged EXACT forward projector (kv_fwd_slab.cu).

The model replays, in numpy float32, what the kernel does with indexes:
the per-view tables (restated from exact_build_tables in kv_exact.cu), the
placement of every slab's shared-memory box from the tile's corner rays,
the start column / row of each ray in each slice, the row descriptors, and
every (row, column) pair with a positive length.  It checks that each pair
the kernel would read lies inside its box (the kernel's own guards never
fire), and that the line integrals it sums agree with the FP64 oracle.
Run on the test geometries in full and on sampled views / rows of the
chest-DT geometry, before the kernel runs on a GPU.
"""
import numpy as np
import pytest

from kevernals_gb300.geometry import config_chest, config_small, linear_sweep

f32 = np.float32


def fma32(a, b, c):
    return (np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64)).astype(f32)


def tables(g):
    """exact_build_tables restated: double precision, stored as float32."""
    nx, ny, nz = g.nx, g.ny, g.nz
    X0, Y0 = -0.5 * nx * float(g.dx), -0.5 * ny * float(g.dy)
    Ztop = 0.5 * nz * float(g.dz)
    Zbot = -Ztop
    P = g.n_views
    xt = np.zeros((P, g.nu, 4), f32)
    xi = np.zeros((P, g.nu), np.int64)
    yt = np.zeros((P, g.nv, 4), f32)
    yi = np.zeros((P, g.nv), np.int64)
    hr = np.zeros((P, nz + 1), f32)
    for p in range(P):
        sx, sy, sz = (float(v) for v in g.src[p])
        ox, oy, zd = (float(v) for v in g.det_origin[p])
        H = sz - zd
        dh, hmid = float(g.dz) / H, -zd / H
        hr[p] = ((Zbot + np.arange(nz + 1) * float(g.dz)) / H).astype(f32)

        def axis(n, o, d, s, B0, sp, tab, ib):
            pc = o + (np.arange(n) + 0.5) * d
            c = (pc - B0) / sp
            gr = (s - pc) / sp
            gr = np.where(np.abs(gr) < 1e-20, np.where(gr < 0, -1e-20, 1e-20), gr)
            cm = c + gr * hmid
            base = np.floor(cm)
            tab[:, 0] = cm - base
            tab[:, 1] = gr
            tab[:, 2] = -1.0 / (gr * dh)
            tab[:, 3] = s - pc
            ib[:] = base.astype(np.int64)

        axis(g.nu, ox, float(g.du), sx, X0, float(g.dx), xt[p], xi[p])
        axis(g.nv, oy, float(g.dv), sy, Y0, float(g.dy), yt[p], yi[p])
    return xt, xi, yt, yi, hr


def cross(plane, ft, iz):
    return ((plane - ft).astype(f32) * iz).astype(f32)


def start_cell(T, h):
    """Start column (float, relative to the table base) of each ray at the top plane h."""
    ft = fma32(T[..., 1], h, T[..., 0])
    fl = np.floor(ft).astype(f32)
    neg = T[..., 2] < 0
    fi = np.where(neg & (fl == ft), fl - f32(1), fl).astype(f32)
    return ft, fi, neg


def span2(T, base, ia, ib_, h0, h1):
    vals = []
    for i in (ia, ib_):
        for h in (h0, h1):
            vals.append(base[i] + int(np.floor(fma32(T[i, 1], h, T[i, 0]))))
    return min(vals), max(vals)


def box_origins(g, xt, xi, yt, yi, hr, R, S, align):
    """Per view: x0[ut, s], y0[vt, s] and the box extent needed over all of them."""
    TV = 8 * R
    n_ut, n_vt, nslab = -(-g.nu // 32), -(-g.nv // TV), -(-g.nz // S)
    x0 = np.zeros((g.n_views, n_ut, nslab), np.int64)
    y0 = np.zeros((g.n_views, n_vt, nslab), np.int64)
    bx = by = 0
    for p in range(g.n_views):
        for s in range(nslab):
            h0, h1 = hr[p, s * S], hr[p, min(s * S + S, g.nz)]
            for ut in range(n_ut):
                cmin, cmax = span2(xt[p], xi[p], ut * 32, min(ut * 32 + 31, g.nu - 1), h0, h1)
                o = (cmin - 3) - ((cmin - 3) % align)
                x0[p, ut, s] = o
                bx = max(bx, cmax + 3 - o + 1)
            for vt in range(n_vt):
                rmin, rmax = span2(yt[p], yi[p], vt * TV, min(vt * TV + TV - 1, g.nv - 1), h0, h1)
                y0[p, vt, s] = rmin - 2
                by = max(by, rmax + 2 - (rmin - 2) + 1)
    bx = -(-bx // align) * align
    return x0, y0, bx, by


def emulate(g, vol, R=4, S=4, align=4, views=None, rows=None):
    """The kernel's forward projection (no ray factor: sum of slice-local
    lengths times voxel values) with every read checked against its box.
    Returns (sums [P, nv, nu] float64, number of pairs read, bx, by)."""
    xt, xi, yt, yi, hr = tables(g)
    assert np.all(np.abs(xt[..., 2]) >= 0.5) and np.all(np.abs(yt[..., 2]) >= 0.25)
    x0, y0, bx, by = box_origins(g, xt, xi, yt, yi, hr, R, S, align)
    TV = 8 * R
    views = range(g.n_views) if views is None else views
    rows = np.arange(g.nv) if rows is None else np.asarray(rows)
    us = np.arange(g.nu)
    out = np.zeros((g.n_views, g.nv, g.nu))
    reads = 0
    for p in views:
        X = xt[p][us]
        ib = xi[p][us]
        nc3 = np.zeros(g.nu, bool)
        for ut in range(-(-g.nu // 32)):     # a warp's lanes share the column count
            sl = slice(ut * 32, ut * 32 + 32)
            nc3[sl] = np.any(np.abs(X[sl, 2]) < 1.0)
        Y = yt[p][rows]
        jb = yi[p][rows]
        sx = np.where(X[:, 2] < 0, -1, 1)
        sy = np.where(Y[:, 2] < 0, -1, 1)
        acc = np.zeros((len(rows), g.nu))
        for k in range(g.nz):
            s = k // S
            h = hr[p, k + 1]
            ftx, fi, negx = start_cell(X, h)
            e1 = np.where(negx, f32(0), f32(1))
            e2 = np.where(negx, f32(-1), f32(2))
            X1 = cross((fi + e1).astype(f32), ftx, X[:, 2])
            X2 = np.where(nc3, cross((fi + e2).astype(f32), ftx, X[:, 2]), f32(2))
            colb = fi.astype(np.int64) + ib - x0[p, us // 32, s]
            assert np.all((colb >= 2) & (colb <= bx - 3)), f"view {p} slice {k}: start column outside the box"
            fty, fj, negy = start_cell(Y, h)
            p1 = (fj + np.where(negy, f32(0), f32(1))).astype(f32)
            ys = [cross(p1, fty, Y[:, 2])]
            for i in range(3):
                ys.append(cross((p1 + (i + 1) * sy).astype(f32), fty, Y[:, 2]))
            nr = 1 + sum((y < 1).astype(np.int64) for y in ys)
            js = fj.astype(np.int64) + jb - y0[p, rows // TV, s]
            je = js + (nr - 1) * sy
            assert np.all((np.minimum(js, je) >= 0) & (np.maximum(js, je) < by)), \
                f"view {p} slice {k}: rows outside the box"
            yc = [np.minimum(f32(1), y) for y in ys] + [np.full(len(rows), f32(1))]
            slab = vol[k]
            col_abs = fi.astype(np.int64) + ib
            row_abs = fj.astype(np.int64) + jb
            for r in range(5):
                live = r < nr
                lo = np.zeros(len(rows), f32) if r == 0 else yc[r - 1]
                hi = yc[r]
                rr = row_abs + r * sy
                los = [np.zeros(g.nu, f32), X1, X2]       # column c covers [X_c, X_{c+1}]
                his = [X1, X2, np.full(g.nu, f32(2))]      # X2 = 2 (beyond the slice) without nc3
                for c in range(3):
                    use = nc3[None, :] if c == 2 else np.ones((1, g.nu), bool)
                    w = (np.minimum(hi[:, None], his[c][None, :]) - np.maximum(lo[:, None], los[c][None, :])).astype(f32)
                    m = (w > 0) & live[:, None] & use
                    if not m.any():
                        continue
                    cc = col_abs + c * sx
                    # box-relative indexes of the pairs read
                    bc = np.broadcast_to((cc - x0[p, us // 32, s])[None, :], m.shape)
                    br = np.broadcast_to((rr - y0[p, rows // TV, s])[:, None], m.shape)
                    assert np.all((bc[m] >= 0) & (bc[m] < bx) & (br[m] >= 0) & (br[m] < by)), \
                        f"view {p} slice {k}: a pair outside the box"
                    inside = (cc[None, :] >= 0) & (cc[None, :] < g.nx) & (rr[:, None] >= 0) & (rr[:, None] < g.ny)
                    mm = m & inside
                    ri, ci = np.nonzero(mm)
                    acc[ri, ci] += w[ri, ci].astype(np.float64) * slab[rr[ri], cc[ci]]
                    reads += int(m.sum())
        out[p][rows] = acc
    return out, reads, bx, by


def ray_factor(g):
    P = g.n_views
    xt, xi, yt, yi, hr = tables(g)
    out = np.zeros((P, g.nv, g.nu))
    for p in range(P):
        H = float(g.src[p, 2]) - float(g.det_origin[p, 2])
        ax = xt[p, :, 3].astype(np.float64)[None, :]
        ay = yt[p, :, 3].astype(np.float64)[:, None]
        out[p] = np.sqrt(ax * ax + ay * ay + H * H) * float(g.dz) / H
    return out


def small_geometries():
    return [
        linear_sweep(48, 40, 12, 0.5, 0.5, 1.0, 7, 64, 56, 0.4, 0.4, 15.0),
        linear_sweep(40, 36, 10, 0.4, 0.5, 1.25, 5, 72, 40, 0.3, 0.45, 20.0),
    ]


@pytest.mark.parametrize("gi", [0, 1])
@pytest.mark.parametrize("R,S", [(4, 4), (2, 8), (2, 2)])
def test_slab_model_matches_fp64_oracle(gi, R, S):
    from oracle import oracle as O
    g = small_geometries()[gi]
    rng = np.random.default_rng(gi)
    vol = rng.random(g.volume_shape).astype(np.float32)
    sums, reads, bx, by = emulate(g, vol, R=R, S=S)
    got = sums * ray_factor(g)
    ref = O.exact_forward(g, vol.astype(np.float64))
    err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert err < 2e-6, err
    assert reads > 0 and bx <= 256 and by <= 256


def test_slab_indexes_inside_boxes_chest_dt():
    """Chest-DT geometry: every pair read by the kernel lies in its box, on
    the first, middle and last views and every 61st detector row."""
    g = config_chest()
    vol = np.zeros(g.volume_shape, np.float32)
    _, reads, bx, by = emulate(g, vol, R=4, S=4, views=[0, g.n_views // 2, g.n_views - 1],
                               rows=np.arange(0, g.nv, 61))
    assert reads > 0
    assert bx <= 64 and by <= 64, (bx, by)


def test_slab_indexes_inside_boxes_small_config():
    g = config_small()
    vol = np.zeros(g.volume_shape, np.float32)
    _, reads, bx, by = emulate(g, vol, R=4, S=4, views=[0, 7, 14], rows=np.arange(0, g.nv, 5))
    assert reads > 0
