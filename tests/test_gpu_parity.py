"""GPU parity tests: the CUDA path, called through the C ABI, against the
oracle (FP32 restatement of the reference for RC, FP64 Siddon for EXACT) and
against the golden outputs of the reference kernels."""
import hashlib
import json
import os

import numpy as np
import pytest

from kevernals_gb300 import build, engine, phantom as ph
from kevernals_gb300._lib import KvError
from kevernals_gb300.geometry import Geometry, config_chest, config_small, linear_sweep, scaled
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")

# Tolerances (stated): EXACT FP32 GPU vs FP64 oracle
EXACT_FWD_REL_L2 = 2e-6
EXACT_BACK_REL_L2 = 2e-6
DOT_REL = 1e-6


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def ctx():
    build.build()
    return engine.Context(0)


def golden_cases():
    z = np.load(os.path.join(GOLDEN, "golden_small.npz"))
    out = {}
    for name in ("a", "b", "c"):
        nx, ny, nz, nu, nv = (int(t) for t in z[f"{name}_dims"])
        dx, dy, dz, du, dv, fz = (float(t) for t in z[f"{name}_spacing"])
        g = Geometry(nx, ny, nz, dx, dy, dz, nu, nv, du, dv, z[f"{name}_src"], z[f"{name}_det"], fz)
        out[name] = (g, {k[len(name) + 1:]: z[k] for k in z.files if k.startswith(name + "_")})
    return out


def small_geoms():
    return [
        linear_sweep(40, 36, 12, 0.5, 0.5, 1.0, 5, 48, 44, 0.4, 0.4, 15.0),
        linear_sweep(33, 29, 7, 0.7, 0.45, 1.3, 4, 37, 41, 0.55, 0.35, 22.0),
        linear_sweep(64, 64, 16, 0.4, 0.4, 2.5, 9, 96, 96, 0.2, 0.2, 17.5),
    ]


def phantom_for(g, n=8, seed=5):
    return O.phantom(g, ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, n, seed))


# ---------------------------------------------------------------- RC family

@pytest.mark.parametrize("name", ["a", "b", "c"])
def test_rc_forward_back_bitexact_vs_reference_golden(ctx, name):
    g, d = golden_cases()[name]
    plan = engine.Plan(ctx, g, "rc")
    vol = engine.phantom(ctx, g, d["params"])
    assert np.array_equal(vol, d["vol"])
    f = plan.forward(vol)
    assert np.array_equal(f, d["fwd"]), f"max diff {np.abs(f - d['fwd']).max()}"
    assert np.array_equal(plan.back(d["fwd"]), d["back"])
    assert np.array_equal(plan.back(d["y"]), d["back_y"])


def test_rc_config1_bitexact_vs_reference_digests(ctx):
    info = json.load(open(os.path.join(GOLDEN, "golden_config1.json")))
    g = config_small()
    params = ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, 40, info["seed"])
    vol = engine.phantom(ctx, g, params)
    dg = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()  # noqa: E731
    assert dg(vol) == info["phantom_sha256"]
    plan = engine.Plan(ctx, g, "rc")
    f = plan.forward(vol)
    assert dg(f) == info["ref_forward_sha256"]
    assert dg(plan.back(f)) == info["ref_back_of_forward_sha256"]


def test_rc_drivers_match_oracle(ctx):
    g = small_geoms()[0]
    truth = phantom_for(g)
    p = O.rc_forward(g, truth)
    plan = engine.Plan(ctx, g, "rc")
    for relax in (1.0, 0.5):
        x = np.ones(g.volume_shape, np.float32)
        plan.mlem(p, x, 3, relax)
        assert np.array_equal(x, O.rc_mlem(g, p, np.ones(g.volume_shape, np.float32), 3, relax))
        x = np.ones(g.volume_shape, np.float32)
        plan.sart(p, x, 3, relax)
        assert np.array_equal(x, O.rc_art(g, p, np.ones(g.volume_shape, np.float32), 3, relax))
    # the callback path (unfused ratio) gives the same iterate
    x1 = np.ones(g.volume_shape, np.float32)
    hist = plan.mlem(p, x1, 3, 0.5, callback=lambda it, r, ll: False)
    assert len(hist) == 3 and hist[0][1] > hist[-1][1]
    assert np.array_equal(x1, O.rc_mlem(g, p, np.ones(g.volume_shape, np.float32), 3, 0.5))


def test_rc_random_geometries_match_oracle(ctx):
    rng = np.random.default_rng(11)
    for g in small_geoms():
        vol = rng.random(g.volume_shape, dtype=np.float32)
        plan = engine.Plan(ctx, g, "rc")
        f = plan.forward(vol)
        assert np.array_equal(f, O.rc_forward(g, vol))
        assert np.array_equal(plan.back(f), O.rc_back(g, f))


# ------------------------------------------------------------- EXACT family

@pytest.mark.parametrize("gi", [0, 1, 2])
def test_exact_forward_vs_fp64_oracle(ctx, gi):
    g = small_geoms()[gi]
    vol = phantom_for(g)
    plan = engine.Plan(ctx, g, "exact")
    f = plan.forward(vol)
    ref = O.exact_forward(g, vol.astype(np.float64))
    assert rel_l2(f, ref) < EXACT_FWD_REL_L2
    rng = np.random.default_rng(gi)
    x = rng.random(g.volume_shape, dtype=np.float32)
    assert rel_l2(plan.forward(x), O.exact_forward(g, x.astype(np.float64))) < 1e-5


@pytest.mark.parametrize("gi", [0, 1, 2])
def test_exact_back_vs_fp64_oracle(ctx, gi):
    g = small_geoms()[gi]
    rng = np.random.default_rng(gi + 10)
    y = rng.random(g.proj_shape, dtype=np.float32)
    plan = engine.Plan(ctx, g, "exact")
    b = plan.back(y)
    assert rel_l2(b, O.exact_back(g, y.astype(np.float64))) < EXACT_BACK_REL_L2


@pytest.mark.parametrize("gi", [0, 1, 2])
def test_exact_dot_product(ctx, gi):
    g = small_geoms()[gi]
    rng = np.random.default_rng(gi + 20)
    x = rng.random(g.volume_shape, dtype=np.float32)
    y = rng.random(g.proj_shape, dtype=np.float32)
    plan = engine.Plan(ctx, g, "exact")
    lhs = np.vdot(plan.forward(x).astype(np.float64), y.astype(np.float64))
    rhs = np.vdot(x.astype(np.float64), plan.back(y).astype(np.float64))
    assert abs(lhs - rhs) <= DOT_REL * abs(lhs)


@pytest.mark.parametrize("gi,half_taps", [(0, 8), (2, 64)])
def test_exact_fbp_vs_fp64_oracle(ctx, gi, half_taps):
    """Filtered backprojection (Shepp-Logan ramp along v, then A^T and the
    sensitivity normalisation) against its FP64 restatement."""
    g = small_geoms()[gi]
    vol = phantom_for(g)
    plan = engine.Plan(ctx, g, "exact")
    p = plan.forward(vol)
    x = plan.fbp(p, half_taps)
    ref = O.exact_fbp(g, p, half_taps)
    assert rel_l2(x, ref) < 1e-5
    # the ramp sharpens: closer to the phantom than the plain normalised backprojection
    sens = O.exact_back(g, np.ones(g.proj_shape))
    saa = np.where(sens > 0, O.exact_back(g, p) / np.where(sens > 0, sens, 1.0), 0.0)
    if half_taps >= 16:
        assert rel_l2(x, vol) < rel_l2(saa, vol)
    with pytest.raises(KvError):
        plan.fbp(p, 0)
    with pytest.raises(KvError):
        plan.fbp(p, 257)


def test_exact_sensitivity_vs_oracle(ctx):
    g = small_geoms()[0]
    plan = engine.Plan(ctx, g, "exact")
    s = plan.sensitivity()
    assert rel_l2(s, O.exact_back(g, np.ones(g.proj_shape))) < 1e-6


def test_exact_mlem_sart_vs_fp64_oracle(ctx):
    g = small_geoms()[0]
    truth = phantom_for(g)
    p = O.exact_forward(g, truth.astype(np.float64)).astype(np.float32)
    plan = engine.Plan(ctx, g, "exact")
    x = np.ones(g.volume_shape, np.float32)
    hist = plan.mlem(p, x, 5, callback=lambda *a: False)
    xo = O.exact_mlem(g, p.astype(np.float64), np.ones(g.volume_shape), 5)
    assert rel_l2(x, xo) < 1e-5
    assert all(b[1] < a[1] for a, b in zip(hist, hist[1:]))
    x = np.zeros(g.volume_shape, np.float32)
    plan.sart(p, x, 5, 0.5)
    xo = O.exact_sart(g, p.astype(np.float64), np.zeros(g.volume_shape), 5, 0.5)
    assert rel_l2(x, xo) < 1e-5


def test_exact_residual_matches_numpy(ctx):
    g = small_geoms()[1]
    truth = phantom_for(g)
    p = O.exact_forward(g, truth.astype(np.float64)).astype(np.float32)
    plan = engine.Plan(ctx, g, "exact")
    x = np.full(g.volume_shape, 0.01, np.float32)
    r, ll = plan.residual(p, x)
    q = O.exact_forward(g, x.astype(np.float64))
    pd = p.astype(np.float64)
    assert r == pytest.approx(np.linalg.norm(q - pd) / np.linalg.norm(pd), rel=1e-5)
    llo = np.sum(np.where(q > 0, pd * np.log(np.maximum(q, 1e-300)), 0.0) - q)
    assert ll == pytest.approx(llo, rel=1e-5)


def test_mixed_precision_close_to_fp32(ctx):
    g = small_geoms()[0]
    truth = phantom_for(g)
    p = O.exact_forward(g, truth.astype(np.float64)).astype(np.float32)
    ref = np.ones(g.volume_shape, np.float32)
    engine.Plan(ctx, g, "exact").mlem(p, ref, 5)
    for storage, tol in (("bf16", 2e-2), ("f16", 3e-3)):
        x = np.ones(g.volume_shape, np.float32)
        engine.Plan(ctx, g, "exact", storage).mlem(p, x, 5)
        assert rel_l2(x, ref) < tol, storage


# ----------------------------------------------------------- shift-and-add

@pytest.mark.parametrize("family,rule", [("rc", 0), ("exact", 1)])
def test_shift_and_add_vs_oracle(ctx, family, rule):
    g = small_geoms()[2]
    rng = np.random.default_rng(4)
    p = rng.random(g.proj_shape, dtype=np.float32)
    out = engine.Plan(ctx, g, family).shift_and_add(p)
    ref = O.saa(g, p, rule)
    assert np.abs(out - ref).max() <= 1e-6 * np.abs(ref).max()


def test_shift_and_add_staged_equals_direct(ctx):
    """The staged shift-and-add (TMA-loaded row bands; detector widths that
    are whole 16-byte units) and the direct kernel (any width) add the same
    rows in the same order: a detector widened by three columns, whose first
    columns are the narrow one's, gives the narrow one's slices bit for bit;
    both against the oracle, on geometries whose shifts leave the detector."""
    for g in (small_geoms()[2], linear_sweep(48, 40, 9, 0.5, 0.5, 3.0, 11, 64, 56, 0.4, 0.4, 35.0)):
        assert g.nu % 4 == 0
        rng = np.random.default_rng(9)
        p = rng.random(g.proj_shape, dtype=np.float32)
        gw = Geometry(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, g.nu + 3, g.nv, g.du, g.dv, g.src, g.det_origin,
                      g.fulcrum_z)
        pw = np.concatenate([p, rng.random((g.n_views, g.nv, 3), dtype=np.float32)], axis=2)
        staged = engine.Plan(ctx, g, "exact").shift_and_add(p)
        direct = engine.Plan(ctx, gw, "exact").shift_and_add(pw)
        assert np.array_equal(staged, direct[:, :, :g.nu])
        ref = O.saa(g, p, 1)
        assert np.abs(staged - ref).max() <= 1e-6 * np.abs(ref).max()


# ---------------------------------------------------------------- edges

def test_device_buffers_match_host(ctx):
    torch = pytest.importorskip("torch")
    g = small_geoms()[0]
    vol = phantom_for(g)
    for fam in ("rc", "exact"):
        plan = engine.Plan(ctx, g, fam)
        fh = plan.forward(vol)
        fd = plan.forward(torch.from_numpy(vol).cuda())
        torch.cuda.synchronize()
        assert np.array_equal(fd.cpu().numpy(), fh)
        bh = plan.back(fh)
        bd = plan.back(torch.from_numpy(fh).cuda())
        torch.cuda.synchronize()
        assert np.array_equal(bd.cpu().numpy(), bh)


@pytest.mark.parametrize("family", ["exact", "rc"])
@pytest.mark.parametrize("gi", [0, 1, 2])
def test_host_mlem_sart_overlapped_equal_device(ctx, gi, family):
    """Host-buffer MLEM / SART (FP32) overlap the copies with the first
    forward projection (view chunks growing 1, 4, 16, ...) and the last
    backprojection (slabs of slices shrinking to 1); the result equals the
    device-buffer call bit for bit for 1 to 4 iterations, with ragged pieces
    (5 views: 1 + 4, 9 views: 1 + 4 + 4; 12 slices: 7 + 4 + 1, 16 slices:
    11 + 4 + 1)."""
    torch = pytest.importorskip("torch")
    g = small_geoms()[gi]
    p = O.exact_forward(g, phantom_for(g).astype(np.float64)).astype(np.float32)
    plan = engine.Plan(ctx, g, family)
    pd = torch.from_numpy(p).cuda()
    for iters in (1, 2, 3, 4):
        for method, relax, x0 in (("mlem", 1.0, 1.0), ("sart", 0.5, 0.0)):
            xh = np.full(g.volume_shape, x0, np.float32)
            getattr(plan, method)(p, xh, iters, relax)
            xd = torch.full(g.volume_shape, x0, dtype=torch.float32, device="cuda")
            getattr(plan, method)(pd, xd, iters, relax)
            torch.cuda.synchronize()
            assert np.array_equal(xd.cpu().numpy(), xh), (method, iters)


def test_rays_missing_the_volume_are_zero(ctx):
    g = linear_sweep(16, 16, 4, 0.5, 0.5, 1.0, 3, 40, 40, 0.5, 0.5, 10.0)
    det = g.det_origin.copy()
    det[:, 0] += 6.0                      # the last columns of the detector see no volume
    g = Geometry(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, g.nu, g.nv, g.du, g.dv, g.src, det, g.fulcrum_z)
    vol = np.ones(g.volume_shape, np.float32)
    for fam in ("rc", "exact"):
        f = engine.Plan(ctx, g, fam).forward(vol)
        assert (f[:, :, -5:] == 0).all() and (f > 0).any()


def test_tiny_and_single_view_geometries(ctx):
    for g in (linear_sweep(1, 1, 1, 1.0, 1.0, 1.0, 1, 3, 3, 0.5, 0.5, 0.0),
              linear_sweep(5, 3, 2, 1.0, 1.0, 1.0, 2, 7, 1, 0.8, 0.8, 5.0)):
        vol = np.arange(1, g.n_voxels + 1, dtype=np.float32).reshape(g.volume_shape)
        pe = engine.Plan(ctx, g, "exact")
        assert rel_l2(pe.forward(vol), O.exact_forward(g, vol.astype(np.float64))) < 1e-5
        pr = engine.Plan(ctx, g, "rc")
        assert np.array_equal(pr.forward(vol), O.rc_forward(g, vol))


def test_single_view_forward(ctx):
    g = small_geoms()[0]
    vol = phantom_for(g)
    for fam in ("rc", "exact"):
        plan = engine.Plan(ctx, g, fam)
        full = plan.forward(vol)
        one = plan.forward_single(vol, g.src[2], g.det_origin[2])
        if fam == "rc":
            assert np.array_equal(one, full[2])
        else:
            assert rel_l2(one, full[2]) < 1e-6


def test_invalid_arguments_return_status(ctx):
    g = small_geoms()[0]
    bad = Geometry(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, g.nu, g.nv, g.du, g.dv,
                   g.src * np.array([1, 1, -1], np.float32), g.det_origin, g.fulcrum_z)
    with pytest.raises(KvError) as e:
        engine.Plan(ctx, bad, "exact")          # source below the volume
    assert e.value.status == 2
    with pytest.raises(KvError) as e:
        engine.Plan(ctx, g, "rc", "bf16")
    assert e.value.status == 7
    plan = engine.Plan(ctx, g, "exact")
    with pytest.raises(ValueError):
        plan.forward(np.zeros(5, np.float32))


def test_chest_scale_exact_properties(ctx):
    """Size-independent checks at the chest-DT geometry (1024^2 x 128 volume,
    60 views of 2048^2): dot-product identity with FP64 reductions, and A 1 equal
    to the chord lengths of a sample of rays from the FP64 oracle."""
    torch = pytest.importorskip("torch")
    g = config_chest()
    plan = engine.Plan(ctx, g, "exact")
    gen = torch.Generator(device="cuda").manual_seed(1)
    x = torch.rand(g.volume_shape, generator=gen, device="cuda")
    y = torch.rand(g.proj_shape, generator=gen, device="cuda")
    ax = plan.forward(x)
    aty = plan.back(y)
    lhs = torch.dot(ax.double().flatten(), y.double().flatten()).item()
    rhs = torch.dot(x.double().flatten(), aty.double().flatten()).item()
    assert abs(lhs - rhs) <= DOT_REL * abs(lhs)
    ones = torch.ones(g.volume_shape, device="cuda")
    a1 = plan.forward(ones).cpu().numpy().reshape(-1)
    rays = np.random.default_rng(0).integers(0, g.n_rays, 20000)
    assert rel_l2(a1[rays], chord_lengths(g, rays)) < 1e-5


def chord_lengths(g, rays):
    """FP64 length of each ray inside the volume box (slab method)."""
    view = rays // (g.nu * g.nv)
    v = (rays // g.nu) % g.nv
    u = rays % g.nu
    s = g.src[view].astype(np.float64)
    p = g.det_origin[view].astype(np.float64)
    p[:, 0] += (u + 0.5) * np.float64(g.du)
    p[:, 1] += (v + 0.5) * np.float64(g.dv)
    d = p - s
    half = 0.5 * np.array([g.nx * g.dx, g.ny * g.dy, g.nz * g.dz])
    with np.errstate(divide="ignore", invalid="ignore"):
        t0 = (-half - s) / d
        t1 = (half - s) / d
    lo = np.maximum(0.0, np.minimum(t0, t1).max(axis=1))
    hi = np.minimum(1.0, np.maximum(t0, t1).min(axis=1))
    return np.maximum(hi - lo, 0.0) * np.linalg.norm(d, axis=1)


# ---------------------------------------------------------------- kernel shapes

def test_forward_slab_shapes_agree_and_match_fp64(ctx):
    """Every slab shape of the forward projector (rays per thread, slices per
    slab, stages, view group) sums each ray in the same order, so all give
    the same projections bit for bit; the one-thread-per-ray kernel sums the
    same weights in another order.  Both against the FP64 oracle."""
    for g in small_geoms():
        vol = phantom_for(g)
        ref = O.exact_forward(g, vol.astype(np.float64))
        plan = engine.Plan(ctx, g, "exact")
        if (g.nx * 4) % 16 != 0:
            # the volume's rows are no whole number of 16-byte TMA units: the
            # plan keeps the one-thread-per-ray kernel and refuses slab shapes
            assert plan.slab[0] == 0
            with pytest.raises(KvError):
                plan.set_slab(4, 4, 3, 16)
            assert rel_l2(plan.forward(vol), ref) < EXACT_FWD_REL_L2
            plan.close()
            continue
        assert plan.slab[0] > 0                              # the default path is the slab kernel
        outs = []
        for shape in [(8, 4, 2, 16), (4, 4, 3, 16), (4, 2, 2, 2), (2, 8, 2, 1), (2, 1, 4, 3)]:
            plan.set_slab(*shape)
            assert plan.slab == shape[:3] + (min(shape[3], g.n_views),)
            outs.append(plan.forward(vol))
        for o in outs[1:]:
            assert np.array_equal(o, outs[0])
        assert rel_l2(outs[0], ref) < EXACT_FWD_REL_L2
        plan.set_slab(0)
        assert plan.slab[0] == 0
        per_ray = plan.forward(vol)
        assert rel_l2(per_ray, ref) < EXACT_FWD_REL_L2
        assert rel_l2(outs[0], per_ray) < 1e-6
        plan.close()


def test_back_shapes_bit_identical(ctx):
    """The gather backprojector's work shapes (voxel rows and slices per
    thread, or one voxel per thread) evaluate the same weights in the same
    order per voxel: identical volumes, and the FP64 oracle within tolerance;
    likewise the FP64 sensitivity image.  The last geometry's detector rows
    are 40 times finer than its voxel rows (40-odd candidate rows per voxel
    row), so the candidate intervals take several fill passes and row chunks."""
    fine_rows = linear_sweep(24, 12, 6, 1.0, 2.0, 1.0, 5, 96, 640, 0.3, 0.05, 15.0)
    for g in small_geoms() + [fine_rows]:
        y = np.random.default_rng(3).random(g.proj_shape, dtype=np.float32)
        ref = O.exact_back(g, y.astype(np.float64))
        plan = engine.Plan(ctx, g, "exact")
        assert plan.back_shape == (8, 1)
        outs, sens = [], []
        for shape in [(0, 1), (1, 1), (2, 1), (2, 2), (4, 1), (4, 2), (8, 1)]:
            plan.set_back_shape(*shape)
            outs.append(plan.back(y))
            plan2 = engine.Plan(ctx, g, "exact")
            plan2.set_back_shape(*shape)
            sens.append(plan2.sensitivity())
            plan2.close()
        for o in outs[1:]:
            assert np.array_equal(o, outs[0])
        for s in sens[1:]:
            assert np.array_equal(s, sens[0])
        assert rel_l2(outs[0], ref) < EXACT_BACK_REL_L2
        with pytest.raises(KvError):
            plan.set_back_shape(1, 2)
        with pytest.raises(KvError):
            plan.set_back_shape(3, 1)
        plan.close()


def test_back_staging_bit_identical(ctx):
    """The TMA-staged backprojector (each view's detector patch in shared
    memory, one view ahead) against the gather kernel: identical volumes for
    the plain backprojection and after MLEM / SART iterations (fused
    updates), on every geometry whose detector rows are a whole number of 16
    bytes; the others (nu = 37) are refused, as are 16-bit storage and bad
    shapes.  The last geometry's detector rows are 20 times finer than its
    voxel rows (up to 25 candidate rows per voxel row: several fill passes)
    and its 88 x 244 patches leave room for two stages only."""
    torch = pytest.importorskip("torch")
    fine_rows = linear_sweep(24, 12, 6, 1.0, 1.0, 1.0, 5, 96, 256, 0.3, 0.05, 15.0)
    staged = 0
    for gi, g in enumerate(small_geoms() + [fine_rows]):
        y = np.random.default_rng(4).random(g.proj_shape, dtype=np.float32)
        plan = engine.Plan(ctx, g, "exact")
        ref = plan.back(y)
        p = O.exact_forward(g, phantom_for(g).astype(np.float64)).astype(np.float32)
        pd = torch.from_numpy(p).cuda()
        runs = {}
        for shape in [(0, 2), (4, 2), (8, 2), (4, 3)]:
            if shape[0]:
                try:
                    plan.set_back_staging(*shape)
                except KvError:
                    assert g.nu % 4 != 0 or (gi == 3 and shape == (4, 3)), (gi, shape)
                    continue
                staged += 1
                assert plan.back_staging[:2] == shape
                assert np.array_equal(plan.back(y), ref), shape
            else:
                plan.set_back_staging(0)
            out = []
            for method, relax, x0 in (("mlem", 1.0, 1.0), ("sart", 0.5, 0.0)):
                x = torch.full(g.volume_shape, x0, dtype=torch.float32, device="cuda")
                getattr(plan, method)(pd, x, 3, relax)
                torch.cuda.synchronize()
                out.append(x.cpu().numpy())
            runs[shape] = out
        for shape, out in runs.items():
            for a, b in zip(out, runs[(0, 2)]):
                assert np.array_equal(a, b), shape
        plan.set_back_staging(0)
        assert plan.back_staging[0] == 0
        plan.close()
    assert staged == 8
    g = small_geoms()[0]
    plan = engine.Plan(ctx, g, "exact", "bf16")
    with pytest.raises(KvError):
        plan.set_back_staging(4, 2)
    plan.close()
    plan = engine.Plan(ctx, g, "exact")
    for bad in [(2, 2), (4, 1), (4, 4)]:
        with pytest.raises(KvError):
            plan.set_back_staging(*bad)
    plan.close()


def test_exact_config1_full_size_vs_fp64(ctx):
    """The whole config-1 workload (256x256x64 voxels, 15 views of 512^2):
    the forward projection of its seeded 40-ellipsoid phantom and the
    backprojection of a seeded random projection stack against the FP64
    oracle, every ray and every voxel."""
    g = config_small()
    vol = O.phantom(g, ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, 40, ph.seed_for(1)))
    plan = engine.Plan(ctx, g, "exact")
    f = plan.forward(vol)
    ref = O.exact_forward(g, vol.astype(np.float64))
    assert rel_l2(f, ref) < EXACT_FWD_REL_L2
    assert np.abs(f - ref).max() < 1e-5 * np.abs(ref).max()
    y = np.random.default_rng(11).random(g.proj_shape, dtype=np.float32)
    b = plan.back(y)
    ref_b = O.exact_back(g, y.astype(np.float64))
    assert rel_l2(b, ref_b) < EXACT_BACK_REL_L2
    assert np.abs(b - ref_b).max() < 1e-5 * np.abs(ref_b).max()
    plan.close()
