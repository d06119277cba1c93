"""CPU tests of the oracle itself: pinned against the reference kernels (run
here when the reference tree is present, and through the committed golden
fixtures everywhere) and against known answers for the FP64 Siddon."""
import hashlib
import json
import os

import numpy as np
import pytest

from kevernals_gb300 import phantom as ph
from kevernals_gb300.geometry import Geometry, config_small, linear_sweep
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def load_small():
    z = np.load(os.path.join(GOLDEN, "golden_small.npz"))
    cases = {}
    for name in ("a", "b", "c"):
        nx, ny, nz, nu, nv = (int(t) for t in z[f"{name}_dims"])
        dx, dy, dz, du, dv, fz = (float(t) for t in z[f"{name}_spacing"])
        g = Geometry(nx, ny, nz, dx, dy, dz, nu, nv, du, dv, z[f"{name}_src"], z[f"{name}_det"], fz)
        cases[name] = (g, {k[len(name) + 1:]: z[k] for k in z.files if k.startswith(name + "_")})
    return cases


@pytest.mark.parametrize("name", ["a", "b", "c"])
def test_rc_oracle_matches_reference_golden(name):
    g, d = load_small()[name]
    vol = O.phantom(g, d["params"])
    assert np.array_equal(vol, d["vol"])
    assert np.array_equal(O.rc_forward(g, vol), d["fwd"])          # bit-exact
    assert np.array_equal(O.rc_back(g, d["fwd"]), d["back"])
    assert np.array_equal(O.rc_back(g, d["y"]), d["back_y"])


def test_golden_covers_missed_rays_and_single_view():
    cases = load_small()
    g, d = cases["b"]
    assert (d["fwd"] == 0).any() and (d["fwd"] > 0).any()
    g, d = cases["c"]
    assert g.n_views == 1


@pytest.mark.skipif(O.ref_lib() is None, reason="reference tree not present")
def test_rc_oracle_matches_reference_kernels_random():
    rng = np.random.default_rng(7)
    for trial in range(3):
        nx, ny, nz = rng.integers(8, 30, 3)
        g = linear_sweep(int(nx), int(ny), int(nz), 0.5, 0.6, 1.1, int(rng.integers(2, 6)),
                         int(rng.integers(10, 40)), int(rng.integers(10, 40)), 0.45, 0.5,
                         float(rng.uniform(5, 25)))
        vol = rng.random(g.volume_shape, dtype=np.float32)
        f_ref = O.ref_forward(g, vol)
        assert np.array_equal(O.rc_forward(g, vol), f_ref)
        assert np.array_equal(O.rc_back(g, f_ref), O.ref_back(g, f_ref))


def test_rc_uniform_volume_known_answer():
    # the reference forward is a path-length weighted mean: 1 on every hitting ray
    g = linear_sweep(20, 20, 8, 0.5, 0.5, 1.0, 3, 30, 30, 0.4, 0.4, 10.0)
    f = O.rc_forward(g, np.ones(g.volume_shape, np.float32))
    assert set(np.unique(f)) <= {0.0, 1.0}
    assert (f == 1.0).mean() > 0.5


def _chord(g, view, u, v):
    """Analytic length of the ray (u, v) inside the volume box (slab method)."""
    s = g.src[view].astype(np.float64)
    p = g.det_origin[view].astype(np.float64) + np.array([(u + .5) * g.du, (v + .5) * g.dv, 0])
    d = p - s
    half = 0.5 * np.array([g.nx * g.dx, g.ny * g.dy, g.nz * g.dz])
    lo, hi = 0.0, 1.0
    for a in range(3):
        if d[a] == 0:
            if not (-half[a] <= s[a] < half[a]):
                return 0.0
            continue
        t0, t1 = sorted(((-half[a] - s[a]) / d[a], (half[a] - s[a]) / d[a]))
        lo, hi = max(lo, t0), min(hi, t1)
    return max(0.0, hi - lo) * np.linalg.norm(d)


def test_exact_oracle_chord_lengths():
    g = linear_sweep(16, 14, 6, 0.5, 0.5, 1.0, 3, 24, 22, 0.5, 0.5, 20.0)
    f = O.exact_forward(g, np.full(g.volume_shape, 2.0))
    for view in range(3):
        for (u, v) in [(0, 0), (5, 7), (12, 11), (23, 21)]:
            assert f[view, v, u] == pytest.approx(2.0 * _chord(g, view, u, v), rel=1e-12, abs=1e-12)
    assert np.allclose(O.exact_ray_lengths(g), f / 2.0, rtol=1e-12, atol=1e-12)


def test_exact_oracle_impulse_response():
    g = linear_sweep(9, 9, 5, 1.0, 1.0, 1.0, 2, 20, 20, 0.7, 0.7, 12.0)
    vol = np.zeros(g.volume_shape)
    vol[2, 4, 4] = 1.0
    f = O.exact_forward(g, vol)
    # the impulse response of each ray is its chord through the voxel box
    box_lo = np.array([4 * 1.0 - 4.5, 4 * 1.0 - 4.5, 2 * 1.0 - 2.5])
    for view in range(2):
        for v in range(20):
            for u in range(20):
                s = g.src[view].astype(np.float64)
                p = g.det_origin[view].astype(np.float64) + np.array([(u + .5) * np.float64(g.du), (v + .5) * np.float64(g.dv), 0])
                d = p - s
                lo, hi = 0.0, 1.0
                for a in range(3):
                    t0, t1 = sorted(((box_lo[a] - s[a]) / d[a], (box_lo[a] + 1 - s[a]) / d[a]))
                    lo, hi = max(lo, t0), min(hi, t1)
                want = max(0.0, hi - lo) * np.linalg.norm(d)
                assert f[view, v, u] == pytest.approx(want, abs=1e-12)


def test_exact_oracle_is_a_transpose():
    g = linear_sweep(12, 10, 6, 0.5, 0.5, 1.0, 4, 18, 16, 0.4, 0.4, 15.0)
    rng = np.random.default_rng(3)
    x = rng.random(g.volume_shape)
    y = rng.random(g.proj_shape)
    lhs = np.vdot(O.exact_forward(g, x), y)
    rhs = np.vdot(x, O.exact_back(g, y))
    assert abs(lhs - rhs) <= 1e-13 * abs(lhs)


def test_exact_oracle_mlem_decreases_residual():
    g = linear_sweep(16, 16, 6, 0.5, 0.5, 1.0, 5, 24, 24, 0.4, 0.4, 15.0)
    params = ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, 5, ph.seed_for(0, 1))
    truth = O.phantom(g, params).astype(np.float64)
    p = O.exact_forward(g, truth)
    res = []
    x = np.ones(g.volume_shape)
    for k in range(4):
        res.append(np.linalg.norm(O.exact_forward(g, x) - p) / np.linalg.norm(p))
        x = O.exact_mlem(g, p, x, 2)
    assert all(b < a for a, b in zip(res, res[1:]))
    assert (x >= 0).all()


def test_saa_shift_rules():
    g = config_small()
    rc = O.saa_shifts(g, 0)
    ex = O.saa_shifts(g, 1)
    assert rc.shape == ex.shape == (g.nz, g.n_views)
    # central view (source y = 0) is never shifted
    assert (rc[:, g.n_views // 2] == 0).all() and (ex[:, g.n_views // 2] == 0).all()
    # shifts are odd in the source position
    assert np.array_equal(ex[:, 0], -ex[:, -1])


def test_fbp_ramp_known_answers():
    """The FBP oracle's Shepp-Logan kernel h[n] = -2 / (pi^2 (4 n^2 - 1)):
    h[0] = 2 / pi^2, h[1] = -2 / (3 pi^2); its frequency response is
    |sin(w / 2)| / pi (the ramp |nu| times the sinc window, nu = w / 2 pi), up
    to the truncation error sum_{n > K} 2 |h[n]| < 1 / (pi^2 K); filtering an
    impulse along v reproduces the kernel; filtering is linear and leaves u
    and the views independent."""
    h = O.ramp_taps(4096)
    assert h[0] == 2.0 / np.pi ** 2 and abs(h[1] + 2.0 / (3.0 * np.pi ** 2)) < 1e-17
    n = np.arange(1, h.size)
    for w in (0.0, 0.3, np.pi / 3, 2.0, np.pi):
        resp = h[0] + 2.0 * np.sum(h[1:] * np.cos(n * w))
        assert abs(resp - abs(np.sin(w / 2.0)) / np.pi) < 1.0 / (np.pi ** 2 * 4096)
    K, nv = 8, 40
    p = np.zeros((2, nv, 3))
    p[1, 20, 2] = 1.0
    f = O.ramp_filter_v(p, K)
    hk = O.ramp_taps(K)
    expect = np.zeros(nv)
    expect[20 - K:20 + K + 1] = np.concatenate([hk[:0:-1], hk])
    assert np.array_equal(f[1, :, 2], expect)
    assert not f[0].any() and not f[1, :, :2].any()
    rng = np.random.default_rng(3)
    a, b = rng.random((2, 2, nv, 3))
    assert np.allclose(O.ramp_filter_v(2.0 * a - b, K), 2.0 * O.ramp_filter_v(a, K) - O.ramp_filter_v(b, K))


def test_siddon_segment_count_matches_oracle():
    """geometry.segments_per_ray -- the gather work the benchmark reports --
    equals the number of voxels the FP64 oracle's transpose of a single ray
    touches, on random rays of three geometries."""
    from kevernals_gb300.geometry import segments_per_ray, siddon_segments
    rng = np.random.default_rng(0)
    for g in (linear_sweep(40, 36, 12, 0.5, 0.5, 1.0, 5, 48, 44, 0.4, 0.4, 15.0),
              linear_sweep(33, 29, 7, 0.7, 0.45, 1.3, 4, 37, 41, 0.55, 0.35, 22.0),
              linear_sweep(64, 64, 16, 0.4, 0.4, 2.5, 9, 96, 96, 0.2, 0.2, 17.5)):
        for r in rng.integers(0, g.n_rays, 100):
            p, rem = divmod(int(r), g.nu * g.nv)
            v, u = divmod(rem, g.nu)
            vol = np.zeros(g.n_voxels)
            O.exact_back_rays(g, np.ones(1), np.array([r]), vol)
            assert int(segments_per_ray(g, p, u + 0.5, v + 0.5)) == np.count_nonzero(vol)
        # the sampled total extrapolates the full one closely
        full = siddon_segments(g, 1)
        assert abs(siddon_segments(g, 4) - full) <= 0.02 * full


def test_splitmix64_known_values():
    # first outputs of splitmix64 seeded with 0 (published reference sequence)
    r = ph.SplitMix64(0)
    assert r.next_u64() == 0xE220A8397B1DCDAF
    assert r.next_u64() == 0x6E789E6AA1B965F4
    a = ph.ellipsoid_params(64, 64, 16, 0.5, 0.5, 1.0, 10, 123)
    b = ph.ellipsoid_params(64, 64, 16, 0.5, 0.5, 1.0, 10, 123)
    assert np.array_equal(a, b) and a.shape == (11, 16)


def test_config1_digests_from_reference():
    info = json.load(open(os.path.join(GOLDEN, "golden_config1.json")))
    g = config_small()
    params = ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, 40, info["seed"])
    vol = O.phantom(g, params)
    d = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()  # noqa: E731
    assert d(vol) == info["phantom_sha256"]
    assert d(O.rc_forward(g, vol)) == info["ref_forward_sha256"]


def test_reference_gpu_guard_agrees_with_reference_hit_test():
    """oracle/ref_gpu.py launches the reference forward kernel only on
    geometries where every ray crosses the volume (the kernel has no defined
    result for a missed ray, Projector.cu:79-85).  Its host guard must never
    accept a geometry in which the reference's own hit test
    (FindProjectionAlphas_d's box clip, restated as kvo_rc_ray_hits) misses a
    ray, and it must refuse the config-1 geometry, whose detector extends
    past the volume's shadow."""
    from oracle import ref_gpu
    lib = O.lib()
    accepted = [linear_sweep(256, 256, 64, 0.5, 0.5, 1.0, 15, 224, 224, 0.4, 0.4, 15.0),
                linear_sweep(64, 48, 16, 0.5, 0.5, 1.0, 5, 40, 30, 0.4, 0.4, 10.0)]
    for g in accepted:
        assert ref_gpu.all_rays_cross_volume(g)
        cg = O.cgeom(g)
        for p in range(g.n_views):
            for v in range(0, g.nv, 3):
                for u in range(0, g.nu, 3):
                    assert lib.kvo_rc_ray_hits(cg, p, u, v)
    assert not ref_gpu.all_rays_cross_volume(config_small())
    assert not ref_gpu.all_rays_cross_volume(linear_sweep(64, 48, 16, 0.5, 0.5, 1.0, 5, 80, 60, 0.4, 0.4, 20.0))


def test_oracle_runs_clean_under_sanitizers(tmp_path):
    """The C oracle built with AddressSanitizer and UBSan, driven through its
    Python wrapper in a child process on geometries with missed rays, odd
    sizes and oblique sweeps: no sanitizer report, same results as the
    normal build."""
    import shutil
    import subprocess
    import sys
    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    runtimes = [subprocess.run(["gcc", f"-print-file-name={n}"], capture_output=True, text=True).stdout.strip()
                for n in ("libasan.so", "libubsan.so")]
    if not all(os.path.isabs(r) and os.path.exists(r) for r in runtimes):
        pytest.skip("sanitizer runtimes not available")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    so = str(tmp_path / "liboracle_asan.so")
    subprocess.run(["gcc", "-std=c11", "-O1", "-g", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                    "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
                    os.path.join(root, "oracle", "kvtomo_oracle.c"), "-o", so, "-lm"], check=True)
    script = f"""
import sys
sys.path.insert(0, {root!r})
import numpy as np
from oracle import build as b
b.build_oracle = lambda *a, **k: {so!r}
from oracle import oracle as O
from kevernals_gb300 import phantom as ph
from kevernals_gb300.geometry import linear_sweep
out = []
for g in (linear_sweep(33, 29, 7, 0.7, 0.45, 1.3, 4, 37, 41, 0.55, 0.35, 22.0),
          linear_sweep(16, 16, 4, 0.5, 0.5, 1.0, 3, 64, 48, 0.4, 0.4, 10.0)):
    vol = O.phantom(g, ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, 5, 3))
    p = O.rc_forward(g, vol)
    e = O.exact_forward(g, vol.astype(np.float64))
    out += [p, O.rc_back(g, p), O.rc_mlem(g, p, np.ones(g.volume_shape, np.float32), 2, 0.5),
            O.rc_art(g, p, np.ones(g.volume_shape, np.float32), 2, 0.5), e, O.exact_back(g, e),
            O.exact_mlem(g, e, np.ones(g.volume_shape), 2), O.exact_fbp(g, e, 8), O.saa_shifts(g, 0)]
np.savez({str(tmp_path / "asan.npz")!r}, *out)
"""
    env = dict(os.environ, LD_PRELOAD=":".join(runtimes), ASAN_OPTIONS="detect_leaks=0:halt_on_error=1",
               OMP_NUM_THREADS="2")
    r = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0 and "ERROR" not in r.stderr and "runtime error" not in r.stderr, r.stderr[-3000:]
    got = np.load(tmp_path / "asan.npz")
    i = 0
    for g in (linear_sweep(33, 29, 7, 0.7, 0.45, 1.3, 4, 37, 41, 0.55, 0.35, 22.0),
              linear_sweep(16, 16, 4, 0.5, 0.5, 1.0, 3, 64, 48, 0.4, 0.4, 10.0)):
        vol = O.phantom(g, ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, 5, 3))
        p = O.rc_forward(g, vol)
        assert np.array_equal(got[f"arr_{i}"], p)
        assert np.array_equal(got[f"arr_{i + 1}"], O.rc_back(g, p))
        i += 9


def _ref_tools():
    """(fixture module, fixtures or None, live checkers built?)"""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import make_ref_tools_golden as G
    from oracle import build as ob
    ob.build_ref()
    live = os.path.exists(ob.REF_DRIVERS) and os.path.exists(ob.REF_GEOMETRY)
    fix = G.load()
    if not live and fix is None:
        pytest.skip("neither the reference checkers nor their fixtures")
    return G, fix, live, ob


def test_rc_drivers_match_reference_drivers(tmp_path):
    """The oracle's restated ART and MLEM (the drivers the engine's RC path
    reproduces bit for bit) against the reference's own drivers --
    recons::ART / recons::MLEM of Reconstructors.h with PhantomMaker's uniform
    start, compiled from the reference tree and run on the reference's
    kernels built for the host (oracle/_ref/ref_drivers), or the digests of
    their results committed in tests/golden -- on a geometry read by the
    reference's reader, with rays that miss the volume: equal bit for bit,
    for 3 iterations at relax 0.5 and 1.0."""
    import subprocess
    G, fix, live, ob = _ref_tools()
    from test_geometry_xml import write_xml
    xml = str(tmp_path / "geo.xml")
    write_xml(xml, **G.DRIVER_CASE["xml"])
    if live:
        flat = G.last_json([ob.REF_GEOMETRY, xml])
        assert fix is None or json.loads(flat) == json.loads(str(fix["drv_geometry"])), "stale fixtures"
    else:
        flat = str(fix["drv_geometry"])
    g, p = G.driver_inputs(flat=flat)
    assert 0 < np.count_nonzero(p) < p.size           # some rays miss the volume
    p.tofile(tmp_path / "proj.raw")
    for method, restated in (("mlem", O.rc_mlem), ("art", O.rc_art)):
        for relax in (0.5, 1.0):
            ours = G.digest(restated(g, p, np.ones(g.volume_shape, np.float32), G.DRIVER_CASE["iterations"], relax))
            key = f"drv_{method}_{relax}"
            if live:
                subprocess.run([ob.REF_DRIVERS, xml, str(tmp_path / "proj.raw"), method,
                                str(G.DRIVER_CASE["iterations"]), str(relax), str(tmp_path / "x.raw")],
                               check=True, capture_output=True)
                ref = G.digest(np.fromfile(tmp_path / "x.raw", np.float32))
                assert fix is None or str(fix[key]) == ref, f"{key}: stale fixtures"
            else:
                ref = str(fix[key])
            assert ours == ref, (method, relax)


def test_rc_shift_rule_matches_reference_code(tmp_path):
    """The row shifts of the RC shift-and-add -- the C ABI's rule
    (kv_shift_and_add_shifts) and the oracle's -- against those the
    reference's own recons::ShiftAndAdd computes (Reconstructors.h:287-331),
    read back from its VTK filter calls by oracle/_ref/ref_drivers (or their
    committed fixtures), on geometry files read by the reference's reader:
    equal."""
    from kevernals_gb300 import build as kb, engine
    G, fix, live, ob = _ref_tools()
    kb.build()
    from test_geometry_xml import write_xml
    xml = str(tmp_path / "geo.xml")
    for k, kw in enumerate(G.SHIFT_CASES):
        if live:
            write_xml(xml, **kw)
            flat = G.last_json([ob.REF_GEOMETRY, xml])
            r = json.loads(G.last_json([ob.REF_DRIVERS, xml, "saa-shifts"]))
            assert r["status"] == "ok"
            ref = np.asarray(r["shifts"], np.int32)
            if fix is not None:
                assert json.loads(flat) == json.loads(str(fix[f"shift_geometry_{k}"])), "stale fixtures"
                assert np.array_equal(ref.reshape(fix[f"shifts_{k}"].shape), fix[f"shifts_{k}"]), "stale fixtures"
        else:
            flat, ref = str(fix[f"shift_geometry_{k}"]), fix[f"shifts_{k}"]
        g = G.geometry_from_flat(json.loads(flat))
        ref = np.asarray(ref, np.int32).reshape(g.nz, g.n_views)
        assert np.array_equal(engine.shift_and_add_shifts(g, "rc"), ref), kw
        assert np.array_equal(O.saa_shifts(g, 0), ref), kw
