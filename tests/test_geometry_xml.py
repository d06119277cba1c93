"""The drop-in header's reader of the reference's XML geometry files
(TomoGeometry(path), source/modules/geometry/TomoGeometry.cpp:13-434), on
the host: a synthetic file in that schema is read and its flattened
description is compared with the derivation restated here in float32
(TomoTable.cpp:4-19, TomoProjectionsSet.cpp:152-190, PixelSpacing.cpp,
Projector.cu:917-940).  The reference ships no geometry files, so this
reader's parity is pinned by the restated derivation only."""
import json
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
f32 = np.float32


def write_xml(path, centre=(10.0, 20.0, 40.0), res=(16, 64, 48), scale=(1.0, 0.5, 0.5), views=5,
              roi="10 20 0 0 89 79", rois=None, drop=None):
    cx, cy, cz = centre
    ys = np.linspace(-150.0, 150.0, views)
    parts = ['<?xml version="1.0" encoding="UTF-8"?>', "<!-- synthetic linear-sweep geometry -->", "<Geometry>"]
    if drop != "Rotation":
        parts.append(f"  <Rotation><center>{cx} {cy} {cz + 150.0}</center></Rotation>")
    if drop != "Grid":
        parts.append(f"  <Grid><center>{cx} {cy} {cz}</center><scale>{scale[0]} {scale[1]} {scale[2]}</scale>"
                     f"<resolution>{res[0]} {res[1]} {res[2]}</resolution></Grid>")
    parts.append("  <XRay><sources>")
    for i, y in enumerate(ys):
        parts.append(f"    <source>{cx + 0.25 * i} {cy + y} {cz + 900.0 + 0.1 * i}</source>")
    parts.append("  </sources></XRay>")
    parts.append("  <Camera><totalWidth>40</totalWidth><totalHeight>30</totalHeight>"
                 "<pixelWidth>100</pixelWidth><pixelHeight>75</pixelHeight><references>")
    for i in range(views):
        parts.append(f"    <reference>{cx - 20.0 + 0.01 * i} {cy - 15.0} {cz - 60.0 + 0.001 * i}</reference>")
    parts.append("  </references></Camera>")
    parts.append("  <Radios><rois>")
    for i in range(views):
        parts.append(f"    <roi>{rois[i] if rois else roi}</roi>")
    parts.append("  </rois></Radios>")
    parts.append("</Geometry>")
    with open(path, "w") as fh:
        fh.write("\n".join(parts) + "\n")


@pytest.fixture(scope="module")
def dumper(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("xml") / "geometry_xml_dump")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "geometry_xml_dump.cpp"), "-o", exe], check=True)
    return exe


def read(dumper, path):
    out = subprocess.run([dumper, path], check=True, capture_output=True, text=True).stdout
    return json.loads(out)


def expected(centre, res, scale, views, roi_bl, roi_tr):
    cx, cy, cz = (f32(c) for c in centre)
    ys = np.linspace(-150.0, 150.0, views)
    src = [(f32(cx + 0.25 * i) - cx, f32(cy + y) - cy, f32(cz + 900.0 + 0.1 * i) - cz) for i, y in enumerate(ys)]
    sx = f32(0)
    sz = f32(0)
    for s in src:
        sx = f32(sx + s[0])
        sz = f32(sz + s[2])
    sx = f32(sx / f32(views))
    sz = f32(sz / f32(views))
    det_bl = [(f32(cx - 20.0 + 0.01 * i) - cx, f32(cy - 15.0) - cy) for i in range(views)]
    zsum = 0.0
    for i in range(views):
        zsum += float(f32(cz - 60.0 + 0.001 * i) - cz)
    detz = f32(f32(zsum) / f32(views))
    du, dv = f32(f32(40) / f32(100)), f32(f32(30) / f32(75))
    det = []
    for x, y in det_bl:
        for _ in range(roi_bl[0]):
            x = f32(x + du)
        for _ in range(roi_bl[1]):
            y = f32(y + dv)
        det.append((x, y, detz))
    return {"n": [res[2], res[1], res[0]], "d": [scale[2], scale[1], scale[0]], "views": views,
            "det": [roi_tr[0] - roi_bl[0] + 1, roi_tr[1] - roi_bl[1] + 1], "pitch": [du, dv],
            "fulcrum_z": f32(centre[2] + 150.0),   # Rotation/center stays in the file's frame
            "src": [v for s in src for v in (sx, f32(s[1]), sz)], "det_origin": [v for d in det for v in d]}


def test_xml_geometry_matches_restated_derivation(dumper, tmp_path):
    path = str(tmp_path / "geo.xml")
    write_xml(path)
    got = read(dumper, path)
    assert got["valid"], got
    # the ROI's top row 79 is clamped to the detector's last row, 74
    exp = expected((10.0, 20.0, 40.0), (16, 64, 48), (1.0, 0.5, 0.5), 5, (10, 20), (89, 74))
    assert got["n"] == exp["n"] and got["views"] == exp["views"] and got["det"] == exp["det"]
    for k in ("d", "pitch", "src", "det_origin"):
        assert np.array_equal(np.asarray(got[k], np.float32), np.asarray(exp[k], np.float32)), k
    assert np.float32(got["fulcrum_z"]) == exp["fulcrum_z"]


def test_xml_geometry_rejects_bad_files(dumper, tmp_path):
    path = str(tmp_path / "bad.xml")
    write_xml(path, drop="Grid")
    got = read(dumper, path)
    assert not got["valid"] and "Grid" in got["error"]
    write_xml(path, rois=["10 20 0 0 89 79"] * 2 + ["11 20 0 0 89 79"] + ["10 20 0 0 89 79"] * 2)
    got = read(dumper, path)
    assert not got["valid"] and "ROI" in got["error"]
    with open(path, "w") as fh:
        fh.write("<Geometry><Grid><center>1 2 3</center>")
    got = read(dumper, path)
    assert not got["valid"] and "XML" in got["error"]
    got = read(dumper, str(tmp_path / "missing.xml"))
    assert not got["valid"] and "cannot open" in got["error"]


def test_xml_geometry_rejects_out_of_range_values(dumper, tmp_path):
    """Values a float cannot hold, non-positive counts and spacings, and
    non-finite positions are refused with a reason (not passed on)."""
    path = str(tmp_path / "geo.xml")
    write_xml(path)
    txt = open(path).read()
    cases = [("<scale>1.0 0.5 0.5</scale>", "<scale>1.0 1e40 0.5</scale>", "Grid/scale"),
             ("<scale>1.0 0.5 0.5</scale>", "<scale>1.0 -0.5 0.5</scale>", "Grid/scale"),
             ("<resolution>16 64 48</resolution>", "<resolution>16 0 48</resolution>", "Grid/resolution"),
             ("<resolution>16 64 48</resolution>", "<resolution>16 1e12 48</resolution>", "Grid/resolution"),
             ("<pixelWidth>100</pixelWidth>", "<pixelWidth>nan</pixelWidth>", "pixel counts"),
             ("<totalWidth>40</totalWidth>", "<totalWidth>-40</totalWidth>", "pitch"),
             ("<source>10.0 -130.0 940.0</source>", "<source>10.0 -130.0 inf</source>", "source"),
             ("<center>10.0 20.0 190.0</center>", "<center>10.0 20.0 1e39</center>", "fulcrum"),
             ("<roi>10 20 0 0 89 79</roi>", "<roi>10 20 0 0 1e30 79</roi>", "Radios/rois")]
    for old, new, why in cases:
        assert old in txt, old
        with open(path, "w") as fh:
            fh.write(txt.replace(old, new, 1))
        got = read(dumper, path)
        assert not got["valid"] and why in got["error"], (new, got)


def test_xml_reader_survives_hostile_files(tmp_path):
    """Truncations, seeded byte corruptions and out-of-range numbers of a good
    file, deep nesting and an entity flood, read by the dump tool built with
    AddressSanitizer and UBSan (plain when the compiler lacks them): each
    ends within a time limit with a result or a printable error."""
    import re
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "geometry_xml_dump")
    base = ["g++", "-std=c++17", "-O1", "-g", "-I", os.path.join(ROOT, "include"),
            os.path.join(ROOT, "tests", "cpp", "geometry_xml_dump.cpp"), "-o", exe]
    if subprocess.run(base + ["-fsanitize=address,undefined", "-fno-sanitize-recover=undefined"],
                      capture_output=True).returncode != 0:
        subprocess.run(base, check=True)
    good = str(tmp_path / "good.xml")
    write_xml(good)
    raw = open(good, "rb").read()
    rng = np.random.default_rng(2)
    variants = [raw[:c] for c in range(0, len(raw), 11)]
    for _ in range(80):
        b = bytearray(raw)
        for pos in rng.integers(0, len(raw), size=rng.integers(1, 4)):
            b[pos] = rng.integers(0, 256)
        variants.append(bytes(b))
    txt = raw.decode()
    spans = [m.span() for m in re.finditer(r"-?\d+(\.\d+)?", txt)]
    for bad in ("1e40", "nan", "-inf", "99999999999", "-2147483649", ""):
        for k in rng.choice(len(spans), 6, replace=False):
            a, b = spans[k]
            variants.append((txt[:a] + bad + txt[b:]).encode())
    variants.append(("<Geometry>" + "<a>" * 100000 + "</a>" * 100000 + "</Geometry>").encode())
    variants.append(("<Geometry><Rotation><center>" + "&amp;" * 200000 + "</center></Rotation></Geometry>").encode())
    path = str(tmp_path / "v.xml")
    for v in variants:
        with open(path, "wb") as fh:
            fh.write(v)
        r = subprocess.run([exe, path], capture_output=True, timeout=20)
        assert r.returncode == 0 and b"ERROR" not in r.stderr and b"runtime error" not in r.stderr, r.stderr[-1500:]
        out = json.loads(r.stdout.decode("ascii"))
        assert out["valid"] or out["error"]


def test_demonstration_adaptations(dumper, tmp_path):
    """PerformCheatingAdaptationsForDemonstration (TomoGeometry.cpp:593-611),
    as mainReconstruct.cpp applies it.  Indices {3, 0, 9, 3} of 5 views,
    erased in decreasing order as the reference does: 9 is out of range, the
    repeated 3 erases the view that moved into that slot (view 4), so views
    1 and 2 remain.  100 slices, a 3048 x 3048 ROI whose pitch is the
    detector width / 3048; the common source x / z and the remaining ROI
    corners keep their values."""
    path = str(tmp_path / "geo.xml")
    write_xml(path)
    before = read(dumper, path)
    out = subprocess.run([dumper, path, "adapt", "3", "0", "9", "3"], check=True, capture_output=True,
                         text=True).stdout
    after = json.loads(out)
    assert after["valid"] and after["views"] == 2
    assert after["n"] == [before["n"][0], before["n"][1], 100] and after["d"] == before["d"]
    assert after["det"] == [3048, 3048]
    assert np.float32(after["pitch"][0]) == f32(f32(40) / f32(3048))
    assert np.float32(after["pitch"][1]) == f32(f32(30) / f32(3048))
    keep = [1, 2]
    src = np.asarray(before["src"], np.float32).reshape(-1, 3)
    det = np.asarray(before["det_origin"], np.float32).reshape(-1, 3)
    assert np.array_equal(np.asarray(after["src"], np.float32).reshape(-1, 3), src[keep])
    assert np.array_equal(np.asarray(after["det_origin"], np.float32).reshape(-1, 3), det[keep])


def _positions(first, step, n):
    out = [f32(first)]
    for _ in range(n - 1):
        out.append(f32(out[-1] + f32(step)))
    return np.asarray(out, np.float32)


def test_geometry_accessors(dumper, tmp_path):
    """The reference's value accessors (TomoGeometry.h:34-89 over TomoVolume
    and TomoProjectionsSet) against their construction restated in float32:
    extents count x spacing, the volume centred, positions by repeated
    addition of the spacing or pitch from the corner, the grid z-major, the
    detector and ROI sets each with its own corners, size, pitch and extent;
    then the same after the demonstration adaptation."""
    path = str(tmp_path / "geo.xml")
    write_xml(path, res=(3, 4, 5), roi="1 2 0 0 6 5")
    got = json.loads(subprocess.run([dumper, path, "accessors"], check=True, capture_output=True,
                                    text=True).stdout)
    n, d = (5, 4, 3), (f32(0.5), f32(0.5), f32(1.0))
    w = np.array([f32(n[k]) * d[k] for k in range(3)], np.float32)
    blf = (f32(-0.5) * w).astype(np.float32)
    eq = lambda a, b: np.array_equal(np.asarray(a, np.float32), np.asarray(b, np.float32))  # noqa: E731
    assert eq(got["wsize"], w) and eq(got["blf"], blf) and eq(got["trb"], blf + w)
    assert eq(got["volume_size"], [f32(f32(w[0] * w[1]) * w[2])])
    axes = [_positions(blf[k], d[k], n[k]) for k in range(3)]
    assert eq(got["xs"], axes[0]) and eq(got["ys"], axes[1]) and eq(got["zs"], axes[2])
    grid = [(x, y, z) for z in axes[2] for y in axes[1] for x in axes[0]]
    assert eq(np.asarray(got["grid"]).reshape(-1, 3), grid)
    pitch = (f32(f32(40) / f32(100)), f32(f32(30) / f32(75)))
    assert eq(got["det_wsize"], [40, 30]) and eq(got["det_pitch"], pitch) and eq(got["roi_pitch"], pitch)
    assert got["det_size"] == [100, 75] and got["roi_size"] == [6, 4]
    assert eq(got["roi_wsize"], [f32(6) * pitch[0], f32(4) * pitch[1]])
    exp = expected((10.0, 20.0, 40.0), (3, 4, 5), (1.0, 0.5, 0.5), 5, (1, 2), (6, 5))
    det_bl = [(f32(10.0 - 20.0 + 0.01 * i) - f32(10.0), f32(20.0 - 15.0) - f32(20.0)) for i in range(5)]
    assert eq(np.asarray(got["det_bl"]).reshape(-1, 2), det_bl)
    assert eq(got["det_x1"], _positions(det_bl[1][0], pitch[0], 100))
    assert eq(got["det_y1"], _positions(det_bl[1][1], pitch[1], 75))
    roi_bl = np.asarray(exp["det_origin"], np.float32).reshape(-1, 3)[:, :2]
    assert eq(got["roi_x1"], _positions(roi_bl[1][0], pitch[0], 6))
    assert eq(got["roi_y1"], _positions(roi_bl[1][1], pitch[1], 4))
    rois = np.asarray(got["roi_positions"]).reshape(5, 4, 6, 2)
    assert eq(rois[1, :, :, 0], np.tile(got["roi_x1"], (4, 1)))
    assert eq(rois[1, :, :, 1], np.tile(np.asarray(got["roi_y1"])[:, None], (1, 6)))
    assert np.asarray(got["det_positions"]).size == 2 * 5 * 75 * 100
    assert got["n_voxel_indices"] == 60 and got["last_voxel_index"] == 59
    assert got["n_det_indices"] == 5 * 75 * 100 and got["n_roi_indices"] == 5 * 4 * 6
    # after the demonstration adaptation: 100 slices from the same corner (the
    # volume no longer centred in z, as in the reference), 3048^2 detector and
    # ROI, the detector pitch from its extent, the ROI keeping its own pitch
    got = json.loads(subprocess.run([dumper, path, "adapt", "0", "accessors"], check=True,
                                    capture_output=True, text=True).stdout)
    assert eq(got["blf"], blf) and eq(got["zs"], _positions(blf[2], d[2], 100))
    assert got["det_size"] == [3048, 3048] and got["roi_size"] == [3048, 3048]
    assert eq(got["det_pitch"], [f32(40) / f32(3048), f32(30) / f32(3048)]) and eq(got["roi_pitch"], pitch)
    assert eq(got["roi_wsize"], [f32(3048) * pitch[0], f32(3048) * pitch[1]])
    assert eq(np.asarray(got["det_bl"]).reshape(-1, 2), det_bl[1:])
    assert got["n_roi_indices"] == 4 * 3048 * 3048


# ---- against the reference's own reader ------------------------------------

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_ref_tools_golden as G  # noqa: E402


@pytest.fixture(scope="module")
def ref_reader():
    """The reference's XML reader (its geometry module and tinyxml2, compiled
    from the reference tree by oracle/build_ref.sh), or None without the tree:
    the tests then use the fixtures tests/golden/make_ref_tools_golden.py
    recorded from it."""
    from oracle import build as ob
    ob.build_ref()
    return ob.REF_GEOMETRY if os.path.exists(ob.REF_GEOMETRY) else None


def _reference(ref_reader, key, args, reduce=False):
    """The reference reader's output for `args`: run live when it is built
    (the committed fixture must then agree with it), else the fixture."""
    fix = G.load()
    fixed = json.loads(str(fix[key])) if fix is not None and key in fix else None
    if ref_reader is None:
        if fixed is None:
            pytest.skip("neither the reference reader nor its fixtures")
        return fixed
    live = json.loads(G.last_json([ref_reader, *args]))
    if reduce:
        live = G.reduce_lists(live)
    assert fixed is None or live == fixed, f"{key}: tests/golden/golden_ref_tools.npz is stale"
    return live


def _same(ours, ref, keys):
    for k in keys:
        a, b = ours[k], ref[k]
        if isinstance(b, list) and b and isinstance(b[0], float):
            assert np.array_equal(np.asarray(a, np.float32), np.asarray(b, np.float32)), k
        else:
            assert a == b, k


@pytest.mark.parametrize("i", range(len(G.VARIANTS)))
def test_xml_reader_matches_reference_reader(dumper, ref_reader, tmp_path, i):
    """The drop-in's reader and the reference's own reader on the same files:
    what the projector receives is equal bit for bit."""
    path = str(tmp_path / "geo.xml")
    write_xml(path, **G.VARIANTS[i])
    ours, ref = read(dumper, path), _reference(ref_reader, f"xml_flat_{i}", [path])
    assert ours["valid"] and ref["valid"], (ours, ref)
    assert np.float32(ours["fulcrum_z"]) == np.float32(ref["fulcrum_z"])
    _same(ours, ref, ("n", "views", "det", "d", "pitch", "src", "det_origin"))


@pytest.mark.parametrize("j", range(len(G.ACCESSOR_ARGS)))
def test_xml_accessors_match_reference_reader(dumper, ref_reader, tmp_path, j):
    """Every value accessor, before and after the demonstration adaptation,
    equal to the reference reader's (long position lists compared through
    the SHA-256 of their float32 values)."""
    path = str(tmp_path / "geo.xml")
    write_xml(path, **G.ACCESSOR_XML)
    args = G.ACCESSOR_ARGS[j]
    ours = G.reduce_lists(json.loads(subprocess.run([dumper, path, *args], check=True, capture_output=True,
                                                    text=True).stdout))
    ref = _reference(ref_reader, f"xml_acc_{j}", [path, *args], reduce=True)
    assert set(ours) == set(ref)
    _same(ours, ref, sorted(ref))


def test_xml_invalid_files_match_reference_reader(dumper, ref_reader, tmp_path):
    """Files both readers refuse: a missing section, ROIs that differ between
    views (run live only)."""
    if ref_reader is None:
        pytest.skip("reference reader not built (needs the reference tree)")
    path = str(tmp_path / "bad.xml")
    for kw in ({"drop": "Grid"}, {"drop": "Rotation"},
               {"rois": ["10 20 0 0 89 79"] * 2 + ["11 20 0 0 89 79"] + ["10 20 0 0 89 79"] * 2}):
        write_xml(path, **kw)
        assert not read(dumper, path)["valid"] and not json.loads(G.last_json([ref_reader, path]))["valid"], kw


def test_geometry_part_views(dumper, tmp_path):
    """GetVolume / GetProjections / GetProjectionsRois / GetTable
    (TomoGeometry.h:86-89): read-only views whose accessors (the reference's
    TomoVolume, TomoProjectionsSet and TomoTable getters) return exactly the
    geometry's own values, before and after the demonstration adaptation."""
    path = str(tmp_path / "geo.xml")
    write_xml(path, res=(3, 4, 5), roi="1 2 0 0 6 5")
    for extra in ([], ["adapt", "1"]):
        got = json.loads(subprocess.run([dumper, path, *extra, "views"], check=True, capture_output=True,
                                        text=True).stdout)
        assert got["volume"] and got["projections"] and got["rois"] and got["table"], got
    assert got["voxels"] == 5 * 4 * 100 and got["views"] == 4
