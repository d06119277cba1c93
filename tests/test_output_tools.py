"""Output and post-processing of the C++ drop-in (include/kevernals_output.hpp):
multi-page TIFF writers, the 16-bit rescale of the reference's tomosynthesis
reconstructor (vtkImageShiftScale, TomosynthesisFBPReconstructor.cpp:57-66)
and its histogram tools (HistogramMatchingTools.h:12-179), checked against
numpy restatements; the TIFF files are read back by a small parser here."""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def read_tiff(path):
    """Pages of an uncompressed little-endian TIFF, top row first, with tags."""
    b = open(path, "rb").read()
    assert b[:4] == b"II*\0"
    off = struct.unpack_from("<I", b, 4)[0]
    pages = []
    while off:
        n = struct.unpack_from("<H", b, off)[0]
        tags = {}
        for i in range(n):
            t, typ, cnt = struct.unpack_from("<HHI", b, off + 2 + 12 * i)
            v = struct.unpack_from("<H" if typ == 3 else "<I", b, off + 10 + 12 * i)[0]
            tags[t] = v
        w, h, bits, fmt = tags[256], tags[257], tags[258], tags[339]
        dt = {(32, 3): "<f4", (16, 1): "<u2"}[(bits, fmt)]
        assert tags[259] == 1 and tags[277] == 1
        data = np.frombuffer(b, dt, w * h, tags[273]).reshape(h, w)
        pages.append(data)
        off = struct.unpack_from("<I", b, off + 2 + 12 * n)[0]
    return np.stack(pages)


def rescale_u16(x):
    v = x.astype(np.float64) * ((65535 - 1) / float(x.max()))
    return np.clip(v, 0, 65535).astype(np.uint16)


def hist_match(expected, img, slice_pixels):
    expected = np.asarray(expected, np.float64).copy()
    orig = np.bincount(img.ravel(), minlength=65536).astype(np.float64)
    first = int(np.argmax(expected != 0))
    if expected[first] == slice_pixels:
        return np.full_like(img, first)
    expected[0] = 0
    orig[0] = 0
    ce = np.cumsum(expected)
    co = np.cumsum(orig)
    ce /= ce[-1]
    co /= co[-1]
    up = np.searchsorted(ce, co, side="right")
    lut = np.empty(65536, np.int64)
    for g in range(65536):
        u = up[g]
        if u == 65536:
            lut[g] = g
        elif u > 0 and co[g] - ce[u - 1] < ce[u] - co[g]:
            lut[g] = u - 1
        else:
            lut[g] = u
    return np.clip(lut, 0, 65535).astype(np.uint16)[img]


@pytest.fixture(scope="module")
def tool(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("out") / "output_dump")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "output_dump.cpp"), "-o", exe], check=True)
    return exe


def test_tiff_rescale_and_histogram_tools(tool, tmp_path):
    nx, ny, nz = 37, 23, 3
    rng = np.random.default_rng(5)
    vol = (rng.gamma(2.0, 0.01, size=(nz, ny, nx))).astype(np.float32)
    vol[0, :4, :5] = 0.0                                  # a masked (zero) patch
    raw = tmp_path / "vol.raw"
    vol.tofile(raw)
    subprocess.run([tool, str(raw), str(nx), str(ny), str(nz), str(tmp_path)], check=True)
    # float TIFF: one page per slice, rows written top first
    pages = read_tiff(str(tmp_path / "vol.tif"))
    assert pages.shape == (nz, ny, nx)
    assert np.array_equal(pages[:, ::-1, :], vol)
    u16 = np.fromfile(tmp_path / "u16.raw", np.uint16).reshape(nz, ny, nx)
    assert np.array_equal(u16, rescale_u16(vol))
    assert np.array_equal(read_tiff(str(tmp_path / "u16.tif"))[:, ::-1, :], u16)
    uni = np.fromfile(tmp_path / "uniform.raw", np.uint16).reshape(nz, ny, nx)
    assert np.array_equal(uni, hist_match(np.ones(65536), u16, nx * ny))
    assert np.array_equal(read_tiff(str(tmp_path / "uniform.tif"))[:, ::-1, :], uni)
    half = np.fromfile(tmp_path / "halftop.raw", np.uint16).reshape(nz, ny, nx)
    exp = np.ones(65536)
    exp[:1000] *= 20
    assert np.array_equal(half, hist_match(exp, u16, nx * ny))
    # uniformisation spreads the grey levels over the whole range
    assert int(uni.max()) > 60000 and np.count_nonzero(uni[0, :4, :5]) == 0


def test_rescale_handles_non_finite_voxels(tool, tmp_path):
    """NaN voxels map to 0 and +-inf to the ends of the range; the scale comes
    from the largest finite voxel."""
    nx, ny, nz = 8, 4, 2
    vol = np.linspace(0.0, 2.0, nx * ny * nz, dtype=np.float32).reshape(nz, ny, nx)
    vol[0, 0, :3] = [np.nan, np.inf, -np.inf]
    raw = tmp_path / "vol.raw"
    vol.tofile(raw)
    subprocess.run([tool, str(raw), str(nx), str(ny), str(nz), str(tmp_path)], check=True)
    u16 = np.fromfile(tmp_path / "u16.raw", np.uint16).reshape(nz, ny, nx)
    assert list(u16[0, 0, :3]) == [0, 65535, 0]
    finite = np.isfinite(vol)
    exp = rescale_u16(np.where(finite, vol, 0.0).astype(np.float32))
    assert np.array_equal(u16[finite], exp[finite])


def test_histogram_tools_match_reference(tool, tmp_path):
    """HistUniformization16Bit / HistHalfTop16Bit of the drop-in against the
    reference's own header (HistogramMatchingTools.h, compiled from the
    reference tree by oracle/build_ref.sh, or its results committed in
    tests/golden) on the same 16-bit images: a rescaled gamma volume with a
    zero (masked) patch, a few-level image, and an image with one non-zero
    level.  Equal bit for bit."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_ref_tools_golden as G
    from oracle import build as ob
    ob.build_ref()
    live = os.path.exists(ob.REF_HISTOGRAM)
    fix = G.load()
    if not live and fix is None:
        pytest.skip("neither the reference histogram tools nor their fixtures")
    nz, ny, nx = G.HIST_SHAPE
    for k, vol in enumerate(G.hist_cases()):
        case = tmp_path / f"case{k}"
        case.mkdir()
        vol.tofile(case / "vol.raw")
        subprocess.run([tool, str(case / "vol.raw"), str(nx), str(ny), str(nz), str(case)], check=True)
        u16 = np.fromfile(case / "u16.raw", np.uint16)
        assert np.array_equal(u16, rescale_u16(vol).ravel())
        if live:
            ref = case / "ref"
            ref.mkdir()
            subprocess.run([ob.REF_HISTOGRAM, str(case / "u16.raw"), str(nx), str(ny), str(nz), str(ref) + "/"],
                           check=True)
            assert np.array_equal(np.fromfile(ref / "hist.raw", np.int32), np.bincount(u16, minlength=65536))
        for name in ("uniform", "halftop"):
            if live:
                expect = np.fromfile(ref / f"{name}.raw", np.uint16)
                assert fix is None or np.array_equal(fix[f"hist_{k}_{name}"].ravel(), expect), "stale fixtures"
            else:
                expect = fix[f"hist_{k}_{name}"].ravel()
            assert np.array_equal(np.fromfile(case / f"{name}.raw", np.uint16), expect), (k, name)
