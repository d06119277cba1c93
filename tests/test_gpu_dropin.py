"""The C++ drop-in API (include/kevernals_tomo.hpp) compiled and run as a
reference caller would use it, checked against the oracle."""
import os
import subprocess

import numpy as np
import pytest

from kevernals_gb300 import build
from kevernals_gb300.geometry import Geometry, linear_sweep
from kevernals_gb300 import phantom as ph
from oracle import oracle as O

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_dropin(tmp_path):
    lib = build.build()
    exe = tmp_path / "test_dropin"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "test_dropin.cpp"), "-o", str(exe),
                    "-L", os.path.dirname(lib), "-lkvtomo", "-Wl,-rpath," + os.path.dirname(lib)],
                   check=True)
    g0 = linear_sweep(40, 36, 12, 0.5, 0.5, 1.0, 5, 48, 44, 0.4, 0.4, 15.0)
    # the drop-in geometry keeps one source x / z and one detector z (TomoTable)
    src = g0.src.copy()
    src[:, 0] = np.float32(np.sum(src[:, 0], dtype=np.float32) / np.float32(g0.n_views))
    src[:, 2] = np.float32(np.sum(src[:, 2], dtype=np.float32) / np.float32(g0.n_views))
    g = Geometry(g0.nx, g0.ny, g0.nz, g0.dx, g0.dy, g0.dz, g0.nu, g0.nv, g0.du, g0.dv, src,
                 g0.det_origin, g0.fulcrum_z)
    vol = O.phantom(g, ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, 6, 99))
    proj = O.rc_forward(g, vol)
    case = tmp_path / "case.bin"
    with open(case, "wb") as f:
        f.write(np.array([g.nx, g.ny, g.nz, g.nu, g.nv, g.n_views], np.int32).tobytes())
        f.write(np.array([g.dx, g.dy, g.dz, g.du, g.dv, g.fulcrum_z, g.det_origin[0, 2]],
                         np.float32).tobytes())
        f.write(g.src.tobytes())
        f.write(np.ascontiguousarray(g.det_origin[:, :2]).tobytes())
        f.write(vol.tobytes())
        f.write(proj.tobytes())
    r = subprocess.run([str(exe), str(case), str(tmp_path) + "/"], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)

    def load(name, shape):
        return np.fromfile(tmp_path / name, np.float32).reshape(shape)
    assert np.array_equal(load("rc_fwd.raw", g.proj_shape), proj)
    assert np.array_equal(load("rc_back.raw", g.volume_shape), O.rc_back(g, proj))
    ones = np.ones(g.volume_shape, np.float32)
    assert np.array_equal(load("rc_mlem.raw", g.volume_shape), O.rc_mlem(g, proj, ones, 3, 0.5))
    assert np.array_equal(load("rc_art.raw", g.volume_shape), O.rc_art(g, proj, ones, 3, 0.5))
    saa = load("rc_saa.raw", (g.nz, g.nv, g.nu))
    ref = O.saa(g, proj, 0)
    assert np.abs(saa - ref).max() <= 1e-6 * np.abs(ref).max()
    e = load("exact_fwd.raw", g.proj_shape).astype(np.float64)
    eo = O.exact_forward(g, vol.astype(np.float64))
    assert np.linalg.norm(e - eo) <= 2e-6 * np.linalg.norm(eo)
    assert np.array_equal(load("rc_single.raw", (g.nv, g.nu)), proj[0])
    fbp = load("exact_fbp.raw", g.volume_shape).astype(np.float64)
    ref = O.exact_fbp(g, load("exact_fwd.raw", g.proj_shape), 16)
    assert np.linalg.norm(fbp - ref) <= 1e-5 * np.linalg.norm(ref)
    # verbose MLEM: TIFF pages (rows top first) equal the iterates, the
    # projections A x and the corrected projections 0.5 p / A x (A x where 0)
    from test_output_tools import read_tiff
    tif = lambda name: read_tiff(str(tmp_path / name))[:, ::-1, :]  # noqa: E731
    x = ones
    for it in range(2):
        q = O.rc_forward(g, x)
        assert np.array_equal(tif(f"verbose_currentProjectionStep{it}.tiff"), q)
        corrected = np.where(q != 0, np.float32(0.5) * (proj / np.where(q != 0, q, np.float32(1))), q)
        assert np.array_equal(tif(f"verbose_currentCorrectedProjectionStep{it}.tiff"), corrected.astype(np.float32))
        x = O.rc_mlem(g, proj, x, 1, 0.5)
        assert np.array_equal(tif(f"verbose_reconstructionstep{it}.tiff"), x)
    assert np.array_equal(read_tiff(str(tmp_path / "verbose_initialVolume.tiff"))[:, ::-1, :], ones)
