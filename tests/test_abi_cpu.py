"""CPU tests of the C-ABI library: it builds, loads, exports every symbol the
header declares, and its host-only logic works without a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from kevernals_gb300 import _lib, build, engine
from kevernals_gb300.geometry import config_small, linear_sweep
from oracle import oracle as O

HEADER = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include", "kvtomo.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(kv_[a-z0-9_]+)\s*\(", text)) - {"kv_iter_cb"})


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.lib()


def test_header_declares_the_api():
    syms = declared_symbols()
    for s in ("kv_forward", "kv_back", "kv_mlem", "kv_sart", "kv_shift_and_add", "kv_plan_create"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    for s in declared_symbols():
        assert hasattr(lib, s), s
    assert set(declared_symbols()) <= set(_lib.SIGNATURES), "binding misses a declared symbol"


def test_status_strings(lib):
    assert lib.kv_status_string(0) == b"ok"
    assert b"sm_103" in lib.kv_status_string(8)
    assert lib.kv_version().startswith(b"kvtomo")


def test_no_device_is_reported_not_fatal(lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = C.c_void_p()
    assert lib.kv_ctx_create(0, C.byref(h)) == 8   # KV_ERR_NO_DEVICE
    assert not h.value
    assert lib.kv_ctx_destroy(None) == 1


@pytest.mark.parametrize("family,rule", [("rc", 0), ("exact", 1)])
def test_shift_rule_matches_oracle(lib, family, rule):
    for g in (config_small(), linear_sweep(32, 32, 17, 0.4, 0.4, 2.5, 9, 64, 64, 0.3, 0.3, 25.0)):
        assert np.array_equal(engine.shift_and_add_shifts(g, family), O.saa_shifts(g, rule))


def test_shift_rule_rejects_degenerate_geometry(lib):
    g = linear_sweep(8, 8, 1, 0.5, 0.5, 1.0, 3, 8, 8, 0.5, 0.5, 10.0)   # one slice
    with pytest.raises(_lib.KvError):
        engine.shift_and_add_shifts(g, "rc")
    g = linear_sweep(8, 8, 4, 0.5, 0.5, 1.0, 1, 8, 8, 0.5, 0.5, 10.0)   # one view
    with pytest.raises(_lib.KvError):
        engine.shift_and_add_shifts(g, "exact")


def test_shift_rule_refuses_non_finite_values(lib):
    import dataclasses
    g = linear_sweep(8, 8, 4, 0.5, 0.5, 1.0, 3, 8, 8, 0.5, 0.5, 10.0)
    bad_src = g.src.copy()
    bad_src[1, 1] = np.nan
    for bad in (dataclasses.replace(g, fulcrum_z=float("nan")), dataclasses.replace(g, dy=float("inf")),
                dataclasses.replace(g, dv=0.0), dataclasses.replace(g, src=bad_src)):
        for family in ("rc", "exact"):
            with pytest.raises(_lib.KvError):
                engine.shift_and_add_shifts(bad, family)


@pytest.mark.parametrize("family,rule", [("rc", 0), ("exact", 1)])
def test_shift_rule_keeps_shifts_beyond_the_detector(lib, family, rule):
    """A detector of 4 rows under a +-25 deg sweep: most shifts exceed the
    row count and are returned as the rule gives them (the device copy
    limits them to +-nv, the same sum)."""
    g = linear_sweep(32, 32, 17, 0.4, 0.4, 2.5, 9, 64, 4, 0.3, 0.3, 25.0)
    ref = O.saa_shifts(g, rule)
    assert (np.abs(ref) > g.nv).any()
    assert np.array_equal(engine.shift_and_add_shifts(g, family), ref)


def test_cpp_dropin_compiles_and_links(lib, tmp_path):
    """The C++ drop-in headers (kevernals_tomo.hpp, kevernals_dicom.hpp,
    kevernals_output.hpp) compile with warnings as errors and the drop-in
    driver links against libkvtomo.so (running it needs a GPU)."""
    import shutil
    import subprocess
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    root = os.path.dirname(os.path.dirname(__file__))
    so = os.path.dirname(build.build())
    src = tmp_path / "all_headers.cpp"
    # the TIFF writer refuses a file beyond classic TIFF's 32-bit offsets
    # (without reading the data) and writes a small one
    src.write_text('#include "kevernals_tomo.hpp"\n#include "kevernals_dicom.hpp"\n'
                   '#include "kevernals_output.hpp"\n'
                   'int main(int, char **argv) {\n'
                   '    const uint8_t px[4] = {0, 0, 128, 63};\n'
                   '    if (kvtomo_detail::write_tiff_pages(argv[1], 70000, 70000, 1, 4, 3, px)) return 1;\n'
                   '    if (!kvtomo_detail::write_tiff_pages(argv[1], 1, 1, 1, 4, 3, px)) return 2;\n'
                   '    Result<ImageDataPtr> r = ReconstructorsErrorCode::MLEM;\n'
                   '    if (PrintErrorCode(r.error()) != "Reconstructors:4 MLEM reconstruction failed. Details: none.")\n'
                   '        return 3;\n'
                   '    TomoGeometry g({8, 8, 4}, {1.f, 1.f, 1.f}, {{0.f, -5.f, 100.f}, {0.f, 5.f, 100.f}},\n'
                   '                   {{-4.f, -4.f}, {-4.f, -4.f}}, -10.f, {8, 8}, {1.f, 1.f});\n'
                   '    std::ostringstream os;\n'
                   '    os << g;\n'
                   '    for (const char *h : {"volume ", "projections: ", "projections Rois: ", "table: "})\n'
                   '        if (os.str().find(h) == std::string::npos) return 4;\n'
                   '    auto im = ImageData::New();\n'
                   '    im->SetDimensions(3, 2, 2);\n'
                   '    im->SetSpacing(0.5, 0.25, 2.0);\n'
                   '    im->AllocateScalars();\n'
                   '    im->SetScalarComponentFromFloat(2, 1, 1, 0, 7.f);\n'
                   '    if (im->data()[(1 * 2 + 1) * 3 + 2] != 7.f || im->GetScalarComponentAsFloat(2, 1, 1, 0) != 7.f)\n'
                   '        return 5;\n'
                   '    if (im->GetScalarPointer(3, 0, 0) != nullptr || im->GetNumberOfPoints() != 12) return 6;\n'
                   '    int ext[6];\n'
                   '    im->GetExtent(ext);\n'
                   '    if (ext[1] != 2 || ext[3] != 1 || ext[5] != 1 || im->GetSpacing()[2] != 2.0) return 7;\n'
                   '    auto cp = ImageData::New();\n'
                   '    cp->DeepCopy(im);\n'
                   '    im->data()[0] = 1.f;\n'
                   '    if (cp->data()[0] != 0.f || cp->data()[11] != 7.f || cp->GetSpacing()[0] != 0.5) return 8;\n'
                   '    return 0;\n}\n')
    example = os.path.join(root, "tests", "cpp", "reconstruct_example.cpp")
    for f in (str(src), os.path.join(root, "tests", "cpp", "test_dropin.cpp"), example):
        r = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I",
                            os.path.join(root, "include"), f, "-o", str(tmp_path / "a.out"), "-L", so,
                            "-lkvtomo", "-Wl,-rpath," + so], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        if f == str(src):
            tif = tmp_path / "one.tif"
            assert subprocess.run([str(tmp_path / "a.out"), str(tif)]).returncode == 0
            assert tif.stat().st_size == 8 + 2 + 11 * 12 + 4 + 4
        if f == example:
            # the reference main's flow: errors before any device work are reported, not fatal
            from test_geometry_xml import write_xml
            run = lambda *a: subprocess.run([str(tmp_path / "a.out"), *a], capture_output=True,  # noqa: E731
                                            text=True)
            r = run(str(tmp_path / "missing.xml"), str(tmp_path), str(tmp_path) + "/")
            assert r.returncode == 1 and "invalid geometry: cannot open" in r.stdout
            write_xml(str(tmp_path / "geo.xml"))
            r = run(str(tmp_path / "geo.xml"), str(tmp_path / "no_series"), str(tmp_path) + "/")
            assert r.returncode == 1 and "does not exist" in r.stdout and "projections Rois:" in r.stdout


def test_host_entry_points_run_clean_under_sanitizers(lib, tmp_path):
    """kv_api.cu (the C ABI's host logic) rebuilt with AddressSanitizer and
    UBSan and linked with the normal kernel objects, then driven in a child
    process through the host-only entry points: the shift-and-add rule on
    ordinary, oblique and hostile geometries (huge shifts are limited, NaN
    refused), status strings and the no-device path.  No sanitizer report."""
    import shutil
    import subprocess
    import sys
    runtimes = [subprocess.run(["gcc", f"-print-file-name={n}"], capture_output=True, text=True).stdout.strip()
                for n in ("libasan.so", "libubsan.so")]
    if shutil.which("gcc") is None or not all(os.path.isabs(r) and os.path.exists(r) for r in runtimes):
        pytest.skip("sanitizer runtimes not available")
    from kevernals_gb300 import build as kb
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    csrc = os.path.join(root, "kevernals_gb300", "csrc")
    api = str(tmp_path / "kv_api.o")
    subprocess.run([kb.nvcc(), "-std=c++17", "-O1", "-g", *kb.ARCH, "-Xcompiler",
                    "-fPIC,-fsanitize=address,-fsanitize=undefined,-fno-omit-frame-pointer",
                    "-I", os.path.join(root, "include"), "-I", csrc, "-c", os.path.join(csrc, "kv_api.cu"),
                    "-o", api], check=True, capture_output=True)
    objs = [os.path.join(kb.BUILD, os.path.splitext(s)[0] + ".o") for s in kb.SOURCES if s != "kv_api.cu"]
    so = str(tmp_path / "libkvtomo_asan.so")
    subprocess.run([kb.nvcc(), "-shared", *kb.ARCH, "-o", so, api, *objs, "-lcudart", "-Xcompiler",
                    "-fsanitize=address,-fsanitize=undefined"], check=True, capture_output=True)
    script = f"""
import dataclasses, sys
sys.path.insert(0, {root!r})
import ctypes as C
import numpy as np
from kevernals_gb300 import _lib
_lib.LIB_PATH = {so!r}
from kevernals_gb300 import engine
from kevernals_gb300.geometry import config_chest, config_small, linear_sweep
L = _lib.lib()
assert L.kv_status_string(0) == b"ok"
h = C.c_void_p()
assert L.kv_ctx_create(0, C.byref(h)) == 8 and L.kv_ctx_destroy(None) == 1
for g in (config_small(), config_chest(), linear_sweep(32, 32, 17, 0.4, 0.4, 2.5, 9, 64, 4, 0.3, 0.3, 25.0),
          linear_sweep(8, 8, 2, 0.5, 0.5, 1.0, 3, 8, 8, 0.5, 0.5, 89.0)):
    for fam in ("rc", "exact"):
        engine.shift_and_add_shifts(g, fam)
g = linear_sweep(8, 8, 4, 0.5, 0.5, 1.0, 3, 8, 8, 0.5, 0.5, 10.0)
src = g.src.copy()
src[:, 1] = np.float32(3e38)
assert np.abs(engine.shift_and_add_shifts(dataclasses.replace(g, src=src), "rc")).max() == 1 << 30
for bad in (dataclasses.replace(g, fulcrum_z=float("nan")), dataclasses.replace(g, dz=float("inf"))):
    for fam in ("rc", "exact"):
        try:
            engine.shift_and_add_shifts(bad, fam)
            raise SystemExit("accepted a non-finite geometry")
        except _lib.KvError:
            pass
"""
    env = dict(os.environ, LD_PRELOAD=":".join(runtimes), ASAN_OPTIONS="detect_leaks=0:halt_on_error=1",
               UBSAN_OPTIONS="halt_on_error=1")
    r = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0 and "ERROR" not in r.stderr and "runtime error" not in r.stderr, r.stderr[-3000:]


def test_python_handles_are_context_managers():
    """Context, Plan and UNet close their handles on leaving a with block
    (checked on a stand-in handle: creating one needs a GPU)."""
    for cls in (engine.Context, engine.Plan, engine.UNet):
        obj = cls.__new__(cls)
        obj._h = None                       # nothing to destroy
        with obj as same:
            assert same is obj
        assert obj._h is None
