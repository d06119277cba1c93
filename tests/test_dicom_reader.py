"""Projection ingestion of the C++ drop-in (include/kevernals_dicom.hpp):
DICOMReader::ReadDirectory (DICOMReader.cpp:85-203) and the log(1 + x)
preprocessing (mainReconstruct.cpp:113-124), on synthetic DICOM files written
here (Explicit and Implicit VR Little Endian, an undefined-length sequence
to skip, shuffled file names, acquisition times out of order).  The
reference reads DICOM through vtk-dicom, which is not available, so the
expected values restate its conventions (time-ordered, bottom-up rows, ROI
crop); parity with vtk-dicom itself is unpinned."""
import json
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from test_geometry_xml import write_xml

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LONG_VR = {"OB", "OD", "OF", "OL", "OV", "OW", "SQ", "SV", "UC", "UN", "UR", "UT", "UV"}
EXPLICIT_LE, IMPLICIT_LE = "1.2.840.10008.1.2.1", "1.2.840.10008.1.2"


def _pad(v, fill=b" "):
    return v + fill if len(v) % 2 else v


def _elem(group, element, vr, value, explicit):
    tag = struct.pack("<HH", group, element)
    if not explicit:
        return tag + struct.pack("<I", len(value)) + value
    if vr in LONG_VR:
        return tag + vr.encode() + b"\0\0" + struct.pack("<I", len(value)) + value
    return tag + vr.encode() + struct.pack("<H", len(value)) + value


def write_dicom(path, pixels, time, patient=True, explicit=True):
    rows, cols = pixels.shape
    us = lambda v: struct.pack("<H", v)  # noqa: E731
    ts = _pad(EXPLICIT_LE.encode() if explicit else IMPLICIT_LE.encode(), b"\0")
    meta = _elem(0x0002, 0x0010, "UI", ts, True)
    ds = b""
    ds += _elem(0x0008, 0x0032, "TM", _pad(time.encode()), explicit)
    # an undefined-length sequence with one undefined-length item, to be skipped
    item_body = _elem(0x0008, 0x1150, "UI", _pad(b"1.2.3", b"\0"), explicit)
    seq = (struct.pack("<HH", 0xFFFE, 0xE000) + struct.pack("<I", 0xFFFFFFFF) + item_body +
           struct.pack("<HHI", 0xFFFE, 0xE00D, 0) + struct.pack("<HHI", 0xFFFE, 0xE0DD, 0))
    tag = struct.pack("<HH", 0x0008, 0x1140)
    ds += (tag + b"SQ\0\0" + struct.pack("<I", 0xFFFFFFFF) if explicit else tag + struct.pack("<I", 0xFFFFFFFF)) + seq
    if patient:
        ds += _elem(0x0010, 0x0020, "LO", _pad(b"SYNTH01"), explicit)
    ds += _elem(0x0028, 0x0002, "US", us(1), explicit)
    ds += _elem(0x0028, 0x0010, "US", us(rows), explicit)
    ds += _elem(0x0028, 0x0011, "US", us(cols), explicit)
    ds += _elem(0x0028, 0x0100, "US", us(16), explicit)
    ds += _elem(0x0028, 0x0103, "US", us(0), explicit)
    ds += _elem(0x7FE0, 0x0010, "OW", pixels.astype("<u2").tobytes(), explicit)
    with open(path, "wb") as fh:
        fh.write(b"\0" * 128 + b"DICM" + meta + ds)


@pytest.fixture(scope="module")
def dumper(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("dicom") / "dicom_dump")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "dicom_dump.cpp"), "-o", exe], check=True)
    return exe


def test_read_directory_orders_crops_and_log_scales(dumper, tmp_path):
    # geometry: a 100 x 75 pixel detector, ROI from pixel (10, 20) to (89, 74)
    geo = str(tmp_path / "geo.xml")
    write_xml(geo, roi="10 20 0 0 29 33")               # ROI 20 x 14 pixels at (10, 20)
    d = tmp_path / "series"
    d.mkdir()
    rng = np.random.default_rng(3)
    times = ["101501.250", "101500.000", "101502.500", "101500.750", "101501.000"]
    imgs = [rng.integers(0, 4000, size=(75, 100)).astype(np.uint16) for _ in times]
    for i, (t, im) in enumerate(zip(times, imgs)):
        write_dicom(str(d / f"proj_{(7 * i) % 5}.dcm"), im, t, explicit=(i % 2 == 0))
    (d / "notes.txt").write_text("not a DICOM file")
    out = json.loads(subprocess.run([dumper, geo, str(d), "3"], check=True, capture_output=True,
                                    text=True).stdout)
    assert out["ok"], out
    order = sorted(range(len(times)), key=lambda i: times[i])
    del order[3]
    exp = np.stack([imgs[i][::-1][20:34, 10:30] for i in order]).astype(np.float32)
    assert out["dims"] == [20, 14, 4]
    got = np.asarray(out["data"], np.float32).reshape(4, 14, 20)
    assert np.array_equal(got, exp)
    assert np.allclose(np.asarray(out["log"], np.float32).reshape(4, 14, 20), np.log1p(exp.astype(np.float64)),
                       rtol=1e-6)


def test_read_directory_errors(dumper, tmp_path):
    geo = str(tmp_path / "geo.xml")
    write_xml(geo, roi="10 20 0 0 29 33")
    d = tmp_path / "bad"
    d.mkdir()
    write_dicom(str(d / "a.dcm"), np.zeros((75, 100), np.uint16), "1")
    with open(d / "b.dcm", "wb") as fh:
        fh.write(b"\0" * 128 + b"DICM" + _elem(0x0002, 0x0010, "UI", _pad(b"1.2.840.10008.1.2.4.50", b"\0"), True))
    out = json.loads(subprocess.run([dumper, geo, str(d)], check=True, capture_output=True, text=True).stdout)
    assert not out["ok"] and "transfer syntax" in out["error"] and out["code"] == "DICOM file reading failed"
    out = json.loads(subprocess.run([dumper, geo, str(tmp_path / "missing")], check=True, capture_output=True,
                                    text=True).stdout)
    assert not out["ok"] and "does not exist" in out["error"]
    small = tmp_path / "small"
    small.mkdir()
    write_dicom(str(small / "a.dcm"), np.zeros((20, 20), np.uint16), "1")
    out = json.loads(subprocess.run([dumper, geo, str(small)], check=True, capture_output=True, text=True).stdout)
    assert not out["ok"] and "ROI" in out["error"]


@pytest.fixture(scope="module")
def checked_dumper(tmp_path_factory):
    """The dump tool built with AddressSanitizer and UBSan (plain when the
    compiler lacks them)."""
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("dicom_asan") / "dicom_dump")
    base = ["g++", "-std=c++17", "-O1", "-g", "-I", os.path.join(ROOT, "include"),
            os.path.join(ROOT, "tests", "cpp", "dicom_dump.cpp"), "-o", exe]
    san = ["-fsanitize=address,undefined", "-fno-sanitize-recover=undefined"]
    if subprocess.run(base + san, capture_output=True).returncode != 0:
        subprocess.run(base, check=True)
    return exe


def test_malformed_files_are_errors_not_crashes(checked_dumper, tmp_path):
    """Every prefix of a file's header (and a few cuts inside the pixel data)
    and seeded byte corruptions of the header, in both VR encodings: the
    reader returns a result or an error with a printable message, within a
    time limit, with no sanitizer report."""
    geo = str(tmp_path / "geo.xml")
    write_xml(geo, roi="10 20 0 0 29 33")
    rng = np.random.default_rng(5)
    variants = []
    for explicit in (True, False):
        good = tmp_path / f"good_{explicit}.dcm"
        write_dicom(str(good), rng.integers(0, 4000, (75, 100)).astype(np.uint16), "101500", explicit=explicit)
        raw = good.read_bytes()
        hdr = len(raw) - 75 * 100 * 2
        variants += [raw[:cut] for cut in list(range(0, hdr + 8, 3)) + [hdr + 101, len(raw) - 1]]
        for _ in range(60):
            b = bytearray(raw)
            for pos in rng.integers(128, hdr, size=rng.integers(1, 4)):
                b[pos] = rng.integers(0, 256)
            variants.append(bytes(b))
    d = tmp_path / "series"
    d.mkdir()
    for v in variants:
        (d / "x.dcm").write_bytes(v)
        r = subprocess.run([checked_dumper, geo, str(d)], capture_output=True, timeout=20)
        assert r.returncode == 0 and b"ERROR" not in r.stderr and b"runtime error" not in r.stderr, r.stderr[-1500:]
        out = json.loads(r.stdout.decode("ascii"))
        assert out["ok"] or out["error"]
