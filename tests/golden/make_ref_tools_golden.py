"""Generates tests/golden/golden_ref_tools.npz from the REFERENCE's own code,
compiled from the reference tree by oracle/build_ref.sh:

  xml_flat_<i>, xml_acc_<j>   what the reference's XML geometry reader
                              (oracle/_ref/ref_geometry) prints for the files
                              of tests/test_geometry_xml.py (VARIANTS[i];
                              ACCESSOR_ARGS[j]), as JSON text, lists longer
                              than 1000 values replaced by the SHA-256 of
                              their float32 bytes (reduce_lists)
  drv_<method>_<relax>        SHA-256 of the volume the reference's
                              recons::MLEM / recons::ART
                              (oracle/_ref/ref_drivers) computes in 3
                              iterations on the seeded case of DRIVER_CASE
  drv_geometry                the driver case's geometry as the reference's
                              reader flattens it (JSON text)
  shifts_<k>, shift_geometry_<k>  the row shifts of the reference's
                              recons::ShiftAndAdd for SHIFT_CASES[k], and
                              that case's flattened geometry
  hist_<k>_<name>             the reference's HistUniformization16Bit /
                              HistHalfTop16Bit (oracle/_ref/ref_histogram) on
                              the 16-bit images of HIST_CASES[k]

so that the tests that compare the drop-in and the oracle with that code
still check something where the reference tree is absent.  Run in a
checkout where the reference tree is present:
    python tests/golden/make_ref_tools_golden.py
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from kevernals_gb300 import phantom as ph  # noqa: E402
from kevernals_gb300.geometry import Geometry  # noqa: E402
from oracle import build as ob  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.join(HERE, "golden_ref_tools.npz")

# the XML files (keyword arguments of test_geometry_xml.write_xml)
VARIANTS = [
    {},
    {"centre": (-3.5, 7.25, 12.0), "res": (7, 33, 21), "scale": (2.5, 0.4, 0.3), "views": 9,
     "roi": "0 0 0 0 99 74"},
    {"roi": "-5 3 0 0 150 90"},
    {"views": 1, "roi": "40 30 0 0 40 30"},
    {"centre": (0.125, -250.0, 600.0), "res": (64, 16, 8), "scale": (0.7, 1.1, 0.9), "views": 4},
]
ACCESSOR_XML = {"res": (3, 4, 5), "roi": "1 2 0 0 6 5"}
ACCESSOR_ARGS = [("accessors",), ("adapt", "3", "0", "9", "3", "accessors")]
DRIVER_CASE = {"xml": {"res": (8, 40, 36), "scale": (1.0, 0.5, 0.5), "roi": "30 20 0 0 79 59"},
               "ellipsoids": 6, "seed": 9, "iterations": 3}
SHIFT_CASES = [VARIANTS[0], DRIVER_CASE["xml"], VARIANTS[1], VARIANTS[4]]
HIST_SHAPE = (3, 17, 29)


def reduce_lists(d):
    """A JSON object with every list of more than 1000 values replaced by the
    SHA-256 of its values as float32 (bit-exact comparisons either way)."""
    out = {}
    for k, v in d.items():
        if isinstance(v, list) and len(v) > 1000:
            v = "sha256:" + hashlib.sha256(np.asarray(v, np.float32).tobytes()).hexdigest()
        out[k] = v
    return out


def digest(a):
    return "sha256:" + hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def last_json(cmd):
    out = subprocess.run(cmd, capture_output=True, text=True, check=True).stdout
    return [ln for ln in out.splitlines() if ln.startswith("{")][-1]


def geometry_from_flat(f):
    return Geometry(*f["n"], *f["d"], *f["det"], *f["pitch"], np.asarray(f["src"], np.float32).reshape(-1, 3),
                    np.asarray(f["det_origin"], np.float32).reshape(-1, 3), f["fulcrum_z"])


def driver_inputs(xml=None, flat=None):
    """The driver case's geometry (as the reference reads `xml`, or from its
    flattened JSON) and projections."""
    g = geometry_from_flat(json.loads(flat if flat is not None else last_json([ob.REF_GEOMETRY, xml])))
    c = DRIVER_CASE
    vol = O.phantom(g, ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, c["ellipsoids"], c["seed"]))
    return g, O.rc_forward(g, vol)


def hist_cases():
    """Float volumes whose 16-bit rescale feeds the histogram tools."""
    rng = np.random.default_rng(11)
    gamma = rng.gamma(2.0, 0.01, size=HIST_SHAPE).astype(np.float32)
    gamma[0, :4, :5] = 0.0
    levels = rng.integers(0, 4, size=HIST_SHAPE).astype(np.float32) * 0.25
    single = np.zeros(HIST_SHAPE, np.float32)
    single[1, 5:9, 3:12] = 1.0
    return [gamma, levels, single]


def load():
    """The fixtures, or None when they have not been generated."""
    return dict(np.load(OUT)) if os.path.exists(OUT) else None


def main():
    from test_geometry_xml import write_xml
    from test_output_tools import rescale_u16
    ob.build_ref()
    for f in (ob.REF_GEOMETRY, ob.REF_DRIVERS, ob.REF_HISTOGRAM):
        if not os.path.exists(f):
            raise SystemExit(f"{f} missing: the reference tree is needed")
    out = {}
    with tempfile.TemporaryDirectory() as d:
        xml = os.path.join(d, "geo.xml")
        for i, kw in enumerate(VARIANTS):
            write_xml(xml, **kw)
            out[f"xml_flat_{i}"] = np.array(last_json([ob.REF_GEOMETRY, xml]))
        write_xml(xml, **ACCESSOR_XML)
        for j, args in enumerate(ACCESSOR_ARGS):
            out[f"xml_acc_{j}"] = np.array(json.dumps(reduce_lists(json.loads(last_json([ob.REF_GEOMETRY, xml, *args])))))
        write_xml(xml, **DRIVER_CASE["xml"])
        out["drv_geometry"] = np.array(last_json([ob.REF_GEOMETRY, xml]))
        g, p = driver_inputs(xml)
        p.tofile(os.path.join(d, "proj.raw"))
        for method in ("mlem", "art"):
            for relax in (0.5, 1.0):
                res = os.path.join(d, "x.raw")
                subprocess.run([ob.REF_DRIVERS, xml, os.path.join(d, "proj.raw"), method,
                                str(DRIVER_CASE["iterations"]), str(relax), res], check=True, capture_output=True)
                out[f"drv_{method}_{relax}"] = np.array(digest(np.fromfile(res, np.float32)))
        for k, kw in enumerate(SHIFT_CASES):
            write_xml(xml, **kw)
            flat = last_json([ob.REF_GEOMETRY, xml])
            out[f"shift_geometry_{k}"] = np.array(flat)
            g = geometry_from_flat(json.loads(flat))
            r = json.loads(last_json([ob.REF_DRIVERS, xml, "saa-shifts"]))
            out[f"shifts_{k}"] = np.asarray(r["shifts"], np.int32).reshape(g.nz, g.n_views)
        nz, ny, nx = HIST_SHAPE
        for k, vol in enumerate(hist_cases()):
            rescale_u16(vol).tofile(os.path.join(d, "u16.raw"))
            subprocess.run([ob.REF_HISTOGRAM, os.path.join(d, "u16.raw"), str(nx), str(ny), str(nz), d + "/"],
                           check=True)
            for name in ("uniform", "halftop"):
                out[f"hist_{k}_{name}"] = np.fromfile(os.path.join(d, f"{name}.raw"), np.uint16).reshape(HIST_SHAPE)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({os.path.getsize(OUT)} bytes, {len(out)} arrays)")


if __name__ == "__main__":
    main()
