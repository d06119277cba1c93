"""Generates the golden fixtures of tests/golden from the REFERENCE itself.

The reference's projector kernels (Kevernals source/modules/reconstruction/
Projector.cu: CudaPerformProjection and CudaPerformBackProjection) are
compiled for the host by oracle/build_ref.sh and run on seeded inputs:

  golden_small.npz    small geometries (inputs + reference outputs), used by
                      the CPU oracle tests and the GPU parity tests.
  golden_config1.json SHA-256 digests and summary statistics of the
                      reference outputs at the 256x256x64 / 15 x 512^2
                      workload (too large to store), so that the GPU path can
                      be checked bit for bit at full size.

Run in a checkout where the reference tree is present:
    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from kevernals_gb300 import phantom as ph  # noqa: E402
from kevernals_gb300.geometry import Geometry, config_small, linear_sweep  # noqa: E402
from oracle import oracle as O  # noqa: E402


def small_cases():
    """Small geometries covering the reference's regimes."""
    cases = {}
    # a: regular linear sweep
    cases["a"] = linear_sweep(40, 36, 12, 0.5, 0.5, 1.0, 5, 48, 44, 0.4, 0.4, 15.0)
    # b: anisotropic voxels, detector ROI shifted so that some rays miss the volume
    g = linear_sweep(24, 30, 9, 0.7, 0.45, 1.3, 4, 40, 36, 0.55, 0.35, 22.0)
    det = g.det_origin.copy()
    det[:, 0] += 9.0
    det[:, 1] -= 6.0
    cases["b"] = Geometry(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, g.nu, g.nv, g.du, g.dv,
                          g.src, det, g.fulcrum_z)
    # c: single view, odd sizes, source off the y axis in x
    g = linear_sweep(17, 23, 5, 0.6, 0.6, 2.0, 1, 29, 31, 0.5, 0.5, 0.0)
    src = g.src.copy()
    src[:, 0] = 13.0
    cases["c"] = Geometry(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, g.nu, g.nv, g.du, g.dv,
                          src, g.det_origin, g.fulcrum_z)
    return cases


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    if O.ref_lib() is None:
        raise SystemExit("reference kernels unavailable (reference tree absent)")
    out = {}
    for name, g in small_cases().items():
        params = ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, 8, ph.seed_for(1, ord(name)))
        vol = O.phantom(g, params)
        fwd = O.ref_forward(g, vol)
        back = O.ref_back(g, fwd)
        rng = np.random.default_rng(ord(name))
        y = rng.random(g.proj_shape, dtype=np.float32)
        back_rand = O.ref_back(g, y)
        out.update({f"{name}_src": g.src, f"{name}_det": g.det_origin,
                    f"{name}_dims": np.array([g.nx, g.ny, g.nz, g.nu, g.nv], np.int32),
                    f"{name}_spacing": np.array([g.dx, g.dy, g.dz, g.du, g.dv, g.fulcrum_z], np.float32),
                    f"{name}_params": params, f"{name}_vol": vol, f"{name}_fwd": fwd,
                    f"{name}_back": back, f"{name}_y": y, f"{name}_back_y": back_rand})
    np.savez_compressed(os.path.join(HERE, "golden_small.npz"), **out)

    g = config_small()
    t = time.time()
    params = ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, 40, ph.seed_for(1))
    vol = O.phantom(g, params)
    fwd = O.ref_forward(g, vol)
    back = O.ref_back(g, fwd)
    info = {
        "workload": "256x256x64 @ 0.5x0.5x1.0 mm, 15 views +-15 deg, 512x512 @ 0.4 mm, 40 ellipsoids",
        "seed": ph.seed_for(1),
        "phantom_sha256": digest(vol),
        "ref_forward_sha256": digest(fwd),
        "ref_back_of_forward_sha256": digest(back),
        "ref_forward_sum": float(fwd.astype(np.float64).sum()),
        "ref_back_sum": float(back.astype(np.float64).sum()),
        "seconds": round(time.time() - t, 1),
    }
    with open(os.path.join(HERE, "golden_config1.json"), "w") as f:
        json.dump(info, f, indent=1)
    print(json.dumps(info, indent=1))


if __name__ == "__main__":
    main()
