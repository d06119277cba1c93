"""Host-side helpers of bench.py that need no GPU."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from kevernals_gb300.geometry import config_small, segments_per_ray, siddon_segments  # noqa: E402


def test_gather_rate_counts_siddon_segments():
    g = config_small()
    seg = siddon_segments(g, 8)
    r = bench.gather_rate("exact_fwd", g, 4, 4, 10.0)
    assert r["segments_per_launch"] == seg and r["gather_bytes"] == 4 * seg
    assert abs(r["gather_gbs"] - 4 * seg / 1e-2 / 1e9) < 1e-9 * r["gather_gbs"]
    # the central ray of the central view crosses every slice
    assert segments_per_ray(g, g.n_views // 2, g.nu / 2, g.nv / 2) >= g.nz
    assert bench.gather_rate("exact_back", g, 2, 2, 10.0)["gather_bytes"] == 2 * seg
    assert bench.gather_rate("rc_back", g, 4, 4, 10.0) == {}
    assert "gather_unavailable" in bench.gather_rate("exact_fwd", None, 4, 4, 10.0)


def test_reference_cpu_step_is_one_reference_mlem_iteration():
    """With the whole workload as its sample, a step of the timed reference
    arm is one iteration of the reference's MLEM (forward, ratio loop,
    backprojection, update loop) from the uniform start, bit for bit."""
    import numpy as np
    from kevernals_gb300 import phantom as ph
    from kevernals_gb300.geometry import linear_sweep
    from oracle import oracle as O
    g = linear_sweep(24, 20, 6, 0.5, 0.5, 1.0, 5, 24, 20, 0.4, 0.4, 10.0)
    truth = O.phantom(g, ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, 5, 7))
    times, units, desc, kind, cores, x = bench.reference_cpu_steps(g, truth, 1, 0, fraction=1.0)
    p = O.rc_forward(g, truth)
    want = O.rc_mlem(g, p, np.ones(g.volume_shape, np.float32), 1, 1.0)
    assert np.array_equal(x, want)
    assert units == 2 * g.n_rays and len(times) == 1 and "whole iterations" in desc
