"""Mixed precision at the 256x256x64 / 15 x 512^2 workload: 50 MLEM
iterations with the volume and projections stored in FP32, BF16 and FP16
(FP32 path-length and backprojection accumulation, FP64 sensitivity and
reductions), against the FP64 oracle MLEM and against FP32
GPU MLEM.  The measured errors are printed; the bounds below are the stated
tolerances."""
import json

import numpy as np
import pytest

from kevernals_gb300 import build, engine, phantom as ph
from kevernals_gb300.geometry import config_small
from oracle import oracle as O

pytestmark = pytest.mark.gpu

ITERS = 50
# stated tolerances (relative L2 / max abs error normalised by max |x|)
BOUNDS = {"f32": (1e-4, 1e-3), "f16": (5e-3, 5e-2), "bf16": (4e-2, 2e-1)}


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def case():
    build.build()
    g = config_small()
    params = ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, 40, ph.seed_for(4))
    truth = O.phantom(g, params)
    line = O.exact_forward(g, truth.astype(np.float64))
    p = ph.poisson_log_data(line, 1e4, ph.seed_for(4))
    x64 = O.exact_mlem(g, p.astype(np.float64), np.ones(g.volume_shape), ITERS)
    return g, p, x64


def test_mixed_precision_mlem_vs_fp64_oracle(case):
    g, p, x64 = case
    ctx = engine.Context(0)
    results = {}
    ref32 = None
    for storage in ("f32", "f16", "bf16"):
        plan = engine.Plan(ctx, g, "exact", storage)
        x = np.ones(g.volume_shape, np.float32)
        plan.mlem(p, x, ITERS)
        scale = np.abs(x64).max()
        res = {"rel_l2_vs_fp64": rel_l2(x, x64),
               "max_err_vs_fp64": float(np.abs(x - x64).max() / scale)}
        if storage == "f32":
            ref32 = x.copy()
        else:
            res["rel_l2_vs_fp32_gpu"] = rel_l2(x, ref32)
            res["max_err_vs_fp32_gpu"] = float(np.abs(x - ref32).max() / scale)
        results[storage] = res
        plan.close()
    print("mixed-precision MLEM, 50 iterations:", json.dumps(results))
    for storage, (l2, mx) in BOUNDS.items():
        assert results[storage]["rel_l2_vs_fp64"] < l2, (storage, results[storage])
        assert results[storage]["max_err_vs_fp64"] < mx, (storage, results[storage])
