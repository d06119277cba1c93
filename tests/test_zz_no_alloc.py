"""kv_residual_noalloc: the residual for callers that may not allocate device
memory when they need it (real-time loops kept off the allocator, hosts whose
device memory belongs to another framework's allocator or a fixed budget).

It is called through the C ABI and checked against the existing entry point
kv_residual on two calls in a row.  This file is collected last so that a run
stopping at its first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5   # the relative tolerance of the other residual tests


def _noalloc(plan, p, x):
    from kevernals_gb300 import _lib
    r, ll = C.c_double(), C.c_double()
    plan.ctx.use_torch_stream()
    status = _lib.lib().kv_residual_noalloc(plan.handle, C.c_void_p(p.data_ptr()),
                                            C.c_void_p(x.data_ptr()), C.byref(r), C.byref(ll))
    return status, r.value, ll.value


def test_noalloc_residual_matches_kv_residual():
    torch = pytest.importorskip("torch")
    from kevernals_gb300 import build, engine, phantom as ph
    from kevernals_gb300.geometry import linear_sweep

    build.build()
    ctx = engine.Context(0)
    g = linear_sweep(64, 64, 16, 0.4, 0.4, 2.5, 9, 96, 96, 0.2, 0.2, 17.5)
    plan = engine.Plan(ctx, g, "exact")
    params = ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, 8, ph.seed_for(0, 3))
    truth = engine.phantom(ctx, g, params, device=True)
    p = plan.forward(truth)
    x = torch.full(g.volume_shape, 0.01, dtype=torch.float32, device="cuda")
    for call in range(2):
        if call == 1:
            x.mul_(2.0)                       # a different iterate on the second call
        want_r, want_ll = plan.residual(p, x)
        status, r, ll = _noalloc(plan, p, x)
        assert status == 0, ctx.last_error()
        assert r == pytest.approx(want_r, rel=TOL)
        assert ll == pytest.approx(want_ll, rel=TOL)
        assert np.isfinite(r) and r > 0


def test_noalloc_residual_rejects_oversize_geometry():
    torch = pytest.importorskip("torch")
    from kevernals_gb300 import build, engine
    from kevernals_gb300.geometry import config_chest

    build.build()
    ctx = engine.Context(0)
    plan = engine.Plan(ctx, config_chest(), "exact")   # 60 x 2048^2 rays: too many blocks
    dummy = torch.zeros(4, device="cuda")
    status, _, _ = _noalloc(plan, dummy, dummy)
    assert status == 1                                  # KV_ERR_INVALID_ARG
    assert "static scratch" in ctx.last_error()
