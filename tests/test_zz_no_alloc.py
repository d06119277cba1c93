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


def test_noalloc_residual_block_limit_is_exact():
    """At exactly KV_NOALLOC_MAX_BLOCKS forward blocks the call is accepted
    and matches kv_residual; one block more is refused.  Blocks are
    ceil(nu / 32) * ceil(nv / fwd_rows) * n_views with the plan's forward
    block height, set here to one row."""
    torch = pytest.importorskip("torch")
    from kevernals_gb300 import build, engine
    from kevernals_gb300.geometry import linear_sweep

    build.build()
    max_blocks = 65536
    ctx = engine.Context(0)
    # 1 column tile x 1024 rows x 64 views = 65536 blocks of 32 x 1 rays
    g = linear_sweep(32, 32, 8, 0.5, 0.5, 1.0, 64, 32, 1024, 0.4, 0.0125, 15.0)
    plan = engine.Plan(ctx, g, "exact")
    plan.set_tuning(1, 8)
    assert ((g.nu + 31) // 32) * g.nv * g.n_views == max_blocks
    x = torch.rand(g.volume_shape, device="cuda") + 0.5
    p = plan.forward(x) * 1.01
    for call in range(2):
        want_r, want_ll = plan.residual(p, x)
        status, r, ll = _noalloc(plan, p, x)
        assert status == 0, ctx.last_error()
        assert r == pytest.approx(want_r, rel=TOL) and ll == pytest.approx(want_ll, rel=TOL)
        x.mul_(1.1)
    # one block more: 65537 rows of one view
    g2 = linear_sweep(32, 32, 8, 0.5, 0.5, 1.0, 1, 32, max_blocks + 1, 0.4, 0.0002, 15.0)
    plan2 = engine.Plan(ctx, g2, "exact")
    plan2.set_tuning(1, 8)
    dummy = torch.zeros(4, device="cuda")
    status, _, _ = _noalloc(plan2, dummy, dummy)
    assert status == 1 and "static scratch" in ctx.last_error()
