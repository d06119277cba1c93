"""Batched uneven solves (one persistent launch per phase, the iteration loop
captured as a CUDA graph), graph-captured single-plan loops and the
autotuner."""
import time

import numpy as np
import pytest

from kevernals_gb300 import build, engine, phantom as ph
from kevernals_gb300.geometry import linear_sweep, uneven_cases

pytestmark = pytest.mark.gpu


def batch_cases(n, seed, scale=1):
    return uneven_cases(n, seed, scale)


def make_data(ctx, g, seed):
    import torch
    params = ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, 20, seed)
    truth = engine.phantom(ctx, g, params, device=True)
    p = engine.Plan(ctx, g, "exact").forward(truth)
    gen = torch.Generator(device="cuda").manual_seed(seed)
    counts = torch.poisson(1e4 * torch.exp(-p.double()), generator=gen)
    return torch.log(1e4 / counts.clamp_min(1.0)).clamp_min(0.0).float().contiguous()


@pytest.fixture(scope="module")
def ctx():
    build.build()
    return engine.Context(0)


def test_graph_captured_loop_matches_stepwise(ctx):
    g = linear_sweep(64, 48, 12, 0.5, 0.5, 1.0, 7, 80, 72, 0.4, 0.4, 15.0)
    p = make_data(ctx, g, 5).cpu().numpy()
    for fam in ("exact", "rc"):
        plan = engine.Plan(ctx, g, fam)
        x1 = np.ones(g.volume_shape, np.float32)
        plan.mlem(p, x1, 6, 0.9)                                  # captured as a graph
        x2 = np.ones(g.volume_shape, np.float32)
        plan.mlem(p, x2, 6, 0.9, callback=lambda *a: False)       # launched one by one
        assert np.array_equal(x1, x2), fam
        x3 = np.ones(g.volume_shape, np.float32)
        plan.mlem(p, x3, 6, 0.9)                                  # cached graph, relaunched
        assert np.array_equal(x1, x3), fam


def test_batch_matches_one_by_one(ctx):
    """The persistent batch (one-thread-per-ray forward tiles) against each
    plan's own solve (the slab forward projector where the geometry suits
    it: the same weights, summed in another order) and against the FP64
    oracle's MLEM."""
    import torch
    from oracle import oracle as O
    cases = batch_cases(6, 321, scale=4)
    plans = [engine.Plan(ctx, g, "exact") for g in cases]
    data = [make_data(ctx, g, 100 + i) for i, g in enumerate(cases)]
    xs = [torch.ones(g.volume_shape, device="cuda") for g in cases]
    engine.batch_mlem(ctx, plans, data, xs, 5)
    for plan, p, x in zip(plans, data, xs):
        ref = torch.ones(plan.geometry.volume_shape, device="cuda")
        plan.mlem(p, ref, 5)
        torch.cuda.synchronize()
        assert float((x - ref).norm() / ref.norm()) < 1e-5
    smallest = sorted(zip(cases, data, xs), key=lambda c: c[0].n_voxels + c[0].n_rays)[:2]
    for g, p, x in smallest:                            # the two smallest cases against FP64
        xo = O.exact_mlem(g, p.cpu().numpy().astype(np.float64), np.ones(g.volume_shape), 5)
        xg = x.cpu().numpy()
        assert np.linalg.norm(xg - xo) / np.linalg.norm(xo) < 1e-5
    # host buffers through the same entry point
    hp = [p.cpu().numpy() for p in data]
    hx = [np.ones(g.volume_shape, np.float32) for g in cases]
    engine.batch_mlem(ctx, plans, hp, hx, 5)
    for x, hxx in zip(xs, hx):
        assert np.array_equal(x.cpu().numpy(), hxx)


def test_batch_throughput_vs_one_by_one(ctx):
    """32 seeded uneven cases x 30 MLEM iterations: batched vs sequential."""
    import torch
    cases = batch_cases(32, 20261203 + 3000)
    plans = [engine.Plan(ctx, g, "exact") for g in cases]
    data = [make_data(ctx, g, 3000 + i) for i, g in enumerate(cases)]
    for plan in plans:                  # sensitivity images outside the timing
        plan.sensitivity(device=True)
    xs = [torch.ones(g.volume_shape, device="cuda") for g in cases]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    engine.batch_mlem(ctx, plans, data, xs, 30)
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    ys = [torch.ones(g.volume_shape, device="cuda") for g in cases]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for plan, p, y in zip(plans, data, ys):
        plan.mlem(p, y, 30)
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0
    rays = sum(2 * g.n_rays for g in cases) * 30
    print(f"batch of 32 uneven cases x 30 MLEM iterations: batched {t_batch:.3f} s "
          f"({rays / t_batch:.3e} rays/s), one by one {t_seq:.3f} s ({rays / t_seq:.3e} rays/s), "
          f"speed-up {t_seq / t_batch:.2f}x")
    for x, y in zip(xs, ys):
        assert float((x - y).norm() / y.norm()) < 1e-4


def test_autotune_picks_valid_shapes(ctx):
    g = linear_sweep(128, 128, 32, 0.5, 0.5, 1.0, 9, 256, 256, 0.4, 0.4, 15.0)
    plan = engine.Plan(ctx, g, "exact")
    f, b = plan.autotune()
    assert f in (1, 2, 4, 8) and b in (2, 4, 8)
    vol = np.random.default_rng(0).random(g.volume_shape, dtype=np.float32)
    tuned = plan.forward(vol)
    plan.set_tuning(4, 8)
    assert np.array_equal(tuned, plan.forward(vol))   # the shape changes the speed, not the result
    with pytest.raises(engine.KvError):
        plan.set_tuning(0, 8)
