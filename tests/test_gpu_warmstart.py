"""What the learned warm start gains over plain MLEM, at a small scale.

Triples (shift-and-add, 30-iteration MLEM target) are generated by the engine
on 128x128x32 crops (chest-DT voxel size, 30 views over +-17.5 deg), the
U-Net is trained briefly, and on held-out phantoms the number of MLEM
iterations needed to reach the residual of 15 plain MLEM iterations (within
1%) is compared for three starts: uniform (plain MLEM), the shift-and-add
volume alone (the untrained network is the identity), and the trained
network.  Plain MLEM stays the arbiter: a start with a worse residual than the
uniform start is rejected.
"""
import numpy as np
import pytest

from kevernals_gb300 import build, engine, phantom as ph, warmstart as ws
from kevernals_gb300.geometry import linear_sweep

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

PLAIN_ITERS = 15


def geom():
    return linear_sweep(128, 128, 32, 0.4, 0.4, 2.5, 30, 512, 512, 0.2, 0.2, 17.5)


def iters_from(plan, p, x0, target):
    n, r = ws.iterations_to_residual(plan, p, x0.clone(), target, 3 * PLAIN_ITERS)
    return n, r


def test_learned_warm_start_gains_over_plain_mlem():
    build.build()
    ctx = engine.Context(0)
    ctx.use_torch_stream()
    g = geom()
    triples = [ws.make_triple(ctx, g, ph.seed_for(5, 10 + i), n_ellipsoids=20, target_iters=30)[:2]
               for i in range(24)]
    net = engine.UNet(ctx, seed=7)
    untrained = engine.UNet(ctx, seed=7)
    hist = ws.train(net, triples, epochs=6, lr=1e-3)
    assert hist[-1] < hist[0]
    results = []
    for case in range(3):
        seed = ph.seed_for(5, 900 + case)
        params = ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, 20, seed)
        truth = engine.phantom(ctx, g, params, device=True)
        plan = engine.Plan(ctx, g, "exact")
        p = ws.noisy_data(ctx, plan, truth, 5e4, seed)
        x = torch.ones(g.volume_shape, device="cuda")
        plan.mlem(p, x, PLAIN_ITERS)
        target = plan.residual(p, x)[0] * 1.01
        ones = torch.ones(g.volume_shape, device="cuda")
        n_uniform, _ = iters_from(plan, p, ones, target)
        x_saa, acc_saa, _, _ = ws.warm_start(plan, untrained, p)
        n_saa, _ = iters_from(plan, p, x_saa, target)
        x_net, acc_net, r_net, r_uni = ws.warm_start(plan, net, p)
        n_net, r_end = iters_from(plan, p, x_net, target)
        results.append((n_uniform, n_saa, n_net, acc_net))
        plan.close()
    print("iterations to the 15-iteration plain-MLEM residual (uniform / shift-and-add / trained U-Net):",
          results, "training loss", [round(h, 6) for h in hist])
    for n_uniform, n_saa, n_net, acc in results:
        assert acc
        assert n_net < n_uniform
    assert sum(r[2] for r in results) <= sum(r[1] for r in results)


def test_warm_start_elementwise_kernels_match_their_definitions():
    """The warm start's ray ratio, FP64 normalisation and blind-spot fill
    (kv_warm_ratio / kv_warm_normalize / kv_warm_fill) against the same
    formulas in PyTorch, bit for bit; the uniform start's residual against
    an FP64 norm."""
    build.build()
    ctx = engine.Context(0)
    g = geom()
    plan = engine.Plan(ctx, g, "exact")
    params = ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, 10, ph.seed_for(5, 1))
    truth = engine.phantom(ctx, g, params, device=True)
    p = ws.noisy_data(ctx, plan, truth, 5e4, 3)
    c = ws.prepare(plan)
    s, r_u = ws._saa_from_prepared(plan, c, p)
    a1, sens = c["a1"], c["sens"]
    r = torch.where(a1 > 0, p / torch.where(a1 > 0, a1, torch.ones_like(a1)), torch.zeros_like(p))
    b = plan.back(r.contiguous())
    want = torch.where(sens > 0, b.double() / torch.where(sens > 0, sens, torch.ones_like(sens)),
                       torch.zeros_like(sens)).float()
    assert torch.equal(s, want)
    pd = p.double()
    assert r_u == pytest.approx(float((a1.double() - pd).norm() / pd.norm()), rel=1e-12)
    net = engine.UNet(ctx, seed=0)
    x0, r_u2 = ws._start_estimate(plan, net, p)
    y = net.forward(s)
    want0 = torch.where(c["seen"], y, s).clamp(min=ws.EPS)
    assert torch.equal(x0, want0) and r_u2 == r_u
    net.close()
    plan.close()
