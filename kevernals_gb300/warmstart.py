"""Learned warm start for MLEM.

Input of the network: the volume-grid shift-and-add,
    s = A^T (p / A 1) / A^T 1,
the mean attenuation of the rays through each voxel averaged over the views --
exactly one SART step from zero (kv_sart, relax 1).  Target: the MLEM iterate
after `target_iters` iterations from the uniform start.  Training triples
(phantom, shift-and-add, MLEM target) are generated by the engine itself.

warm_start_mlem() keeps plain MLEM as the arbiter: the network's estimate is
used only if its data residual ||A x0 - p|| / ||p|| is no worse than the
uniform start's; otherwise MLEM starts from the uniform volume.

CLI (writes a checkpoint and a JSON report):
    python -m kevernals_gb300.warmstart train --out DIR [--triples N] ...
    python -m kevernals_gb300.warmstart evaluate --ckpt FILE [--cases N] ...
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import time

import numpy as np

from . import engine, phantom as ph
from .geometry import Geometry, config_chest, linear_sweep

EPS = 1e-4   # MLEM needs a strictly positive start


def crop_geometry(nx=256, ny=256, nz=64, n_views=60, half_angle=17.5) -> Geometry:
    """Training crop at the chest-DT voxel size (0.4 x 0.4 x 2.5 mm) and
    acquisition (60 views over +-17.5 deg); a 1024^2 detector at 0.2 mm covers
    the crop and its oblique shadows."""
    return linear_sweep(nx, ny, nz, 0.4, 0.4, 2.5, n_views, 1024, 1024, 0.2, 0.2, half_angle)


def column_geometry(centre_mm, nx=128, ny=256, full: Geometry = None) -> Geometry:
    """A full-thickness column of the chest-DT volume (nx x ny x 128 voxels,
    the chest's voxel grid, centred laterally at `centre_mm` in the chest
    frame, a multiple of the voxel pitch) seen by the chest's own sources and
    detector pixels: per view, the detector ROI is the pixel box covering the
    column's shadow (a common nu x nv for all views, per-view origins on the
    chest's pixel grid).  The column problem's rays are chest rays; its
    voxels are chest voxels."""
    g = config_chest() if full is None else full
    cx, cy = (round(float(c) / p) * p for c, p in zip(centre_mm, (g.dx, g.dy)))
    hx, hy, hz = 0.5 * nx * g.dx, 0.5 * ny * g.dy, 0.5 * g.nz * g.dz
    src = g.src.astype(np.float64)
    det = g.det_origin.astype(np.float64)
    zd = det[0, 2]
    boxes = []
    for p in range(g.n_views):
        s = src[p]
        pts = []
        for x in (cx - hx, cx + hx):
            for y in (cy - hy, cy + hy):
                for z in (-hz, hz):
                    a = (zd - s[2]) / (z - s[2])
                    pts.append((s[0] + a * (x - s[0]), s[1] + a * (y - s[1])))
        pts = np.asarray(pts)
        u0 = int(np.floor((pts[:, 0].min() - det[p, 0]) / g.du)) - 1
        u1 = int(np.ceil((pts[:, 0].max() - det[p, 0]) / g.du)) + 1
        v0 = int(np.floor((pts[:, 1].min() - det[p, 1]) / g.dv)) - 1
        v1 = int(np.ceil((pts[:, 1].max() - det[p, 1]) / g.dv)) + 1
        boxes.append((u0, u1, v0, v1))
    nu = max(b[1] - b[0] for b in boxes)
    nv = max(b[3] - b[2] for b in boxes)
    org = np.zeros((g.n_views, 3))
    for p, (u0, u1, v0, v1) in enumerate(boxes):
        ua = min(max(u0 - (nu - (u1 - u0)) // 2, 0), g.nu - nu)   # common size, inside the chest detector
        va = min(max(v0 - (nv - (v1 - v0)) // 2, 0), g.nv - nv)
        org[p] = (det[p, 0] + ua * g.du - cx, det[p, 1] + va * g.dv - cy, zd)
    src_c = src - np.array([cx, cy, 0.0])
    return Geometry(nx, ny, g.nz, g.dx, g.dy, g.dz, nu, nv, g.du, g.dv, src_c, org,
                    fulcrum_z=g.fulcrum_z), (cx, cy)


def chest_crops(s, x, nx, ny, n, seed):
    """n seeded full-thickness nx x ny crops (input, target) of a whole-volume
    triple; crop corners anywhere in the volume (edges included)."""
    rng = ph.SplitMix64(seed ^ 0x9E3779B97F4A7C15)
    D, H, W = s.shape
    out = []
    for _ in range(n):
        x0 = min(int(rng.uniform(0, W - nx + 1)), W - nx)
        y0 = min(int(rng.uniform(0, H - ny + 1)), H - ny)
        out.append((s[:, y0:y0 + ny, x0:x0 + nx].contiguous(), x[:, y0:y0 + ny, x0:x0 + nx].contiguous()))
    return out


def noisy_data(ctx, plan, truth, i0, seed):
    import torch
    line = plan.forward(truth)
    gen = torch.Generator(device=line.device).manual_seed(int(seed))
    counts = torch.poisson(i0 * torch.exp(-line.double()), generator=gen)
    return torch.log(i0 / counts.clamp_min(1.0)).clamp_min(0.0).float().contiguous()


def shift_and_add_volume(plan, p):
    """A^T(p / A1) / A^T1: one SART step (relax 1) from zero.  With the
    plan's prepare() quantities at hand it is one backprojection and two
    elementwise divisions; otherwise one kv_sart step (a forward projection
    of zeros, whose epilogue forms A1, and a backprojection)."""
    import torch
    c = getattr(plan, "_warm_cache", None)
    if c is not None:
        return _saa_from_prepared(plan, c, p)[0]
    x = torch.zeros(plan.geometry.volume_shape, dtype=torch.float32, device=p.device)
    plan.sart(p, x, 1, 1.0)
    return x


def _saa_from_prepared(plan, c, p):
    """A^T(p / A1) / A^T 1 from the prepared A1 and A^T 1 with the engine's
    kernels (ray ratio, backprojection, FP64 normalisation), and the uniform
    start's data residual ||A1 - p|| / ||p||, which the ratio pass computes
    on the way."""
    import torch
    from ._lib import lib
    ctx = plan.ctx
    p = p.contiguous()
    r = torch.empty_like(p)
    res = C.c_double()
    ctx.use_torch_stream()
    ctx.check(lib().kv_warm_ratio(ctx.handle, C.c_void_p(p.data_ptr()), C.c_void_p(c["a1"].data_ptr()),
                                  C.c_void_p(r.data_ptr()), p.numel(), C.byref(res)))
    b = plan.back(r)
    out = torch.empty_like(b)
    ctx.check(lib().kv_warm_normalize(ctx.handle, C.c_void_p(b.data_ptr()), C.c_void_p(c["sens"].data_ptr()),
                                      C.c_void_p(out.data_ptr()), b.numel()))
    return out, res.value


def window_params(seed, offset_mm, n_ellipsoids=400):
    """Ellipsoids of a seeded chest-DT phantom (1024 x 1024 x 128 at
    0.4 x 0.4 x 2.5 mm, `n_ellipsoids` plus the background) re-centred so
    that a crop volume centred at the origin shows the window of that
    phantom centred at `offset_mm` (chest frame): the training crops see
    structures of the sizes the chest-DT volumes hold."""
    params = ph.ellipsoid_params(1024, 1024, 128, 0.4, 0.4, 2.5, n_ellipsoids, seed).copy()
    params[:, 0:3] -= np.asarray(offset_mm, np.float32)
    return params


def column_centre(seed, nx=128, ny=256):
    """A seeded column centre (mm, chest frame) anywhere in the room the
    chest-DT volume leaves around an nx x ny column (so columns also cover
    the phantom's outer boundary and the empty corners)."""
    rng = ph.SplitMix64(seed ^ 0x2545F4914F6CDD1D)
    room = (0.5 * (1024 - nx) * 0.4, 0.5 * (1024 - ny) * 0.4)
    return [rng.uniform(-r, r) for r in room]


# Lateral margin (voxels) of a column whose MLEM target is not used for
# training: the column's side faces cut through tissue, and MLEM piles up
# values there that the full volume does not have.
COLUMN_MARGIN = 8


def mask_margin(x, margin=COLUMN_MARGIN):
    """The target with its lateral margin set to NaN (no target there)."""
    t = x.clone()
    t[:, :, :margin] = float("nan")
    t[:, :, -margin:] = float("nan")
    t[:, :margin, :] = float("nan")
    t[:, -margin:, :] = float("nan")
    return t


def window_offset(seed, crop: Geometry):
    """A seeded window centre inside 0.8 x the room the chest-DT volume
    leaves around the crop."""
    rng = ph.SplitMix64(seed ^ 0x5DEECE66D)
    room = [0.5 * (1024 * 0.4 - crop.nx * crop.dx), 0.5 * (1024 * 0.4 - crop.ny * crop.dy),
            0.5 * (128 * 2.5 - crop.nz * crop.dz)]
    return [rng.uniform(-0.8 * r, 0.8 * r) if r > 0 else 0.0 for r in room]


# A voxel is "seen" when its sensitivity (A^T 1) is at least this fraction of
# the median over voxels that some ray crosses.  At the chest-DT geometry the
# cone misses the lateral edges of the upper slices: MLEM never updates those
# voxels (they keep the start value), and voxels crossed by only a few views
# are barely constrained, so neither carries a usable training target.
SEEN_FRACTION = 0.1


def prepare(plan):
    """Per-geometry quantities of the warm start, computed once per plan
    (like the sensitivity image, which they include) and kept on it: the ray
    lengths A1 (a forward projection of ones), the FP64 sensitivity A^T 1 and
    the mask of seen voxels (sensitivity at least SEEN_FRACTION of the median
    over the voxels some ray crosses)."""
    import torch
    c = getattr(plan, "_warm_cache", None)
    if c is None:
        g = plan.geometry
        a1 = plan.forward(torch.ones(g.volume_shape, dtype=torch.float32, device="cuda"))
        sens = plan.sensitivity(device=True)
        pos = sens[sens > 0]
        seen = sens >= SEEN_FRACTION * float(pos.float().median()) if pos.numel() else sens > 0
        c = {"a1": a1, "sens": sens, "seen": seen, "seen_u8": seen.to(torch.uint8).contiguous()}
        plan._warm_cache = c
    return c


def seen_mask(plan):
    """Boolean volume: voxels whose sensitivity reaches SEEN_FRACTION of the
    median sensitivity of the voxels crossed by any ray."""
    return prepare(plan)["seen"]


def make_triple(ctx, g, seed, n_ellipsoids=40, i0=5e4, target_iters=100, params=None, mask_unseen=False):
    """(shift-and-add, MLEM target, data) for one seeded phantom, on the GPU;
    `params` (ellipsoid rows) overrides the phantom drawn for g.  With
    mask_unseen the target is NaN (no training target) outside seen_mask()."""
    import torch
    if params is None:
        params = ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, n_ellipsoids, seed)
    truth = engine.phantom(ctx, g, params, device=True)
    plan = engine.Plan(ctx, g, "exact")
    p = noisy_data(ctx, plan, truth, i0, seed)
    s = shift_and_add_volume(plan, p)
    x = torch.ones(g.volume_shape, dtype=torch.float32, device=p.device)
    plan.mlem(p, x, target_iters)
    if mask_unseen:
        x[~seen_mask(plan)] = float("nan")
    torch.cuda.synchronize()
    plan.close()
    return s, x, p


def train(net, triples, epochs, lr=1e-3, seed=0, log=None, on_epoch=None):
    rng = np.random.default_rng(seed)
    history = []
    for ep in range(epochs):
        order = rng.permutation(len(triples))
        losses = [net.train_step(triples[i][0], triples[i][1], lr) for i in order]
        history.append(float(np.mean(losses)))
        if log:
            log(f"epoch {ep + 1}/{epochs}: mean loss {history[-1]:.4e}")
        if on_epoch:
            on_epoch(ep, history)
    return history


def warm_start(plan, net, p):
    """Initial estimate: the network's, if its data residual is no worse than
    the uniform start's; returns (x0, accepted, residual_warm, residual_uniform)."""
    import torch
    s = shift_and_add_volume(plan, p)
    x0 = net.forward(s).clamp_(min=EPS)
    # voxels outside the network's training support (unseen or barely seen
    # by the rays) start from the shift-and-add value
    unseen = ~seen_mask(plan)
    x0[unseen] = s[unseen].clamp(min=EPS)
    ones = torch.ones_like(x0)
    r_w, _ = plan.residual(p, x0)
    r_u, _ = plan.residual(p, ones)
    if r_w <= r_u:
        return x0, True, r_w, r_u
    return ones, False, r_w, r_u


def iterations_to_residual(plan, p, x, target, max_iters, reject_above=None):
    """MLEM from x until ||Ax - p|| / ||p|| <= target; returns (iterations,
    residual).  With reject_above, also the start's own residual and whether
    it was rejected: a start whose residual exceeds reject_above is rejected
    before any update, (0, r0, r0, True)."""
    state = {"n": max_iters, "r": None, "r0": None, "rejected": False}

    def cb(it, res, ll):
        # res is the residual of the iterate entering iteration `it`, i.e.
        # after `it` updates; stopping here skips that update
        state["r"] = res
        state["n"] = it
        if it == 0:
            state["r0"] = res
        if it == 0 and reject_above is not None and res > reject_above:
            state["rejected"] = True
            return True
        return res <= target or it >= max_iters
    plan.mlem(p, x, max_iters + 1, callback=cb)
    if reject_above is not None:
        return state["n"], state["r"], state["r0"], state["rejected"]
    return state["n"], state["r"]


def _start_estimate(plan, net, p):
    """The network's start (blind spots filled from the shift-and-add volume)
    and the uniform start's residual from the prepared A1."""
    import torch
    from ._lib import lib
    c = prepare(plan)
    s, r_u = _saa_from_prepared(plan, c, p)
    y = net.forward(s)
    x0 = torch.empty_like(y)
    ctx = plan.ctx
    ctx.check(lib().kv_warm_fill(ctx.handle, C.c_void_p(y.data_ptr()), C.c_void_p(s.data_ptr()),
                                 C.c_void_p(c["seen_u8"].data_ptr()), float(EPS), C.c_void_p(x0.data_ptr()),
                                 x0.numel()))
    return x0, r_u


def warm_start_mlem(plan, net, p, target, max_iters):
    """The learned warm start followed by MLEM until the residual reaches
    `target`.  The network's estimate is kept only if its data residual is
    no worse than the uniform start's; that check reads the residual the
    first MLEM iteration computes anyway (the fused forward projection), and
    the uniform start's residual comes from the prepared ray lengths A1.  A
    rejected estimate falls back to MLEM from the uniform start.
    Returns (x, iterations, residual, accepted, start_residual, uniform_residual)."""
    import torch
    x0, r_u = _start_estimate(plan, net, p)
    n, r, r_start, rejected = iterations_to_residual(plan, p, x0, target, max_iters, reject_above=r_u)
    if rejected:
        x0 = torch.ones_like(x0)
        n, r = iterations_to_residual(plan, p, x0, target, max_iters)
    return x0, n, r, not rejected, r_start, r_u


def evaluate_case(ctx, net, g, seed, plain_iters=50, tol=0.01, i0=5e4, n_ellipsoids=400, params=None,
                  max_iters=None):
    """Plain MLEM (uniform start, plain_iters iterations) vs the warm start
    reaching the same data residual within `tol` (at most `max_iters`
    iterations, default plain_iters): iterations and wall time."""
    import torch
    if params is None:
        params = ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, n_ellipsoids, seed)
    truth = engine.phantom(ctx, g, params, device=True)
    plan = engine.Plan(ctx, g, "exact")
    p = noisy_data(ctx, plan, truth, i0, seed)
    # one-time set-up, outside both timings: per geometry A1, the sensitivity
    # image and the seen mask; per volume shape the network's workspace; per
    # process the first use of the elementwise tensor operations of the start
    # (a fresh process loads / compiles them on first use, which took ~3 s)
    prepare(plan)
    _start_estimate(plan, net, p)
    torch.cuda.synchronize()
    # plain MLEM
    x = torch.ones(g.volume_shape, dtype=torch.float32, device="cuda")
    t0 = time.perf_counter()
    plan.mlem(p, x, plain_iters)
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    r_plain, _ = plan.residual(p, x)
    target = r_plain * (1.0 + tol)
    # warm start
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    x0, n_w, r_end, accepted, r_w, r_u = warm_start_mlem(plan, net, p, target, max_iters or plain_iters)
    torch.cuda.synchronize()
    t_warm = time.perf_counter() - t0
    # the cost of the start itself (shift-and-add + network), timed separately
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    net.forward(shift_and_add_volume(plan, p))
    torch.cuda.synchronize()
    t_start = time.perf_counter() - t1
    reached = r_end is not None and r_end <= target
    out = {"seed": seed, "plain_iters": plain_iters, "plain_s": t_plain, "plain_residual": r_plain,
           "warm_accepted": accepted, "warm_start_residual": r_w, "uniform_start_residual": r_u,
           "warm_start_s": t_start, "warm_iters": n_w, "warm_s": t_warm, "warm_residual": r_end,
           "reached": reached,
           "speedup": t_plain / t_warm if reached else None}
    plan.close()
    return out


def _cli():
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["train", "evaluate"])
    ap.add_argument("--out", default="warmstart_out")
    ap.add_argument("--ckpt", default=None)
    ap.add_argument("--triples", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--target-iters", type=int, default=100)
    ap.add_argument("--lr", type=float, default=3e-4)
    ap.add_argument("--crop", default="128,256",
                    help="training volume nx,ny[,nz] (nz only for the centred crop geometries)")
    ap.add_argument("--cases", type=int, default=50)
    ap.add_argument("--case-size", default="1024,1024,128")
    ap.add_argument("--case-kind", choices=["volume", "column"], default="volume",
                    help="evaluation cases: whole volumes of --case-size, or held-out chest-DT columns "
                         "(--case-size gives nx,ny)")
    ap.add_argument("--max-iters", type=int, default=None,
                    help="most MLEM iterations the warm start may take (default: the plain count)")
    ap.add_argument("--seed", type=int, default=5000)
    ap.add_argument("--phantom", choices=["chest", "column", "window", "crop"], default="chest",
                    help="training cases: crops (--crop gives nx,ny; full thickness) of whole chest-DT "
                         "triples (--triples of them, --crops-per-volume crops each), full-thickness "
                         "columns of chest-DT phantoms seen by the chest geometry's own rays, windows of "
                         "chest-DT phantoms in the centred crop geometry, or phantoms drawn for the crop")
    ap.add_argument("--crops-per-volume", type=int, default=16)
    ap.add_argument("--init", default=None,
                    help="start training from this checkpoint (full state or weights only)")
    ap.add_argument("--first-case", type=int, default=0,
                    help="seed index of the first training phantom (continue with fresh phantoms)")
    args = ap.parse_args()
    import torch
    os.makedirs(args.out, exist_ok=True)
    ctx = engine.Context(0)
    ctx.use_torch_stream()
    net = engine.UNet(ctx, seed=args.seed)
    report = {}
    log = lambda s: print(s, flush=True)  # noqa: E731
    if args.cmd == "train":
        dims = [int(t) for t in args.crop.split(",")]
        nx, ny = dims[0], dims[1]
        nz = dims[2] if len(dims) > 2 else 128
        g = crop_geometry(nx, ny, nz)
        t0 = time.perf_counter()
        triples = []
        if args.init:
            net.load(args.init)
        for i in range(args.first_case, args.first_case + args.triples):
            seed = ph.seed_for(5, i)
            params = None
            if args.phantom == "chest":
                gc = config_chest()
                s, x, _ = make_triple(ctx, gc, seed, n_ellipsoids=400, target_iters=args.target_iters,
                                      mask_unseen=True)
                triples.extend(chest_crops(s, x, nx, ny, args.crops_per_volume, seed))
                del s, x
                if (i + 1 - args.first_case) % 4 == 0:
                    log(f"{i + 1 - args.first_case} chest triples, {time.perf_counter() - t0:.1f} s")
                continue
            if args.phantom == "column":
                g, centre = column_geometry(column_centre(seed, nx, ny), nx, ny)
                nz = g.nz
                params = window_params(seed, (centre[0], centre[1], 0.0))
            elif args.phantom == "window":
                params = window_params(seed, window_offset(seed, g))
            s, x, _ = make_triple(ctx, g, seed, target_iters=args.target_iters, params=params)
            triples.append((s, mask_margin(x) if args.phantom == "column" else x))
            if (i + 1) % 50 == 0:
                log(f"{i + 1} triples, {time.perf_counter() - t0:.1f} s")
        torch.cuda.synchronize()
        t_gen = time.perf_counter() - t0
        log(f"generated {len(triples)} triples in {t_gen:.1f} s")
        t0 = time.perf_counter()
        path = os.path.join(args.out, "unet.npz")
        n_val = max(1, len(triples) // 16)
        val, triples = triples[-n_val:], triples[:-n_val]

        def validate():
            def mse(a, b):
                d = (a - b) ** 2
                return float(d[~torch.isnan(d)].mean())
            mse_net = np.mean([mse(net.forward(a), b) for a, b in val])
            mse_id = np.mean([mse(a, b) for a, b in val])
            return float(mse_net), float(mse_id)

        val_hist = []

        def on_epoch(ep, h):
            net.save(path)
            val_hist.append(validate())
            log(f"  held-out MSE: network {val_hist[-1][0]:.4e}, shift-and-add itself {val_hist[-1][1]:.4e}")
        hist = train(net, triples, args.epochs, args.lr, log=log, on_epoch=on_epoch)
        t_train = time.perf_counter() - t0
        report = {"triples": len(triples), "crop": [nx, ny, nz], "target_iters": args.target_iters,
                  "phantom": args.phantom, "volumes": args.triples, "first_case": args.first_case,
                  "init": args.init,
                  "epochs": args.epochs, "lr": args.lr, "generate_s": t_gen, "train_s": t_train,
                  "loss_history": hist, "held_out_mse": val_hist, "checkpoint": path}
    else:
        net.load(args.ckpt)
        nx, ny, nz = (int(t) for t in args.case_size.split(","))
        cases = []
        for i in range(args.cases):
            seed = ph.seed_for(5, 100000 + i)
            if args.case_kind == "column":
                g, centre = column_geometry(column_centre(seed, nx, ny), nx, ny)
                params = window_params(seed, (centre[0], centre[1], 0.0))
                cases.append(evaluate_case(ctx, net, g, seed, params=params, max_iters=args.max_iters))
            else:
                g = config_chest() if (nx, ny, nz) == (1024, 1024, 128) else \
                    linear_sweep(nx, ny, nz, 0.4, 0.4, 2.5, 60, 2 * nx, 2 * ny, 0.2, 0.2, 17.5)
                cases.append(evaluate_case(ctx, net, g, seed, max_iters=args.max_iters))
            log(json.dumps(cases[-1]))
        sp = [c["speedup"] for c in cases if c["speedup"]]
        report = {"cases": cases, "case_size": [nx, ny, nz], "checkpoint": args.ckpt,
                  "reached": sum(c["reached"] for c in cases), "accepted": sum(c["warm_accepted"] for c in cases),
                  "median_speedup": float(np.median(sp)) if sp else None,
                  "min_speedup": float(np.min(sp)) if sp else None,
                  "max_speedup": float(np.max(sp)) if sp else None,
                  "at_least_3x": sum(1 for v in sp if v >= 3.0),
                  "median_warm_iters": float(np.median([c["warm_iters"] for c in cases]))}
    with open(os.path.join(args.out, f"{args.cmd}_report.json"), "w") as f:
        json.dump(report, f, indent=1)
    log(json.dumps({k: v for k, v in report.items() if k != "cases"}))


if __name__ == "__main__":
    _cli()
