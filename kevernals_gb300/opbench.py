"""Per-operator timings of the engine (one JSON line per operator).

    python -m kevernals_gb300.opbench [--ops a,b,...] [--workload W] [--reps N] [--warmup N]

Operators: exact_fwd, exact_back, mlem_iter, sart_iter, rc_fwd,
rc_back, saa, phantom, unet_fwd, unet_train.  Workloads: chest (1024x1024x128,
60 views of 2048^2), chest4 (the same, first 4 views), small (256x256x64,
15 views of 512^2), column (a 128x256x128 full-thickness chest-DT column).
Inputs are device-resident; each line gives the median time of `reps` calls
(CUDA events around each call), the algorithmic bytes of one call (every
input read once, every output written once) and the rate they imply.  Also
the program run under ncu for the per-kernel captures (run it with --reps 1 --warmup 0
under ncu's kernel filter).
"""
from __future__ import annotations

import argparse
import json

# U-Net FLOP per input voxel of one forward: 2 * 27 * Cin * Cout / 8^level
# summed over the thirteen 3x3x3 convolutions (levels 0-3, channels
# 16/32/64/128, concatenated skips), plus the 1->16 input and 16->1 output
# layers.  A training step adds the backward-data and backward-weight
# convolutions: ~3x.
UNET_FLOP_PER_VOXEL = (sum(2 * 27 * cin * cout / 8 ** lvl for cin, cout, lvl in (
    (16, 16, 0), (16, 32, 1), (32, 32, 1), (32, 64, 2), (64, 64, 2), (64, 128, 3), (128, 128, 3),
    (192, 64, 2), (64, 64, 2), (96, 32, 1), (32, 32, 1), (48, 16, 0), (16, 16, 0))) + 2 * 27 * 16 + 2 * 16)

OPS = ["exact_fwd", "exact_back", "mlem_iter", "sart_iter", "rc_fwd", "rc_back", "saa",
       "phantom", "unet_fwd", "unet_train", "batch_small"]


def _geometry(name):
    from .geometry import config_chest, config_small
    from .warmstart import column_geometry
    if name == "chest":
        return config_chest(), 400, 2
    if name == "chest4":
        import numpy as np
        return config_chest().subset_views(np.arange(4)), 400, 2
    if name == "small":
        return config_small(), 40, 1
    if name == "column":
        g, _ = column_geometry((0.0, 0.0))
        return g, 400, 2
    raise ValueError(name)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--ops", default=",".join(OPS))
    ap.add_argument("--workload", default="chest4", choices=["chest", "chest4", "small", "column"])
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--back-shape", default="",
                    help="gather backprojector: rows,slices per thread (rows 0: one voxel per thread)")
    ap.add_argument("--back-staging", default="",
                    help="TMA-staged backprojector: rows,stages (rows 0: off)")
    ap.add_argument("--slab", default="",
                    help="forward projector shape: 'off' (one thread per ray) or R,S,stages,group")
    args = ap.parse_args(argv)
    import torch

    from . import engine, phantom as ph
    ctx = engine.Context(0)
    ctx.use_torch_stream()
    g, n_ell, cfg = _geometry(args.workload)
    params = ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, n_ell, ph.seed_for(cfg, 0))
    V, R = g.n_voxels, g.n_rays

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        ts = []
        for _ in range(args.reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return sorted(ts)[len(ts) // 2]

    def report(op, ms, byts, units, unit_name):
        print(json.dumps({"op": op, "workload": args.workload, "ms": ms, "algorithmic_bytes": byts,
                          "GB/s": byts / (ms * 1e-3) / 1e9 if byts else None,
                          unit_name: units / (ms * 1e-3)}), flush=True)

    truth = engine.phantom(ctx, g, params, device=True)
    plans = {}

    def plan(family):
        if family not in plans:
            plans[family] = engine.Plan(ctx, g, family)
            if family == "exact" and args.slab:
                shape = [0] if args.slab == "off" else [int(v) for v in args.slab.split(",")]
                plans[family].set_slab(*shape)
            if family == "exact" and args.back_shape:
                plans[family].set_back_shape(*[int(v) for v in args.back_shape.split(",")])
            if family == "exact" and args.back_staging:
                plans[family].set_back_staging(*[int(v) for v in args.back_staging.split(",")])
        return plans[family]

    p = plan("exact").forward(truth)
    ops = [o for o in args.ops.split(",") if o]
    for op in ops:
        if op == "exact_fwd":
            out = torch.empty_like(p)
            report(op, timed(lambda: plan("exact").forward(truth, out=out)), 4 * (V + R), R, "rays/s")
        elif op == "exact_back":
            out = torch.empty_like(truth)
            report(op, timed(lambda: plan("exact").back(p, out=out)), 4 * (V + R), V * g.n_views,
                   "voxel-views/s")
        elif op == "mlem_iter":
            x = torch.ones_like(truth)
            plan("exact").sensitivity(device=True)
            report(op, timed(lambda: plan("exact").mlem(p, x, 1)), 4 * (3 * V + 3 * R) + 8 * V, 2 * R,
                   "rays/s")
        elif op == "sart_iter":
            x = torch.ones_like(truth)
            plan("exact").sensitivity(device=True)
            report(op, timed(lambda: plan("exact").sart(p, x, 1, 0.5)), 4 * (3 * V + 4 * R) + 8 * V, 2 * R,
                   "rays/s")
        elif op == "rc_fwd":
            out = torch.empty_like(p)
            report(op, timed(lambda: plan("rc").forward(truth, out=out)), 4 * (V + R), R, "rays/s")
        elif op == "rc_back":
            out = torch.empty_like(truth)
            report(op, timed(lambda: plan("rc").back(p, out=out)), 4 * (V + R), V * g.n_views,
                   "voxel-views/s")
        elif op == "saa":
            out = plan("exact").shift_and_add(p)
            report(op, timed(lambda: plan("exact").shift_and_add(p, out=out)), 4 * (R + g.nu * g.nv * g.nz),
                   g.nu * g.nv * g.nz, "pixels-slices/s")
        elif op == "phantom":
            report(op, timed(lambda: engine.phantom(ctx, g, params, device=True)), 4 * V,
                   V * len(params), "voxel-ellipsoids/s")
        elif op in ("unet_fwd", "unet_train"):
            if g.nx % 128 or g.ny % 8 or g.nz % 8:
                print(json.dumps({"op": op, "workload": args.workload, "skipped": "volume not a multiple of "
                                  "128 (x) / 8 (y, z)"}), flush=True)
                continue
            net = engine.UNet(ctx, seed=1)
            y = torch.empty_like(truth)
            flop_fwd = UNET_FLOP_PER_VOXEL * V
            if op == "unet_fwd":
                ms = timed(lambda: net.forward(truth, out=y))
                print(json.dumps({"op": op, "workload": args.workload, "ms": ms,
                                  "TFLOP/s": flop_fwd / (ms * 1e-3) / 1e12}), flush=True)
            else:
                ms = timed(lambda: net.train_step(truth, truth, 1e-4))
                print(json.dumps({"op": op, "workload": args.workload, "ms": ms,
                                  "TFLOP/s": 3 * flop_fwd / (ms * 1e-3) / 1e12}), flush=True)
            net.close()
        elif op == "batch_small":
            # many small problems: 256 seeded uneven cases at a quarter of the
            # batched workload's sizes, 30 MLEM iterations, one persistent
            # launch per phase (kv_batch_mlem) against solving one by one
            from .geometry import uneven_cases
            cases = uneven_cases(256, 20261203 + 3000, scale=4)
            bplans, data = [], []
            for ci, gc in enumerate(cases):
                pc = engine.Plan(ctx, gc, "exact")
                tc = engine.phantom(ctx, gc, ph.ellipsoid_params(gc.nx, gc.ny, gc.nz, gc.dx, gc.dy, gc.dz, 20,
                                                                   3000 + ci), device=True)
                data.append(pc.forward(tc))
                pc.sensitivity(device=True)
                bplans.append(pc)
            xs = [torch.ones(gc.volume_shape, device="cuda") for gc in cases]
            t_batch = timed(lambda: [x.fill_(1.0) for x in xs] and engine.batch_mlem(ctx, bplans, data, xs, 30))
            t_seq = timed(lambda: [pc.mlem(d, x.fill_(1.0), 30) for pc, d, x in zip(bplans, data, xs)])
            rays = sum(2 * gc.n_rays for gc in cases) * 30
            print(json.dumps({"op": op, "cases": len(cases), "iterations": 30, "batched_ms": t_batch,
                              "one_by_one_ms": t_seq, "speedup": t_seq / t_batch,
                              "batched_rays_per_s": rays / (t_batch * 1e-3)}), flush=True)
            for pc in bplans:
                pc.close()
        else:
            raise SystemExit(f"unknown op {op}")
    for pl in plans.values():
        pl.close()


if __name__ == "__main__":
    main()
