#!/usr/bin/env python
"""Chest-DT MLEM benchmark of the kvtomo engine (one JSON line on stdout).

Workload (default): the chest-DT acquisition -- volume 1024x1024x128 at
0.4x0.4x2.5 mm, 60 views over +-17.5 deg, 2048^2 detector at 0.2 mm,
SID 1000 mm, SOD 850 mm -- with a seeded 400-ellipsoid phantom and Poisson
data at I0 = 5e4 (synthetic: no dataset is involved).  One step = one plain
MLEM iteration from the uniform start (forward projection with the fused
ratio, backprojection with the fused multiplicative update).

  value      projector rays/s = 2 * P * D rays (A and A^T) per iteration,
             inputs resident in HBM, CUDA events on the launching stream.
  e2e        the same metric through the C ABI with HOST buffers: every step
             copies the projections and the iterate in and the iterate out.
  roofline   the dominant kernel's algorithmic bytes per launch over its
             live average duration (per-launch CUDA events), against the
             measured HBM copy bandwidth.
  cpu_baseline  the reference's CPU MLEM iteration (as --impl reference) on
             a bounded sample of the same workload, all host cores.

--impl reference times the reference's own CPU path for the same metric:
its MLEM iteration (forward projection with the reference's selection sort,
11x11-window backprojection, the serial host ratio and update loops) on the
host cores -- the reference's Projector.cu kernels compiled for the host
where they were built (oracle/_ref), else their restatement in oracle/ --
whole iterations at the small workload, a bounded sample of rays and voxels
per step at chest-DT; rate = work done / measured step time.

Multi-GPU (torchrun): replicas only -- each rank solves its own seeded case;
value = all ranks' rays / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "chest-DT time-to-residual (learned vs plain GPU MLEM); projector rays/s, %HBM"
UNIT = "rays/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["kvtomo", "reference"], default="kvtomo")
    ap.add_argument("--family", choices=["exact", "rc"], default="exact")
    ap.add_argument("--storage", choices=["f32", "bf16", "f16"], default="f32")
    ap.add_argument("--workload", choices=["chest", "small"], default="chest")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-seconds", type=float, default=None,
                    help="reference arm: size each step's sample to about this many seconds "
                         "(default: whole iterations at the small workload, 5 s at chest-DT)")
    ap.add_argument("--no-ttr", action="store_true",
                    help="skip the learned-warm-start time-to-residual comparison")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the accuracy check and the SAA / SART / RC / storage runs")
    ap.add_argument("--no-ref-gpu", action="store_true",
                    help="skip timing the reference's own CUDA kernels on a sample")
    ap.add_argument("--views", type=int, default=0,
                    help="keep only the first N views (smaller case for profiling captures)")
    return ap.parse_args()


def geometry(workload):
    from kevernals_gb300.geometry import config_chest, config_small
    if workload == "chest":
        return config_chest(), 400, 5e4, 2, (
            "chest-DT: 1024x1024x128 @ 0.4x0.4x2.5 mm, 60 views +-17.5 deg, 2048^2 @ 0.2 mm, "
            "SID 1000 / SOD 850 mm")
    return config_small(), 40, 1e4, 1, (
        "small: 256x256x64 @ 0.5x0.5x1.0 mm, 15 views +-15 deg, 512^2 @ 0.4 mm")


# ----------------------------------------------------------------- helpers

class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.out = None

    def start(self):
        try:
            self.out = open(os.devnull if False else "/tmp/kv_clocks_%d.csv" % os.getpid(), "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)], stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.out.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.out.name):
            parts = [t.strip() for t in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.out.name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(path))["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic(kernel, workload):
    """DRAM traffic per launch from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        d = json.load(open(path))
        return d[workload][kernel]["bytes_per_launch"]
    except Exception:
        return None


def algorithmic_bytes(kernel, g, sv, sp):
    """Compulsory bytes of one launch (every input read once, every output
    written once) for the fused MLEM kernels."""
    V, PD = g.n_voxels, g.n_rays
    return {
        "exact_fwd": sv * V + 2 * sp * PD,            # read x, p; write ratio
        "exact_back": sp * PD + 2 * sv * V + 8 * V,   # read ratio; read+write x; read FP64 sens
        "rc_fwd": 4 * V + 8 * PD,
        "rc_back": 4 * PD + 8 * V,
    }.get(kernel)


# ---------------------------------------------------------------- the arms

def reference_cpu_steps(g, truth, steps, warmup, seconds=None, fraction=None, seed=1):
    """The reference's MLEM iteration (Reconstructors.h:182-242: forward
    projection, host ratio loop, backprojection, host update loop) on the
    host cores, each step on a bounded sample: a fraction f of the rays and
    the same fraction of the voxels.  The kernels are the reference's own
    Projector.cu compiled for the host (oracle/_ref, all cores) where the
    reference tree was present at build time, else their restatement in the
    oracle (the reference's selection sort and 11x11-window backprojector);
    the host loops are the reference's serial loops restated.  f = 1 runs
    whole iterations; otherwise f is sized so that a step takes about
    `seconds`.  Returns (step times, units of work per step, description,
    kind, cores, the iterate after the last step)."""
    from oracle import oracle as O
    use_ref = O.ref_lib() is not None
    rng = np.random.default_rng(seed)
    x = np.ones(g.volume_shape, np.float32)          # the uniform start
    p = np.zeros(g.proj_shape, np.float32)           # measurements at the sampled rays
    q = np.zeros(g.proj_shape, np.float32)           # forward projection, then ratio
    b = np.zeros(g.volume_shape, np.float32)         # backprojection
    relax = 1.0

    def forward(vol, rays, out):
        if use_ref:
            O.ref_forward_rays(g, vol, rays, out)
        else:
            out.reshape(-1)[rays] = O.rc_forward_rays_refcost(g, vol, rays)

    def back(proj, vox, out):
        if use_ref:
            O.ref_back_voxels(g, proj, vox, out)
        else:
            out.reshape(-1)[vox] = O.rc_back_voxels(g, proj, vox)

    def sample(f):
        if f >= 1.0:
            return np.arange(g.n_rays, dtype=np.int64), np.arange(g.n_voxels, dtype=np.int64)
        nr, nv = max(1, int(round(f * g.n_rays))), max(1, int(round(f * g.n_voxels)))
        return (np.unique(rng.integers(0, g.n_rays, nr)), np.unique(rng.integers(0, g.n_voxels, nv)))

    def step(rays, vox):
        t0 = time.perf_counter()
        forward(x, rays, q)
        O.rc_mlem_host_loops(p, q, rays, x, b, vox[:0], relax)       # ratio loop
        back(q, vox, b)
        O.rc_mlem_host_loops(p, q, rays[:0], x, b, vox, relax)       # update loop
        return time.perf_counter() - t0

    if fraction is None:
        fraction = 1.0
        if seconds is not None:
            f0 = min(1.0, 4096.0 / g.n_rays)
            rays, vox = sample(f0)
            forward(truth, rays, p)
            t = step(rays, vox)
            fraction = min(1.0, f0 * seconds / max(t, 1e-4))
    rays, vox = sample(fraction)
    forward(truth, rays, p)                          # the sampled rays' measurements
    for _ in range(warmup):
        step(rays, vox)
    gc.collect()
    gc.disable()                       # as in the GPU arm's timed loops
    times = [step(rays, vox) for _ in range(steps)]
    gc.enable()
    units = len(rays) + len(vox) * g.n_rays / g.n_voxels     # rays, and voxels in ray units
    what = ("the reference's Projector.cu kernels compiled for the host (OpenMP)" if use_ref
            else "the oracle's restatement of the reference kernels (selection sort, 11x11 window; OpenMP)")
    desc = (f"{'whole iterations' if fraction >= 1.0 else f'{len(rays)} random rays and {len(vox)} random voxels per step (fraction {fraction:.3g} of an iteration)'}"
            f" of the reference's MLEM: {what}, with its serial host ratio and update loops; "
            f"rate = (rays + voxels x P*D/V) per step / step time")
    return times, units, desc, ("reference" if use_ref else "port"), O.num_threads(), x


def reference_arm(args, g, desc):
    """The reference's MLEM iteration on the host cores (reference_cpu_steps)."""
    from kevernals_gb300 import phantom as ph
    from oracle import oracle as O
    _, n_ell, i0, cfg, _ = geometry(args.workload)
    params = ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, n_ell, ph.seed_for(cfg))
    truth = O.phantom(g, params)
    seconds = args.ref_seconds if args.ref_seconds is not None else (None if args.workload == "small" else 5.0)
    times, units, sample, kind, cores, _ = reference_cpu_steps(g, truth, args.steps, args.warmup, seconds=seconds)
    t = statistics.mean(times)
    value = units / t
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded ellipsoid phantom", "config": {"workload": desc, "family": "rc",
                                                                       "step": sample, "rays_per_step": units},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_baseline(g, truth_np, seconds):
    """The reference's CPU MLEM iteration on a bounded sample of the same
    workload (about `seconds` of host work), rays/s."""
    times, units, sample, kind, cores, _ = reference_cpu_steps(g, truth_np, 1, 0, seconds=seconds)
    return {"value": units / times[0], "unit": UNIT, "cores": cores, "kind": kind, "sample": sample}


def reference_gpu(g, truth):
    """The reference's own CUDA kernels (Projector.cu:227-785, compiled from
    source by oracle/build_ref.sh) timed on this GPU on a sample of the
    workload: the same volume and views 0, 1/3, 2/3 and last.  The forward
    kernel runs on a central 256 x 256 detector ROI (it has no defined
    result for rays that miss the volume, so the sample keeps every ray
    inside it) and is extrapolated by rays; the backprojector runs on the
    full detector and is extrapolated by views.  Kernel time only -- the
    reference's per-call allocations, copies and host ratio/update loops are
    not included."""
    import dataclasses

    import torch

    from oracle import ref_gpu
    if not ref_gpu.available("fma"):
        return {"unavailable": "reference kernels not compiled (oracle/build_ref.sh needs the reference sources)"}
    roi = 256
    views = sorted({0, g.n_views // 3, (2 * g.n_views) // 3, g.n_views - 1})
    det = g.det_origin.copy()
    det[:, 0] += 0.5 * (g.nu - roi) * g.du
    det[:, 1] += 0.5 * (g.nv - roi) * g.dv
    gs = dataclasses.replace(g, nu=roi, nv=roi, det_origin=det).subset_views(views)
    if not ref_gpu.all_rays_cross_volume(gs):
        return {"unavailable": "sample geometry has rays that miss the volume"}

    def timed(fn):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        out = fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), out

    gb = g.subset_views(views)
    ref_gpu.forward(gs, truth)                       # module load and warm-up
    f_ms, _ = timed(lambda: ref_gpu.forward(gs, truth))
    proj = torch.ones(gb.proj_shape, dtype=torch.float32, device=truth.device)
    b_ms, _ = timed(lambda: ref_gpu.back(gb, proj))
    fwd = f_ms * g.n_rays / gs.n_rays
    back = b_ms * g.n_views / gb.n_views
    return {"kind": "reference kernels compiled from source for sm_103a (nvcc defaults), run on this GPU",
            "sample": f"views {views}: forward on a central {roi}x{roi} detector ROI {f_ms:.1f} ms, "
                      f"backprojection (full detector) {b_ms:.1f} ms; extrapolated by rays / views",
            "forward_ms": fwd, "back_ms": back, "iteration_ms": fwd + back,
            "value": 2 * g.n_rays / ((fwd + back) * 1e-3), "unit": UNIT}


WEIGHTS = os.path.join(ROOT, "kevernals_gb300", "weights", "unet_chest_dt.npz")


def time_to_residual(ctx, g, cfg, rank, plain_iters=50):
    """The headline comparison on the bench's own case (same seeded phantom
    and Poisson data): plain GPU MLEM from the uniform start for
    `plain_iters` iterations, against the learned warm start (shift-and-add
    volume through the trained U-Net, kept only if its data residual is no
    worse than the uniform start's) followed by MLEM until the plain
    residual is reached within 1 %.  Wall time of each, sensitivity image
    precomputed for both."""
    from kevernals_gb300 import engine, phantom as ph, warmstart as ws
    if not os.path.exists(WEIGHTS):
        return {"unavailable": "no trained U-Net checkpoint in kevernals_gb300/weights/"}
    net = engine.UNet(ctx, seed=0)
    net.load(WEIGHTS)
    r = ws.evaluate_case(ctx, net, g, ph.seed_for(cfg, rank), plain_iters=plain_iters)
    net.close()
    return {"plain_iters": plain_iters, "plain_s": r["plain_s"], "plain_residual": r["plain_residual"],
            "warm_start_s": r["warm_start_s"], "warm_iters": r["warm_iters"], "warm_s": r["warm_s"],
            "warm_residual": r["warm_residual"], "accepted": r["warm_accepted"], "reached": r["reached"],
            "speedup": r["speedup"], "checkpoint": os.path.relpath(WEIGHTS, ROOT)}


def gather_rate(kernel, g, sv, sp, avg_ms):
    """The projector's gather work, beside the compulsory bytes: one element
    read per Siddon segment (a voxel for a forward walk, a ray value for the
    EXACT gather backprojector; the RC backprojector scans pixel windows
    instead and gets no figure); segments counted from the geometry on every
    8th detector row and column and scaled to all rays.  Mostly served by
    L1 / L2, so it is a rate of work, not of DRAM traffic."""
    try:
        if kernel not in ("exact_fwd", "exact_back", "rc_fwd"):
            return {}
        from kevernals_gb300.geometry import siddon_segments
        seg = siddon_segments(g, 8)
        elem = sv if kernel.endswith("fwd") else sp
        return {"segments_per_launch": seg, "gather_bytes": elem * seg,
                "gather_gbs": elem * seg / (avg_ms * 1e-3) / 1e9}
    except Exception as e:          # a missing figure must not cost the line
        return {"gather_unavailable": f"{type(e).__name__}: {e}"}


def cuda_ms(fn, reps=3, warmup=1):
    """Median wall time of fn() in ms, CUDA events on the current stream."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return sorted(ts)[len(ts) // 2]


def accuracy_vs_fp64(g, plan, truth, n_rays=4096, seed=7):
    """The stated error of the benchmarked EXACT pair against the FP64
    oracle on the bench's own phantom: the GPU forward projection on a
    seeded sample of rays against the oracle's FP64 Siddon line integrals,
    and the GPU backprojection of a projection stack that is zero except on
    those rays (seeded float32 values) against the oracle's FP64 transpose
    of the same rays, over the whole volume."""
    import torch
    from oracle import oracle as O
    rng = np.random.default_rng(seed)
    rays = np.unique(rng.integers(0, g.n_rays, n_rays))
    idx = torch.from_numpy(rays).to(truth.device)
    fwd = plan.forward(truth)
    got = fwd.reshape(-1)[idx].double().cpu().numpy()
    del fwd
    ref = O.exact_forward_rays(g, truth.double().cpu().numpy(), rays)
    vals = rng.random(len(rays)).astype(np.float32)
    y = torch.zeros(g.proj_shape, dtype=torch.float32, device=truth.device)
    y.view(-1)[idx] = torch.from_numpy(vals).to(truth.device)
    b = plan.back(y).double().cpu().numpy()
    del y
    ref_b = np.zeros(g.volume_shape, np.float64)
    O.exact_back_rays(g, vals.astype(np.float64), rays, ref_b)
    nz = ref_b != 0
    return {"forward": {"rays": int(len(rays)), "rel_l2": float(np.linalg.norm(got - ref) / np.linalg.norm(ref)),
                        "max_abs": float(np.abs(got - ref).max()),
                        "max_rel_to_max": float(np.abs(got - ref).max() / np.abs(ref).max())},
            "back": {"rays": int(len(rays)), "voxels_touched": int(nz.sum()),
                     "rel_l2": float(np.linalg.norm(b - ref_b) / np.linalg.norm(ref_b)),
                     "max_abs": float(np.abs(b - ref_b).max()),
                     "max_rel_to_max": float(np.abs(b - ref_b).max() / np.abs(ref_b).max())},
            "oracle": "FP64 Siddon (oracle/kvtomo_oracle.c), tolerance 2e-6 relative L2 (tests)"}


def config2_runs(ctx, g, plan, p, peak):
    """The rest of the chest-DT run set beside the MLEM step: shift-and-add,
    20 SART iterations at relaxation 0.5, the reference-compatible (RC)
    family's MLEM iteration (the reference's own operator, like-for-like
    with the reference arm), and BF16 / FP16 storage against FP32."""
    import torch
    from kevernals_gb300 import engine
    out = {}
    # shift-and-add (detector-sized slices, Reconstructors.h:263-379)
    saa = plan.shift_and_add(p)
    ms = cuda_ms(lambda: plan.shift_and_add(p, out=saa))
    byts = 4 * (g.n_rays + g.nu * g.nv * g.nz)
    out["shift_and_add"] = {"ms": ms, "algorithmic_bytes": byts, "GB/s": byts / (ms * 1e-3) / 1e9,
                            "frac_hbm": byts / (ms * 1e-3) / 1e9 / peak,
                            "parity": "shift rule equal to the reference's own code; zero padding and the 1/P "
                                      "weighted sum restated (VTK absent): parity unpinned at that boundary"}
    del saa
    # 20 SART iterations, relaxation 0.5, from zero (graph-captured loop)
    x = torch.zeros(g.volume_shape, dtype=torch.float32, device=p.device)
    plan.sart(p, x, 20, 0.5)                     # capture + sensitivity, untimed
    x.zero_()
    ms = cuda_ms(lambda: plan.sart(p, x.zero_(), 20, 0.5), reps=1, warmup=0)
    res, _ = plan.residual(p, x)
    out["sart_20"] = {"iterations": 20, "relax": 0.5, "ms": ms, "ms_per_iteration": ms / 20,
                      "rays_per_s": 2 * g.n_rays * 20 / (ms * 1e-3), "rel_residual": res}
    del x
    # RC family: the reference's operator on this GPU
    rc = engine.Plan(ctx, g, "rc")
    xr = torch.ones(g.volume_shape, dtype=torch.float32, device=p.device)
    ms = cuda_ms(lambda: rc.mlem(p, xr, 1), reps=2, warmup=1)
    out["rc_mlem_iteration"] = {"ms": ms, "rays_per_s": 2 * g.n_rays / (ms * 1e-3), "family": "rc",
                                "note": "reference-compatible operator (bit-identical to the reference's kernels)"}
    rc.close()
    del xr
    # storage precision: iteration time against FP32 (5 iterations per call)
    times = {}
    for storage in ("f32", "bf16", "f16"):
        ps = engine.Plan(ctx, g, "exact", storage)
        xs = torch.ones(g.volume_shape, dtype=torch.float32, device=p.device)
        ms = cuda_ms(lambda: ps.mlem(p, xs, 5), reps=2, warmup=1)
        times[storage] = ms / 5
        ps.close()
        del xs
    out["storage_mlem_ms_per_iteration"] = times
    out["storage_speedup_vs_f32"] = {k: times["f32"] / v for k, v in times.items() if k != "f32"}
    return out


def max_over_ranks(ms, world, device):
    """The slowest rank's time: replicas finish when the last one does.  One
    all-reduce (MAX) over the process group; the identity on one rank."""
    if world == 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gpu_arm(args, g, n_ell, i0, cfg, desc, rank, world):
    import torch

    from kevernals_gb300 import engine, phantom as ph
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    ctx = engine.Context(dev)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)

    # data: seeded phantom, EXACT line integrals, Poisson counts
    params = ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, n_ell, ph.seed_for(cfg, rank))
    truth = engine.phantom(ctx, g, params, device=True)
    gen_plan = engine.Plan(ctx, g, "exact")
    line = gen_plan.forward(truth)
    gen = torch.Generator(device=f"cuda:{dev}").manual_seed(ph.seed_for(cfg, rank))
    counts = torch.poisson(i0 * torch.exp(-line.double()), generator=gen)
    p = torch.log(i0 / counts.clamp_min(1.0)).clamp_min(0.0).float().contiguous()
    del counts, line
    gen_plan.close()

    plan = engine.Plan(ctx, g, args.family, args.storage)
    x = plan.uniform_volume(device=True)
    for _ in range(args.warmup):
        plan.mlem(p, x, 1)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # ---- timed region: device-resident inputs (both larger than L2).  As in
    # timeit, Python's garbage collector is run before and held off during
    # the timed loops: its pauses between two calls of the C ABI would idle
    # the GPU (measured: periodic 5-15 ms stalls of the host-buffer loop).
    sampler = ClockSampler(dev)
    sampler.start()
    ctx.set_timing(True)
    barrier()
    torch.cuda.synchronize()
    gc.collect()
    gc.disable()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        plan.mlem(p, x, 1)
    e1.record(stream)
    torch.cuda.synchronize()
    gc.enable()
    barrier()
    ms = e0.elapsed_time(e1)
    kernels = ctx.read_timing()
    ctx.set_timing(False)
    clocks = sampler.stop()
    ms = max_over_ranks(ms, world, f"cuda:{dev}")
    rays_per_step = 2 * g.n_rays
    value = world * rays_per_step * args.steps / (ms * 1e-3)
    gpu_launches = sum(n for n, _ in kernels.values())

    # ---- roofline of the dominant kernel
    sv = sp = 2 if args.storage != "f32" else 4
    dom = max(kernels.items(), key=lambda kv: kv[1][1])[0] if kernels else None
    roof = None
    if dom is not None:
        n, tot = kernels[dom]
        byt = algorithmic_bytes(dom, g, sv, sp)
        peak, src = measured_hbm()
        if byt is not None:
            ach = byt / (tot / n * 1e-3) / 1e9
            roof = {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": peak, "unit": "GB/s",
                    "frac": ach / peak, "peak_source": src, "algorithmic_bytes": byt,
                    "traffic": committed_traffic(dom, args.workload), "avg_ms": tot / n}
            roof.update(gather_rate(dom, g, sv, sp, tot / n))

    # ---- end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        ph_p = torch.empty(g.proj_shape, dtype=torch.float32).pin_memory()
        ph_x = torch.empty(g.volume_shape, dtype=torch.float32).pin_memory()
        ph_p.copy_(p.cpu())
        hp, hx = ph_p.numpy(), ph_x.numpy()
        hx[...] = 1.0
        plan.mlem(hp, hx, 1)          # warm the staging buffers
        barrier()
        torch.cuda.synchronize()
        gc.collect()
        gc.disable()
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        for _ in range(args.steps):
            plan.mlem(hp, hx, 1)
        a1.record(stream)
        torch.cuda.synchronize()
        gc.enable()
        barrier()
        ems = max_over_ranks(a0.elapsed_time(a1), world, f"cuda:{dev}")
        e2e = {"value": world * rays_per_step * args.steps / (ems * 1e-3), "unit": UNIT,
               "h2d_bytes_per_step": 4 * (g.n_rays + g.n_voxels), "d2h_bytes_per_step": 4 * g.n_voxels,
               "ms_per_step": ems / args.steps}

    acc = extra = None
    if not args.no_extras and args.family == "exact" and args.storage == "f32":
        acc = accuracy_vs_fp64(g, plan, truth)
        extra = config2_runs(ctx, g, plan, p, measured_hbm()[0])

    # the learned-warm-start comparison runs before the CPU and reference
    # legs, on a GPU and host that nothing else is using
    ttr = None
    if (not args.no_ttr and args.workload == "chest" and args.family == "exact"
            and args.storage == "f32" and args.views == 0):
        del x
        plan.close()
        ttr = time_to_residual(ctx, g, cfg, rank)
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(g, truth.cpu().numpy(), args.cpu_seconds)
    ref_gpu_line = reference_gpu(g, truth) if rank == 0 and not args.no_ref_gpu else None

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.storage == "f32" else args.storage,
            "data": f"synthetic: seeded {n_ell}-ellipsoid phantom, EXACT line integrals, Poisson I0={i0:g}",
            "config": {"workload": desc, "family": args.family, "storage": args.storage,
                       "step": "one MLEM iteration (forward+ratio, backprojection+update)",
                       "rays_per_step": rays_per_step, "l2": "inputs larger than L2 (no flush)",
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
            "clocks": clocks, "e2e": e2e, "gpu_launches": gpu_launches, "roofline": roof,
            "cpu_baseline": cpu, "reference_gpu": ref_gpu_line, "time_to_residual": ttr,
            "accuracy_vs_fp64": acc, "chest_runs": extra,
            "kernels": {k: {"launches": n, "avg_ms": t / n} for k, (n, t) in kernels.items()},
        }
        print(json.dumps(out), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    g, n_ell, i0, cfg, desc = geometry(args.workload)
    if args.views > 0:
        g = g.subset_views(np.arange(min(args.views, g.n_views)))
        desc += f" (first {g.n_views} views only)"
    if args.impl == "reference":
        if rank == 0:
            reference_arm(args, g, desc)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    try:
        gpu_arm(args, g, n_ell, i0, cfg, desc, rank, world)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
