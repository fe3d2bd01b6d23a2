#!/usr/bin/env python
"""Benchmark of the GB300 pressure projection.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gbp|reference]
                    [--workload liquid3_128|smoke3_256|liquid2_128]
                    [--solver cg|mgpcg] [--precision fp64|mixed]

A step is one projection (face fractions, labelling, operator and
right-hand side assembly, the solve to a relative residual of 1e-6, the
pressure-gradient velocity update) of one synthetic scene. The default
workload is the 3D smoke scene at 256^3 (every cell fluid, Neumann box walls,
a solid cylinder of radius 0.1 along z, face velocities N(0, 1)), the
configuration the mixed-vs-FP64 metric is quoted on. Inputs are seeded
synthetic data with the shapes and value distributions of that workload.

The headline path is multigrid-preconditioned CG with an FP32 inner solve
inside FP64 iterative refinement (--solver mgpcg --precision mixed); the FP64
MGPCG path and the reference's own algorithm (plain FP64 CG) are measured on
the same scene and reported under `compare`, with the mixed/FP64 ratio.
`accuracy` gives each path's result against the oracle's FP64 solve of the
same scene (the C restatement of the reference, one full projection: max-norm
pressure difference, with the mean over the unknowns removed on an
all-Neumann scene, and velocity difference) and the divergence left after
projection. `batched` and `served` hold the batched workload (64 scenes,
one launch per kernel for all) and the served stream (continuous batching),
each mixed and FP64.

Prints one JSON line. `value` is solves/s over all ranks with inputs resident
in HBM (the velocity is reset from a device copy before each step, inside
the timed region); `e2e` is the same through the host-array C ABI call
(gbp_project: host->device copies of the inputs and device->host copies of
the projected velocity and pressure inside the timing). `roofline` times the
dominant kernel alone with CUDA events. `cpu_baseline` is the oracle's CPU
projection of the same scene on this host.

--impl reference times the reference's CPU implementation of the path on
the host cores instead: the reference built from its sources
(oracle/_ref) where it is present, else the oracle's C restatement.
Multi-GPU (torchrun): independent replicas, one per rank, no collective on
the data path ("replicas only").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "liquid3_128": dict(kind="liquid3", n=128, desc="3D liquid 128^3, solid sphere r=0.12, pool y<0.35 + drop r=0.18"),
    "smoke3_256": dict(kind="smoke3", n=256, desc="3D smoke 256^3, all fluid, solid cylinder r=0.1 along z"),
    "liquid2_128": dict(kind="liquid2", n=128, desc="2D liquid 128^2, pool y<0.3 + circle r=0.15"),
    "served": dict(kind="served", n=0, desc="served stream: Poisson arrivals (seed 5, 8 requests/s), 70% liquid / 30% "
                   "smoke, edge in {32,64,96,128,192,256}, 50 steps each, warm start, 150 GB HBM budget; "
                   "--steps = number of requests"),
    "batch64_liquid3": dict(kind="batch", n=64, desc="64 independent 3D liquid scenes, edge log-uniform in "
                            "[32, 160], fluid fraction U[0.1, 0.6], one batched solve per step"),
    "advect_smoke3_256": dict(kind="advect", n=256, desc="MAC advection of the 3D smoke scene 256^3 (macsmoke3's "
                              "step: density U[0,1) by the velocity, then the velocity by itself; MacCormack, "
                              "bilinear, TrimNarrowBand 1); --steps = chained advection steps"),
}
ADVECT_METRIC = "3D MAC advection steps/s (MacCormack, density + velocity)"
METRIC = "3D pressure solves/s at 1e-6 resid"
L2_BYTES = 129 * 2 ** 20
REFERENCE_BUDGET_S = 150.0


def make_scene(name):
    from shiokaze_gb300 import scenes
    w = WORKLOADS[name]
    if w["kind"] == "liquid3":
        return scenes.liquid3(w["n"], seed=2)
    if w["kind"] == "smoke3":
        return scenes.smoke3(w["n"], seed=3)
    return scenes.liquid2(w["n"], seed=1)


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Ranks:
    """The ranks of one bench run, one process per GPU (torchrun env).

    Each rank projects its own replica of the workload: the projection has
    no exchange step between GPUs, so no collective touches the data path.
    The timed region is bracketed by barriers on every rank, the job's time
    is the slowest rank's (all_reduce MAX) and the job's rate is the units
    all ranks processed over that time. backend "nccl" runs on the GPUs;
    "gloo" runs the same logic on CPU processes."""

    def __init__(self, backend="nccl", device=None):
        self.rank, self.world, self.local = dist_info()
        self.backend = backend
        self.device = device
        if self.world > 1:
            import torch.distributed as dist
            if backend == "nccl":
                dist.init_process_group("nccl", device_id=device)
            else:
                dist.init_process_group(backend)

    def barrier(self):
        if self.world > 1:
            import torch.distributed as dist
            dist.barrier()

    def max_ms(self, ms):
        """The slowest rank's time; every rank must call it."""
        if self.world <= 1:
            return float(ms)
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(ms)], dtype=torch.float64,
                         device=self.device if self.backend == "nccl" else "cpu")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def rate(self, units_per_rank, ms):
        """Whole-job units/s: all ranks' units over the slowest rank's time."""
        return self.world * units_per_rank / (self.max_ms(ms) / 1000.0)

    def close(self):
        if self.world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[2:6]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_gbs():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def committed_traffic(workload, kernel):
    """DRAM bytes per launch of `kernel` on `workload` from the committed ncu
    summary (profiles/traffic.json), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            t = json.load(f)
        return t.get(workload, {}).get(kernel)
    except (OSError, ValueError):
        return None


def oracle_solve(scene):
    """One full projection of the scene by the oracle (the C restatement of
    the reference) on this host, timed: the CPU baseline, and the FP64
    solution the GPU results are measured against. The oracle's CG runs its
    matrix-vector products, vector updates and maximum norms on all host
    cores and its dot products serially in the reference's order, so its
    result is bit-identical to the single-threaded restatement."""
    import oracle
    threads = oracle.set_threads(None)
    t0 = time.perf_counter()
    r = oracle.project_scene(scene, "port", residual=1e-6)
    dt = time.perf_counter() - t0
    base = {"value": round(1.0 / dt, 5), "unit": "solves/s", "cores": threads, "kind": "port",
            "sample": f"one full projection of the same scene by the oracle's C restatement of the reference "
                      f"(plain FP64 CG to 1e-6, {r.iterations} iterations; element-wise loops on {threads} "
                      f"threads, dot products serial in the reference's order), {dt:.1f} s",
            "seconds_per_solve": round(dt, 3), "iterations": r.iterations}
    return r, base


def accuracy(scene, ref, outputs):
    """Each GPU path's result against the oracle's FP64 solve `ref`:
    max-norm pressure difference over the unknowns relative to |p_ref|_inf
    (on an all-Neumann scene, whose pressure is defined up to a constant,
    with each side's mean over the unknowns removed), max-norm velocity
    difference relative to |u_ref|_inf, and the divergence left after the
    projection relative to the divergence before it (max over the unknowns
    of |sum sgn area u / dx|, the oracle's face fractions)."""
    import oracle
    pj = oracle.PortProjector(scene.dim, scene.nx, scene.ny, scene.nz, scene.dx, residual=1e-6)
    area, _ = pj.face_fractions(scene.solid, scene.fluid)
    pj.close()
    unk = ref.unknown
    vel_in = tuple(a for a in (scene.u, scene.v, scene.w) if a is not None)
    div_in = oracle.divergence(area, vel_in, scene.dx, unk)
    neumann = bool((scene.fluid < 0).all())  # no air cell: no Dirichlet condition anywhere
    pr = ref.pressure[unk].astype(np.float64)
    if neumann:
        pr = pr - pr.mean()
    pr_inf = max(float(np.max(np.abs(pr))), 1e-300)
    vel_ref = tuple(a for a in (ref.u, ref.v, ref.w) if a is not None)
    u_inf = max(float(max(np.max(np.abs(a)) for a in vel_ref)), 1e-300)
    out = {"oracle": {"iterations": ref.iterations, "reresid": ref.reresid,
                      "divergence_rel": oracle.divergence(area, vel_ref, scene.dx, unk) / div_in},
           "divergence_before": div_in, "pressure_mean_removed": neumann}
    for name, (p, vel) in outputs.items():
        pg = p[unk].astype(np.float64)
        if neumann:
            pg = pg - pg.mean()
        out[name] = {
            "pressure_rel_inf": float(np.max(np.abs(pg - pr))) / pr_inf,
            "velocity_rel_inf": max(float(np.max(np.abs(g.astype(np.float64) - r.astype(np.float64))))
                                    for g, r in zip(vel, vel_ref)) / u_inf,
            "divergence_rel": oracle.divergence(area, vel, scene.dx, unk) / div_in,
            "zero_off_unknowns": not bool((p[~unk] != 0).any()),
        }
    return out


def _measure(gb, torch, pj, ctx, scene, dev_arrays, stream, steps, warmup, ranks, sampler=None):
    """Times `steps` projections (after `warmup`) with CUDA events on the
    projection's stream; the velocity is reset from a device copy first."""
    solid, fluid, comps, comps0, p = dev_arrays
    sh = stream.cuda_stream

    def step():
        for c, c0 in zip(comps, comps0):
            c.copy_(c0)
        rc = pj.project(scene.dt, tuple(comps), solid, fluid, pressure_out=p, stream=sh)
        if rc != gb.GBP_OK:
            raise RuntimeError(f"projection returned {rc}: {gb.load_library().gbp_strerror(rc).decode()}")

    with torch.cuda.stream(stream):
        for _ in range(warmup):
            step()
    torch.cuda.synchronize()
    ranks.barrier()
    if sampler:
        sampler.start()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    l0 = ctx.launches()
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        ev[0].record(stream)
        for k in range(steps):
            step()
            ev[k + 1].record(stream)
    torch.cuda.synchronize()
    ranks.barrier()
    clocks = sampler.stop() if sampler else None
    per_step = [ev[k].elapsed_time(ev[k + 1]) for k in range(steps)]
    # the last step's results, for the accuracy report (after the timing)
    out = (p.cpu().numpy(), tuple(c.cpu().numpy() for c in comps))
    return {"total_ms": ev[0].elapsed_time(ev[-1]), "per_step": per_step, "launches": ctx.launches() - l0,
            "stats": pj.stats.as_dict(), "clocks": clocks, "out": out}


def run_gbp(args):
    import torch
    import shiokaze_gb300 as gb

    rank, world, local = dist_info()
    ranks = Ranks("nccl", torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    scene = make_scene(args.workload)
    ctx = gb.Context(local)
    stream = torch.cuda.Stream(device=dev)
    sh = stream.cuda_stream

    def dev_t(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    solid, fluid = dev_t(scene.solid), dev_t(scene.fluid)
    comps0 = [dev_t(a) for a in (scene.u, scene.v, scene.w) if a is not None]
    comps = [c.clone() for c in comps0]
    p = torch.zeros(scene.fluid.shape, dtype=torch.float32, device=dev)
    arrays = (solid, fluid, comps, comps0, p)
    torch.cuda.synchronize()

    cfg = dict(Residual=1e-6, Solver=args.solver, Precision=args.precision)
    pj = gb.projector_for(scene, ctx, **cfg)
    main = _measure(gb, torch, pj, ctx, scene, arrays, stream, args.steps, args.warmup, ranks, ClockSampler(local))
    stats = main["stats"]
    total_ms = ranks.max_ms(main["total_ms"])
    value = ranks.rate(args.steps, total_ms)

    # the other GPU paths on the same scene, for comparison (fewer steps)
    compare = {}
    outputs = {f"{args.solver}_{args.precision}": main["out"]}
    if not args.no_compare:
        for solver, precision in (("mgpcg", "mixed"), ("mgpcg", "fp64"), ("cg", "fp64")):
            if (solver, precision) == (args.solver, args.precision):
                continue
            other = gb.projector_for(scene, ctx, Residual=1e-6, Solver=solver, Precision=precision)
            nsteps = 3 if solver == "cg" else max(3, args.steps // 2)
            m = _measure(gb, torch, other, ctx, scene, arrays, stream, nsteps, 3, ranks)
            ms = m["total_ms"] / nsteps
            compare[f"{solver}_{precision}"] = {
                "solves_per_s": round(1000.0 / ms, 3), "ms_per_step": round(ms, 4),
                "iterations": m["stats"]["iterations"], "outer_iterations": m["stats"]["outer_iterations"],
                "true_resid_inf": m["stats"]["true_resid_inf"], "steps": nsteps}
            outputs[f"{solver}_{precision}"] = m["out"]
            other.close()
        if args.solver == "mgpcg" and args.precision == "mixed" and "mgpcg_fp64" in compare:
            # the headline comparison: mixed precision over plain FP64, same
            # solver, same scene, same relative residual
            compare["mixed_over_fp64"] = round(value / compare["mgpcg_fp64"]["solves_per_s"], 4)

    # end to end through the host-array call, with plain (pageable) numpy
    # arrays as a caller such as the plugin module passes them (its dense
    # copies are std::vectors); the host->device copies of the inputs and
    # the device->host copies of the velocity and pressure are inside the
    # timing
    h_solid, h_fluid = np.ascontiguousarray(scene.solid), np.ascontiguousarray(scene.fluid)
    h0 = [a for a in (scene.u, scene.v, scene.w) if a is not None]
    hc = [np.empty_like(a) for a in h0]
    e2e_pj = gb.projector_for(scene, ctx, **cfg)
    e2e_times = []
    for k in range(args.warmup + args.steps):
        for t, a in zip(hc, h0):
            t[...] = a
        t0 = time.perf_counter()
        e2e_pj.project(scene.dt, tuple(hc), h_solid, h_fluid)
        t1 = time.perf_counter()
        if k >= args.warmup:
            e2e_times.append(t1 - t0)
    e2e_pj.close()
    face_bytes = sum(a.nbytes for a in h0)
    h2d = scene.solid.nbytes + scene.fluid.nbytes + face_bytes
    d2h = face_bytes + scene.fluid.nbytes
    ranks.barrier()
    e2e_value = ranks.rate(len(e2e_times), 1000.0 * sum(e2e_times))

    # the drop-in module's transport (Projection=gbprojection3): the arrays
    # as 8^3 bricks (narrow-band level sets: values within the band listed,
    # whole-fill bricks by flag; a constant array by its background), the
    # bricked call timed with its host<->device copies; the bricks are built
    # before the clock, as the module builds them from the reference's
    # tiled arrays with the reference's own array operations
    e2e_bricks = None
    if scene.dim == 3:
        def level_bricks(a, mode):
            if mode == 1:  # a constant array: every brick reads its background
                return gb.to_bricks(a, np.zeros(a.shape, bool), None, background=float(a.flat[0]))[0]
            return gb.to_bricks(a, np.abs(a) < scene.band, a <= -scene.band, background=scene.band,
                                fill=-scene.band)[0]
        b_solid = level_bricks(scene.solid, scene.solid_mode)
        b_fluid = level_bricks(scene.fluid, scene.fluid_mode)
        b_vel = [gb.to_bricks(a, np.ones(a.shape, bool), None)[0] for a in (scene.u, scene.v, scene.w)]
        nbc = b_fluid[0].size
        out_slots = [np.arange(nbc, dtype=np.int32)] + [np.where(b[0] >= 0, b[0], -1).astype(np.int32) for b in b_vel]
        bpj = gb.projector_for(scene, ctx, **cfg)
        b_times, b_out = [], None
        for k in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            brc, b_out = bpj.project_bricks(scene.dt, b_solid, b_fluid, b_vel, out_slots, outputs=b_out)
            t1 = time.perf_counter()
            if brc != gb.GBP_OK:
                raise RuntimeError(f"bricked projection returned {brc}")
            if k >= args.warmup:
                b_times.append(t1 - t0)
        bpj.close()
        h2d_b = sum(b[0].nbytes + b[1].nbytes for b in [b_solid, b_fluid] + b_vel)
        d2h_b = sum(int((sl >= 0).sum()) * gb.BRICK_CELLS * 5 for sl in out_slots)  # values + active flags
        e2e_bricks = {"value": round(ranks.rate(len(b_times), 1000.0 * sum(b_times)), 3), "unit": "solves/s",
                      "h2d_bytes_per_step": int(h2d_b), "d2h_bytes_per_step": int(d2h_b),
                      "call": "gbp_project_bricks (the plugin module's transport), pageable host buffers",
                      "listed_bricks": {"solid": int((b_solid[0] >= 0).sum()), "fluid": int((b_fluid[0] >= 0).sum()),
                                        "velocity": [int((b[0] >= 0).sum()) for b in b_vel], "of": int(nbc)}}

    # roofline: the path's fine-level kernels timed alone, each launched once
    # per iteration; the slowest is the dominant one
    if args.solver == "mgpcg":
        kernels = {10: "presmooth_kernel", 12: "restrict_kernel", 13: "post_black_kernel",
                   14: "red_dot_kernel", 15: "direction_kernel", 16: "spmv_kernel", 17: "update_kernel"}
    else:
        kernels = {0: "cg_spmv_kernel", 1: "cg_update_kernel", 2: "cg_direction_kernel"}
    timed = {}
    for kid, name in kernels.items():
        ms, nbytes = pj.bench_kernel(kid, reps=50, stream=sh)
        timed[name] = (ms, nbytes)
    dom = max(timed, key=lambda n: timed[n][0])
    ms, nbytes = timed[dom]
    peak, peak_kind = measured_peak_gbs()
    achieved = nbytes / (ms * 1e-3) / 1e9
    traffic = committed_traffic(f"{args.workload}/{args.solver}_{args.precision}", dom)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": nbytes, "ms_per_launch": round(ms, 5),
                "kernels": {n: {"ms": round(t[0], 5), "GBps": round(t[1] / (t[0] * 1e-3) / 1e9, 1)}
                            for n, t in timed.items()}}

    ms_step = total_ms / args.steps
    per_step = main["per_step"]
    out = {
        "metric": METRIC, "value": round(value, 3), "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic (seeded scene generator, shapes and distributions of the workload)",
        "config": {"workload": args.workload, "desc": WORKLOADS[args.workload]["desc"],
                   "grid": [scene.nx, scene.ny, scene.nz], "solver": args.solver, "precision": args.precision,
                   "residual": 1e-6, "unknowns": stats["unknowns"], "iterations": stats["iterations"],
                   "outer_iterations": stats["outer_iterations"], "parallelism": f"replicas x{world}",
                   "l2": "no flush: working set above the 129 MB L2 (operator + vectors + inputs)"},
        "latency_ms": {"p50": round(float(np.percentile(per_step, 50)), 4),
                       "p99": round(float(np.percentile(per_step, 99)), 4)},
        "voxel_updates_per_s": round(scene.cells * stats["iterations"] / (stats["ms_solve"] * 1e-3), 1)
        if stats["ms_solve"] > 0 else None,
        "phase_ms": {"assemble": round(stats["ms_assemble"], 4), "solve": round(stats["ms_solve"], 4),
                     "update": round(stats["ms_update"], 4)},
        "compare": compare,
        "e2e": {"value": round(e2e_value, 3), "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "host_buffers": "pageable numpy arrays",
                "ms_per_step": {"p50": round(1000.0 * float(np.median(e2e_times)), 3),
                                "max": round(1000.0 * float(np.max(e2e_times)), 3)}},
        "e2e_bricks": e2e_bricks,
        "roofline": roofline,
        "clocks": main["clocks"],
        "gpu_launches": int(main["launches"]),
        "residual": {"reresid": stats["reresid"], "true_inf": stats["true_resid_inf"],
                     "true_l2": stats["true_resid_l2"]},
    }
    if not args.no_extra and args.workload == "smoke3_256":
        # the batched and served workloads of the same metric, in this line
        out["batched"] = run_gbp_batch(args, ranks=ranks, workload="batch64_liquid3", steps=5, warmup=3, ctx=ctx)
        out["served"] = run_gbp_served(args, ranks=ranks, nreq=16, ctx_device=local)
    if rank == 0 and not args.no_cpu_baseline:
        ref, out["cpu_baseline"] = oracle_solve(scene)
        out["accuracy"] = accuracy(scene, ref, outputs)
    if rank == 0:
        print(json.dumps(out), flush=True)
    ranks.close()


def run_gbp_batch(args, ranks=None, workload=None, steps=None, warmup=None, ctx=None):
    """A step is one batched projection of all scenes of the batch. Called
    with `ranks`, it runs inside another workload's bench and returns its
    figures instead of printing a line."""
    import torch
    import shiokaze_gb300 as gb
    from shiokaze_gb300 import scenes as scn

    sub = ranks is not None
    workload = workload or args.workload
    steps = steps or args.steps
    warmup = warmup or args.warmup
    rank, world, local = dist_info()
    if not sub:
        ranks = Ranks("nccl", torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    scs = scn.batch_liquid3(WORKLOADS[workload]["n"], seed=4)
    ctx = ctx or gb.Context(local)
    stream = torch.cuda.Stream(device=dev)
    sh = stream.cuda_stream

    def dev_t(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    solids = [dev_t(sc.solid) for sc in scs]
    fluids = [dev_t(sc.fluid) for sc in scs]
    vel0 = [tuple(dev_t(a) for a in (sc.u, sc.v, sc.w)) for sc in scs]
    vel = [tuple(t.clone() for t in v) for v in vel0]
    ps = [torch.zeros(sc.fluid.shape, dtype=torch.float32, device=dev) for sc in scs]
    cells = sum(sc.cells for sc in scs)

    def make(precision):
        cfg = dict(Residual=1e-6, Solver="mgpcg", Precision=precision)
        pjs = [gb.projector_for(sc, ctx, **cfg) for sc in scs]
        return pjs, gb.Batch(pjs, ctx, **cfg)

    def measure(batch, steps, warmup, sampler=None):
        def step():
            for v, v0 in zip(vel, vel0):
                for t, t0 in zip(v, v0):
                    t.copy_(t0)
            rc = batch.project([sc.dt for sc in scs], vel, solids, fluids, ps, stream=sh)
            if rc != gb.GBP_OK:
                raise RuntimeError(f"batched projection returned {rc}")
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                step()
        torch.cuda.synchronize()
        ranks.barrier()
        if sampler:
            sampler.start()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        l0 = ctx.launches()
        with torch.cuda.stream(stream):
            ev[0].record(stream)
            for k in range(steps):
                step()
                ev[k + 1].record(stream)
        torch.cuda.synchronize()
        ranks.barrier()
        clocks = sampler.stop() if sampler else None
        per = [ev[k].elapsed_time(ev[k + 1]) for k in range(steps)]
        return ranks.max_ms(ev[0].elapsed_time(ev[-1])), per, ctx.launches() - l0, clocks

    pjs, batch = make(args.precision)
    total_ms, per, launches, clocks = measure(batch, steps, warmup, None if sub else ClockSampler(local))
    iters = [batch.stats[i].iterations for i in range(len(scs))]
    value = ranks.rate(len(scs) * steps, total_ms)
    compare = {}
    if not args.no_compare:
        other = "fp64" if args.precision == "mixed" else "mixed"
        pjs2, batch2 = make(other)
        t2, _, _, _ = measure(batch2, max(3, steps // 2), 3)
        compare[f"batch_mgpcg_{other}"] = {"solves_per_s": round(len(scs) * max(3, steps // 2) / (t2 / 1000), 2)}
        if other == "fp64":
            compare["mixed_over_fp64"] = round(value / compare["batch_mgpcg_fp64"]["solves_per_s"], 4)
        batch2.close()
        for pj in pjs2:
            pj.close()
        # the same scenes one projection call at a time (no batching)
        seq = [gb.projector_for(sc, ctx, Residual=1e-6, Solver="mgpcg", Precision=args.precision) for sc in scs]
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            for rep in range(2):
                if rep == 1:
                    e0.record(stream)
                for i, pj in enumerate(seq):
                    for t, t0 in zip(vel[i], vel0[i]):
                        t.copy_(t0)
                    pj.project(scs[i].dt, vel[i], solids[i], fluids[i], pressure_out=ps[i], stream=sh)
            e1.record(stream)
        torch.cuda.synchronize()
        compare[f"sequential_mgpcg_{args.precision}"] = {"solves_per_s": round(len(scs) / (e0.elapsed_time(e1) / 1000), 2)}
        for pj in seq:
            pj.close()
    batch.close()
    for pj in pjs:
        pj.close()
    if sub:
        return {"workload": workload, "desc": WORKLOADS[workload]["desc"], "solves_per_s": round(value, 3),
                "ms_per_step": round(total_ms / steps, 4), "steps": steps, "scenes": len(scs), "cells": cells,
                "precision": args.precision, "iterations_max": max(iters),
                "iterations_mean": float(np.mean(iters)), "compare": compare, "gpu_launches": int(launches)}
    out = {
        "metric": METRIC, "value": round(value, 3), "unit": "solves/s", "n_gpus": world, "steps": steps,
        "warmup": warmup, "ms_per_step": round(total_ms / steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic (seeded scene generator, shapes and distributions of the workload)",
        "config": {"workload": workload, "desc": WORKLOADS[workload]["desc"], "scenes": len(scs),
                   "cells": cells, "edges": [sc.nx for sc in scs], "solver": "mgpcg", "precision": args.precision,
                   "residual": 1e-6, "iterations_max": max(iters), "iterations_mean": float(np.mean(iters)),
                   "parallelism": f"replicas x{world}", "l2": "no flush: batch working set above the 129 MB L2"},
        "latency_ms": {"p50": round(float(np.percentile(per, 50)), 4), "p99": round(float(np.percentile(per, 99)), 4)},
        "compare": compare, "clocks": clocks, "gpu_launches": int(launches),
    }
    if rank == 0:
        print(json.dumps(out), flush=True)
    ranks.close()


def run_gbp_served(args, ranks=None, nreq=None, ctx_device=None):
    """Continuous-batching server on a seeded Poisson request stream; the
    same stream served with the mixed and the FP64 solver. Called with
    `ranks`, it runs inside another workload's bench and returns its figures
    instead of printing a line."""
    import torch
    from shiokaze_gb300.serving import ProjectionServer, poisson_requests

    sub = ranks is not None
    rank, world, local = dist_info()
    if not sub:
        ranks = Ranks("nccl", torch.device("cuda", local))
    torch.cuda.set_device(local)
    nreq = nreq or max(4, args.steps)
    results = {}
    sampler = ClockSampler(local)
    for precision in ([args.precision] + ([] if args.no_compare else
                                          ["fp64" if args.precision == "mixed" else "mixed"])):
        warm = ProjectionServer(budget_bytes=150e9, precision=precision, device=local)
        warm.serve(poisson_requests(3, 50.0, seed=99, edges=(32, 64), steps=3))  # JIT/graph warm-up
        srv = ProjectionServer(budget_bytes=150e9, precision=precision, device=local)
        reqs = poisson_requests(nreq, 8.0, seed=5, steps=50)
        if precision == args.precision and not sub:
            sampler.start()
        torch.cuda.synchronize()
        ranks.barrier()
        l0 = srv.ctx.launches()
        done, out = srv.serve(reqs)
        torch.cuda.synchronize()
        ranks.barrier()
        out["gpu_launches"] = srv.ctx.launches() - l0
        if precision == args.precision and not sub:
            out["clocks"] = sampler.stop()
        results[precision] = out
    main = results[args.precision]
    value = ranks.rate(main["solves"], 1000.0 * main["wall_s"])
    if sub:
        sv = {"workload": "served", "desc": WORKLOADS["served"]["desc"], "requests": nreq,
              "precision": args.precision, "solves_per_s": round(value, 3),
              "step_latency_ms": main["step_latency_ms"], "request_latency_s": main["request_latency_s"],
              "serving": {k: main[k] for k in ("solves", "wall_s", "ticks", "mean_batch", "max_batch",
                                               "batch_rebuilds", "peak_bytes", "admission_waits")},
              "compare": {p: {"solves_per_s": round(r["solves_per_s"], 3), "step_latency_ms": r["step_latency_ms"]}
                          for p, r in results.items() if p != args.precision},
              "gpu_launches": int(main["gpu_launches"])}
        if "fp64" in sv["compare"]:
            sv["compare"]["mixed_over_fp64"] = round(value / sv["compare"]["fp64"]["solves_per_s"], 4)
        return sv
    out = {
        "metric": METRIC, "value": round(value, 3), "unit": "solves/s", "n_gpus": world, "steps": nreq,
        "warmup": args.warmup, "ms_per_step": round(1000.0 / main["solves_per_s"], 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic (seeded Poisson request stream and scene generator)",
        "config": {"workload": "served", "desc": WORKLOADS["served"]["desc"], "requests": nreq,
                   "solver": "mgpcg", "precision": args.precision, "residual": 1e-6,
                   "parallelism": f"replicas x{world}", "l2": "no flush: working set above the 129 MB L2"},
        "latency_ms": main["step_latency_ms"],
        "request_latency_s": main["request_latency_s"],
        "serving": {k: main[k] for k in ("requests", "solves", "wall_s", "ticks", "mean_batch", "max_batch",
                                         "batch_rebuilds", "peak_bytes", "admission_waits")},
        "compare": {p: {"solves_per_s": round(r["solves_per_s"], 3), "step_latency_ms": r["step_latency_ms"]}
                    for p, r in results.items() if p != args.precision},
        "clocks": main.get("clocks"), "gpu_launches": int(main["gpu_launches"]),
    }
    if rank == 0:
        print(json.dumps(out), flush=True)
    ranks.close()


def advect_scene(name):
    """The smoke scene of an advection workload and its density field."""
    from shiokaze_gb300 import scenes
    scene = scenes.smoke3(WORKLOADS[name]["n"], seed=3)
    density = np.random.default_rng(6).random(scene.fluid.shape, dtype=np.float32)
    return scene, density


def advect_bytes(scene):
    """Algorithmic DRAM bytes of one MacCormack step (density + velocity):
    per cell 32 B in each scalar pass (the density, the three velocity
    components' faces counted once, the fluid level set, the forward value
    and limiter record); per face 17.3 B forward (the component, the level
    set shared by three faces, the forward value and the 8-byte limiter
    record) and 20 B backward (forward value, record, input, result)."""
    cells = scene.cells
    faces = scene.u.size + scene.v.size + scene.w.size
    return 64.0 * cells + (4 + 4 / 3 + 12 + 20) * faces


def run_gbp_advect(args):
    import torch
    import shiokaze_gb300 as gb

    rank, world, local = dist_info()
    ranks = Ranks("nccl", torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    scene, density = advect_scene(args.workload)
    ctx = gb.Context(local)
    stream = torch.cuda.Stream(device=dev)
    sh = stream.cuda_stream

    def dev_t(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    u, v, w, fluid, q = (dev_t(a) for a in (scene.u, scene.v, scene.w, scene.fluid, density))
    torch.cuda.synchronize()
    adv = gb.MacAdvection3(scene.nx, scene.ny, scene.nz, scene.dx, context=ctx)

    def step():
        adv.advect_step((u, v, w), fluid, scene.dt, scalar=q, stream=sh)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ranks.barrier()
    sampler = ClockSampler(local)
    sampler.start()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    l0 = ctx.launches()
    torch.cuda.synchronize()
    ev[0].record(stream)
    for k in range(args.steps):
        step()
        ev[k + 1].record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    launches = ctx.launches() - l0
    per_step = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    total_ms = ranks.max_ms(ev[0].elapsed_time(ev[-1]))
    value = ranks.rate(args.steps, total_ms)

    # end to end through the host-array call, plain (pageable) numpy arrays
    hu, hv, hw, hf, hq = (np.array(a, dtype=np.float32) for a in (scene.u, scene.v, scene.w, scene.fluid, density))
    e2e_times = []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        adv.advect_step((hu, hv, hw), hf, scene.dt, scalar=hq)
        t1 = time.perf_counter()
        if k >= args.warmup:
            e2e_times.append(t1 - t0)
    face_bytes = scene.u.nbytes + scene.v.nbytes + scene.w.nbytes
    h2d = face_bytes + scene.fluid.nbytes + density.nbytes
    d2h = face_bytes + density.nbytes
    ranks.barrier()
    e2e_value = ranks.rate(len(e2e_times), 1000.0 * sum(e2e_times))

    # the two halves of the step timed alone with CUDA events: the face
    # passes (velocity forward + backward) dominate, the cell passes carry
    # the density
    def timed(fn, reps=10):
        fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps
    face_ms = timed(lambda: adv.advect_vector((u, v, w), (u, v, w), fluid, scene.dt, stream=sh))
    # the solid constraint that follows the projection (macutility3::constrain_velocity)
    solid = dev_t(scene.solid)
    util = gb.MacUtility3(scene.nx, scene.ny, scene.nz, scene.dx, context=ctx)
    constrain_ms = timed(lambda: util.constrain_velocity(solid, (u, v, w), stream=sh))
    cell_ms = timed(lambda: adv.advect_scalar(q, (u, v, w), fluid, scene.dt, stream=sh))
    # velocity extrapolation (array_extrapolator3, 3 rounds) of the u
    # component from the faces inside a ball of radius 0.3 (a liquid's
    # narrow-band velocity), restored from a saved copy before each round of
    # timing; only the extrapolation is between the events
    zc, yc, xc = np.meshgrid(*(np.arange(m) for m in scene.u.shape), indexing="ij")
    ball = (((xc * scene.dx - 0.5) ** 2 + ((yc + 0.5) * scene.dx - 0.5) ** 2 + ((zc + 0.5) * scene.dx - 0.5) ** 2)
            < 0.3 ** 2)
    m0 = dev_t(ball.astype(np.uint8))
    e0 = dev_t(np.where(ball, scene.u, 0.0).astype(np.float32))
    ev_, em_ = e0.clone(), m0.clone()
    ext_ms, ext_added = [], 0
    for r in range(6):
        ev_.copy_(e0)
        em_.copy_(m0)
        a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a_.record(stream)
        ext_added = util.extrapolate(ev_, em_, 3, stream=sh)
        b_.record(stream)
        torch.cuda.synchronize()
        if r:
            ext_ms.append(a_.elapsed_time(b_))
    # the 2D step (macadvection2: velocity and density) on a 2048^2 smoke scene
    from shiokaze_gb300 import scenes
    sc2 = scenes.smoke2(2048, seed=3)
    u2, v2, f2 = dev_t(sc2.u), dev_t(sc2.v), dev_t(sc2.fluid)
    q2 = dev_t(np.random.default_rng(6).random(sc2.fluid.shape, dtype=np.float32))
    adv2 = gb.MacAdvection2(sc2.nx, sc2.ny, sc2.dx, context=ctx)
    advect2_ms = timed(lambda: adv2.advect_step((u2, v2), f2, sc2.dt, scalar=q2, stream=sh))
    faces = scene.u.size + scene.v.size + scene.w.size
    face_bytes_alg = (4 + 4 / 3 + 12 + 20) * faces
    cell_bytes_alg = 64.0 * scene.cells

    ms_step = total_ms / args.steps
    nbytes = advect_bytes(scene)
    peak, peak_kind = measured_peak_gbs()
    achieved = face_bytes_alg / (face_ms * 1e-3) / 1e9
    out = {
        "metric": ADVECT_METRIC, "value": round(value, 3), "unit": "steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 storage, f64 traces (the reference's)",
        "data": "synthetic (seeded smoke scene: velocity N(0,1) faces, density U[0,1))",
        "config": {"workload": args.workload, "desc": WORKLOADS[args.workload]["desc"],
                   "grid": [scene.nx, scene.ny, scene.nz], "parallelism": f"replicas x{world}",
                   "l2": "no flush: inputs and scratch (~1.1 GB) above the 129 MB L2"},
        "latency_ms": {"p50": round(float(np.percentile(per_step, 50)), 4),
                       "p99": round(float(np.percentile(per_step, 99)), 4)},
        "cell_updates_per_s": round(scene.cells / (ms_step * 1e-3), 1),
        "e2e": {"value": round(e2e_value, 3), "unit": "steps/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "roofline": {"bound": "hbm", "kernel": "adv_face_forward + adv_face_backward (velocity passes)",
                     "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": committed_traffic(args.workload, "face_passes"), "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": face_bytes_alg, "ms_per_launch": round(face_ms, 5),
                     "limiter": "FP64 pipe: the reference's double-precision traces and trilinear weights",
                     "kernels": {"face_passes": {"ms": round(face_ms, 5),
                                                 "GBps": round(face_bytes_alg / (face_ms * 1e-3) / 1e9, 1)},
                                 "cell_passes": {"ms": round(cell_ms, 5),
                                                 "GBps": round(cell_bytes_alg / (cell_ms * 1e-3) / 1e9, 1)}},
                     "step_GBps": round(nbytes / (ms_step * 1e-3) / 1e9, 1)},
        "constrain_velocity_ms": round(constrain_ms, 4),
        "extrapolate": {"ms": round(float(np.median(ext_ms)), 4), "rounds": 3, "activated": int(ext_added),
                        "array": f"u component {list(scene.u.shape)}, active inside a ball of radius 0.3"},
        "advect2": {"ms": round(advect2_ms, 4), "grid": [sc2.nx, sc2.ny],
                    "desc": "2D MacCormack step (velocity, then density), smoke 2048^2"},
        "clocks": clocks,
        "gpu_launches": int(launches),
    }
    if rank == 0 and not args.no_cpu_baseline:
        import oracle
        t0 = time.perf_counter()
        oracle.advect3(scene.u, scene.v, scene.w, scene.fluid, scene.dx, scene.dt, q=density)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(1.0 / dt, 5), "unit": "steps/s", "cores": 1, "kind": "port",
                               "sample": f"one full advection step of the same scene by the oracle's C "
                                         f"restatement of the reference's macadvection3, single thread, "
                                         f"{dt:.1f} s"}
    if rank == 0:
        print(json.dumps(out), flush=True)
    ranks.close()


def run_reference_advect(args):
    rank, world, local = dist_info()
    if rank != 0:
        return
    import oracle
    scene, density = advect_scene(args.workload)
    kind = "reference" if oracle.reference_available() else "port"
    times = []
    for k in range(args.steps):
        t0 = time.perf_counter()
        oracle.advect3(scene.u, scene.v, scene.w, scene.fluid, scene.dx, scene.dt, q=density, impl=kind,
                       fluid_mode=scene.fluid_mode, band=scene.band)
        times.append(time.perf_counter() - t0)
        if sum(times) > REFERENCE_BUDGET_S:
            break
    value = len(times) / sum(times)
    what = ("the reference's macadvection3 built from its sources (its own threads)" if kind == "reference"
            else "the oracle's C restatement of the reference's macadvection3, single thread (the reference's "
                 "own build is not on this host)")
    out = {
        "metric": ADVECT_METRIC, "value": round(value, 5), "unit": "steps/s", "n_gpus": world, "steps": len(times),
        "warmup": args.warmup, "ms_per_step": round(1000 * sum(times) / len(times), 2), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 storage, f64 traces", "impl": "reference",
        "data": "synthetic (seeded smoke scene: velocity N(0,1) faces, density U[0,1))",
        "config": {"workload": args.workload, "desc": WORKLOADS[args.workload]["desc"],
                   "grid": [scene.nx, scene.ny, scene.nz]},
        "cpu_baseline": {"value": round(value, 5), "unit": "steps/s",
                         "cores": (os.cpu_count() or 1) if kind == "reference" else 1, "kind": kind,
                         "sample": f"{len(times)} full advection steps of the workload by {what}"},
        "e2e": {"value": round(value, 5), "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def run_reference(args):
    rank, world, local = dist_info()
    if rank != 0:
        return
    import oracle
    if WORKLOADS[args.workload]["kind"] == "batch":
        from shiokaze_gb300 import scenes as scn
        scene = min(scn.batch_liquid3(WORKLOADS[args.workload]["n"], seed=4), key=lambda sc: sc.cells)
    elif WORKLOADS[args.workload]["kind"] == "served":
        scene = make_scene("liquid3_128")
    else:
        scene = make_scene(args.workload)
    kind = "port"
    if oracle.reference_available():
        try:
            oracle._ref_lib()
            kind = "reference"
        except OSError:
            kind = "port"
    # warm-up on a small scene (loader, page faults); every timed step is one
    # full projection of the workload. A CPU solve takes tens of seconds, so
    # the timed steps stop before the next one would pass REFERENCE_BUDGET_S
    # (at least one). The oracle's CG runs its element-wise loops on every
    # host core and its dot products serially, in the reference's order.
    from shiokaze_gb300 import scenes
    threads = oracle.set_threads(None) if kind == "port" else 1
    small = scenes.liquid3(32, seed=2)
    for _ in range(max(1, min(args.warmup, 3))):
        oracle.project_scene(small, kind, residual=1e-6)
    times, iters = [], []
    for k in range(args.steps):
        t0 = time.perf_counter()
        r = oracle.project_scene(scene, kind, residual=1e-6)
        dt = time.perf_counter() - t0
        times.append(dt)
        iters.append(r.iterations)
        if sum(times) + dt > REFERENCE_BUDGET_S:
            break
    value = len(times) / sum(times)
    what = ("the reference's macpressuresolver built from its sources" if kind == "reference"
            else f"the oracle's C restatement of the reference's macpressuresolver (the reference's own build "
                 f"is not on this host; CG element-wise loops on {threads} threads, dot products serial as in the "
                 f"reference, bit-identical to one thread)")
    out = {
        "metric": METRIC, "value": round(value, 5), "unit": "solves/s", "n_gpus": world, "steps": len(times),
        "warmup": args.warmup, "ms_per_step": round(1000 * sum(times) / len(times), 2), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
        "data": "synthetic (seeded scene generator, shapes and distributions of the workload)",
        "config": {"workload": args.workload, "desc": WORKLOADS[args.workload]["desc"],
                   "grid": [scene.nx, scene.ny, scene.nz], "solver": "cg (reference pcg, identity preconditioner)",
                   "residual": 1e-6, "iterations": iters[-1] if iters else None},
        "cpu_baseline": {"value": round(value, 5), "unit": "solves/s", "cores": threads, "kind": kind,
                         "sample": f"{len(times)} full projections of the workload by {what}; warm-up on a "
                                   f"32^3 scene"},
        "e2e": {"value": round(value, 5), "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbp", choices=["gbp", "reference"])
    ap.add_argument("--workload", default="smoke3_256", choices=sorted(WORKLOADS))
    ap.add_argument("--solver", default="mgpcg", choices=["cg", "mgpcg"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-compare", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="leave out the batched and served sub-objects")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gbp":
        args.warmup = 3
    if args.impl == "reference" and WORKLOADS[args.workload]["kind"] == "advect":
        run_reference_advect(args)
    elif args.impl == "reference":
        run_reference(args)
    elif WORKLOADS[args.workload]["kind"] == "batch":
        run_gbp_batch(args)
    elif WORKLOADS[args.workload]["kind"] == "served":
        run_gbp_served(args)
    elif WORKLOADS[args.workload]["kind"] == "advect":
        run_gbp_advect(args)
    else:
        run_gbp(args)


if __name__ == "__main__":
    main()
