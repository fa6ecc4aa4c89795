"""Benchmark: 2D Newtonian SLIC (MinBee), FP32 bulk vs FP64, 4096 x 4096 cells, periodic.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--n 4096]

One "step" is one Strang step X(dt/2) Y(dt) X(dt/2) of the whole grid with the time step computed
on the device from the previous step's CFL reduction (the reference's solve2D loop body,
Solvers/EulerSecondOrderSolver.cpp:131-146).  Metric: cell-updates per second.

Our arm prints one JSON line with
  value           FP32 cell-updates/s with the state resident in HBM (CUDA events on the library's
                  stream around K graph-replayed steps; the 335 MB state exceeds the 129 MB L2, so no
                  flush is needed between steps),
  e2e             the same steps through the C ABI with pinned host buffers: every step copies the
                  grid's primitive state (5 doubles per cell) host->device, runs the step and copies
                  the state back (the reference-facing per-step call, whose grids live on the host),
  fp64            the plain FP64 (reference-exact) path on the same workload,
  l1_rho_fp32_vs_fp64  relative L1 density error of the FP32 run against the FP64 run,
  roofline        per-kernel achieved HBM GB/s for the dominant kernel (the X sweep) against the
                  measured copy bandwidth in MEASURED_PEAKS.json,
  cpu_baseline    the CPU oracle (FP64 restatement of the reference) on the host cores, bounded sample.
--impl reference times the CPU path alone (all host threads) on the same workload.
"""
import argparse
import ctypes
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
sys.path.insert(0, os.path.join(ROOT, "tests"))

WORKLOAD = "2D Newtonian Euler SLIC MinBee, 4096x4096 on [0,1]^2, gamma 1.4, CFL 0.9, periodic, " \
           "four-quadrant Riemann data (seed 2)"
METRIC = "cell-updates/s"


def four_quadrant(n, seed):
    import cases
    return cases.four_quadrant(n, seed)


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Ranks:
    """The bookkeeping of a run launched one process per GPU (torchrun; RANK / WORLD_SIZE from the
    environment): barriers around timed regions, the maximum of a time over ranks, and whole-job
    throughput (units per rank x ranks / the slowest rank's time).  The ranks run independent
    replicas; the process group carries only these scalars.  backend "nccl" with device "cuda" on
    GPUs, "gloo" with "cpu" on hosts."""

    def __init__(self, backend="nccl", device="cuda"):
        self.rank, self.world, _ = dist_env()
        self.device = device
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist
            if not dist.is_initialized():
                dist.init_process_group(backend)
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()
        if self.device == "cuda":
            import torch
            torch.cuda.synchronize()

    def max(self, v):
        if not self.dist:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def throughput(self, units_per_rank, ms):
        """Whole-job units per second from this rank's time in ms (the slowest rank's time counts)."""
        return units_per_rank * self.world / (self.max(ms) * 1e-3)


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, gpu):
        self.gpu, self.samples, self.proc = gpu, [], None

    def __enter__(self):
        q = "clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
            "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
            "clocks_event_reasons.sw_power_cap,utilization.gpu"
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        load = [s for s in self.samples if num(s[7]) and num(s[7]) > 50] or self.samples
        sm = [num(s[0]) for s in load if num(s[0])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in load for k in range(4) if s[3 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": num(load[0][1]), "reasons": reasons, "samples": len(self.samples),
                "samples_under_load": len(load)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_per_launch(kernel):
    """DRAM bytes per launch from the committed ncu summary (profiles/traffic.json), if present."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            t = json.load(f)
        return t.get(kernel)
    except Exception:
        return None


def cpu_baseline(n, seconds=12.0, threads=None):
    """Time the CPU oracle (FP64 restatement of the reference, line-parallel on all host cores) on
    the same workload: as many full-size Strang steps as fit in `seconds` (at least one)."""
    from oracle.pyoracle import Oracle
    O = Oracle()
    cores = threads or os.cpu_count() or 1
    O.set_threads(cores)
    s = four_quadrant(n, 2)
    t0 = time.perf_counter()
    steps = 0
    while True:
        s, k, _, _ = O.solve(0, s, 2, 1.0 / n, 0.9, 1e9, 0.0, 2, 1.4, 1, max_steps=1)
        steps += k
        el = time.perf_counter() - t0
        if el >= seconds or steps >= 50:
            break
    rate = steps * n * n / el
    return {"value": rate, "unit": METRIC, "cores": cores, "kind": "port",
            "sample": f"{steps} full {n}x{n} Strang steps of the FP64 oracle (restatement of the reference, "
                      f"bit-identical to it) in {el:.1f} s on {cores} host threads"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    n = args.n
    base = cpu_baseline(n, seconds=max(8.0, 2.0 * args.steps))
    line = {"metric": METRIC, "value": base["value"], "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": n * n / base["value"] * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": WORKLOAD, "n": n, "cells": n * n},
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import cosmos_gb300 as cg
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    ranks = Ranks("nccl", "cuda")
    L = cg.load()
    ctx = cg.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    n = args.n
    s0 = four_quadrant(n, 2)
    cells = n * n
    barrier, max_over_ranks = ranks.barrier, ranks.max

    # ---------------- FP32 resident: value
    g = cg.Grid(cg.NEWTONIAN, (n, n), 1.0 / n, 1.4, cg.FP32, cg.BC_PERIODIC, ctx=ctx)
    g.set_prim(s0)
    g.run_begin(2, 0.9, 1e30, 0.0, cg.MINBEE)
    g.run_steps(args.warmup)
    ctx.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = L.cosmos_kernel_launches()
    barrier()
    with Clocks(local) as clk:
        with torch.cuda.stream(stream):
            e0.record(stream)
            g.run_steps(args.steps)
            e1.record(stream)
        e1.synchronize()
    barrier()
    launches = L.cosmos_kernel_launches() - launches0
    ms = max_over_ranks(e0.elapsed_time(e1)) / args.steps
    r = g.run_end()
    value = ranks.throughput(cells, ms)

    # ---------------- per-kernel durations for the roofline (individual launches, events between)
    dt_probe = 0.5 * 0.9 / n / 2.0
    kern = {"x": [], "y": []}
    with torch.cuda.stream(stream):
        for _ in range(3):
            g.sweep(0, 2, dt_probe, 0.0, cg.MINBEE)
            g.sweep(1, 2, dt_probe, 0.0, cg.MINBEE)
        for _ in range(max(4, args.steps // 2)):
            for ax, key in ((0, "x"), (1, "y")):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                g.sweep(ax, 2, dt_probe, 0.0, cg.MINBEE)
                b.record(stream)
                kern[key].append((a, b))
    torch.cuda.synchronize()
    kx = statistics.mean(a.elapsed_time(b) for a, b in kern["x"])
    ky = statistics.mean(a.elapsed_time(b) for a, b in kern["y"])
    peak, peak_kind = peaks()
    bytes_sweep = cells * 40  # 5 FP32 fields read + 5 written per cell (halo re-reads not counted)
    x_gbs = bytes_sweep / (kx * 1e-3) / 1e9
    y_gbs = bytes_sweep / (ky * 1e-3) / 1e9
    step_gbs = cells * 120 / (ms * 1e-3) / 1e9

    # ---------------- e2e: per step, host state in -> step -> host state out (pinned buffers)
    host_in = torch.empty((n, n, 5), dtype=torch.float64, pin_memory=True)
    host_out = torch.empty((n, n, 5), dtype=torch.float64, pin_memory=True)
    host_in.numpy()[...] = s0
    ge = cg.Grid(cg.NEWTONIAN, (n, n), 1.0 / n, 1.4, cg.FP32, cg.BC_PERIODIC, ctx=ctx)
    ge.set_prim(s0)
    ge.run_begin(2, 0.9, 1e30, 0.0, cg.MINBEE)
    nbytes = cells * 5 * 8
    e2e_steps = max(3, min(args.steps, 10))
    for _ in range(2):
        L.cosmos_grid_set_prim(ge.h, host_in.data_ptr(), cells * 5)
        ge.run_steps(1)
        L.cosmos_grid_get_prim(ge.h, host_out.data_ptr(), cells * 5)
    barrier()
    with torch.cuda.stream(stream):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(e2e_steps):
            cg._lib.check(L.cosmos_grid_set_prim(ge.h, host_in.data_ptr(), cells * 5))
            ge.run_steps(1)
            cg._lib.check(L.cosmos_grid_get_prim(ge.h, host_out.data_ptr(), cells * 5))
        b.record(stream)
        b.synchronize()
    e2e_ms = max_over_ranks(a.elapsed_time(b)) / e2e_steps
    e2e_value = ranks.throughput(cells, e2e_ms)
    ge.close()

    # ---------------- FP64 (reference-exact) on the same workload, and the FP32-vs-FP64 error
    nerr = args.err_steps
    g32 = cg.Grid(cg.NEWTONIAN, (n, n), 1.0 / n, 1.4, cg.FP32, cg.BC_PERIODIC, ctx=ctx)
    g32.set_prim(s0)
    g32.solve(2, 0.9, 1e30, 0.0, cg.MINBEE, max_steps=nerr)
    rho32 = g32.get_prim()[..., 0].copy()
    g32.close()
    g64 = cg.Grid(cg.NEWTONIAN, (n, n), 1.0 / n, 1.4, cg.FP64, cg.BC_PERIODIC, ctx=ctx)
    g64.set_prim(s0)
    g64.run_begin(2, 0.9, 1e30, 0.0, cg.MINBEE, max_steps=nerr)
    with torch.cuda.stream(stream):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        g64.run_steps(nerr)
        b.record(stream)
        b.synchronize()
    ms64 = max_over_ranks(a.elapsed_time(b)) / nerr
    g64.run_end()
    rho64 = g64.get_prim()[..., 0]
    g64.close()
    l1 = float(np.abs(rho32 - rho64).mean() / np.abs(rho64).mean())

    if rank != 0:
        return
    base = cpu_baseline(n, seconds=args.cpu_seconds) if not args.no_cpu else None
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "n": n, "cells_per_gpu": cells, "precision": "fp32 bulk",
                   "l2": "state 335 MB > 129 MB L2 (no flush needed)", "parallelism": f"replicas x{world}",
                   "device_dt": True, "graph_replay": True, "steps_completed": r.steps},
        "fp64": {"value": cells * world / (ms64 * 1e-3), "ms_per_step": ms64, "steps": nerr,
                 "path": "plain FP64, bit-identical to the reference"},
        "l1_rho_fp32_vs_fp64": l1, "l1_steps": nerr,
        "fp32_over_fp64": ms64 / ms,
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "ms_per_step": e2e_ms, "steps": e2e_steps,
                "what": "per step: pinned host AoS FP64 primitives -> device, one Strang step, state -> host"},
        "roofline": {"bound": "hbm", "kernel": "sweep_x_pair_kernel (X sweep, FP32 cell pairs)",
                     "achieved": x_gbs, "peak": peak, "unit": "GB/s", "frac": x_gbs / peak,
                     "peak_source": peak_kind, "traffic": traffic_per_launch("sweep_x_fp32"),
                     "algorithmic_bytes_per_launch": bytes_sweep, "ms_per_launch": kx,
                     "y_sweep": {"achieved": y_gbs, "frac": y_gbs / peak, "ms_per_launch": ky},
                     "step": {"achieved": step_gbs, "frac": step_gbs / peak, "bytes_per_cell_update": 120}},
        "clocks": clk.summary(),
        "gpu_launches": int(launches),
        "status": r.status,
    }
    if base:
        line["cpu_baseline"] = base
    print(json.dumps(line), flush=True)


BATCH_WORKLOAD = "256 independent Newtonian Euler grids (1D and 2D), every side log-uniform in " \
                 "[128, 2048] cells (seed 5), seeded Riemann data, SLIC MinBee, CFL 0.9, transmissive, dx = 1/nx"


def batch_problem():
    import cases
    shapes = cases.batch_shapes()
    states = [cases.riemann(sh, 1000 + k) for k, sh in enumerate(shapes)]
    dxs = [1.0 / sh[-1] for sh in shapes]
    return shapes, states, dxs


def batch_cpu_baseline(shapes, states, dxs, seconds=12.0):
    """The CPU oracle on the batched workload: one step of each grid in turn (the grids are
    independent) until `seconds` have passed; cell-updates per second."""
    from oracle.pyoracle import Oracle
    O = Oracle()
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    t0 = time.perf_counter()
    cells = grids = 0
    for k in range(len(shapes)):
        O.solve(0, states[k], 2, dxs[k], 0.9, 1e9, 0.0, 2, 1.4, 0, max_steps=1)
        cells += int(np.prod(shapes[k]))
        grids += 1
        if time.perf_counter() - t0 >= seconds:
            break
    el = time.perf_counter() - t0
    return {"value": cells / el, "unit": METRIC, "cores": cores, "kind": "port",
            "sample": f"one FP64 oracle step of each of the first {grids} grids ({cells} cells) in {el:.1f} s "
                      f"on {cores} host threads"}


def run_batch(args):
    import torch
    import cosmos_gb300 as cg
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    L = cg.load()
    ctx = cg.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    shapes, states, dxs = batch_problem()
    cells = sum(int(np.prod(sh)) for sh in shapes)
    bytes_step = sum(int(np.prod(sh)) * (120 if len(sh) == 2 else 40) for sh in shapes)

    def timed(fn):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            a.record(stream)
            fn()
            b.record(stream)
        b.synchronize()
        return a.elapsed_time(b)

    b = cg.Batch(shapes, dxs, 1.4, cg.FP32, cg.BC_TRANSMISSIVE, ctx=ctx)
    for k, s in enumerate(states):
        b.set_prim(k, s)
    b.run_begin(0.9, 1e30, 0.0, cg.MINBEE)
    tile_ms = {f"{nt}x{seg}{'c' if cap else ''}": b.time_shape(nt, seg, cap, steps=5)
               for nt in (128, 256) for seg in (32, 64) for cap in (0, 1)}
    tuned, _ = b.autotune(None)
    b.run_steps(args.warmup)
    launches0 = L.cosmos_kernel_launches()
    with Clocks(local) as clk:
        ms = timed(lambda: b.run_steps(args.steps)) / args.steps
    launches = L.cosmos_kernel_launches() - launches0
    res = b.run_end()
    value = cells / (ms * 1e-3)
    peak, peak_kind = peaks()
    gbs = bytes_step / (ms * 1e-3) / 1e9

    # the same grids advanced one by one (each its own graph-replayed steps), for comparison
    ku = 5
    singles = []
    for k, sh in enumerate(shapes):
        g = cg.Grid(cg.NEWTONIAN, sh, dxs[k], 1.4, cg.FP32, cg.BC_TRANSMISSIVE, ctx=ctx)
        g.set_prim(states[k])
        g.run_begin(2, 0.9, 1e30, 0.0, cg.MINBEE)
        g.run_steps(3)
        singles.append(g)
    ms_u = timed(lambda: [g.run_steps(ku) for g in singles]) / ku
    for g in singles:
        g.close()

    # FP64 batch (bit-identical to the reference per grid) and the FP32-vs-FP64 density error
    nerr = 10
    b64 = cg.Batch(shapes, dxs, 1.4, cg.FP64, cg.BC_TRANSMISSIVE, ctx=ctx)
    b32 = cg.Batch(shapes, dxs, 1.4, cg.FP32, cg.BC_TRANSMISSIVE, ctx=ctx)
    for k, s in enumerate(states):
        b64.set_prim(k, s)
        b32.set_prim(k, s)
    b64.run_begin(0.9, 1e30, 0.0, cg.MINBEE, max_steps=nerr)
    b64.autotune(None)
    ms64 = timed(lambda: b64.run_steps(nerr)) / nerr
    b64.run_end()
    b32.run_begin(0.9, 1e30, 0.0, cg.MINBEE, max_steps=nerr)
    b32.set_shape(*tuned)
    b32.run_steps(nerr)
    b32.run_end()
    num = den = 0.0
    for k in range(len(shapes)):
        r64 = b64.get_prim(k)[..., 0]
        num += float(np.abs(b32.get_prim(k)[..., 0] - r64).sum())
        den += float(np.abs(r64).sum())
    b64.close()
    b32.close()

    # e2e: per step, every grid's primitive state host -> device, one batched step, state -> host
    hosts = [torch.empty(sh + (5,), dtype=torch.float64, pin_memory=True) for sh in shapes]
    for h, s in zip(hosts, states):
        h.numpy()[...] = s
    be = cg.Batch(shapes, dxs, 1.4, cg.FP32, cg.BC_TRANSMISSIVE, ctx=ctx)
    be.set_shape(*tuned)
    be.run_begin(0.9, 1e30, 0.0, cg.MINBEE)

    def e2e_step():
        for k, h in enumerate(hosts):
            cg._lib.check(L.cosmos_batch_set_prim(be.h, k, h.data_ptr(), h.numel()))
        be.run_steps(1)
        for k, h in enumerate(hosts):
            cg._lib.check(L.cosmos_batch_get_prim(be.h, k, h.data_ptr(), h.numel()))
    e2e_step()
    e2e_steps = 3
    e2e_ms = timed(lambda: [e2e_step() for _ in range(e2e_steps)]) / e2e_steps
    be.close()
    nbytes = cells * 5 * 8

    adj = adjoint_measure(cg, ctx)
    base = None if args.no_cpu else batch_cpu_baseline(shapes, states, dxs, args.cpu_seconds)
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": BATCH_WORKLOAD, "grids": len(shapes), "grids_2d": sum(len(s) == 2 for s in shapes),
                   "cells": cells, "precision": "fp32 bulk", "tile_shape": list(tuned),
                   "l2": f"state {cells * 40 / 1e9:.2f} GB > 129 MB L2 (no flush needed)",
                   "launch": "one persistent cooperative kernel per 10 steps, replayed from a CUDA graph"},
        "tile_ms_per_step": tile_ms,
        "unbatched": {"value": cells / (ms_u * 1e-3), "ms_per_step": ms_u,
                      "what": "the same grids stepped one after another, each by its own graph-replayed steps"},
        "fp64": {"value": cells / (ms64 * 1e-3), "ms_per_step": ms64, "steps": nerr,
                 "path": "FP64 batch, bit-identical to the reference per grid"},
        "l1_rho_fp32_vs_fp64": num / den, "l1_steps": nerr,
        "e2e": {"value": cells / (e2e_ms * 1e-3), "unit": METRIC, "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes, "ms_per_step": e2e_ms, "steps": e2e_steps,
                "what": "per step: each grid's pinned host AoS FP64 primitives -> device, one batched step, "
                        "states -> host"},
        "roofline": {"bound": "hbm", "kernel": "batch_pair_kernel (whole step, FP32 cell pairs)",
                     "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak, "peak_source": peak_kind,
                     "traffic": (traffic_per_launch("batch_step_fp32_ratio") or 0.0) * bytes_step or None,
                     "traffic_note": "per step; ncu ratio traffic/algorithmic of a 64-grid capture x this "
                                     "workload's algorithmic bytes", "algorithmic_bytes_per_step": bytes_step,
                     "bytes_per_cell_update": "40 (1D), 120 (2D)"},
        "adjoint": adj,
        "clocks": clk.summary(),
        "gpu_launches": int(launches),
        "status": [r.status for r in res if r.status][:8],
    }
    if base:
        line["cpu_baseline"] = base
    print(json.dumps(line), flush=True)


def adjoint_measure(cg, ctx, n=2048, nsteps=100, every=10):
    """Adjoint of `nsteps` SLIC steps (checkpoint every `every`) of the loss 1/2 |rho_T - target|^2 on
    the batch's largest grid size (n x n, FP32, seeded Riemann data, seeded target), timed against
    its forward pass; plus a central finite-difference check of the FP64 gradient at 64 x 64."""
    import cases
    p0 = cases.riemann((n, n), 77)
    rng = np.random.default_rng(78)
    target = p0[..., 0] * (1.0 + 0.05 * rng.standard_normal((n, n)))
    g = cg.Grid(cg.NEWTONIAN, (n, n), 1.0 / n, 1.4, cg.FP32, cg.BC_TRANSMISSIVE, ctx=ctx)
    runs = []
    for _ in range(3):
        g.set_prim(p0)
        runs.append(g.adjoint(target, nsteps, 0.9, 0.0, cg.MINBEE, checkpoint_every=every)[3])
    g.close()
    fwd = statistics.median(r[0] for r in runs)
    bwd = statistics.median(r[1] for r in runs)
    # finite differences of the FP64 forward (same fixed dts) in one seeded direction
    m = 64
    q0 = cases.smooth_state((m, m), 5)
    tq = cases.smooth_state((m, m), 6)[..., 0]
    gq = cg.Grid(cg.NEWTONIAN, (m, m), 1.0 / m, 1.4, cg.FP64, cg.BC_TRANSMISSIVE, ctx=ctx)
    gq.set_prim(q0)
    _, grad, dts, _ = gq.adjoint(tq, nsteps, 0.9, 0.0, cg.MINBEE, checkpoint_every=every)
    d = np.random.default_rng(79).standard_normal(q0.shape)
    # The step map is piecewise smooth (limiter branches): a central difference whose +-h stencil
    # crosses a branch point measures neither one-sided derivative.  h shrinks by decades until two
    # successive differences agree to 1e-5 (no crossing in either stencil, round-off still small);
    # the larger h of that pair is reported.
    def central(h):
        ls = []
        for sgn in (1.0, -1.0):
            gq.set_prim(q0 + sgn * h * d)
            ls.append(gq.adjoint(tq, nsteps, 0.9, 0.0, cg.MINBEE, checkpoint_every=every, dts=dts)[0])
        return (ls[0] - ls[1]) / (2 * h)
    hs = [1e-6, 1e-7, 1e-8, 1e-9, 1e-10]
    fds = [central(hs[0])]
    h, fd = hs[-1], None
    for i in range(1, len(hs)):
        fds.append(central(hs[i]))
        if abs(fds[i] - fds[i - 1]) <= 1e-5 * abs(fds[i]):
            h, fd = hs[i - 1], fds[i - 1]
            break
    if fd is None:
        fd = fds[-1]
    gq.close()
    an = float(np.sum(grad * d))
    return {"grid": f"{n}x{n} FP32, seeded Riemann data", "steps": nsteps, "checkpoint_every": every,
            "forward_ms": fwd, "backward_ms": bwd, "adjoint_over_forward": bwd / fwd,
            "what": "backward = recomputation of each checkpoint segment + the sweep adjoints, per forward "
                    "pass of the same steps (graph-replayed, checkpoints stored)",
            "fd_check": {"grid": f"{m}x{m} FP64 smooth data", "steps": nsteps, "h": h,
                         "rule": "h = 1e-6, 1e-7, ... until two successive central differences agree to 1e-5",
                         "fd_by_h": {f"{x:.0e}": v for x, v in zip(hs, fds)},
                         "directional_adjoint": an, "directional_fd": fd, "rel_err": abs(fd - an) / abs(an)}}


def run_batch_reference(args):
    rank, _, _ = dist_env()
    if rank != 0:
        return
    shapes, states, dxs = batch_problem()
    cells = sum(int(np.prod(sh)) for sh in shapes)
    base = batch_cpu_baseline(shapes, states, dxs, max(8.0, 2.0 * args.steps))
    line = {"metric": METRIC, "value": base["value"], "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": cells / base["value"] * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": BATCH_WORKLOAD, "grids": len(shapes), "cells": cells},
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- SR (2048^2 Kelvin-Helmholtz) and GR (1024^2 accretion)
SR_WORKLOAD = "2D special-relativistic Euler (gamma 5/3), SLIC MinBee, CFL 0.9, 2048x2048 on the periodic " \
              "unit square, Kelvin-Helmholtz shear layers (vx = +-0.5 tanh profile, rho in {1, 2}, p = 1, " \
              "vy = 0.01 sin(4 pi x + phase), phase seed 3; Lorentz factor <= 1.16); 200 steps"
GR_WORKLOAD = "2D black-hole Euler in Kerr-Schild Schwarzschild spacetime (M = 1), SLIC van Leer + " \
              "RK4 source (BlackHoleEulerForcingSolver, one subcycle), CFL 0.9, 1024x1024 on [-10, 10]^2 " \
              "(dx = 20/1024, hole at (10, 10) of the grid's coordinates), excision r <= 2M, rho = 1 with 1% " \
              "log-normal noise (seed 4), p = 0.01, transmissive; 100 steps"


def gr_state(n, seed=4):
    rng = np.random.default_rng(seed)
    s = np.zeros((n, n, 5))
    s[..., 0] = np.exp(0.01 * rng.standard_normal((n, n)))
    s[..., 4] = 0.01
    return s


def grid_problem(kind, n):
    """(system, state, dx, gamma, boundary, limiter, black hole, subcycles)"""
    import cases
    if kind == "sr":
        return 1, cases.kelvin_helmholtz(n, 3), 1.0 / n, 5.0 / 3.0, 1, 2, None, 1
    return 2, gr_state(n), 20.0 / n, 5.0 / 3.0, 0, 1, (1.0, 0.0, 10.0, 10.0, 0.0), 1


def grid_cpu_baseline(kind, n, seconds):
    """The CPU oracle (FP64 restatement of the reference, line-parallel on all host cores) on the
    full-size grid: whole steps until `seconds` have passed (at least one)."""
    from oracle.pyoracle import Oracle
    O = Oracle()
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    system, s, dx, gam, bc, lim, bh, sub = grid_problem(kind, n)
    t0 = time.perf_counter()
    steps = 0
    while True:
        s, k, _, _ = O.solve(system, s, 2, dx, 0.9, 1e9, 0.0, lim, gam, bc, subcycles=sub, bh=bh, max_steps=1)
        steps += k
        el = time.perf_counter() - t0
        if el >= seconds or steps >= 20:
            break
    return {"value": steps * n * n / el, "unit": METRIC, "cores": cores, "kind": "port",
            "sample": f"{steps} full {n}x{n} steps of the FP64 oracle (bit-identical restatement of the reference) "
                      f"in {el:.1f} s on {cores} host threads"}


def run_grid(args, kind):
    """One SR or GR grid: FP32 (SR) or FP64 (GR) steps resident in HBM, e2e through the C ABI with
    host buffers, the FP64 path and the FP32-vs-FP64 density error (SR)."""
    import torch
    import cosmos_gb300 as cg
    _, _, local = dist_env()
    torch.cuda.set_device(local)
    L = cg.load()
    ctx = cg.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    n = args.n if args.n != 4096 else (2048 if kind == "sr" else 1024)
    system, s0, dx, gam, bc, lim, bh, sub = grid_problem(kind, n)
    cells = n * n
    bhs = cg.BlackHoleSpacetime(*bh) if bh else None
    prec = cg.FP32

    def timed(fn):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            a.record(stream)
            fn()
            b.record(stream)
        b.synchronize()
        return a.elapsed_time(b)

    def make(precision, above=2.0):
        g = cg.Grid(system, (n, n), dx, gam, precision, bc, bhs, ctx=ctx, sr_c2p64_above=above)
        g.set_prim(s0)
        g.run_begin(2, 0.9, 1e30, 0.0, lim, subcycles=sub)
        return g

    steps = args.steps if args.steps != 200 or kind == "sr" else 100
    g = make(prec)
    g.run_steps(args.warmup)
    launches0 = L.cosmos_kernel_launches()
    with Clocks(local) as clk:
        ms = timed(lambda: g.run_steps(steps)) / steps
    launches = L.cosmos_kernel_launches() - launches0
    r = g.run_end()
    g.close()
    value = cells / (ms * 1e-3)
    extra = {}
    nerr = 10 if kind == "sr" else 5
    if kind == "gr":
        # FP64 over the same window as the FP32 value (the per-step cost grows as the inflow reaches
        # the horizon, where the recovery meets states without a physical root)
        g64 = make(cg.FP64)
        g64.run_steps(args.warmup)
        ms64 = timed(lambda: g64.run_steps(steps)) / steps
        g64.close()
        g64 = make(cg.FP64)
        g64.run_steps(nerr)
        rho64 = g64.get_prim()[..., 0]
        g64.close()
        g32 = make(cg.FP32)
        g32.run_steps(nerr)
        rho32 = g32.get_prim()[..., 0]
        g32.close()
        x = np.arange(n) * dx
        X, Y = np.meshgrid(x, x)
        outside = np.sqrt((X - bh[2]) ** 2 + (Y - bh[3]) ** 2) > 2.0 * bh[0] + 3 * dx
        extra = {"fp64": {"value": cells / (ms64 * 1e-3), "ms_per_step": ms64, "steps": steps,
                          "path": "plain FP64, bit-identical to the reference (same steps as value)"},
                 "l1_rho_vs_fp64": float(np.abs(rho32[outside] - rho64[outside]).mean() / np.abs(rho64[outside]).mean()),
                 "l1_cells": "outside r > 2M + 3 dx (the excised region keeps its initial state in both)",
                 "l1_steps": nerr, "fp32_over_fp64": ms64 / ms}
    if kind == "sr":
        # FP32 with the FP64 Newton stage in every primitive recovery
        ga = make(cg.FP32, 0.0)
        ga.run_steps(args.warmup)
        ms_a = timed(lambda: ga.run_steps(steps)) / steps
        ga.close()
        # the FP64 (reference-exact) path and the density errors after nerr steps
        g64 = make(cg.FP64)
        ms64 = timed(lambda: g64.run_steps(nerr)) / nerr
        rho64 = g64.get_prim()[..., 0]
        g64.close()
        errs = {}
        for tag, above in (("fp32", 2.0), ("fp32_c2p64_always", 0.0)):
            gg = make(cg.FP32, above)
            gg.run_steps(nerr)
            rr = gg.get_prim()[..., 0]
            gg.close()
            errs[tag] = float(np.abs(rr - rho64).mean() / np.abs(rho64).mean())
        extra = {"fp64": {"value": cells / (ms64 * 1e-3), "ms_per_step": ms64, "steps": nerr,
                          "path": "plain FP64, bit-identical to the reference"},
                 "fp32_c2p64_always": {"value": cells / (ms_a * 1e-3), "ms_per_step": ms_a,
                                       "what": "FP32 with the FP64 Newton stage in every primitive recovery"},
                 "l1_rho_vs_fp64": errs, "l1_steps": nerr, "fp32_over_fp64": ms64 / ms}
    # e2e: per step, host primitives -> device, one step, state -> host (pinned buffers)
    host = torch.empty((n, n, 5), dtype=torch.float64, pin_memory=True)
    host.numpy()[...] = s0
    ge = make(prec)
    nbytes = cells * 5 * 8

    def e2e_step():
        cg._lib.check(L.cosmos_grid_set_prim(ge.h, host.data_ptr(), cells * 5))
        ge.run_steps(1)
        cg._lib.check(L.cosmos_grid_get_prim(ge.h, host.data_ptr(), cells * 5))
    e2e_step()
    e2e_steps = 3
    e2e_ms = timed(lambda: [e2e_step() for _ in range(e2e_steps)]) / e2e_steps
    ge.close()
    peak, peak_kind = peaks()
    word = 4 if prec == cg.FP32 else 8
    bpc = (30 if kind == "sr" else 50) * word  # 3 sweeps x 10 words (+ 2 RK source passes for GR)
    gbs = cells * bpc / (ms * 1e-3) / 1e9
    base = None if args.no_cpu else grid_cpu_baseline(kind, n, args.cpu_seconds)
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 1, "steps": steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if prec == cg.FP32 else "f64", "data": "synthetic",
        "config": {"workload": SR_WORKLOAD if kind == "sr" else GR_WORKLOAD, "n": n, "cells": cells,
                   "precision": "fp32 bulk; primitive recovery finishes in FP64 for W > 2 or when the FP32 "
                                "Newton iteration does not converge" + ("" if kind == "sr" else
                                "; metric, its derivatives and inverses from FP64 tables built once"),
                   "l2": f"state {cells * 10 * word / 1e6:.0f} MB (two buffers) > 129 MB L2 (no flush needed)"
                   if cells * 10 * word > 129e6 else "state fits in L2",
                   "device_dt": True, "graph_replay": True, "steps_completed": r.steps},
        **extra,
        "e2e": {"value": cells / (e2e_ms * 1e-3), "unit": METRIC, "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes, "ms_per_step": e2e_ms, "steps": e2e_steps,
                "what": "per step: pinned host AoS FP64 primitives -> device, one step, state -> host"},
        "roofline": {"bound": "hbm", "kernel": "whole step (X, Y, X sweeps" + (", RK source" if kind == "gr" else "") + ")",
                     "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak, "peak_source": peak_kind,
                     "traffic": None, "bytes_per_cell_update": bpc,
                     "note": "compute-bound: primitive recovery (FP32 Newton, FP64 stage above W = 2)" +
                             ("; RK4 source: 38 recoveries per cell per source step" if kind == "gr" else "")},
        "clocks": clk.summary(), "gpu_launches": int(launches), "status": r.status,
    }
    if base:
        line["cpu_baseline"] = base
    print(json.dumps(line), flush=True)


def run_grid_reference(args, kind):
    rank, _, _ = dist_env()
    if rank != 0:
        return
    n = args.n if args.n != 4096 else (2048 if kind == "sr" else 1024)
    base = grid_cpu_baseline(kind, n, max(8.0, 2.0 * args.steps))
    line = {"metric": METRIC, "value": base["value"], "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": n * n / base["value"] * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": SR_WORKLOAD if kind == "sr" else GR_WORKLOAD, "n": n},
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- Level-1 AMR (EulerAMR::solve2DLevel1AMR)
AMR_WORKLOAD = "Level-1 AMR, EulerAMR::solve2DLevel1AMR: 2D Newtonian cylindrical explosion (rho, p = 1, 1 inside " \
               "r <= 0.2, 0.125, 0.1 outside), 512x512 coarse cells on [0,1]^2 (1024x1024 fine), gamma 1.4, " \
               "CFL 0.95, SLIC (bias 0, van Leer, as the driver fixes them), AMRTolerance 25.6, transmissive, " \
               "t_final 0.125; one step = one whole driver run"
AMR_N, AMR_T, AMR_TOL, AMR_CFL = 512, 0.125, 25.6, 0.95


def amr_problem(n):
    """The reference's 2D AMR test layout (Tests/EulerAMRTests.cpp:33-62) on n x n coarse cells."""
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    inside = np.sqrt((i - 0.5 * n) ** 2 + (j - 0.5 * n) ** 2) <= 0.2 * n
    s = np.zeros((n, n, 5))
    s[..., 0] = np.where(inside, 1.0, 0.125)
    s[..., 4] = np.where(inside, 1.0, 0.1)
    return s


def amr_cpu_baseline(n, t_sample):
    """The oracle's Level-1 driver (FP64 restatement, bit-identical to the reference's) on all host
    cores, run to t_sample; cell-updates = coarse steps x coarse cells + fine steps taken x fine cells."""
    from oracle.pyoracle import Oracle
    O = Oracle()
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    s = amr_problem(n)
    fr = []
    t0 = time.perf_counter()
    nc, _, _, _, _, _ = O.amr_level1(0, s, 1.0 / n, AMR_CFL, t_sample, AMR_TOL * n / AMR_N, 2, 1.4, fine_run=fr)
    el = time.perf_counter() - t0
    cells = nc * n * n + fr[0] * 4 * n * n
    return {"value": cells / el, "unit": METRIC, "cores": cores, "kind": "port", "sample_ms": el * 1e3,
            "sample": f"the oracle's Level-1 AMR driver on the same {n}x{n} problem to t = {t_sample} "
                      f"({nc} coarse and {fr[0]} fine steps, {cells / 1e6:.0f} M cell-updates) in {el:.1f} s "
                      f"on {cores} host threads (sweeps line-parallel; flag, exchange and derefinement passes serial)"}


def run_amr(args):
    """Level-1 AMR runs (FP64, bit-identical to the reference's driver; FP32 beside it), state
    resident in HBM between runs; e2e with host buffers through the C ABI."""
    import torch
    import cosmos_gb300 as cg
    _, _, local = dist_env()
    torch.cuda.set_device(local)
    L = cg.load()
    ctx = cg.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    n = args.n if args.n != 4096 else AMR_N
    tol = AMR_TOL * n / AMR_N
    s0 = amr_problem(n)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def timed(fn):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            a.record(stream)
            fn()
            b.record(stream)
        b.synchronize()
        return a.elapsed_time(b)

    def measure(precision, runs, warm):
        # every run starts from the initial cells (a run leaves its final cells in the coarse grid)
        a = cg.AMR(cg.NEWTONIAN, (n, n), 1.0 / n, 1.4, precision, ctx=ctx)
        for _ in range(warm):
            a.set_prim(s0)
            a.solve(AMR_CFL, AMR_T, tol, 2)
        times, info = [], None
        for _ in range(runs):
            a.set_prim(s0)
            flush.fill_(1)  # evict the previous run's state from L2
            r = []
            times.append(timed(lambda: r.append(a.solve(AMR_CFL, AMR_T, tol, 2))))
            info = (r[0], a.fine_run)
        cp, fp, cf, ff = a.get()
        a.close()
        return times, info, cp, cf

    steps = args.steps if args.steps != 200 else 3
    launches0 = L.cosmos_kernel_launches()
    with Clocks(local) as clk:
        t64, (r64, run64), cp64, cf64 = measure(cg.FP64, steps, args.warmup)
    launches = (L.cosmos_kernel_launches() - launches0) // (steps + args.warmup)
    ms = statistics.median(t64)
    ncoarse, nfine = r64[0], run64
    cells = ncoarse * n * n + nfine * 4 * n * n
    value = cells / (ms * 1e-3)
    t32, (r32, run32), cp32, cf32 = measure(cg.FP32, steps, 1)
    ms32 = statistics.median(t32)
    cells32 = r32[0] * n * n + run32 * 4 * n * n

    def measure_level2(precision):
        """The Level-2 driver (three levels) on the same problem: one warm-up run, one timed run."""
        a = cg.AMR(cg.NEWTONIAN, (n, n), 1.0 / n, 1.4, precision, ctx=ctx, levels=2)
        a.set_prim(s0)
        a.solve(AMR_CFL, AMR_T, tol, 2)
        a.set_prim(s0)
        flush.fill_(1)
        r = []
        ms2 = timed(lambda: r.append(a.solve(AMR_CFL, AMR_T, tol, 2)))
        c2 = r[0][0] * n * n + a.mid_run * 4 * n * n + a.fine_run * 16 * n * n
        out = {"value": c2 / (ms2 * 1e-3), "ms_per_run": ms2, "coarse_steps": r[0][0],
               "intermediate_steps": a.mid_run, "fine_steps": a.fine_run, "cell_updates_per_run": c2}
        a.close()
        return out
    level2 = {"fp64": measure_level2(cg.FP64), "fp32": measure_level2(cg.FP32),
              "what": "EulerAMR::solve2DLevel2AMR on the same problem (coarse 512^2, intermediate 1024^2, fine "
                      "2048^2); cell-updates count every level's steps taken"}
    # e2e: pinned host primitives -> device, one driver run, both levels and flags -> host
    host = torch.empty((n, n, 5), dtype=torch.float64, pin_memory=True)
    host.numpy()[...] = s0
    hc = torch.empty((n, n, 5), dtype=torch.float64, pin_memory=True)
    hf = torch.empty((2 * n, 2 * n, 5), dtype=torch.float64, pin_memory=True)
    hcf = torch.empty((n, n), dtype=torch.uint8, pin_memory=True)
    hff = torch.empty((2 * n, 2 * n), dtype=torch.uint8, pin_memory=True)
    ae = cg.AMR(cg.NEWTONIAN, (n, n), 1.0 / n, 1.4, cg.FP64, ctx=ctx)
    res = cg._lib.AmrResult()

    def e2e_run():
        cg._lib.check(L.cosmos_amr_set_prim(ae.h, host.data_ptr(), n * n * 5))
        cg._lib.check(L.cosmos_amr_solve(ae.h, AMR_CFL, AMR_T, tol, 2, ctypes.byref(res)))
        cg._lib.check(L.cosmos_amr_get(ae.h, hc.data_ptr(), hf.data_ptr(), hcf.data_ptr(), hff.data_ptr()))
    e2e_run()
    e2e_ms = timed(e2e_run)
    ae.close()
    h2d = n * n * 5 * 8
    d2h = n * n * 5 * 8 + 4 * n * n * 5 * 8 + 5 * n * n
    peak, peak_kind = peaks()
    gbs = cells * 240 / (ms * 1e-3) / 1e9
    base = None if args.no_cpu else amr_cpu_baseline(n, AMR_T / 4)
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 1, "steps": steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": AMR_WORKLOAD, "n": n, "tolerance": tol, "coarse_steps": ncoarse, "fine_steps": nfine,
                   "cell_updates_per_run": cells, "refined_coarse_cells_at_end": int((~cf64).sum()),
                   "cell_updates": "coarse steps x coarse cells + fine steps taken x fine cells (every cell of a "
                                   "level is swept; flagged-off cells are copied)",
                   "l2": "256 MB buffer written between timed runs (the two levels' states, 105 MB, fit in L2)",
                   "host_round_trips": "one per coarse step and one per fine step (time-step control stays on "
                                       "the host, as in the reference)"},
        "fp32": {"value": cells32 / (ms32 * 1e-3), "ms_per_step": ms32, "coarse_steps": r32[0], "fine_steps": run32,
                 "l1_rho_vs_fp64": float(np.abs(cp32[..., 0] - cp64[..., 0]).sum() / np.abs(cp64[..., 0]).sum()),
                 "coarse_flags_equal_fp64": float(np.mean(cf32 == cf64))},
        "level2": level2,
        "e2e": {"value": cells / (e2e_ms * 1e-3), "unit": METRIC, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_ms, "what": "pinned host primitives -> device, one driver run, both levels' "
                                               "primitives and flags -> host"},
        "roofline": {"bound": "hbm", "kernel": "whole driver run (masked sweeps, CFL reductions, flag, exchange "
                                               "and derefinement passes)",
                     "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak, "peak_source": peak_kind,
                     "traffic": None, "bytes_per_cell_update": 240,
                     "note": "FP64 sweeps in the reference's operation order are FP64-issue-bound on GB300; the "
                             "run also waits on one host round trip per level step"},
        "clocks": clk.summary(), "gpu_launches": int(launches), "status": r64[3],
    }
    if base:
        line["cpu_baseline"] = base
    print(json.dumps(line), flush=True)


def run_amr_reference(args):
    rank, _, _ = dist_env()
    if rank != 0:
        return
    n = args.n if args.n != 4096 else AMR_N
    base = amr_cpu_baseline(n, AMR_T / 4)
    line = {"metric": METRIC, "value": base["value"], "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": base["sample_ms"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": AMR_WORKLOAD, "n": n},
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="grid", choices=["grid", "batch", "sr", "gr", "amr"],
                    help="grid: one 4096^2 Newtonian grid (default); batch: 256 uneven grids in one persistent "
                         "launch; sr: 2048^2 special-relativistic Kelvin-Helmholtz; gr: 1024^2 black-hole accretion; "
                         "amr: Level-1 AMR driver runs on a 512^2 cylindrical explosion")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=4096)
    ap.add_argument("--err-steps", type=int, default=10)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.workload == "batch":
        run_batch_reference(args) if args.impl == "reference" else run_batch(args)
    elif args.workload == "amr":
        run_amr_reference(args) if args.impl == "reference" else run_amr(args)
    elif args.workload in ("sr", "gr"):
        run_grid_reference(args, args.workload) if args.impl == "reference" else run_grid(args, args.workload)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
