"""Benchmark: 2D Newtonian SLIC (MinBee), FP32 bulk vs FP64, 4096 x 4096 cells, periodic -- and,
in the same default run, every other configuration of the solver's workload set.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--no-extras]
    python bench.py --workload {grid,sod,batch,sr,gr,adjoint,amr} ...   (one configuration per line)

One "step" is one Strang step X(dt/2) Y(dt) X(dt/2) of the whole grid with the time step computed
on the device from the previous step's CFL reduction (the reference's solve2D loop body,
Solvers/EulerSecondOrderSolver.cpp:131-146).  Metric: cell-updates per second.

The default line (our arm) carries
  value           FP32 cell-updates/s with the state resident in HBM (CUDA events on the library's
                  stream around K graph-replayed steps; the 335 MB state exceeds the 129 MB L2, so no
                  flush is needed between steps),
  e2e             the same K steps through the C ABI with one pinned host buffer: every step copies
                  the grid's primitive state (5 doubles per cell) host->device, runs the step and
                  copies the state back into the same buffer, which the next step reads (the
                  reference-facing per-step call, whose grids live on the host); split into the
                  upload, the step and the download,
  roofline        per-kernel achieved HBM GB/s of the dominant kernel (the X sweep) against the
                  measured copy bandwidth in MEASURED_PEAKS.json, with the Y sweep and the whole step,
  cpu_baseline    the CPU oracle (FP64 restatement of the reference) on the host cores, bounded sample,
  configs         the other configurations, each with its own value, the FP64 path on the same
                  steps, the FP32-vs-FP64 density error over the configuration's full step count,
                  conservation drift, an e2e over the same steps and the roofline fraction:
                  sod (1000-cell shock tube, FP64), grid_parity (this workload at 200 steps in FP32
                  and FP64), sr (2048^2 Kelvin-Helmholtz), gr (1024^2 black-hole accretion), batch
                  (256 uneven grids in one persistent launch), adjoint (Newtonian 2048^2, 100 steps,
                  checkpoint every 10, finite-difference check) and rel_adjoint (special-relativistic
                  and black-hole adjoints, bounded step counts).
--impl reference times the CPU path alone (all host threads) on the same workload, W untimed and
K timed full-size steps.
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
import traceback

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
    """nvidia-smi sampling while the GPU works."""

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


def grid_config(n, gpus):
    """The headline workload's config; both arms print exactly this dict."""
    return {"workload": WORKLOAD, "n": n, "cells_per_gpu": n * n, "precision": "fp32 bulk (reference arm: fp64)",
            "l2": "state 335 MB > 129 MB L2 (no flush needed)" if n >= 4096 else "state size n^2 x 20 B",
            "parallelism": f"replicas x{gpus}", "step": "X(dt/2) Y(dt) X(dt/2), dt from the CFL rule"}


def rel_l1(a, b):
    """Relative L1 difference of a against the reference values b."""
    return float(np.abs(a - b).sum() / np.abs(b).sum())


def newton_totals(prim, gamma):
    """Total mass and total energy (the reference's conserved density and energy, in FP64)."""
    rho, vx, vy, vz, p = (prim[..., k] for k in range(5))
    e = rho * (0.5 * (vx * vx + vy * vy + vz * vz)) + p / (gamma - 1.0)
    return float(np.sum(rho, dtype=np.float64)), float(np.sum(e, dtype=np.float64))


def sr_totals(prim, gamma):
    """Total conserved density D = rho W and energy tau = rho h W^2 - p - rho W (FP64)."""
    rho, vx, vy, vz, p = (prim[..., k] for k in range(5))
    W = 1.0 / np.sqrt(1.0 - (vx * vx + vy * vy + vz * vz))
    h = 1.0 + p / rho * gamma / (gamma - 1.0)
    return float(np.sum(rho * W)), float(np.sum(rho * h * W * W - p - rho * W))


def drift(t0, t1):
    return {"mass": abs(t1[0] - t0[0]) / abs(t0[0]), "energy": abs(t1[1] - t0[1]) / abs(t0[1])}


class Clock:
    """CUDA-event timing on one stream (the library context's)."""

    def __init__(self, stream):
        self.stream = stream

    def __call__(self, fn):
        import torch
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(self.stream):
            a.record(self.stream)
            fn()
            b.record(self.stream)
        b.synchronize()
        return a.elapsed_time(b)

    def event(self):
        import torch
        e = torch.cuda.Event(enable_timing=True)
        e.record(self.stream)
        return e


def e2e_chain(cg, L, g, clock, nsteps, host):
    """nsteps steps through the C ABI, each: the pinned host buffer `host` (primitives) -> device,
    one step of the run begun on g, the state -> the same buffer (which the next step reads).
    Returns (total ms, upload ms, step ms, download ms) summed over the steps."""
    import torch
    n = host.numel()
    ev = []
    with torch.cuda.stream(clock.stream):
        for _ in range(nsteps):
            e0 = clock.event()
            cg._lib.check(L.cosmos_grid_set_prim(g.h, host.data_ptr(), n))
            e1 = clock.event()
            g.run_steps(1)
            e2 = clock.event()
            cg._lib.check(L.cosmos_grid_get_prim(g.h, host.data_ptr(), n))
            e3 = clock.event()
            ev.append((e0, e1, e2, e3))
    ev[-1][3].synchronize()
    up = sum(a.elapsed_time(b) for a, b, _, _ in ev)
    st = sum(b.elapsed_time(c) for _, b, c, _ in ev)
    dn = sum(c.elapsed_time(d) for _, _, c, d in ev)
    return ev[0][0].elapsed_time(ev[-1][3]), up, st, dn


def guarded(fn):
    """Runs one configuration's measurement; an exception becomes an error entry of the line."""
    try:
        return fn()
    except Exception as e:  # the headline line still prints
        return {"error": f"{type(e).__name__}: {e}", "trace": traceback.format_exc(limit=3)[-600:]}


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
    """The CPU arm: the oracle (bit-identical restatement of the reference) on all host threads, W
    untimed and K timed full-size Strang steps of the headline workload."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle.pyoracle import Oracle
    O = Oracle()
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    n = args.n
    s = four_quadrant(n, 2)
    s, _, _, _ = O.solve(0, s, 2, 1.0 / n, 0.9, 1e9, 0.0, 2, 1.4, 1, max_steps=args.warmup)
    t0 = time.perf_counter()
    s, k, _, _ = O.solve(0, s, 2, 1.0 / n, 0.9, 1e9, 0.0, 2, 1.4, 1, max_steps=args.steps)
    el = time.perf_counter() - t0
    value = k * n * n / el
    base = {"value": value, "unit": METRIC, "cores": cores, "kind": "port",
            "sample": f"{args.warmup} untimed and {k} timed full {n}x{n} Strang steps of the FP64 oracle "
                      f"(restatement of the reference, bit-identical to it) in {el:.1f} s on {cores} host threads"}
    line = {"metric": METRIC, "value": value, "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / k * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": grid_config(n, args.gpus), "cpu_baseline": base,
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- the headline workload
def run_ours(args):
    import torch
    import cosmos_gb300 as cg
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    ranks = Ranks("nccl", "cuda")
    L = cg.load()
    ctx = cg.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    clock = Clock(stream)
    n = args.n
    s0 = four_quadrant(n, 2)
    cells = n * n

    # ---------------- FP32 resident: value
    g = cg.Grid(cg.NEWTONIAN, (n, n), 1.0 / n, 1.4, cg.FP32, cg.BC_PERIODIC, ctx=ctx)
    g.set_prim(s0)
    g.run_begin(2, 0.9, 1e30, 0.0, cg.MINBEE)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:  # sampled over the warm-up and the timed steps
        g.run_steps(args.warmup)
        ctx.synchronize()
        launches0 = L.cosmos_kernel_launches()
        ranks.barrier()
        with torch.cuda.stream(stream):
            e0.record(stream)
            g.run_steps(args.steps)
            e1.record(stream)
        e1.synchronize()
        ranks.barrier()
    launches = L.cosmos_kernel_launches() - launches0
    ms = ranks.max(e0.elapsed_time(e1)) / args.steps
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
                a = clock.event()
                g.sweep(ax, 2, dt_probe, 0.0, cg.MINBEE)
                kern[key].append((a, clock.event()))
    torch.cuda.synchronize()
    g.close()
    kx = statistics.mean(a.elapsed_time(b) for a, b in kern["x"])
    ky = statistics.mean(a.elapsed_time(b) for a, b in kern["y"])
    peak, peak_kind = peaks()
    bytes_sweep = cells * 40  # 5 FP32 fields read + 5 written per cell (halo re-reads not counted)
    x_gbs = bytes_sweep / (kx * 1e-3) / 1e9
    y_gbs = bytes_sweep / (ky * 1e-3) / 1e9
    step_gbs = cells * 120 / (ms * 1e-3) / 1e9

    # ---------------- e2e: K steps chained through one pinned host buffer
    host = torch.empty((n, n, 5), dtype=torch.float64, pin_memory=True)
    host.numpy()[...] = s0
    ge = cg.Grid(cg.NEWTONIAN, (n, n), 1.0 / n, 1.4, cg.FP32, cg.BC_PERIODIC, ctx=ctx)
    ge.set_prim(s0)
    ge.run_begin(2, 0.9, 1e30, 0.0, cg.MINBEE)
    e2e_chain(cg, L, ge, clock, 2, host)  # warm-up (staging, conversion kernels)
    host.numpy()[...] = s0
    ranks.barrier()
    tot, up, st, dn = e2e_chain(cg, L, ge, clock, args.steps, host)
    ge.close()
    e2e_ms = ranks.max(tot) / args.steps
    nbytes = cells * 5 * 8

    if rank != 0:
        return
    base = cpu_baseline(n, seconds=args.cpu_seconds) if not args.no_cpu else None
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": grid_config(n, args.gpus),
        "run": {"device_dt": True, "graph_replay": True, "steps_completed": r.steps, "status": r.status},
        "e2e": {"value": ranks.throughput(cells, e2e_ms), "unit": METRIC, "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes, "ms_per_step": e2e_ms, "steps": args.steps,
                "h2d_ms": up / args.steps, "compute_ms": st / args.steps, "d2h_ms": dn / args.steps,
                "h2d_gbs": nbytes / (up / args.steps * 1e-3) / 1e9, "d2h_gbs": nbytes / (dn / args.steps * 1e-3) / 1e9,
                "what": "per step: pinned host AoS FP64 primitives -> device (copy + conversion to FP32 conserved), "
                        "one Strang step, state -> the same host buffer, which the next step reads"},
        "roofline": {"bound": "hbm", "kernel": "sweep_x_ring_kernel (X sweep, FP32 cell pairs staged by bulk copies)",
                     "achieved": x_gbs, "peak": peak, "unit": "GB/s", "frac": x_gbs / peak,
                     "peak_source": peak_kind, "traffic": traffic_per_launch("sweep_x_fp32"),
                     "algorithmic_bytes_per_launch": bytes_sweep, "ms_per_launch": kx,
                     "y_sweep": {"achieved": y_gbs, "frac": y_gbs / peak, "ms_per_launch": ky},
                     "step": {"achieved": step_gbs, "frac": step_gbs / peak, "bytes_per_cell_update": 120}},
        "clocks": clk.summary(),
        "gpu_launches": int(launches),
    }
    if base:
        line["cpu_baseline"] = base
    if not args.no_extras:
        with Clocks(local) as clk2:
            line["configs"] = all_configs(cg, L, ctx, stream, args)
        line["clocks_configs"] = clk2.summary()
    print(json.dumps(line), flush=True)


def all_configs(cg, L, ctx, stream, args):
    """Every other configuration, measured in this process after the headline (state resident in
    HBM unless an e2e says otherwise); an exception in one becomes that entry's error."""
    out = {}
    steps = [("sod", lambda: measure_sod(cg, ctx, stream)),
             ("grid_parity", lambda: measure_grid_parity(cg, ctx, stream, args.n, args.parity_steps)),
             ("sr", lambda: measure_sr(cg, L, ctx, stream, 2048, args.sr_steps, args.warmup)),
             ("gr", lambda: measure_gr(cg, L, ctx, stream, 1024, args.gr_steps, args.warmup)),
             ("batch", lambda: measure_batch(cg, L, ctx, stream, max(args.steps, 20), args.warmup)),
             ("adjoint", lambda: adjoint_measure(cg, ctx)),
             ("rel_adjoint", lambda: measure_rel_adjoint(cg, ctx))]
    for name, fn in steps:
        t0 = time.perf_counter()
        out[name] = guarded(fn)
        out[name]["wall_s"] = time.perf_counter() - t0
    return out


# ---------------------------------------------------------------- Sod shock tube, 1000 cells, FP64
SOD_WORKLOAD = "1D Newtonian Euler Sod shock tube, SLIC van Leer, FP64, 1000 cells on [0,1], gamma 1.4, CFL 0.9, " \
               "transmissive, t = 0.25"
# The reference's own run of this problem (built from its sources): 613 steps, rho[500] at t = 0.25.
SOD_STEPS, SOD_RHO500 = 613, 0.42639270172959448


def measure_sod(cg, ctx, stream):
    import cases
    import torch
    clock = Clock(torch.cuda.ExternalStream(ctx.stream))
    s = cases.sod(1000)
    g = cg.Grid(cg.NEWTONIAN, (1000,), 1.0 / 1000, 1.4, cg.FP64, ctx=ctx)
    res = []
    for _ in range(2):  # the first solve captures the step graph
        g.set_prim(s)
        ms = clock(lambda: res.append(g.solve(2, 0.9, 0.25, 0.0, cg.VANLEER)))
    r = res[-1]
    rho = g.get_prim()[..., 0]
    g.close()
    return {"workload": SOD_WORKLOAD, "dtype": "f64", "value": r.steps * 1000 / (ms * 1e-3), "unit": METRIC,
            "ms_per_run": ms, "steps": r.steps, "t": r.t, "rho500": float(rho[500]),
            "matches_reference_run": bool(r.steps == SOD_STEPS and float(rho[500]) == SOD_RHO500),
            "note": "1000 cells: launch-bound (one host round trip per solve, 613 graph-replayed steps)"}


# ---------------------------------------------------------------- the 4096^2 grid at full length
def measure_grid_parity(cg, ctx, stream, n, steps):
    """The headline workload run `steps` steps in FP32 and in the FP64 (reference-exact) path, each
    with its own CFL time steps: the FP64 path's rate, the FP32-vs-FP64 relative L1 density error,
    and both runs' mass and energy drift (periodic boundaries conserve both exactly)."""
    clock = Clock(stream)
    s0 = four_quadrant(n, 2)
    tot0 = newton_totals(s0, 1.4)
    out = {"workload": WORKLOAD, "steps": steps}
    prims = {}
    for prec, tag in ((cg.FP32, "fp32"), (cg.FP64, "fp64")):
        g = cg.Grid(cg.NEWTONIAN, (n, n), 1.0 / n, 1.4, prec, cg.BC_PERIODIC, ctx=ctx)
        g.set_prim(s0)
        g.run_begin(2, 0.9, 1e30, 0.0, cg.MINBEE, max_steps=steps)
        ms = clock(lambda: g.run_steps(steps)) / steps
        r = g.run_end()
        p = g.get_prim()
        sums = g.field_sums() if prec == cg.FP32 else None
        g.close()
        prims[tag] = p
        out[tag] = {"value": n * n / (ms * 1e-3), "ms_per_step": ms, "t": r.t, "steps_completed": r.steps,
                    "status": r.status, "drift": drift(tot0, newton_totals(p, 1.4))}
        if sums is not None:  # the stored FP32 conserved totals, compensated on the device
            out[tag]["drift_stored"] = {"mass": abs(sums[0] - tot0[0]) / tot0[0],
                                        "energy": abs(sums[4] - tot0[1]) / tot0[1]}
    out["l1_rho_fp32_vs_fp64"] = rel_l1(prims["fp32"][..., 0], prims["fp64"][..., 0])
    out["l1_bound"] = 1e-5
    out["fp32_over_fp64"] = out["fp64"]["ms_per_step"] / out["fp32"]["ms_per_step"]
    return out


# ---------------------------------------------------------------- SR Kelvin-Helmholtz, 2048^2
SR_WORKLOAD = "2D special-relativistic Euler (gamma 5/3), SLIC MinBee, CFL 0.9, 2048x2048 on the periodic " \
              "unit square, Kelvin-Helmholtz shear layers (vx = +-0.5 tanh profile, rho in {1, 2}, p = 1, " \
              "vy = 0.01 sin(4 pi x + phase), phase seed 3; Lorentz factor <= 1.16); 200 steps"


def measure_sr(cg, L, ctx, stream, n, steps, warmup):
    """The SR Kelvin-Helmholtz workload as stated (FP32 bulk, every primitive recovery's Newton iterations finished
    in FP64), the FP32-Newton variant (FP64 stage only above a Lorentz factor of 2), and the FP64
    reference-exact path, all over the same `steps` steps from the same data."""
    import cases
    import torch
    clock = Clock(stream)
    s0 = cases.kelvin_helmholtz(n, 3)
    gam = 5.0 / 3.0
    tot0 = sr_totals(s0, gam)
    peak, peak_kind = peaks()

    def make(prec, above):
        g = cg.Grid(cg.SR, (n, n), 1.0 / n, gam, prec, cg.BC_PERIODIC, ctx=ctx, sr_c2p64_above=above)
        g.set_prim(s0)
        return g

    out = {"workload": SR_WORKLOAD, "steps": steps}
    prims = {}
    for tag, prec, above in (("fp32_c2p_fp64", cg.FP32, 0.0), ("fp32_newton_variant", cg.FP32, 2.0),
                             ("fp64", cg.FP64, 2.0)):
        g = make(prec, above)
        if prec == cg.FP32:  # warm-up run (graph capture), then the timed run from the same data
            g.run_begin(2, 0.9, 1e30, 0.0, cg.MINBEE, max_steps=warmup)
            g.run_steps(warmup)
            g.run_end()
            g.set_prim(s0)
        g.run_begin(2, 0.9, 1e30, 0.0, cg.MINBEE, max_steps=steps)
        ms = clock(lambda: g.run_steps(steps)) / steps
        r = g.run_end()
        prims[tag] = g.get_prim()
        g.close()
        bpc = 120 if prec == cg.FP32 else 240
        out[tag] = {"value": n * n / (ms * 1e-3), "ms_per_step": ms, "t": r.t, "steps_completed": r.steps,
                    "status": r.status, "drift": drift(tot0, sr_totals(prims[tag], gam)),
                    "roofline_frac": n * n * bpc / (ms * 1e-3) / 1e9 / peak}
    for tag in ("fp32_c2p_fp64", "fp32_newton_variant"):
        out[tag]["l1_rho_vs_fp64"] = rel_l1(prims[tag][..., 0], prims["fp64"][..., 0])
    out["fp32_c2p_fp64"]["what"] = "as stated: FP32 bulk, FP64 Newton iterations in every primitive recovery"
    out["fp32_newton_variant"]["what"] = "variant: FP32 Newton iterations, FP64 only above Lorentz factor 2 " \
                                         "(not reached here) or on FP32 non-convergence"
    out["value"] = out["fp32_c2p_fp64"]["value"]
    # e2e of the as-stated path over the same steps, chained through one pinned host buffer
    host = torch.empty((n, n, 5), dtype=torch.float64, pin_memory=True)
    host.numpy()[...] = s0
    ge = make(cg.FP32, 0.0)
    ge.run_begin(2, 0.9, 1e30, 0.0, cg.MINBEE, max_steps=steps)
    tot, up, st, dn = e2e_chain(cg, L, ge, clock, steps, host)
    ge.close()
    nb = n * n * 40
    out["e2e"] = {"value": n * n * steps / (tot * 1e-3), "ms_per_step": tot / steps, "steps": steps,
                  "h2d_bytes_per_step": nb, "d2h_bytes_per_step": nb, "h2d_ms": up / steps,
                  "compute_ms": st / steps, "d2h_ms": dn / steps}
    out["roofline_note"] = "compute-bound: five primitive recoveries per cell per sweep"
    return out


# ---------------------------------------------------------------- black-hole accretion, 1024^2
GR_WORKLOAD = "2D black-hole Euler in Kerr-Schild Schwarzschild spacetime (M = 1), SLIC van Leer + " \
              "RK4 source (BlackHoleEulerForcingSolver, one subcycle), CFL 0.9, 1024x1024 on [-10, 10]^2 " \
              "(dx = 20/1024, hole at (10, 10) of the grid's coordinates), excision r <= 2M, rho = 1 with 1% " \
              "log-normal noise (seed 4), p = 0.01, transmissive; 100 steps"
GR_HOLE = (1.0, 0.0, 10.0, 10.0, 0.0)


def gr_state(n, seed=4):
    rng = np.random.default_rng(seed)
    s = np.zeros((n, n, 5))
    s[..., 0] = np.exp(0.01 * rng.standard_normal((n, n)))
    s[..., 4] = 0.01
    return s


def gr_step_fixed(g, dt, nsub=1, lim=1):
    """One solver step with a given dt, as the library's run enqueues it: the RK source half-steps,
    X(dt/2) Y(dt) X(dt/2), the RK source half-steps (Solvers/BlackHoleEulerSecondOrderSolver.cpp:181-218)."""
    for _ in range(nsub):
        g.rk_source(0.5 * (dt / nsub), 0.0, 1)
    g.sweep(0, 2, 0.5 * dt, 0.0, lim)
    g.sweep(1, 2, dt, 0.0, lim)
    g.sweep(0, 2, 0.5 * dt, 0.0, lim)
    for _ in range(nsub):
        g.rk_source(0.5 * (dt / nsub), 0.0, 1)


def measure_gr(cg, L, ctx, stream, n, steps, warmup, r_cut=5.0):
    """Black-hole accretion: the FP32 bulk path's own run (CFL time steps), the FP64 reference-exact path
    over the same number of steps driven by its own CFL rule, and the FP32 path driven by the FP64
    run's time-step sequence, so that the density error over r > r_cut M compares the solutions at
    equal times (the free-running runs' time steps part where the horizon cells' speeds differ)."""
    import torch
    clock = Clock(stream)
    s0 = gr_state(n)
    dx = 20.0 / n
    bh = cg.BlackHoleSpacetime(*GR_HOLE)
    x = np.arange(n) * dx
    X, Y = np.meshgrid(x, x)
    rr = np.sqrt((X - GR_HOLE[2]) ** 2 + (Y - GR_HOLE[3]) ** 2)
    far = rr > r_cut * GR_HOLE[0]
    peak, peak_kind = peaks()

    def make(prec, above=2.0):
        g = cg.Grid(cg.GR, (n, n), dx, 5.0 / 3.0, prec, cg.BC_TRANSMISSIVE, bh, ctx=ctx, sr_c2p64_above=above)
        g.set_prim(s0)
        return g

    out = {"workload": GR_WORKLOAD, "steps": steps}
    # FP32 free-running (own CFL steps): the configuration's value
    g = make(cg.FP32)
    g.run_begin(2, 0.9, 1e30, 0.0, cg.VANLEER, max_steps=warmup)
    g.run_steps(warmup)
    g.run_end()
    g.set_prim(s0)
    g.run_begin(2, 0.9, 1e30, 0.0, cg.VANLEER, max_steps=steps)
    ms = clock(lambda: g.run_steps(steps)) / steps
    r = g.run_end()
    g.close()
    out["fp32"] = {"value": n * n / (ms * 1e-3), "ms_per_step": ms, "t": r.t, "steps_completed": r.steps,
                   "status": r.status, "roofline_frac": n * n * 200 / (ms * 1e-3) / 1e9 / peak,
                   "what": "FP32 bulk; metric from FP64 tables; primitive recovery finished in FP64 above W = 2 "
                           "or on FP32 non-convergence"}
    out["value"] = out["fp32"]["value"]
    # the same free run with every primitive recovery's Newton iterations finished in FP64 (the
    # workload's "FP64 con2prim"); the metric is FP64-evaluated in both
    g = make(cg.FP32, 0.0)
    g.run_begin(2, 0.9, 1e30, 0.0, cg.VANLEER, max_steps=steps)
    ms_c = clock(lambda: g.run_steps(steps)) / steps
    r = g.run_end()
    g.close()
    out["fp32_c2p_fp64"] = {"value": n * n / (ms_c * 1e-3), "ms_per_step": ms_c, "t": r.t,
                            "steps_completed": r.steps, "status": r.status,
                            "what": "FP32 bulk; metric from FP64 tables; every primitive recovery's Newton "
                                    "iterations finished in FP64"}
    # FP64 driven by its own CFL rule, and FP32 (as configured, and with the FP64 Newton stage in
    # every primitive recovery) driven by the FP64 run's dts; density errors at checkpoints.  The
    # FP64 run stops where the reference's own arithmetic produces a non-finite state next to the
    # horizon (the reference carries the NaN on; this library reports it).
    g64, g32, g32c = make(cg.FP64), make(cg.FP32), make(cg.FP32, 0.0)
    t, ms64, dts, checks, stop = 0.0, 0.0, [], {}, None
    for it in range(steps):
        try:
            dt = g64.stable_dt(0.9, t, 1e30, it)
            ms64 += clock(lambda: gr_step_fixed(g64, dt))
        except cg.CosmosError as e:
            stop = {"step": it, "t": t, "error": str(e)}
            break
        gr_step_fixed(g32, dt)
        gr_step_fixed(g32c, dt)
        dts.append(dt)
        t += dt
        if (it + 1) in (5, 10, 20, 50, steps) or (it + 1) % 10 == 0:
            p64 = g64.get_prim()
            if not np.isfinite(p64[..., 0][far]).all():
                stop = {"step": it + 1, "t": t, "error": "non-finite FP64 density over r > 5M"}
                break
            checks[it + 1] = {"t": t, "l1": rel_l1(g32.get_prim()[..., 0][far], p64[..., 0][far]),
                              "l1_c2p_fp64": rel_l1(g32c.get_prim()[..., 0][far], p64[..., 0][far])}
    for g in (g64, g32, g32c):
        g.close()
    done = len(dts)
    out["fp64"] = {"value": n * n * done / (ms64 * 1e-3) if done else None, "ms_per_step": ms64 / max(done, 1),
                   "steps": done, "t": t,
                   "path": "plain FP64, bit-identical to the reference; its CFL time steps (host-driven loop)"}
    if stop:
        out["fp64"]["stopped"] = stop
    out["l1_rho_fp32_vs_fp64_same_dts"] = checks
    last = max(checks) if checks else None
    out["l1_last_common_step"] = last
    out["l1_cells"] = f"r > {r_cut} M ({int(far.sum())} cells)"
    out["dt_first_last"] = [dts[0], dts[-1]] if dts else None
    out["l1_note"] = "FP32 and FP64 on the same time steps (the FP64 run's CFL rule); l1_c2p_fp64: the FP32 run " \
                     "with the FP64 Newton stage in every primitive recovery"
    # e2e of the FP32 path over the same steps
    host = torch.empty((n, n, 5), dtype=torch.float64, pin_memory=True)
    host.numpy()[...] = s0
    ge = make(cg.FP32)
    ge.run_begin(2, 0.9, 1e30, 0.0, cg.VANLEER, max_steps=steps)
    tot, up, st, dn = e2e_chain(cg, L, ge, clock, steps, host)
    ge.close()
    nb = n * n * 40
    out["e2e"] = {"value": n * n * steps / (tot * 1e-3), "ms_per_step": tot / steps, "steps": steps,
                  "h2d_bytes_per_step": nb, "d2h_bytes_per_step": nb, "h2d_ms": up / steps,
                  "compute_ms": st / steps, "d2h_ms": dn / steps}
    out["fp32_over_fp64"] = out["fp64"]["ms_per_step"] / ms if done else None
    return out


# ---------------------------------------------------------------- 256 batched uneven grids
BATCH_WORKLOAD = "256 independent Newtonian Euler grids (1D and 2D), every side log-uniform in " \
                 "[128, 2048] cells (seed 5), seeded Riemann data, SLIC MinBee, CFL 0.9, transmissive, dx = 1/nx"


def batch_problem():
    import cases
    shapes = cases.batch_shapes()
    states = [cases.riemann(sh, 1000 + k) for k, sh in enumerate(shapes)]
    dxs = [1.0 / sh[-1] for sh in shapes]
    return shapes, states, dxs


def measure_batch(cg, L, ctx, stream, steps, warmup, l1_steps=20, tiles=False):
    """The 256-grid batch: the FP32 batch in one persistent graph-replayed launch (tile shape from the
    autotuner), the same grids stepped one by one, the FP64 batch and the FP32-vs-FP64 density
    error over `l1_steps` steps, and an e2e over the value's steps."""
    import torch
    clock = Clock(stream)
    shapes, states, dxs = batch_problem()
    cells = sum(int(np.prod(sh)) for sh in shapes)
    bytes_step = sum(int(np.prod(sh)) * (120 if len(sh) == 2 else 40) for sh in shapes)
    peak, peak_kind = peaks()
    ratio = traffic_per_launch("batch_step_fp32_ratio")
    b = cg.Batch(shapes, dxs, 1.4, cg.FP32, cg.BC_TRANSMISSIVE, ctx=ctx)
    for k, s in enumerate(states):
        b.set_prim(k, s)
    b.run_begin(0.9, 1e30, 0.0, cg.MINBEE)
    shapes_tried = [(nt, seg, cap) for nt in (128, 256) for seg in (32, 64) for cap in (0, 1)]
    shapes_tried += [(128, 128, 1), (256, 128, 1)]
    tile_ms = {f"{nt}x{seg}{'c' if cap else ''}": b.time_shape(nt, seg, cap, steps=5)
               for nt, seg, cap in shapes_tried} if tiles else None
    tuned, _ = b.autotune(None)
    b.run_steps(warmup)
    launches0 = L.cosmos_kernel_launches()
    ms = clock(lambda: b.run_steps(steps)) / steps
    launches = L.cosmos_kernel_launches() - launches0
    res = b.run_end()
    b.close()
    out = {"workload": BATCH_WORKLOAD, "grids": len(shapes), "grids_2d": sum(len(s) == 2 for s in shapes),
           "cells": cells, "tile_shape": list(tuned), "steps": steps,
           "value": cells / (ms * 1e-3), "ms_per_step": ms, "gpu_launches": int(launches),
           "roofline": {"bound": "hbm", "kernel": "batch_pair_kernel (whole step)",
                        "achieved": bytes_step / (ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                        "frac": bytes_step / (ms * 1e-3) / 1e9 / peak,
                        "bytes_per_cell_update": "40 (1D), 120 (2D)", "algorithmic_bytes_per_step": bytes_step,
                        "traffic": (ratio * bytes_step) if ratio else None,
                        "traffic_note": "per step: the algorithmic bytes times the DRAM-traffic ratio of an ncu "
                                        "capture of the first 64 grids (every grid is swept the same way)"},
           "status": [x.status for x in res if x.status][:8]}
    if tile_ms:
        out["tile_ms_per_step"] = tile_ms
    # the same grids advanced one by one (each its own graph-replayed steps)
    ku = 5
    singles = []
    for k, sh in enumerate(shapes):
        g = cg.Grid(cg.NEWTONIAN, sh, dxs[k], 1.4, cg.FP32, cg.BC_TRANSMISSIVE, ctx=ctx)
        g.set_prim(states[k])
        g.run_begin(2, 0.9, 1e30, 0.0, cg.MINBEE)
        g.run_steps(3)
        singles.append(g)
    ms_u = clock(lambda: [g.run_steps(ku) for g in singles]) / ku
    for g in singles:
        g.close()
    out["unbatched"] = {"value": cells / (ms_u * 1e-3), "ms_per_step": ms_u}
    # FP64 batch (bit-identical to the reference per grid) and the FP32-vs-FP64 density error
    b64 = cg.Batch(shapes, dxs, 1.4, cg.FP64, cg.BC_TRANSMISSIVE, ctx=ctx)
    b32 = cg.Batch(shapes, dxs, 1.4, cg.FP32, cg.BC_TRANSMISSIVE, ctx=ctx)
    for k, s in enumerate(states):
        b64.set_prim(k, s)
        b32.set_prim(k, s)
    b64.run_begin(0.9, 1e30, 0.0, cg.MINBEE, max_steps=l1_steps)
    b64.autotune(None)
    ms64 = clock(lambda: b64.run_steps(l1_steps)) / l1_steps
    b64.run_end()
    b32.run_begin(0.9, 1e30, 0.0, cg.MINBEE, max_steps=l1_steps)
    b32.set_shape(*tuned)
    b32.run_steps(l1_steps)
    b32.run_end()
    num = den = 0.0
    m32 = m64 = 0.0
    for k in range(len(shapes)):
        r64 = b64.get_prim(k)[..., 0]
        r32 = b32.get_prim(k)[..., 0]
        num += float(np.abs(r32 - r64).sum())
        den += float(np.abs(r64).sum())
        m32 += float(r32.sum())
        m64 += float(r64.sum())
    b64.close()
    b32.close()
    out["fp64"] = {"value": cells / (ms64 * 1e-3), "ms_per_step": ms64, "steps": l1_steps,
                   "path": "FP64 batch, bit-identical to the reference per grid"}
    out["l1_rho_fp32_vs_fp64"] = num / den
    out["l1_steps"] = l1_steps
    out["density_total_diff"] = abs(m32 - m64) / m64
    out["drift_note"] = "transmissive boundaries exchange mass; the FP32-vs-FP64 difference of the density total"
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
    e2e_steps = min(steps, 10)
    e2e_ms = clock(lambda: [e2e_step() for _ in range(e2e_steps)]) / e2e_steps
    be.close()
    nbytes = cells * 5 * 8
    out["e2e"] = {"value": cells / (e2e_ms * 1e-3), "unit": METRIC, "h2d_bytes_per_step": nbytes,
                  "d2h_bytes_per_step": nbytes, "ms_per_step": e2e_ms, "steps": e2e_steps,
                  "what": "per step: each grid's pinned host AoS FP64 primitives -> device, one batched step, "
                          "states -> host (256 calls each way)"}
    return out


# ---------------------------------------------------------------- adjoints
def adjoint_measure(cg, ctx, n=2048, nsteps=100, every=10):
    """Adjoint of `nsteps` SLIC steps (checkpoint every `every`) of the loss 1/2 |rho_T - target|^2 on
    the batch's largest grid size (n x n, FP32, seeded Riemann data, seeded target), timed against
    its forward pass; plus a central finite-difference check of the FP64 gradient at 64 x 64."""
    import cases
    p0 = cases.riemann((n, n), 77)
    rng = np.random.default_rng(78)
    target = p0[..., 0] * (1.0 + 0.05 * rng.standard_normal((n, n)))
    g = cg.Grid(cg.NEWTONIAN, (n, n), 1.0 / n, 1.4, cg.FP32, cg.BC_TRANSMISSIVE, ctx=ctx)
    runs = {}
    for keep in (-1, 0):  # sweep inputs kept from the forward pass (default), or every earlier segment recomputed
        g.set_adjoint_keep(keep)
        runs[keep] = []
        for _ in range(3):
            g.set_prim(p0)
            runs[keep].append(g.adjoint(target, nsteps, 0.9, 0.0, cg.MINBEE, checkpoint_every=every)[3])
    g.close()
    fwd = statistics.median(r[0] for r in runs[-1])
    bwd = statistics.median(r[1] for r in runs[-1])
    fwd0 = statistics.median(r[0] for r in runs[0])
    bwd0 = statistics.median(r[1] for r in runs[0])
    seg_gb = every * 3 * n * n * 5 * 4 / 1e9
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
            "forward_ms": fwd, "backward_ms": bwd, "adjoint_over_forward": bwd / fwd, "target": 3.0,
            "what": f"backward = the sweep adjoints, every segment's sweep inputs kept from the forward pass "
                    f"({nsteps // every} x {seg_gb:.1f} GB in HBM, the default keep budget of half the free "
                    f"memory), per forward pass of the same steps",
            "recompute": {"forward_ms": fwd0, "backward_ms": bwd0, "adjoint_over_forward": bwd0 / fwd0,
                          "what": "keep budget 0: the last segment kept, every earlier one recomputed from its "
                                  "checkpoint on a second stream while the following segment's adjoints run"},
            "fd_check": {"grid": f"{m}x{m} FP64 smooth data", "steps": nsteps, "h": h,
                         "rule": "h = 1e-6, 1e-7, ... until two successive central differences agree to 1e-5",
                         "fd_by_h": {f"{x:.0e}": v for x, v in zip(hs, fds)},
                         "directional_adjoint": an, "directional_fd": fd, "rel_err": abs(fd - an) / abs(an),
                         "bound": 1e-4}}


def measure_rel_adjoint(cg, ctx, sr_n=2048, sr_steps=2, gr_n=1024, gr_steps=1):
    """Adjoint-to-forward cost of the special-relativistic (Kelvin-Helmholtz, FP64) and black-hole
    (accretion, FP64, one RK source half-step on each side of the flux step) adjoints at their
    configurations' sizes, over a bounded number of steps (checkpoint every step)."""
    import cases
    out = {}
    s = cases.kelvin_helmholtz(sr_n, 3)
    g = cg.Grid(cg.SR, (sr_n, sr_n), 1.0 / sr_n, 5.0 / 3.0, cg.FP64, cg.BC_PERIODIC, ctx=ctx)
    g.set_prim(s)
    _, grad, _, ms = g.adjoint(s[..., 0] * 0.99, sr_steps, 0.9, 0.0, cg.MINBEE, checkpoint_every=1)
    g.close()
    out["sr"] = {"grid": f"{sr_n}x{sr_n} FP64 Kelvin-Helmholtz", "steps": sr_steps, "forward_ms": ms[0],
                 "backward_ms": ms[1], "adjoint_over_forward": ms[1] / ms[0], "finite": bool(np.isfinite(grad).all())}
    a = gr_state(gr_n)
    g = cg.Grid(cg.GR, (gr_n, gr_n), 20.0 / gr_n, 5.0 / 3.0, cg.FP64, cg.BC_TRANSMISSIVE,
                cg.BlackHoleSpacetime(*GR_HOLE), ctx=ctx)
    g.set_prim(a)
    _, grad, _, ms = g.adjoint(a[..., 0] * 0.99, gr_steps, 0.9, 0.0, cg.VANLEER, checkpoint_every=1, subcycles=1)
    g.close()
    out["gr"] = {"grid": f"{gr_n}x{gr_n} FP64 accretion, 1 subcycle", "steps": gr_steps, "forward_ms": ms[0],
                 "backward_ms": ms[1], "adjoint_over_forward": ms[1] / ms[0], "finite": bool(np.isfinite(grad).all())}
    out["what"] = ("gather-form vector-Jacobian products in dual numbers (FP64); every step's sweep inputs kept "
                   "from the forward pass (the default keep budget)")
    return out


# ---------------------------------------------------------------- single-configuration lines
def config_line(args, workload, entry, dtype="f32", extra_config=None):
    """A contract line for one configuration measured by the functions above."""
    v = entry["value"]
    ms = entry.get("ms_per_step") or entry.get("fp32", entry.get("fp32_c2p_fp64", {})).get("ms_per_step")
    e = entry.get("e2e", {})
    line = {"metric": METRIC, "value": v, "unit": METRIC, "n_gpus": 1, "steps": entry.get("steps", args.steps),
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": dtype, "data": "synthetic",
            "config": dict({"workload": workload}, **(extra_config or {})), "result": entry}
    if e:
        line["e2e"] = dict({"unit": METRIC}, **e)
    return line


def run_single(args):
    import torch
    import cosmos_gb300 as cg
    _, _, local = dist_env()
    torch.cuda.set_device(local)
    L = cg.load()
    ctx = cg.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    w = args.workload
    with Clocks(local) as clk:
        if w == "sod":
            e, wl, dt = measure_sod(cg, ctx, stream), SOD_WORKLOAD, "f64"
        elif w == "sr":
            e, wl, dt = measure_sr(cg, L, ctx, stream, args.n if args.n != 4096 else 2048, args.sr_steps,
                                   args.warmup), SR_WORKLOAD, "f32"
        elif w == "gr":
            e, wl, dt = measure_gr(cg, L, ctx, stream, args.n if args.n != 4096 else 1024, args.gr_steps,
                                   args.warmup), GR_WORKLOAD, "f32"
        elif w == "batch":
            e, wl, dt = measure_batch(cg, L, ctx, stream, args.steps, args.warmup, tiles=True), BATCH_WORKLOAD, "f32"
        elif w == "adjoint":
            e = adjoint_measure(cg, ctx)
            e["value"] = 2048 * 2048 * e["steps"] / ((e["forward_ms"] + e["backward_ms"]) * 1e-3)
            e["rel"] = measure_rel_adjoint(cg, ctx)
            wl, dt = "adjoint of 100 SLIC steps (checkpoint every 10), Newtonian 2048^2 FP32", "f32"
        else:
            raise ValueError(w)
    line = config_line(args, wl, e, dt)
    line["clocks"] = clk.summary()
    print(json.dumps(line), flush=True)


def run_single_reference(args):
    """CPU arm of a single-configuration line: the oracle on the configuration's full-size data."""
    rank, _, _ = dist_env()
    if rank != 0:
        return
    from oracle.pyoracle import Oracle
    import cases
    O = Oracle()
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    w = args.workload
    if w in ("sr", "gr"):
        n = args.n if args.n != 4096 else (2048 if w == "sr" else 1024)
        if w == "sr":
            sysid, s, dx, gam, bc, lim, bh, wl = 1, cases.kelvin_helmholtz(n, 3), 1.0 / n, 5 / 3, 1, 2, None, SR_WORKLOAD
        else:
            sysid, s, dx, gam, bc, lim, bh, wl = 2, gr_state(n), 20.0 / n, 5 / 3, 0, 1, GR_HOLE, GR_WORKLOAD
        t0 = time.perf_counter()
        steps = 0
        while True:
            s, k, _, _ = O.solve(sysid, s, 2, dx, 0.9, 1e9, 0.0, lim, gam, bc, subcycles=1, bh=bh, max_steps=1)
            steps += k
            el = time.perf_counter() - t0
            if el >= max(8.0, 2.0 * args.steps) or steps >= max(1, args.steps):
                break
        value, cells, sample = steps * n * n / el, n * n, f"{steps} full {n}x{n} steps"
    elif w == "batch":
        shapes, states, dxs = batch_problem()
        t0 = time.perf_counter()
        cells = grids = 0
        for k in range(len(shapes)):
            O.solve(0, states[k], 2, dxs[k], 0.9, 1e9, 0.0, 2, 1.4, 0, max_steps=1)
            cells += int(np.prod(shapes[k]))
            grids += 1
            if time.perf_counter() - t0 >= max(8.0, 2.0 * args.steps):
                break
        el = time.perf_counter() - t0
        value, sample, wl = cells / el, f"one step of each of the first {grids} grids ({cells} cells)", BATCH_WORKLOAD
    elif w == "sod":
        s = cases.sod(1000)
        t0 = time.perf_counter()
        _, k, _, _ = O.solve(0, s, 2, 1e-3, 0.9, 0.25, 0.0, 1, 1.4)
        el = time.perf_counter() - t0
        value, sample, wl = k * 1000 / el, f"the whole {k}-step solve", SOD_WORKLOAD
    else:
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no adjoint"}), flush=True)
        return
    base = {"value": value, "unit": METRIC, "cores": cores, "kind": "port",
            "sample": f"{sample} of the FP64 oracle (restatement of the reference, bit-identical to it) in "
                      f"{el:.1f} s on {cores} host threads"}
    line = {"metric": METRIC, "value": value, "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": wl}, "cpu_baseline": base,
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if w in ("sr", "gr"):
        line["ms_per_step"] = n * n / value * 1e3
        line["config"]["n"] = n
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
    ap.add_argument("--workload", default="grid", choices=["grid", "sod", "batch", "sr", "gr", "adjoint", "amr"],
                    help="grid: one 4096^2 Newtonian grid plus every other configuration as `configs` (default); "
                         "sod: the 1000-cell FP64 shock tube; batch: 256 uneven grids in one persistent launch; "
                         "sr: 2048^2 special-relativistic Kelvin-Helmholtz; gr: 1024^2 black-hole accretion; "
                         "adjoint: the adjoints; amr: Level-1 AMR driver runs on a 512^2 cylindrical explosion")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=4096)
    ap.add_argument("--parity-steps", "--err-steps", dest="parity_steps", type=int, default=200,
                    help="steps of the FP32-vs-FP64 comparison of the headline workload")
    ap.add_argument("--sr-steps", type=int, default=200)
    ap.add_argument("--gr-steps", type=int, default=100)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="the headline workload alone (no `configs`)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.workload == "grid":
        run_reference(args) if args.impl == "reference" else run_ours(args)
    elif args.workload == "amr":
        run_amr_reference(args) if args.impl == "reference" else run_amr(args)
    else:
        run_single_reference(args) if args.impl == "reference" else run_single(args)


if __name__ == "__main__":
    main()
