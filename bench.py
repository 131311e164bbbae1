#!/usr/bin/env python3
"""Throughput of the fused D3Q19 stream-and-collide step on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--storage f32|f16|bf16|f64]
    python bench.py --impl reference ...      # the CPU restatement on the host cores

Workload: the LES cylinder at Re 300, 512 x 256 x 64 cells, cylinder r = 16 at
(128, 128), inflow U = 0.08, free-slip z-walls, periodic y, sponge over the
last 32 x-planes, seeded velocity noise +-1e-3 (synthetic; no dataset). A
"step" is one quiet stream-collide pass over the whole lattice. The metric
is GLUPS (giga lattice-cell updates per second; the reference prints MLUPS,
bench.py:23 there). The population buffer (19 x 4 B x 8.4M = 637 MB in FP32)
is larger than the 129 MB L2, so no flush is needed between steps.

Prints one JSON line. ``value`` is device-timed: K steps between two CUDA
events on the launch stream (quiet steps launched as CUDA graphs of step
pairs), populations resident in HBM; ``e2e`` runs tack-lbm's application
loop through the public Solver API (run_lbm.py:207-225: quiet steps, a report
step and monitors every 10 steps, the coarsened output fields copied to pinned
host memory, a steering input), timed by the host clock; ``roofline`` is the
step kernel's algorithmic bytes (152 B per fluid cell in FP32, 76 B in
FP16/BF16) over its event-timed duration against the measured HBM copy
bandwidth; ``adjoint`` times the drag gradient (256x128x32, 2000 steps);
``next_rows`` times the temperature step, the flutter and FSI wing steps and
the derived fields on their own reference workloads (see ``next_rows``).

Under torchrun (N > 1) every rank runs an independent replica on its own GPU
(the step does not shard: replicas only); rank 0 prints the line.
"""

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "tack-lbm_gb300"))

WORKLOAD = dict(nx=512, ny=256, nz=64, collision="les", reynolds=300.0, u0=0.08, diameter=32.0,
                obstacle="cylinder", center=(128.0, 128.0, 32.0), vertical="slip", lateral="periodic",
                sponge_planes=32, u_noise=1e-3, rho_sigma=0.0, seed=20240601)
BYTES_PER_CELL = {"f32": 152, "f16": 76, "bf16": 76, "f64": 304}
# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) of one step_kernel
# launch of this workload from ncu captures: profiles/step_kernel_les_cylinder_
# 512x256x64_f32.md and ..._f16.md (mean of an even and an odd launch) and
# step_kernel_report_les_cylinder_512x256x64_f32.md.
NCU_TRAFFIC = {("f32", False): 1221.2e6, ("f16", False): 583.3e6, ("f32", True): 1800.9e6}
DTYPE = {"f32": "f32", "f16": "f16 storage, f32 arithmetic", "bf16": "bf16 storage, f32 arithmetic",
         "f64": "f64"}


def workload_config(storage, report=False):
    w = WORKLOAD
    return {"workload": f"LES cylinder Re 300, {w['nx']}x{w['ny']}x{w['nz']}, r 16, slip z, sponge 32"
                        + (", report steps" if report else ""),
            "cells": w["nx"] * w["ny"] * w["nz"], "storage": storage, "collision": w["collision"],
            "l2": "inputs larger than L2 (no flush)", "parallelism": "replicas"}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """Samples nvidia-smi SM clocks and throttle reasons while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index, period_ms=20):
        self.index = index
        self.period_ms = period_ms
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", str(self.period_ms)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        return world, rank, local, dist, torch
    return 1, 0, 0, None, None


def barrier(dist, torch):
    if dist is not None:
        dist.barrier()
        if torch.cuda.is_available():
            torch.cuda.synchronize()


def max_over_ranks(value, dist, torch):
    """The largest value over the ranks (the job's time is its slowest replica's)."""
    if dist is None:
        return value
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# The end-to-end leg follows tack-lbm's application loop (run_lbm.py:207-225):
# interval - 1 quiet steps and one report step, then Solver.monitors (which
# refreshes the coarsened output grid, lbm.py:606-611), the Catalyst adaptor
# reading the output fields on the host (copied here into pinned host buffers)
# and a steering input (Solver.set_actuation). The reference defaults to an
# interval of 100 steps and stride 2; this leg uses 10.
E2E_INTERVAL = 10
E2E_STRIDE = 2


def make_solver(storage, device, path):
    import lbm
    w = WORKLOAD
    return lbm.Solver(w["nx"], w["ny"], w["nz"], collision=w["collision"], obstacle=w["obstacle"],
                      reynolds=w["reynolds"], u0=w["u0"], diameter=w["diameter"],
                      device=f"cuda:{device}", lateral=w["lateral"], vertical=w["vertical"],
                      storage=storage, obstacle_center=w["center"], sponge_planes=w["sponge_planes"],
                      init="random", seed=w["seed"], rho_sigma=w["rho_sigma"], u_noise=w["u_noise"],
                      kernel=path, stride=E2E_STRIDE)


def oracle_config():
    from oracle import lbm_oracle as O
    w = WORKLOAD
    cx, cy, _ = w["center"]
    return O.Config(w["nx"], w["ny"], w["nz"], collision=w["collision"],
                    nu=w["u0"] * w["diameter"] / w["reynolds"], obstacle=w["obstacle"], ox=cx, oy=cy,
                    r=w["diameter"] / 2, u0=w["u0"], sponge_start=w["nx"] - w["sponge_planes"],
                    sponge_strength=1.0, lateral=w["lateral"], vertical=w["vertical"])


def cpu_sample_step(f, cells):
    from oracle import lbm_oracle as O
    O.step(oracle_config(), f, cells=cells, dtype=np.float32)


def cpu_baseline_single(f, target_s=12.0):
    """The oracle step (float32 NumPy, one process) on a growing sample of z-planes."""
    cfg_nxy = WORKLOAD["nx"] * WORKLOAD["ny"]
    planes, elapsed = 1, 0.0
    while True:
        cells = np.arange(planes * cfg_nxy)
        t0 = time.perf_counter()
        cpu_sample_step(f, cells)
        elapsed = time.perf_counter() - t0
        if elapsed >= target_s / 4 or planes >= WORKLOAD["nz"]:
            break
        planes = min(WORKLOAD["nz"], planes * 4)
    return {"value": cells.size / elapsed / 1e9, "unit": "GLUPS", "cores": 1, "kind": "port",
            "sample": f"one step of {planes} z-plane(s) ({cells.size} cells) of the workload, "
                      f"float32 NumPy oracle, {elapsed:.1f} s"}


# ---------------------------------------------------------------------------
# reference arm: the CPU restatement over all host cores

def _worker(args):
    """``reps`` oracle passes over cells [lo, hi) of the shared population array."""
    shm_name, shape, lo, hi, reps = args
    from multiprocessing import shared_memory
    shm = shared_memory.SharedMemory(name=shm_name)
    try:
        f = np.ndarray(shape, dtype=np.float32, buffer=shm.buf)
        cells = np.arange(lo, hi)
        t0 = time.perf_counter()
        for _ in range(reps):
            cpu_sample_step(f, cells)
        return time.perf_counter() - t0
    finally:
        shm.close()


def run_reference(args):
    """The reference arm: the float32 NumPy oracle on every host core.

    Each step is one oracle pass over a sample of the workload's cells, split
    over a spawn-started process pool; every worker runs all of its steps in
    one dispatch, so the pool costs nothing per step. The sample is sized by a
    one-plane calibration pass so that warm-up plus timed steps take about
    ``--ref-seconds`` (between 1024 cells per core and two z-planes per step)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and rank != 0:
        return 0
    import multiprocessing as mp
    from multiprocessing import shared_memory
    from oracle import lbm_oracle as O
    w = WORKLOAD
    cfg = oracle_config()
    f0 = O.init_random(cfg, w["rho_sigma"], w["u_noise"], w["seed"]).astype(np.float32)
    shm = shared_memory.SharedMemory(create=True, size=f0.nbytes)
    try:
        f = np.ndarray(f0.shape, dtype=np.float32, buffer=shm.buf)
        f[...] = f0
        del f0
        cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
        nxy = w["nx"] * w["ny"]

        def jobs(sample, reps):
            bounds = np.linspace(0, sample, cores + 1).astype(int)
            return [(shm.name, f.shape, int(bounds[i]), int(bounds[i + 1]), reps) for i in range(cores)]

        ctx = mp.get_context("spawn")
        with ctx.Pool(cores) as pool:
            pool.map(_worker, jobs(nxy, 1))  # imports, page-in
            t0 = time.perf_counter()
            pool.map(_worker, jobs(nxy, 1))
            per_cell = (time.perf_counter() - t0) / nxy
            total = args.steps + args.warmup
            sample = int(args.ref_seconds / (total * per_cell))
            sample = max(cores * 1024, min(2 * nxy, sample))
            pool.map(_worker, jobs(sample, args.warmup))
            t0 = time.perf_counter()
            pool.map(_worker, jobs(sample, args.steps))
            dt = time.perf_counter() - t0
    finally:
        shm.close()
        shm.unlink()
    value = sample * args.steps / dt / 1e9
    n = w["nx"] * w["ny"] * w["nz"]
    sample_ms = dt / args.steps * 1e3
    desc = (f"one float32 NumPy oracle pass over {sample} cells of the workload (the first "
            f"{sample / nxy:.2f} z-planes) per step, split over {cores} processes; sample sized for "
            f"~{args.ref_seconds:.0f} s of warm-up and timed steps")
    line = {"impl": "reference", "metric": "GLUPS", "value": value, "unit": "GLUPS", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            # one step of the whole lattice at the sample's rate; the sample's own time beside it
            "ms_per_step": sample_ms * n / sample, "sample_ms_per_step": sample_ms, "sample_cells": sample,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": workload_config("f32"),
            "cpu_baseline": {"value": value, "unit": "GLUPS", "cores": cores, "kind": "port", "sample": desc,
                             "cpu_model": cpu_model()},
            "e2e": {"value": value, "unit": "GLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------

def adjoint_timing(device):
    """Gradient of the time-averaged drag coefficient of the LES cylinder at
    Re 100, 256 x 128 x 32, 2000 steps (loss over steps 1001..2000),
    checkpoints every 100 steps, FP32; r = 8 (tanh width 1.5), U = 0.05, Cs = 0.1.
    Timed with CUDA events by the library after one untimed forward/backward."""
    from adjoint import DragAdjoint
    run = DragAdjoint(256, 128, 32, steps=2000, loss_start=1001, checkpoint=100, precision="f32",
                      u0=0.05, reynolds=100.0, cs=0.1, r=8.0, width=1.5, device=device)
    run.forward()
    run.backward()
    loss = run.forward()
    grad = run.backward()
    info = run.info()
    del run
    cells = 256 * 128 * 32
    prod_ms = production_forward_ms(device)
    return {"workload": "LES cylinder Re 100, 256x128x32, 2000 steps, K=100, FP32",
            "loss": loss, "grad": {k: float(v) for k, v in zip(("U", "tau0", "Cs", "r"), grad)},
            "forward_ms": info["forward_ms"], "backward_ms": info["backward_ms"],
            "backward_over_forward": info["backward_ms"] / info["forward_ms"],
            "forward_glups": cells * 2000 / (info["forward_ms"] * 1e-3) / 1e9,
            "production_forward_ms": prod_ms,
            "backward_over_production_forward": info["backward_ms"] / prod_ms,
            "production_forward": "2000 quiet steps of the production step kernel (Solver, FP32, AA in place) "
                                  "on the same lattice: LES Re 100, cylinder r 8 at (0.22 nx, 0.5 ny + 1.7), "
                                  "U 0.05, Cs 0.1, one lbm_run_timed",
            "device_bytes": info["device_bytes"]}


def production_forward_ms(device, steps=2000):
    """CUDA-event time of ``steps`` quiet production steps (step_kernel) on the
    adjoint's lattice and flow: the forward cost the backward pass is held to."""
    import lbm
    s = lbm.Solver(256, 128, 32, collision="les", reynolds=100.0, u0=0.05, diameter=16.0, cs=0.1,
                   device=f"cuda:{device}")
    ms = ctypes.c_double()
    s._h.call("lbm_run_timed", 50, 0, None, ctypes.byref(ms))
    s._h.call("lbm_run_timed", int(steps), 0, None, ctypes.byref(ms))
    return ms.value


# ---------------------------------------------------------------------------
# the widened rows beside the step: temperature, moving wings, derived fields

def _events(torch):
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _coupled(step, count, torch):
    """Host time and device time (events on the legacy stream, which the wing
    and FSI entry points use) of ``count`` coupled fluid-structure steps."""
    dev = 0.0
    a, b = _events(torch)
    t0 = time.perf_counter()
    for _ in range(count):
        a.record()
        step()
        b.record()
        b.synchronize()
        dev += a.elapsed_time(b)
    return (time.perf_counter() - t0) * 1e3 / count, dev / count


NEXT_ROWS = ("heat", "flutter", "fsi", "derived")
STUDY_NAMES = ("c2", "c3", "c5", "collision", "drag_window")


def row_heat(device, peak, torch):
    """The heat-sink duct of heat_check.py (320 x 96 x 128, LES at Re 1000, D 12,
    walls at T = 1): flow step + D3Q7 temperature step, quiet steps as one
    lbm_run_timed. Bytes per step: every fluid cell 152 B (populations) + 16 B
    (aux write) + 16 B (aux read); every cell 56 B (7 temperature populations
    in and out)."""
    import ctypes as C
    import lbm
    s = lbm.Solver(320, 96, 128, collision="les", obstacle="heatsink", reynolds=1000.0, heat=True,
                   diameter=12.0, device=f"cuda:{device}")
    s.set_wall_temperature(1.0)
    ms = C.c_double()
    s._h.call("lbm_run_timed", 50, 1, None, C.byref(ms))
    steps = 400
    s._h.call("lbm_run_timed", steps, 0, None, C.byref(ms))
    n = s.lat.n
    fluid = n - int(s.mask().sum())
    byts = fluid * (152 + 16 + 16) + n * 56
    per = ms.value / steps
    m = s.monitors(100)
    return {"workload": "heat-sink duct, LES Re 1000, D3Q7 temperature, 320x96x128, quiet steps",
            "glups": n / (per * 1e-3) / 1e9, "ms_per_step": per, "bytes_per_step": byts,
            "achieved_gbs": byts / (per * 1e-3) / 1e9, "frac": byts / (per * 1e-3) / 1e9 / peak,
            "finite": bool(np.isfinite(list(m.values())).all())}


def row_flutter(device, peak, torch):
    """FlutterSolver's default lattice (384 x 192 x 4, LES, Re 500), released,
    one coupled step per call (the loads come back to the host integrator
    every step, flutter.py:248-262). 45 MB of populations: the step is
    L2-resident and launch-bound, so no HBM fraction is given."""
    import flutter
    w = flutter.FlutterSolver(384, 192, 4, device=f"cuda:{device}")
    w.release()
    for _ in range(20):
        w.step()
    host_ms, dev_ms = _coupled(w.step, 500, torch)
    n = 384 * 192 * 4
    return {"workload": "pitch-plunge NACA 0012, LES Re 500, 384x192x4, coupled steps",
            "glups": n / (host_ms * 1e-3) / 1e9, "host_ms_per_step": host_ms,
            "device_ms_per_step": dev_ms, "finite": bool(np.isfinite(w.coefficients()).all())}


def row_fsi(device, peak, torch):
    """FSISolver's default lattice (256 x 128 x 104, chord 32, span 64, LES,
    Re 500) with the beam model, released: 152 B per fluid cell plus the
    1-byte mask written and read (154 B)."""
    import fsi
    f = fsi.FSISolver(device=f"cuda:{device}")
    f.release()
    for _ in range(5):
        f.step()
    host_ms, dev_ms = _coupled(f.step, 100, torch)
    n = f.lat.n
    fluid = n - int(f.mask().sum())
    byts = fluid * 152 + 2 * n
    return {"workload": "cantilever wing, beam model, LES Re 500, 256x128x104, coupled steps",
            "glups": n / (host_ms * 1e-3) / 1e9, "host_ms_per_step": host_ms,
            "device_ms_per_step": dev_ms, "bytes_per_step": byts,
            "achieved_gbs": byts / (dev_ms * 1e-3) / 1e9, "frac": byts / (dev_ms * 1e-3) / 1e9 / peak,
            "finite": bool(np.isfinite(f.coefficients()).all())}


def row_derived(device, peak, torch, solver):
    """The default derived fields (|curl u| and Q at cell centres) on the
    cylinder run's stride-2 output grid (256 x 128 x 32), as DerivedFields.
    evaluate() computes them: one lbm_vorticity_q_direct pass reading the
    velocity (12 B per point) and writing both fields (8 B per cell). The
    velocity gradient alone (lbm_velocity_gradient: 12 B read, 36 B written
    per point) and the earlier two-pass path (gradient, then the fields from
    it: + 36 B read per cell) are timed beside it. The 12 MB velocity grid sits
    in the 129 MB L2, so these rates are not HBM-bound figures."""
    import ctypes as C
    solver.update_output()
    mx, my, mz = solver.out_dims
    pts, cells = mx * my * mz, (mx - 1) * (my - 1) * (mz - 1)
    dev = torch.device(f"cuda:{device}")
    jac = torch.empty(9 * pts, dtype=torch.float32, device=dev)
    vort = torch.empty(cells, dtype=torch.float32, device=dev)
    q = torch.empty(cells, dtype=torch.float32, device=dev)
    inv_h = solver.diameter / solver.stride

    def direct():
        solver._h.call("lbm_vorticity_q_direct", float(inv_h), C.c_void_p(vort.data_ptr()),
                       C.c_void_p(q.data_ptr()), 1, None)

    def gradient():
        solver._h.call("lbm_velocity_gradient", C.c_void_p(jac.data_ptr()), float(inv_h), None)

    def two_pass():
        gradient()
        solver._h.call("lbm_vorticity_q", C.c_void_p(jac.data_ptr()), C.c_void_p(vort.data_ptr()),
                       C.c_void_p(q.data_ptr()), 1, None)

    def timed(fn, reps=50):
        for _ in range(3):
            fn()
        a, b = _events(torch)
        a.record()
        for _ in range(reps):
            fn()
        b.record()
        b.synchronize()
        return a.elapsed_time(b) / reps

    per, per_grad, per_two = timed(direct), timed(gradient), timed(two_pass)
    byts = pts * 12 + cells * 8
    return {"workload": f"vorticity + Q at cells from the velocity, {mx}x{my}x{mz} output grid",
            "ms_per_call": per, "bytes": byts, "achieved_gbs": byts / (per * 1e-3) / 1e9,
            "frac": byts / (per * 1e-3) / 1e9 / peak,
            "gradient_ms": per_grad, "gradient_bytes": pts * (12 + 36),
            "two_pass_ms": per_two}


def next_rows(device, peak, torch, solver, rows=NEXT_ROWS):
    """Throughput of the widened rows on their reference workloads (row_*)."""
    out = {}
    for name in rows:
        if name == "derived":
            out[name] = row_derived(device, peak, torch, solver)
        else:
            out[name] = {"heat": row_heat, "flutter": row_flutter, "fsi": row_fsi}[name](device, peak, torch)
    return out


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else platform)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() == "Model name":
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


# The kernel-timing pass (every step's kernels between CUDA events) runs right
# before the timed region, long enough for the clock sampler to see the GPU
# under load whatever --steps is: at least this many seconds of steps.
CLOCK_WINDOW_S = 0.5


def device_leg(s, args, storage, local, dist=None, torch=None, world=1):
    """Warm-up, a kernel-timing pass and the timed region of one solver.

    Returns (value, span_ms, roofline, step_roofline, clocks, extra): value in
    GLUPS over the timed region (K steps between two CUDA events on the launch
    stream), the dominant kernel's roofline from the event-bracketed pass."""
    steps = args.steps
    for _ in range(args.warmup):
        s.step(report=args.report)
    s.sync()

    def run_timed(count, report_last):
        ms = ctypes.c_double()
        s._h.call("lbm_run_timed", int(count), int(report_last), None, ctypes.byref(ms))
        return ms.value

    # one probe step sizes the kernel-timing pass to CLOCK_WINDOW_S (capped by
    # the 4096 event slots of lbm_timing)
    probe = run_timed(20, 0) / 20 if not args.report else run_timed(1, 1)
    kernel_steps = int(min(4000, max(min(steps, 1000), CLOCK_WINDOW_S / max(probe * 1e-3, 1e-6))))
    t = (ctypes.c_double * 7)()
    barrier(dist, torch)
    with Clocks(local) as clocks:
        s._h.call("lbm_timing", 1)
        for _ in range(kernel_steps):
            s.step(report=args.report)
        s.sync()
        s._h.call("lbm_timing_read", t)
        s._h.call("lbm_timing", 0)
        # the timed region: K steps between two CUDA events on the launch
        # stream (lbm_run_timed; quiet steps go as CUDA graphs of step pairs),
        # no events in between; report steps one lbm_run_timed each
        barrier(dist, torch)
        t0 = time.perf_counter()
        if args.report:
            span_ms = sum(run_timed(1, 1) for _ in range(steps))
        else:
            span_ms = run_timed(steps, 0)
        s.sync()
        wall = time.perf_counter() - t0
    barrier(dist, torch)
    span_ms = max_over_ranks(span_ms, dist, torch)
    cells = s.lat.n
    value = world * cells * steps / (span_ms * 1e-3) / 1e9
    bulk_ms = t[0] / max(t[1], 1)
    kernel_name = "stream_kernel (bulk-copy)" if args.path == "bulkcopy" else "step_kernel"
    solid = int(s.mask().sum())
    # a report step also reads 4 and writes 13 float32 fields per cell (lbm.py:493-513)
    bytes_cell = BYTES_PER_CELL[storage] + (68 if args.report else 0)
    # the dominant kernel updates t[2] cells (all but lid rows); its obstacle
    # cells move no bytes on a quiet step, every fluid cell moves bytes_cell
    kernel_bytes = bytes_cell * (t[2] - solid)
    achieved = kernel_bytes / (bulk_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    step_bytes = bytes_cell * (cells - solid)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs (burst copy)",
                "traffic": (NCU_TRAFFIC.get((storage, bool(args.report)))
                            if args.path != "bulkcopy" else None),
                "traffic_unit": "B per launch (ncu dram read + write)",
                "kernel": kernel_name, "bytes_per_cell": bytes_cell,
                "fluid_cells_per_launch": int(t[2] - solid), "ms_per_launch": bulk_ms,
                "timed_launches": kernel_steps}
    step_roofline = {"achieved": step_bytes / (span_ms / steps * 1e-3) / 1e9,
                     "frac": step_bytes / (span_ms / steps * 1e-3) / 1e9 / peak,
                     "lid_row_cells": int(t[5])}
    ck = clocks.summary()
    ck["window"] = (f"kernel-timing pass ({kernel_steps} steps, {t[6]:.0f} ms) + the timed region "
                    f"({steps} steps, {span_ms:.1f} ms), sampled every 20 ms")
    extra = {"wall_s": wall, "lid_row_cells": int(t[5]), "solid": solid}
    return value, span_ms, roofline, step_roofline, ck, extra


def storage_variants(args, local, f32_value, storages=("f16", "bf16")):
    """The FP16/BF16 deviation-storage legs on the same workload, steps and
    warm-up as the FP32 line: GLUPS, ms per step and the step kernel's
    roofline (76 B per fluid cell)."""
    out = {}
    for st in storages:
        s = make_solver(st, local, args.path)
        value, span_ms, roof, step_roof, ck, _ = device_leg(s, args, st, local)
        out[st] = {"value": value, "unit": "GLUPS", "ms_per_step": span_ms / args.steps,
                   "dtype": DTYPE[st], "roofline": roof, "step_roofline": step_roof, "clocks": ck,
                   "config": workload_config(st, args.report)}
        del s
    for st in storages:
        out[f"{st}_over_f32"] = out[st]["value"] / f32_value
    return out


def reference_workload(local, warmup=5, steps=200):
    """tack-lbm's own benchmark (bench.py:9-23 there) through the drop-in: the
    default Solver (384 x 128 x 64, LES, Re 300, cylinder D = 24, U = 0.08,
    periodic y and z, lbm_init start), ``warmup`` steps, then ``steps`` quiet
    Solver.step() calls timed by the host clock with a sync on both sides."""
    import lbm
    t0 = time.perf_counter()
    s = lbm.Solver(collision="les", device=f"cuda:{local}")
    s.sync()
    setup = time.perf_counter() - t0
    for _ in range(warmup):
        s.step()
    s.sync()
    t0 = time.perf_counter()
    for _ in range(steps):
        s.step()
    s.sync()
    dt = time.perf_counter() - t0
    m = s.monitors(steps)
    return {"workload": "tack-lbm bench.py: default Solver, LES Re 300, 384x128x64, cylinder D 24, "
                        f"{warmup} warm-up + {steps} timed Solver.step() calls",
            "steps_per_s": steps / dt, "mlups": s.lat.n * steps / dt / 1e6,
            "glups": s.lat.n * steps / dt / 1e9, "ms_per_step": dt / steps * 1e3,
            "setup_s": setup, "timing": "host clock around the Solver.step() calls, synced both sides",
            "monitors_finite": bool(np.isfinite(list(m.values())).all())}


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--ref-seconds", type=float, default=60.0,
                    help="reference arm: size the per-step CPU sample so warm-up + timed steps take about this")
    ap.add_argument("--storage", default="f32", choices=["f32", "f16", "bf16", "f64"])
    ap.add_argument("--path", default="auto", choices=["auto", "simt", "bulkcopy"],
                    help="step kernel: per-cell (auto, simt) or bulk-copy staged (bulkcopy)")
    ap.add_argument("--e2e-steps", type=int, default=500)
    ap.add_argument("--report", action="store_true",
                    help="time report steps (13 diagnostic fields and FP64 monitor sums every step)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--study", choices=sorted(STUDY_NAMES),
                    help="run a physics/precision study instead of the benchmark (one JSON line)")
    ap.add_argument("--study-steps", type=int, default=None)
    ap.add_argument("--no-adjoint", action="store_true",
                    help="skip the drag-adjoint timing (256x128x32, 2000 steps, FP32)")
    ap.add_argument("--no-next-rows", action="store_true",
                    help="skip the heat, flutter, FSI and derived-field timings")
    ap.add_argument("--no-variants", action="store_true",
                    help="skip the FP16/BF16 storage legs and the reference-workload leg")
    ap.add_argument("--next-rows-only", default=None, metavar="ROWS",
                    help="time only these widened rows (comma list of heat,flutter,fsi,derived) and print "
                         "one JSON line with them")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference(args)
    if args.study:
        import studies
        kw = {} if args.study_steps is None else {"steps": args.study_steps}
        print(json.dumps(studies.STUDIES[args.study](**kw)), flush=True)
        return 0

    world, rank, local, dist, torch = dist_setup(args.gpus)
    import lbm_native as N  # noqa: F401  (loads the library, fails loudly without it)
    if args.next_rows_only:
        import torch as torch_host
        rows = [r.strip() for r in args.next_rows_only.split(",") if r.strip()]
        bad = [r for r in rows if r not in NEXT_ROWS]
        if bad:
            ap.error(f"unknown rows {bad}; choose from {NEXT_ROWS}")
        s = make_solver(args.storage, local, args.path) if "derived" in rows else None
        peak, _ = peaks()
        print(json.dumps({"next_rows": next_rows(local, peak, torch_host, s, rows)}), flush=True)
        return 0
    s = make_solver(args.storage, local, args.path)
    steps = args.steps
    value, span_ms, roofline, step_roofline, clocks, extra = device_leg(s, args, args.storage, local, dist,
                                                                        torch, world)
    cells = s.lat.n
    peak, _ = peaks()

    # end to end through the public API: a report step and monitors() every
    # E2E_INTERVAL steps, the output fields copied to pinned host memory
    intervals = max(1, args.e2e_steps // E2E_INTERVAL)
    import torch as torch_host  # pinned host buffers only
    host_out = {k: torch_host.empty(s.output[k].numpy.size, dtype=torch_host.float32).pin_memory().numpy()
                for k in s.OUTPUT}
    omega = s.omega_rot

    def interval():
        for _ in range(E2E_INTERVAL - 1):
            s.step()
        s.step(report=True)
        m = s.monitors(E2E_INTERVAL)
        s.read_output(host_out)
        s.set_actuation(omega)
        return m

    for _ in range(2):
        interval()
    barrier(dist, torch)
    t0 = time.perf_counter()
    for _ in range(intervals):
        m = interval()
    e2e_wall = max_over_ranks(time.perf_counter() - t0, dist, torch)
    e2e_steps = intervals * E2E_INTERVAL
    e2e_value = world * cells * e2e_steps / e2e_wall / 1e9
    d2h = (sum(a.nbytes for a in host_out.values()) + 7 * 8) / E2E_INTERVAL
    h2d = 8 / E2E_INTERVAL
    finite = all(np.isfinite(v) for v in m.values())

    line = {
        "metric": "GLUPS", "value": value, "unit": "GLUPS", "n_gpus": world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": span_ms / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": DTYPE[args.storage], "data": "synthetic",
        "config": workload_config(args.storage, args.report),
        "e2e": {"value": e2e_value, "unit": "GLUPS", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "api": (f"tack-lbm's run loop: per {E2E_INTERVAL} steps {E2E_INTERVAL - 1} x Solver.step(), "
                        f"Solver.step(report=True), Solver.monitors() (output grid stride {E2E_STRIDE}), "
                        "Solver.read_output() of the 5 output fields into pinned host memory, "
                        "Solver.set_actuation()"),
                "steps": e2e_steps, "ms_per_step": e2e_wall / e2e_steps * 1e3},
        "roofline": roofline,
        "step_roofline": step_roofline,
        "gpu_launches": steps * (2 if extra["lid_row_cells"] > 0 else 1) + (steps if args.report else 0),
        "clocks": clocks,
        "monitors_finite": bool(finite),
        "wall_s": extra["wall_s"],
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        f = s.populations(np.float32)
        line["cpu_baseline"] = cpu_baseline_single(f)
        line["cpu_baseline"]["cpu_model"] = cpu_model()
        line["cpu_baseline"]["host_cores"] = os.cpu_count()
    if world == 1 and not args.no_next_rows:
        line["next_rows"] = next_rows(local, peak, torch_host, s)
    del s
    if world == 1 and not args.no_variants:
        if args.storage == "f32" and not args.report:
            line["storage_variants"] = storage_variants(args, local, value)
        line["reference_workload"] = reference_workload(local)
    if not args.no_adjoint:
        line["adjoint"] = adjoint_timing(local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
