#!/usr/bin/env python3
"""Benchmark: MHD zone-updates/s of the unsplit ideal-MHD step on one GB300.

Workload (the configuration the headline metric is quoted on): 3D MHD blast
wave, 512^3 zones on [-0.5,0.5]^3, periodic, PLM/MC + HLLD + RK2, CFL 0.3,
constrained transport (UCT_HLL).  A zone-update is one zone advanced by one
full step (both RK stages).  The headline ``value`` is the mixed-precision
path (FP32 storage and fluxes, FP64 accumulation / pressure recovery /
face-field update / dt reduction); the plain FP64 path, the per-variable L1
error of mixed against FP64, the roofline of the dominant kernel, the
end-to-end rate through the C ABI with host buffers, and the CPU oracle's
rate on the host cores are reported beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun (N>1) every rank runs an independent replica (the step has no
data-path exchange on one GPU per box); value = N*zones*K / max over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

PEAKS = {"hbm_gbs": 6782.1}
try:
    PEAKS.update(json.loads((ROOT / "MEASURED_PEAKS.json").read_text()))
    PEAK_SRC = "measured"
except Exception:
    PEAK_SRC = "fallback"

METRIC = "MHD zone-updates/s on 1 GB300: mixed vs FP64 at L1 err <=1e-5; % of HBM peak"


# ---------------------------------------------------------------------------
# distributed plumbing (replicas only)
# ---------------------------------------------------------------------------
def dist_init():
    """One process per GPU (torchrun env); NCCL on GPUs, gloo on a host
    without one (the replica plumbing is tested that way)."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        if torch.cuda.is_available():
            local = int(os.environ.get("LOCAL_RANK", "0"))
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:
            dist.init_process_group("gloo")
    return rank, ws


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(x, ws):
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.p = None
        self.lines = []

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.p = None
        return self

    def _read(self):
        for line in self.p.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, val in zip(names, f[3:7]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# algorithmic bytes of the mixed kernels (FP32 storage), per cell of the box
# a launch covers: each compulsory state array read or written once at its
# stored width (FP32 primitives and face fields, FP64 resident accumulators)
# ---------------------------------------------------------------------------
def kernel_bytes(name, n, stage_mix=True):
    """Compulsory HBM bytes of one launch of kernel family ``name`` on an n^3
    periodic grid (state words read once, results written once)."""
    cells = n ** 3
    ext = (n + 2) * (n + 2) * n       # transverse-extended sweep box
    edges = (n + 1) ** 3
    per = {
        "mixed_sweep_x": (ext, 32 + 4 + 20 + 2 + 8 + 12),
        "mixed_sweep_y": (ext, 32 + 4 + 40 + 4 + 8 + 12),
        "mixed_sweep_z": (ext, 32 + 4 + 40 + 4 + 8 + 12),
        "mixed_sweep_x_tma": (ext, 32 + 4 + 20 + 2 + 8 + 12),
        "mixed_sweep_y_tma": (ext, 32 + 4 + 40 + 4 + 8 + 12),
        "mixed_sweep_z_tma": (ext, 32 + 4 + 40 + 4 + 8 + 12),
        "mixed_sweep_y_march": (ext, 32 + 4 + 40 + 4 + 8 + 12),
        "mixed_sweep_z_march": (ext, 32 + 4 + 40 + 4 + 8 + 12),
        "mixed_emf": (edges, 24 + 36 + 12 + 12 + 12),
        "mixed_face": (edges, 12 + 12 + 6 + 12),
        # resident FP64 accumulators: stage 1 reads U0 (5 x 8 B under CT), dU (5 x 4),
        # the faces (3 x 4), C_dt, writes V (8 x 4) and the flag -> 109 B (its
        # conserved result is stored only where a floor changed it); the RK2
        # corrector reads U0, both increments (2 x 5 x 4), the faces and the flag,
        # writes V, U0 (5 x 8) and the flag -> 166 B; mean of the two
        "mixed_final": (cells, 138),
    }
    if name not in per:
        return None
    units, b = per[name]
    return units * b


# ---------------------------------------------------------------------------
# CPU baseline: the oracle (plain-C restatement of the reference path)
# ---------------------------------------------------------------------------
def cpu_rate(n=512, budget_s=15.0, steps=3, threads=None):
    """The oracle's rate on the blast at n^3: `steps` steps of the central
    n x n x nz slab, nz sized (reference_slab) so they take about budget_s."""
    from oracle.oracle import Oracle
    from pluto_gb300 import problems
    threads = threads or os.cpu_count() or 1
    nz, _ = reference_slab(n, steps, budget_s, threads)
    spec, vc, faces = problems.blast3d(n, nz=nz)
    o = Oracle(spec, nthreads=threads)
    o.set_state(vc, faces)
    del vc, faces
    t0 = time.perf_counter()
    dt = 1e-4
    for _ in range(steps):
        inv, _, _ = o.advance(dt)
        dt = min((1.0 / inv) * spec["cfl"], 1.1 * dt)
    el = time.perf_counter() - t0
    return dict(value=n * n * nz * steps / el, unit="zone-updates/s", cores=threads, kind="port",
                sample=f"oracle (C restatement of the reference path, OpenMP over pencils) on the "
                       f"same blast scheme, {steps} steps of the central {n}x{n}x{nz} slab of the {n}^3 "
                       f"grid, {threads} host threads")


def reference_slab(n, steps_total, budget_s, threads):
    """Layers nz of the central n x n x nz slab of the n^3 blast such that
    steps_total oracle steps take about budget_s on `threads` host threads,
    from one timed step of a 16-layer slab (a multiple of 16, at most n)."""
    from oracle.oracle import Oracle
    from pluto_gb300 import problems
    spec, vc, faces = problems.blast3d(n, nz=16)
    o = Oracle(spec, nthreads=threads)
    o.set_state(vc, faces)
    t0 = time.perf_counter()
    o.advance(1e-4)
    per_layer = (time.perf_counter() - t0) / 16
    del o
    nz = int(budget_s / max(steps_total * per_layer, 1e-9)) // 16 * 16
    return max(16, min(n, nz)), per_layer


def reference_arm(args, rank, ws):
    """--impl reference: the reference algorithm on the host cores.  The
    reference C binary cannot be built on the benchmark machine (an Arm host
    without the reference source tree), so the oracle port -- bit-identical
    to it on the golden problems and on the fixtures at the configurations'
    sizes -- is timed with all host threads on the same blast at the GPU
    arm's grid, --n^3.  Each bench step is one full step of the central
    n x n x nz slab of that grid, nz sized so the warm-up and timed steps
    take about --ref-budget seconds (nz = n, the whole grid, when the step
    counts allow; a 512^3 step takes ~20 s on 16 Grace cores)."""
    if rank != 0:
        return
    from oracle.oracle import Oracle, build as obuild
    from pluto_gb300 import problems
    obuild()
    n = args.n
    threads = os.cpu_count() or 1
    nz, per_layer = reference_slab(n, args.steps + args.warmup, args.ref_budget, threads)
    spec, vc, faces = problems.blast3d(n, nz=nz)
    o = Oracle(spec, nthreads=threads)
    o.set_state(vc, faces)
    del vc, faces
    dt = 1e-4
    for _ in range(args.warmup):
        inv, _, _ = o.advance(dt)
        dt = min((1.0 / inv) * spec["cfl"], 1.1 * dt)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        inv, _, _ = o.advance(dt)
        dt = min((1.0 / inv) * spec["cfl"], 1.1 * dt)
    el = time.perf_counter() - t0
    v = n * n * nz * args.steps / el
    sample = (f"oracle port, the whole {n}^3 grid, one step per bench step" if nz == n else
              f"oracle port, one step of the central {n}x{n}x{nz} slab of the {n}^3 grid per bench step "
              f"(periodic in z; nz sized from a timed 16-layer step, {per_layer * 1e3:.1f} ms per layer, "
              f"so the run takes ~{args.ref_budget:g} s)")
    out = {"metric": METRIC, "value": v, "unit": "zone-updates/s", "impl": "reference", "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (blast IC generated in-process)",
           "config": {"workload": f"3D MHD blast {n}^3 periodic, PLM/MC + HLLD + RK2 + CT(UCT_HLL), CFL 0.3",
                      "grid": [n, n, n], "sample_grid": [n, n, nz], "precision": "fp64"},
           "cpu_baseline": {"value": v, "unit": "zone-updates/s", "cores": threads, "kind": "port",
                            "sample": sample},
           "e2e": {"value": v, "unit": "zone-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# ---------------------------------------------------------------------------
# main GPU arm
# ---------------------------------------------------------------------------
def batched_tubes(args):
    """Batched Riemann tubes: 4096 tubes (seeded), N log-uniform in
    [128, 4096], PLM/minmod + HLLD + RK2, CFL 0.8, outflow, 400 steps, every
    tube with its own dt, all in one persistent graph-captured launch; the
    schedule (warps per tube team, teams per SM; largest tube first) from the
    autotuner.  FP64 and mixed precision; mixed-vs-FP64 L1 per tube after the
    run, with each precision's own CFL dt and at equal times (fixed dt)."""
    from pluto_gb300.batch import Batch, tube_family
    spec, ns, dxs, states = tube_family(args.tubes, args.tube_seed, 128, 4096)
    cells = int(ns.sum())
    cfl, first_dt = spec["cfl"], spec["first_dt"]
    res = {"workload": f"{len(ns)} 1D MHD Riemann tubes, N log-uniform in [128, 4096] (seed "
                       f"{args.tube_seed}), PLM/minmod + HLLD + RK2, CFL 0.8, outflow, per-tube dt",
           "tubes": len(ns), "cells": cells, "steps": args.tube_steps,
           "zone_updates": cells * args.tube_steps}
    finals, fixed = {}, {}
    fixed_dt = 1e-5  # below every tube's CFL limit
    for prec, width in (("fp64", 8), ("mixed", 4)):
        b = Batch(spec, ns, dxs, prec)
        b.upload(states)
        tune = b.autotune(args.tube_trial_steps, first_dt, cfl)
        b.upload(states)
        b.run(args.tube_steps, first_dt, cfl)  # builds and warms the graph of this length
        b.upload(states)
        with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
            ms = b.run(args.tube_steps, first_dt, cfl)
        finals[prec] = b.download()
        t, _, nf = b.get()
        # equal times: the same fixed dt in both precisions
        b.upload(states)
        b.run(args.tube_steps, fixed_dt, 0.0)
        fixed[prec] = b.download()
        del b
        zu = cells * args.tube_steps / (ms / 1e3)
        # algorithmic bytes per zone-update: RK2 reads and writes the primitives twice
        # (4 x 8 words at the storage width) plus the resident conserved state (8-byte
        # words: U0 read, U1 written and read, U0 written)
        per_zu = 4 * 8 * width + 4 * 8 * 8
        res[prec] = {"value": zu, "unit": "zone-updates/s", "ms": ms, "schedule": tune,
                     "hbm_gbs_algorithmic": zu * per_zu / 1e9, "bytes_per_zone_update": per_zu,
                     "t_min": float(t.min()), "t_max": float(t.max()), "floor_events": int(nf.sum()),
                     "clocks": clk.summary()}

    def l1_stats(a, b):
        e = sorted(rel_l1(a[q][v], b[q][v]) for q in range(len(ns)) for v in range(8)
                   if np.abs(b[q][v]).sum() > 0)
        return {"median": e[len(e) // 2], "p99": e[int(0.99 * (len(e) - 1))], "max": e[-1]}
    res["l1_mixed_vs_fp64"] = dict(l1_stats(finals["mixed"], finals["fp64"]),
                                   note="each precision takes its own CFL dt sequence; on shock tubes the "
                                        "time offset moves the discontinuities")
    res["l1_mixed_vs_fp64_equal_times"] = dict(l1_stats(fixed["mixed"], fixed["fp64"]),
                                               note=f"both precisions with the fixed dt {fixed_dt:g}, "
                                                    f"{args.tube_steps} steps", bar=1e-5)
    res["mixed_over_fp64"] = res["mixed"]["value"] / res["fp64"]["value"]
    return res


def adjoint_timing():
    """CP-Alfven 128^2 (30 degrees), PLM/MC + HLLD + RK2 + CT, 256 FP64 steps
    with a frozen CFL dt sequence: forward with a checkpoint every 16 steps,
    the adjoint pass (recomputation + reverse kernels), the tangent-linear
    pass, each timed on the host around the C-ABI calls."""
    from pluto_gb300 import problems
    from pluto_gb300.adjoint import Rollout, cfl_dt_sequence, tangent_linear
    spec, vc, f = problems.cp_alfven(128)
    f = [f[0], f[1], None]
    nsteps = 256
    dts = cfl_dt_sequence(spec, vc, f, nsteps, spec["first_dt"], spec["cfl"])
    r = Rollout(spec, dts, every=16)
    r.run(vc, f, checkpoint=True)  # warm
    t0 = time.perf_counter()
    out_vc, _ = r.run(vc, f, checkpoint=False)
    t_plain = time.perf_counter() - t0
    t0 = time.perf_counter()
    out_vc, _ = r.run(vc, f, checkpoint=True)
    t_fwd = time.perf_counter() - t0
    rng = np.random.default_rng(0)
    lam = np.zeros_like(vc)
    lam[0] = rng.normal(size=vc[0].shape)
    t0 = time.perf_counter()
    g_vc, g_f = r.gradient(lam, [np.zeros_like(f[0]), np.zeros_like(f[1]), None])
    t_adj = time.perf_counter() - t0
    d_vc = rng.normal(size=vc.shape)
    d_f = [rng.normal(size=f[0].shape), rng.normal(size=f[1].shape), None]
    t0 = time.perf_counter()
    _, (tv, _) = tangent_linear(spec, dts, vc, f, d_vc, d_f)
    t_tl = time.perf_counter() - t0
    lhs = float(np.dot(lam.ravel(), tv.ravel()))
    rhs = float(np.dot(g_vc.ravel(), d_vc.ravel()) + sum(np.dot(g_f[d].ravel(), d_f[d].ravel()) for d in range(2)))
    cells = 128 * 128
    return {"workload": "CP-Alfven 128^2 rotated 30 deg, PLM/MC + HLLD + RK2 + CT, 256 FP64 steps, "
                        "checkpoint every 16, frozen dt",
            "forward_ms": 1e3 * t_fwd, "forward_plain_ms": 1e3 * t_plain, "adjoint_ms": 1e3 * t_adj,
            "tangent_linear_ms": 1e3 * t_tl, "adjoint_over_forward": t_adj / t_plain,
            "adjoint_zone_updates_per_s": cells * nsteps / t_adj,
            "dot_product_rel_diff": abs(lhs - rhs) / abs(lhs),
            "timing": "host clock around synchronous C-ABI calls (one pg_advance per step)"}


def turbulence_leg(args):
    """Decaying MHD turbulence (768^3 periodic on [0,1]^3, rho = p = 1,
    random-phase solenoidal v and A with E(k) ~ k^-2 on shells 1..4, rms Mach
    1, plasma beta 10; PPM + HLLD + RK3 + CT (UCT_HLL), CFL 0.3): the mixed
    path at full size (zone-updates/s, algorithmic HBM GB/s), the plain FP64
    path at full size when it fits in device memory (else at the L1 grid),
    and the per-variable L1 error of both mixed forms against FP64 after
    ``turb_l1_steps`` steps on a ``turb_l1_n``^3 copy of the same problem."""
    import torch
    from pluto_gb300 import Solver, problems
    n = args.turb_n
    # the initial state is built in host memory (~140 B per zone at its peak)
    try:
        avail = int(next(l for l in open("/proc/meminfo") if l.startswith("MemAvailable")).split()[1]) * 1024
    except Exception:
        avail = None
    host_note = None
    while avail is not None and avail < 160 * n ** 3 and n > 128:
        n //= 2
        host_note = f"grid reduced to {n}^3: {avail / 1e9:.0f} GB of host memory available"
    spec, vc, faces = problems.turbulence3d(n)
    cfl, first_dt = spec["cfl"], spec["first_dt"]
    cells = n ** 3
    mx = Solver(spec, precision="mixed")
    mx.upload(vc, faces)
    mx.run(args.warmup, first_dt, cfl)
    launches = mx.launches_per_step()
    with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        ms = mx.run_timed(args.steps, 0.0, cfl)
    value = cells * args.steps / (ms / 1e3)
    prof = mx.profile_kernels(1, 0.0, cfl)
    info = mx.info()
    del mx
    torch.cuda.empty_cache()
    # plain FP64 path: 75 doubles + 1 flag byte per zone of the ghosted grid
    ng = 3
    need = 601 * (n + 2 * ng) ** 3
    free = torch.cuda.mem_get_info()[0]
    n64 = n if free > 1.05 * need else args.turb_l1_n
    if n64 != n:
        spec64, vc64, faces64 = problems.turbulence3d(n64)
    else:
        spec64, vc64, faces64 = spec, vc, faces
    f64 = Solver(spec64, precision="fp64")
    f64.upload(vc64, faces64)
    f64.run(1, first_dt, cfl)
    ms64 = f64.run_timed(args.fp64_steps, 0.0, cfl)
    value64 = n64 ** 3 * args.fp64_steps / (ms64 / 1e3)
    del f64, vc64, faces64
    del vc, faces
    # L1 of mixed vs FP64 from the same initial state
    nl = args.turb_l1_n
    spec_l, vc_l, faces_l = problems.turbulence3d(nl)
    a = Solver(spec_l, precision="fp64")
    a.upload(vc_l, faces_l)
    a.run(args.turb_l1_steps, first_dt, cfl)
    ra, rb = a.download()
    del a
    names = ["rho", "vx1", "vx2", "vx3", "Bx1", "Bx2", "Bx3", "prs"]
    l1 = {"steps": args.turb_l1_steps, "grid": nl, "bar": 1e-5}
    for prec in ("mixed", "mixed_dw"):
        b = Solver(spec_l, precision=prec)
        b.upload(vc_l, faces_l)
        b.run(args.turb_l1_steps, first_dt, cfl)
        ma, mb = b.download()
        del b
        per = {names[q]: rel_l1(ma[q], ra[q]) for q in range(8)}
        for d in range(3):
            per[f"Bx{d+1}s"] = rel_l1(mb[d], rb[d])
        l1[prec] = {"per_variable": per, "max": max(per.values())}
    peak = PEAKS.get("hbm_gbs", 6782.1)
    algo = 8 * 11 * 4  # RK3: 8W FP32 words per zone-update, W = NVAR + DIMENSIONS = 11
    dom = max(prof, key=lambda k: prof[k][0])
    return {
        "metric": "MHD zone-updates/s on 1 GB300 (3D decaying turbulence)", "value": value,
        "unit": "zone-updates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 storage/fluxes + f64 accumulation",
        "data": "synthetic (seeded random-phase spectrum generated in-process)",
        "config": {"workload": f"3D decaying MHD turbulence {n}^3 periodic, PPM + HLLD + RK3 + CT(UCT_HLL), "
                               "CFL 0.3", "grid": [n, n, n], "precision": "mixed",
                   "l2": "inputs larger than L2, no flush needed", "host_note": host_note},
        "hbm_algorithmic": {"bytes_per_zone_update": algo, "achieved_gbs": value * algo / 1e9,
                            "frac": value * algo / 1e9 / peak, "peak_gbs": peak, "peak_source": PEAK_SRC},
        "fp64": {"value": value64, "grid": n64, "steps": args.fp64_steps, "ms_per_step": ms64 / args.fp64_steps,
                 "speedup_mixed_over_fp64": value / value64},
        "l1_mixed_vs_fp64": l1,
        "kernels": {k: {"ms": v[0], "launches": v[1]} for k, v in prof.items()}, "dominant_kernel": dom,
        "gpu_launches": launches * args.steps, "floors_in_run": info.get("nfail"),
        "clocks": clk.summary(),
    }


def output_timing(n=256, outputs=4, steps_between=50):
    """The device output path (pg_write_output, .dbl single file) against
    download-then-write through the C ABI, on the mixed 3D blast at n^3:
    per output, the time it adds to a run of steps (outputs every
    steps_between steps, a cadence at which the file writes keep up) over the
    same run without outputs.  Two untimed outputs first allocate the
    staging slots (device + pinned host, one output each)."""
    import shutil
    import tempfile

    import torch
    from pluto_gb300 import Solver, problems
    spec, vc, faces = problems.blast3d(n)
    cfl, first_dt = spec["cfl"], spec["first_dt"]
    s = Solver(spec, precision="mixed")
    s.upload(vc, faces)
    s.run(3, first_dt, cfl)
    bytes_out = 8 * (8 * n ** 3 + sum(f.size for f in faces))
    tmp = tempfile.mkdtemp(prefix="pg_out_")
    try:
        if shutil.disk_usage(tmp).free < 4 * bytes_out:
            return {"skipped": "not enough free space for the files under " + tempfile.gettempdir()}
        steps = outputs * steps_between
        for k in range(2):
            s.write_output(tmp, "dbl", 0, write_record=False)
        s.output_wait()
        ms_run = s.run_timed(steps, 0.0, cfl)
        # async device writer
        s.sync()
        t0 = time.perf_counter()
        for k in range(outputs):
            s.write_output(tmp, "dbl", k, time=float(k), dt=first_dt, step=k)
            s.run_async(steps_between, 0.0, cfl)
        s.sync()
        t_async = time.perf_counter() - t0
        s.output_wait()
        t_drain = time.perf_counter() - t0
        # the packing alone (what the compute stream waits for)
        t0 = time.perf_counter()
        s.write_output(tmp, "dbl", outputs, write_record=False)
        s.sync()
        t_pack = time.perf_counter() - t0
        s.output_wait()
        # download the whole state into pinned host arrays, then write the file
        def pinned(shape):
            return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
        hv = pinned(vc.shape)
        hf = [pinned(f.shape) for f in faces]
        t0 = time.perf_counter()
        for k in range(outputs):
            s.download(out=(hv, hf))
            with open(os.path.join(tmp, f"host.{k:04d}.dbl"), "wb") as f:
                for q in range(8):
                    hv[q].tofile(f)
                for a in hf:
                    a.tofile(f)
            s.run_async(steps_between, 0.0, cfl)
        s.sync()
        t_sync = time.perf_counter() - t0
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    base = ms_run / 1e3
    return {"workload": f"mixed 3D blast {n}^3, .dbl single file ({bytes_out / 1e9:.2f} GB) every "
                        f"{steps_between} steps, {outputs} outputs",
            "bytes_per_output": bytes_out, "ms_per_step": ms_run / steps,
            "device_writer": {"added_ms_per_output": (t_async - base) / outputs * 1e3,
                              "pack_ms": t_pack * 1e3, "all_files_written_s": t_drain},
            "download_then_write": {"added_ms_per_output": (t_sync - base) / outputs * 1e3}}


def profile_case(args):
    """--profile-case PROBLEM: ``--steps`` eager steps of one problem on a
    fresh solver at ``--n``^3 (``--precision``), no CUDA graph, so that every
    kernel is a separate launch a profiler can select with -k/-s/-c.  Prints
    one line; no timing is taken."""
    from pluto_gb300 import Solver, problems
    if args.profile_case == "adjoint":  # the adjoint leg's workload at --n^2, --steps steps
        from pluto_gb300.adjoint import Rollout, cfl_dt_sequence
        spec, vc, f = problems.cp_alfven(args.n)
        f = [f[0], f[1], None]
        dts = cfl_dt_sequence(spec, vc, f, args.steps, spec["first_dt"], spec["cfl"])
        r = Rollout(spec, dts, every=16)
        r.run(vc, f, checkpoint=True)
        lam = np.zeros_like(vc)
        lam[0] = np.random.default_rng(0).normal(size=vc[0].shape)
        r.gradient(lam, [np.zeros_like(f[0]), np.zeros_like(f[1]), None])
        print(json.dumps({"profile_case": "adjoint", "n": args.n, "steps": args.steps}), flush=True)
        return
    if args.profile_case == "blast":
        spec, vc, faces = problems.blast3d(args.n)
    elif args.profile_case == "turb":
        spec, vc, faces = problems.turbulence3d(args.n)
    else:
        spec, vc, faces = problems.orszag_tang(args.n)
    s = Solver(spec, precision=args.precision)
    s.upload(vc, faces)
    dt = spec["first_dt"]
    for _ in range(args.steps):
        inv, _, _ = s.advance(dt)
        dt = min((1.0 / inv) * spec["cfl"], 1.1 * dt)
    print(json.dumps({"profile_case": args.profile_case, "n": args.n, "precision": args.precision,
                      "steps": args.steps, "next_dt": dt}), flush=True)


def rel_l1(a, b):
    den = np.abs(b).sum()
    return float(np.abs(a - b).sum() / den) if den > 0 else float(np.abs(a - b).sum())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--l1-steps", type=int, default=100)
    ap.add_argument("--l1-n", type=int, default=512)
    ap.add_argument("--e2e-steps", type=int, default=30)
    ap.add_argument("--ref-budget", type=float, default=150.0,
                    help="seconds the reference arm's warm-up and timed steps should take")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--tubes", type=int, default=4096)
    ap.add_argument("--tube-seed", type=int, default=0)
    ap.add_argument("--tube-steps", type=int, default=400)
    ap.add_argument("--tube-trial-steps", type=int, default=25)
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-output", action="store_true")
    ap.add_argument("--turbulence", action="store_true",
                    help="print the decaying-turbulence line (PPM/RK3, --turb-n^3) instead of the blast line")
    ap.add_argument("--turb-n", type=int, default=768)
    ap.add_argument("--turb-l1-n", type=int, default=256)
    ap.add_argument("--turb-l1-steps", type=int, default=50)
    ap.add_argument("--profile-case", choices=["blast", "turb", "ot", "adjoint"],
                    help="run --steps eager steps of one problem at --n (for ncu to attach to) and exit; "
                         "adjoint: the CP-Alfven --n^2 forward with checkpoints and one gradient")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "mixed_dw", "fp64"],
                    help="precision of --profile-case")
    args = ap.parse_args()
    rank, ws = dist_init()
    if args.impl == "reference":
        reference_arm(args, rank, ws)
        return
    assert args.warmup >= 3, "at least 3 warm-up steps"

    from pluto_gb300 import Solver, problems
    from pluto_gb300 import build as pbuild
    pbuild.build()
    if args.profile_case:
        profile_case(args)
        return
    if args.turbulence:
        if rank == 0:
            print(json.dumps(turbulence_leg(args)), flush=True)
        return

    n = args.n
    spec, vc, faces = problems.blast3d(n)
    cfl, first_dt = spec["cfl"], spec["first_dt"]
    cells = n ** 3

    # the batched-tube and adjoint legs run first, on a GPU not yet heated by
    # the minutes of 512^3 work (their clocks are sampled too)
    batch = None
    if rank == 0 and not args.no_batch:
        batch = batched_tubes(args)
    adj = None
    if rank == 0 and not args.no_adjoint:
        adj = adjoint_timing()

    # ---- mixed precision, resident inputs (headline value) ----
    mx = Solver(spec, precision="mixed")
    mx.upload(vc, faces)
    mx.run(args.warmup, first_dt, cfl)
    launches = mx.launches_per_step()
    barrier(ws)
    with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        ms = mx.run_timed(args.steps, 0.0, cfl)
    barrier(ws)
    ms = allmax(ms, ws)
    value = ws * cells * args.steps / (ms / 1e3)
    clocks = clk.summary()

    # ---- per-kernel profile of the mixed step (events on the solver stream) ----
    prof = mx.profile_kernels(2, 0.0, cfl)
    tot = sum(t for t, _ in prof.values())
    dom_name = max(prof, key=lambda k: prof[k][0])
    dom_ms, dom_cnt = prof[dom_name]
    avg_ms = dom_ms / dom_cnt
    alg = kernel_bytes(dom_name, n)
    achieved = alg / (avg_ms / 1e3) / 1e9 if alg else None
    # per-kernel ncu figures of one RK2 step of the same scheme at 192^3
    # (DRAM bytes and warp instructions per interior zone, the binding unit);
    # scaled to this grid by the zone count
    traffic = traffic_note = limiter = None
    step_bytes_zone = step_winst_zone = None
    pfile = ROOT / "profiles" / "mixed_step_blast192.json"
    if pfile.exists():
        try:
            pj = json.loads(pfile.read_text())
            step_bytes_zone = pj["step"]["dram_bytes_per_zone"]
            step_winst_zone = pj["step"]["warp_inst_per_zone"]
            kd = pj["kernels"].get(dom_name)
            if kd:
                traffic = kd["dram_bytes_per_zone_per_launch"] * cells
                traffic_note = (f"ncu dram__bytes_read+write of {dom_name} per launch at {pj['grid']}^3 "
                                f"({kd['dram_bytes_per_zone_per_launch']:.1f} B/zone), scaled by the zone count")
                limiter = kd["bound"]
        except Exception:
            traffic = None
    mx_info = mx.info()
    del mx

    # ---- same mixed path with the FP64 parts done as FP32 double-word pairs ----
    dwr = Solver(spec, precision="mixed_dw")
    dwr.upload(vc, faces)
    dwr.run(args.warmup, first_dt, cfl)
    ms_dw = allmax(dwr.run_timed(args.steps, 0.0, cfl), ws)
    value_dw = ws * cells * args.steps / (ms_dw / 1e3)
    prof_dw = dwr.profile_kernels(1, 0.0, cfl)
    del dwr

    # ---- plain FP64 path on the same workload ----
    f64 = Solver(spec, precision="fp64")
    f64.upload(vc, faces)
    f64.run(1, first_dt, cfl)
    ms64 = f64.run_timed(args.fp64_steps, 0.0, cfl)
    ms64 = allmax(ms64, ws)
    value64 = ws * cells * args.fp64_steps / (ms64 / 1e3)
    fp64_prof = f64.profile_kernels(1, 0.0, cfl)
    del f64

    # ---- L1 error of mixed vs FP64 after l1_steps from the same IC ----
    l1 = None
    if args.l1_steps > 0 and rank == 0:
        if args.l1_n != n:
            spec_l, vc_l, faces_l = problems.blast3d(args.l1_n)
        else:
            spec_l, vc_l, faces_l = spec, vc, faces
        a = Solver(spec_l, precision="fp64")
        a.upload(vc_l, faces_l)
        a.run(args.l1_steps, first_dt, cfl)
        ra, rb = a.download()
        nf64 = a.info()["nfail"]
        del a
        names = ["rho", "vx1", "vx2", "vx3", "Bx1", "Bx2", "Bx3", "prs"]
        l1 = {"steps": args.l1_steps, "grid": args.l1_n, "bar": 1e-5, "fp64_floor_events_last_step": nf64}
        for prec in ("mixed", "mixed_dw"):
            b = Solver(spec_l, precision=prec)
            b.upload(vc_l, faces_l)
            b.run(args.l1_steps, first_dt, cfl)
            ma, mb = b.download()
            del b
            per = {names[q]: rel_l1(ma[q], ra[q]) for q in range(8)}
            for d in range(3):
                per[f"Bx{d+1}s"] = rel_l1(mb[d], rb[d])
            l1[prec] = {"per_variable": per, "max": max(per.values())}
            del ma, mb
        l1["max"] = l1["mixed"]["max"]
        del ra, rb

    # ---- e2e through the C ABI with host buffers: pg_upload once, then every step
    # ---- pg_advance (host dt in, invDt out) and a pg_download of the whole state into
    # ---- the host arrays (the AdvanceStep shim with PLUTO_GPU_SYNC_EVERY=1; its default
    # ---- downloads only for host readers, see the "output" leg)
    e2e = None
    if args.e2e_steps > 0:
        import torch

        def pinned(shape):
            return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()

        host_vc = pinned(vc.shape)
        host_vc[...] = vc
        host_f = []
        for f in faces:
            h = pinned(f.shape)
            h[...] = f
            host_f.append(h)
        out_vc = pinned(vc.shape)
        out_f = [pinned(f.shape) for f in faces]
        e = Solver(spec, precision="mixed")
        e.upload(host_vc, host_f)
        e.advance(first_dt)  # warm
        e.download(out=(out_vc, out_f))
        ta = time.perf_counter()
        e.upload(host_vc, host_f)
        tb = time.perf_counter()
        e.download(out=(out_vc, out_f))
        tc = time.perf_counter()
        # synchronous form: each download completes before the next step starts
        barrier(ws)
        t0 = time.perf_counter()
        e.upload(host_vc, host_f)
        dt = first_dt
        for _ in range(args.e2e_steps):
            inv, _, _ = e.advance(dt)
            e.download(out=(out_vc, out_f))
            dt = min((1.0 / inv) * cfl, 1.1 * dt)
        el_sync = allmax(time.perf_counter() - t0, ws)
        # pipelined form (headline): step n's state is snapshotted on the device and
        # copied to the host on a second stream while step n+1 runs; every copy has
        # landed in host memory before the clock stops
        e.download_async((out_vc, out_f))
        e.download_wait()
        barrier(ws)
        t0 = time.perf_counter()
        e.upload(host_vc, host_f)
        dt = first_dt
        for _ in range(args.e2e_steps):
            inv, _, _ = e.advance(dt)
            e.download_async((out_vc, out_f))
            dt = min((1.0 / inv) * cfl, 1.1 * dt)
        e.download_wait()
        el = allmax(time.perf_counter() - t0, ws)
        del e
        state_bytes = 8 * (8 * cells + sum(f.size for f in faces))
        e2e = {"value": ws * cells * args.e2e_steps / el, "unit": "zone-updates/s",
               "h2d_bytes_per_step": int(state_bytes / args.e2e_steps + 8),
               "d2h_bytes_per_step": int(state_bytes + 48),
               "path": "pg_upload once (pinned host FP64) + per step pg_advance (host dt in, invDt out, "
                       "synchronous) + pg_download_async of the whole FP64 state into pinned host arrays "
                       "(device snapshot, copy on a second stream overlapping the next step; all copies "
                       "complete inside the timed region)",
               "sync_value": ws * cells * args.e2e_steps / el_sync,
               "sync_path": "the same with a synchronous pg_download after every step",
               "steps": args.e2e_steps,
               "upload_gbs": state_bytes / (tb - ta) / 1e9, "download_gbs": state_bytes / (tc - tb) / 1e9}

    outp = None
    if rank == 0 and not args.no_output:
        try:
            outp = output_timing()
        except Exception as ex:
            outp = {"skipped": f"{type(ex).__name__}: {ex}"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        try:
            cpu = cpu_rate()
        except Exception as ex:  # the oracle needs gcc on the host
            cpu = {"value": None, "unit": "zone-updates/s", "cores": 0, "kind": "port",
                   "sample": f"unavailable: {ex}"}

    if rank != 0:
        return
    peak = PEAKS.get("hbm_gbs", 6782.1)
    algo_bytes_zu = 55 * 4  # 5W words of FP32, W = NVAR + DIMENSIONS = 11
    out = {
        "metric": METRIC, "value": value, "unit": "zone-updates/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 storage/fluxes + f64 accumulation",
        "data": "synthetic (blast IC generated in-process, seedless)",
        "config": {"workload": "3D MHD blast 512^3 periodic, PLM/MC + HLLD + RK2 + CT(UCT_HLL), CFL 0.3",
                   "grid": [n, n, n], "precision": "mixed",
                   "l2": "inputs larger than L2: ~27 GB working set vs 129 MB L2, no flush needed"},
        "fp64": {"value": value64, "unit": "zone-updates/s", "steps": args.fp64_steps,
                 "ms_per_step": ms64 / args.fp64_steps,
                 "speedup_mixed_over_fp64": value / value64,
                 "dominant_kernel": max(fp64_prof, key=lambda k: fp64_prof[k][0])},
        "mixed_dw": {"value": value_dw, "unit": "zone-updates/s", "ms_per_step": ms_dw / args.steps,
                     "note": "same kernels; the FP64 accumulation, pressure recovery, face update and "
                             "dt sums done as FP32 double-word pairs (48-bit significand)",
                     "kernels": {k: {"ms": v[0], "launches": v[1]} for k, v in prof_dw.items()}},
        "l1_mixed_vs_fp64": l1,
        "hbm_fraction_algorithmic": value * algo_bytes_zu / (peak * 1e9),
        # the whole step against HBM: DRAM bytes per zone of every launch of one
        # step (ncu at 192^3, scaled by the zone count) over the step time
        "step_hbm": ({"bytes_per_zone_step": step_bytes_zone,
                      "achieved_gbs": step_bytes_zone * cells / (ms / args.steps / 1e3) / 1e9,
                      "frac": step_bytes_zone * cells / (ms / args.steps / 1e3) / 1e9 / peak,
                      "peak_gbs": peak, "source": "profiles/mixed_step_blast192.json (ncu at 192^3, per zone)"}
                     if step_bytes_zone else None),
        # the whole step against the instruction-issue ceiling: warp instructions
        # per zone-update (ncu at 192^3) over one warp instruction per cycle per
        # scheduler (152 SMs x 4) at the sampled SM clock
        "compute_roofline": ({"warp_inst_per_zone_update": step_winst_zone,
                              "issue_peak_warp_inst_per_s": 152 * 4 * (clocks.get("sm_mhz") or 2070.0) * 1e6,
                              "floor_ms_per_step": step_winst_zone * cells
                              / (152 * 4 * (clocks.get("sm_mhz") or 2070.0) * 1e6) * 1e3,
                              "frac": step_winst_zone * cells / (152 * 4 * (clocks.get("sm_mhz") or 2070.0) * 1e6)
                              / (ms / args.steps / 1e3),
                              "source": "profiles/mixed_step_blast192.json (smsp__inst_executed.sum at 192^3)"}
                             if step_winst_zone else None),
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                     "limiter": limiter, "traffic": traffic, "traffic_note": traffic_note,
                     "step_frac_algorithmic": value * algo_bytes_zu / (peak * 1e9),
                     "avg_launch_ms": avg_ms, "launches": dom_cnt,
                     "share_of_step": dom_ms / tot if tot else None, "peak_source": PEAK_SRC,
                     "kernels": {k: {"ms": v[0], "launches": v[1]} for k, v in prof.items()}},
        "clocks": clocks,
        "e2e": e2e,
        "gpu_launches": launches * args.steps,
        "floors_in_timed_run": mx_info.get("nfail"),
        "cpu_baseline": cpu,
        "batched_tubes": batch,
        "adjoint": adj,
        "output": outp,
    }
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
