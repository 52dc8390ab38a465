#!/usr/bin/env python3
"""Benchmark of the per-stage RHS on the gas-gas triple point, 7168 x 3072 cells.

Workload (the headline configuration): fluid 1 gamma 1.5 for x < 1 and for x >= 1, y >= 1.5,
fluid 2 gamma 1.4 for x >= 1, y < 1.5, both p_inf = 0, on [0,7] x [0,3] with 7168 x 3072 cells and
5 ghost layers; slip (reflective) walls on all four sides; SC scheme with MP5 + THINC +
central-6 reconstruction; CFL 0.4. Data are synthetic (the analytic initial state; the reference
publishes no dataset). A step is one SSP-RK3 step = three RHS stages over the whole grid.

Reported (one JSON line from rank 0):
  value        Mcell-stage/s over all ranks, device-timed with CUDA events around K steps whose
               state (1.8 GB) is already in HBM; the state is larger than L2, so no flush is needed.
  e2e          the same metric through the C ABI with the conserved state (six cell arrays) in
               pinned host memory: every step copies it host->device, rebuilds the primitives on
               the device (update_prims), runs the step and copies the new state back.
  roofline     algorithmic bytes of a stage (128 B per cell-stage: read the stage state and the
               step-start state, write the new state, averaged over the three stages) divided by
               the measured stage time, against the measured HBM copy bandwidth.
  fp64         the face-sweep kernels' binary64 throughput against the device's measured FP64
               FMA peak (GB300's FP64 rate bounds the plain form, not HBM).
  cpu_baseline the CPU oracle (C restatement of the reference kernels, OpenMP on every host core)
               on the same 7168 x 3072 grid, for a bounded number of steps (about 12 s).
With --impl reference the script times that CPU implementation alone (the reference's own path is
NVIDIA Warp, which is not installable here) and prints its line with "impl": "reference".
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "wave-multiphase_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

NX, NY, G = 7168, 3072, 5
WORKLOAD = f"triple_point_{NX}x{NY}"
ALG_BYTES_PER_CELL_STAGE = 128.0     # read stage state + step-start state, write new state (avg)
# Face-sweep binary64 work per face (x or y) and DRAM traffic per cell-stage, from the ncu captures
# summarised in profiles/ (2048 x 1024 triple point, one kernel per capture): 577 binary64 FLOP per
# face (DFMA x 2 + DADD + DMUL over the launch's faces, the face-sweep summary), and the per-kernel
# DRAM bytes of one stage summed (the DRAM-traffic summary).
FP64_FLOP_PER_FACE = 577.3
DRAM_BYTES_PER_CELL_STAGE_FP32 = 869.0
DRAM_BYTES_PER_CELL_STAGE = 1255.0


def params(nx=None, ny=None, precision="fp64"):
    import wavemp

    nx, ny = nx or NX, ny or NY
    return wavemp.SolverParams(dx=7.0 / nx, dy=3.0 / ny, gamma1=1.5, pinf1=0.0, gamma2=1.4,
                               pinf2=0.0, variant="sc", recon="mp5c6", bc=("slip",) * 4, cfl=0.4,
                               precision=precision)


LIMITER_IN_PLACE = None  # the per-solve fused stage's limiter form (--limiter; None: the default)


def time_form(precision, steps, warmup, dev, fp64_switches=True):
    """Device-timed steps of one form on the workload; returns (ms, kernel-group profile)."""
    import torch

    import wavemp

    p = params(precision=precision)
    p.fp64_switches = fp64_switches
    s = wavemp.Solver(p, NX, NY)
    if LIMITER_IN_PLACE is not None:
        s.set_limiter_sweeps(LIMITER_IN_PLACE)
    q = wavemp.ic.triple_point(NX, NY, device=dev)
    old = wavemp.alloc_state(NX, NY, names=wavemp.FIELDS, device=dev)
    s.initialize(q)
    s.init_dt(q)
    for _ in range(warmup):
        s.step(q, old, None, sync=False)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.profile(True)
    s.profile_read(reset=True)
    e0.record(stream)
    for _ in range(steps):
        s.step(q, old, None, sync=False)
    e1.record(stream)
    torch.cuda.synchronize()
    prof = s.profile_read(reset=True)
    s.profile(False)
    ms = e0.elapsed_time(e1)
    finite = all(bool(torch.isfinite(q[k]).all()) for k in wavemp.FIELDS)
    del s, q, old
    torch.cuda.empty_cache()
    return ms, prof, finite


def precision_errors(steps, dev):
    """Per-field L1 / Linf difference of the precision form from the plain binary64 form after
    `steps` steps from the same state with the same dt (interior cells, relative to the binary64
    field's L1 norm and max)."""
    import torch

    import wavemp

    out = {}
    solvers = {}
    for prec in ("fp64", "fp32"):
        s = wavemp.Solver(params(precision=prec), NX, NY)
        q = wavemp.ic.triple_point(NX, NY, device=dev)
        old = wavemp.alloc_state(NX, NY, names=wavemp.FIELDS, device=dev)
        s.initialize(q)
        solvers[prec] = (s, q, old)
    dt = solvers["fp64"][0].get_dt(solvers["fp64"][1])
    for _ in range(steps):
        for prec in ("fp64", "fp32"):
            s, q, old = solvers[prec]
            s.step(q, old, dt, sync=False)
    torch.cuda.synchronize()
    a, b = solvers["fp32"][1], solvers["fp64"][1]
    sl = (slice(G, -G), slice(G, -G))
    rho_a = (a["ar1"] + a["ar2"])[sl]
    rho_b = (b["ar1"] + b["ar2"])[sl]
    pairs = [("rho", rho_a, rho_b)] + [(k, a[k][sl], b[k][sl]) for k in ("ar1", "ar2", "ru", "rv", "E", "al", "p_p")]
    mom = b["ru"][sl].abs() + b["rv"][sl].abs()
    for k, x, y in pairs:
        d = (x - y).abs()
        ref = mom if k in ("ru", "rv") else y.abs()  # momenta against the momentum magnitude
        out[k] = {"l1": float(d.sum() / ref.sum().clamp_min(1e-300)),
                  "linf": float(d.max() / ref.max().clamp_min(1e-300))}
    del solvers
    torch.cuda.empty_cache()
    return out


def precision_m10(dev, steps, nx=4096, ny=2048):
    """Precision form on the Mach-10 shock-water cylinder (M10 scheme as shipped: MUSCL with THINC
    always on the entropy field, staged Wong limiter; water gamma 4.4 / p_inf 6e8, air 1.4; disk R 0.1
    at (0.3, 0.25) in [0,1] x [0,0.5]; transmissive sides; CFL 0.4): `steps` steps of the binary64
    and binary32 forms in lockstep on the binary64 run's dt sequence, then per-field L1 / Linf of
    the binary32 result against the binary64 one (interior cells)."""
    import torch

    import wavemp

    kw = dict(dx=1.0 / nx, dy=0.5 / ny, gamma1=4.4, pinf1=6.0e8, gamma2=1.4, pinf2=0.0,
              bc=("transmissive",) * 4, variant="m10", recon="shipped", cfl=0.4)
    q0 = wavemp.ic.shock_droplet(nx, ny, 1.0, 0.5, mach=10.0, device=dev)
    runs = {}
    for prec in ("fp64", "fp32"):
        s = wavemp.Solver(wavemp.SolverParams(precision=prec, **kw), nx, ny, device=dev)
        q = {k: v.clone() for k, v in q0.items()}
        old = wavemp.alloc_state(nx, ny, names=wavemp.FIELDS, device=dev)
        s.initialize(q)
        runs[prec] = (s, q, old)
    del q0
    stream = torch.cuda.current_stream()
    s64, q64, old64 = runs["fp64"]
    s32, q32, old32 = runs["fp32"]
    dt = s64.get_dt(q64)
    events = []
    t_end = 0.0
    for _ in range(steps):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record(stream)
        dt_next = s64.step(q64, old64, dt, sync=True)  # waits: the next dt of the binary64 run
        ev[1].record(stream)
        s32.step(q32, old32, dt, sync=False)
        ev[2].record(stream)
        events.append(ev)
        t_end += dt
        dt = dt_next
    torch.cuda.synchronize()
    ms = {"fp64": sum(e[0].elapsed_time(e[1]) for e in events),
          "fp32": sum(e[1].elapsed_time(e[2]) for e in events)}
    a, b = runs["fp32"][1], runs["fp64"][1]
    sl = (slice(G, -G), slice(G, -G))
    fields = {}
    pairs = [("rho", (a["ar1"] + a["ar2"])[sl], (b["ar1"] + b["ar2"])[sl])]
    pairs += [(k, a[k][sl], b[k][sl]) for k in ("ar1", "ar2", "ru", "rv", "E", "al", "p_p")]
    mom = (b["ru"][sl].abs() + b["rv"][sl].abs())
    for k, x, y in pairs:
        d = (x - y).abs()
        # momenta relative to the momentum magnitude: rv is zero by symmetry before the shock
        # reaches the cylinder, so its own norm is no scale
        ref = mom if k in ("ru", "rv") else y.abs()
        fields[k] = {"l1": float(d.sum() / ref.sum().clamp_min(1e-300)),
                     "linf": float(d.max() / ref.max().clamp_min(1e-300))}
    finite = all(bool(torch.isfinite(r[1][k]).all()) for r in runs.values() for k in wavemp.FIELDS)
    cs = nx * ny * 3 * steps
    out = {"workload": f"mach10_cylinder_{nx}x{ny}, M10 scheme as shipped, {steps} steps",
           "t_end": t_end, "finite": finite,
           "fp64": {"value": round(cs / (ms["fp64"] * 1e-3) / 1e6, 3), "unit": "Mcell-stage/s"},
           "fp32": {"value": round(cs / (ms["fp32"] * 1e-3) / 1e6, 3), "unit": "Mcell-stage/s"},
           "dt": "the binary64 run's own CFL 0.4 sequence, used by both forms",
           "error_fp32_vs_fp64": fields}
    del runs
    torch.cuda.empty_cache()
    return out


def batched_form(dev, steps, warmup, n=64, sensitivity_eps=0.0):
    """Batched form on the batched workload (64 shock-droplet solves, grids log-uniform 128x64 to
    1024x512, seed 0): `steps` SSP-RK3 steps of every solve in persistent launches, binary64 and
    binary32 forms after the tile-shape autotuner, against the same solves stepped one after the
    other through the plain binary64 per-solve path. Returns (summary, tuned shapes of the
    binary32 batch)."""
    import torch

    import wavemp
    from wavemp.batch import Batch, config3_solves

    specs = config3_solves(n=n, seed=0, steps=0, device=dev)
    cells = sum(sp.nx * sp.ny for sp in specs)
    stream = torch.cuda.current_stream()
    out, batches, shapes32 = {}, {}, {}
    # the binary64 batch records every solve's dt sequence; the binary32 batch replays it, so
    # that the two differ by their arithmetic alone (not by a drift of their time steps)
    logs = [torch.zeros(warmup + steps + 8, dtype=torch.float64, device=dev) for _ in specs]

    def density_l1(qa, qb):
        ra, rb = (qa["ar1"] + qa["ar2"])[5:-5, 5:-5], (qb["ar1"] + qb["ar2"])[5:-5, 5:-5]
        return float((ra - rb).abs().sum() / rb.abs().sum())

    for prec in ("fp64", "fp32", "fp32_switches32"):
        b = Batch(n, precision=prec[:4], device=dev, fp64_switches=not prec.endswith("switches32"))
        for sp, log in zip(specs, logs):
            b.add(sp, dt_log=log, dt_mode="record" if prec == "fp64" else "replay")
        t0 = time.perf_counter()
        report = b.autotune(steps=1, repeats=2)
        tune_s = time.perf_counter() - t0
        b.run(warmup)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.run(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        graph_used = b.info()["graph"]
        b.profile(True)  # a separate short run with per-phase timing
        b.profile_read(reset=True)
        b.run(2)
        phases = b.profile_read(reset=True)
        b.profile(False)
        tot = sum(phases.values())
        st = b.status()
        info = b.info()
        ok = all(x["steps"] == warmup + steps + 2 for x in st[:n])
        out[prec] = {"value": round(cells * 3 * steps / (ms * 1e-3) / 1e6, 3), "unit": "Mcell-stage/s",
                     "ms_per_step": round(ms / steps, 3), "graph": graph_used, "tiles": info["tiles"],
                     "grid": info["grid"], "steps_ok": ok, "autotune_s": round(tune_s, 2),
                     "shapes": {str(c): int(v[0]) for c, v in report.items()},
                     "phases": {k: {"ms_per_step": round(v / 2, 3), "share": round(v / max(tot, 1e-9), 4)}
                                for k, v in phases.items()}}
        batches[prec] = b
        if prec == "fp32":
            shapes32 = {c: int(v[0]) for c, v in report.items()}
        if prec != "fp64":
            l1 = [density_l1(b.slots[k]["q"], batches["fp64"].slots[k]["q"]) for k in range(n)]
            num = den = 0.0
            for k in range(n):
                qa, qb = b.slots[k]["q"], batches["fp64"].slots[k]["q"]
                ra, rb = (qa["ar1"] + qa["ar2"])[5:-5, 5:-5], (qb["ar1"] + qb["ar2"])[5:-5, 5:-5]
                num += float((ra - rb).abs().sum())
                den += float(rb.abs().sum())
            out[prec]["density_l1_vs_fp64"] = {"max": max(l1), "median": float(sorted(l1)[len(l1) // 2]),
                                              "solves_within_1e-5": sum(v <= 1e-5 for v in l1),
                                              "all_solves_together": num / den}
            if prec == "fp32_switches32":  # its memory back before the serial comparison
                b.close()
                del batches[prec]
    # density L1 of the binary32 batch against the binary64 batch after the same number of steps
    l1 = [density_l1(batches["fp32"].slots[k]["q"], batches["fp64"].slots[k]["q"]) for k in range(n)]
    worst = max(l1)
    sensitivity = None
    if sensitivity_eps:
        # conditioning of the solves themselves: the binary64 batch again, from initial partial
        # densities perturbed by a relative sensitivity_eps (seeded), on the same dt sequence
        def perturbed(sp, k):
            def make():
                st = sp.make_state()
                gen = torch.Generator().manual_seed(1000 + k)
                noise = torch.randn(tuple(st["ar1"].shape), generator=gen, dtype=torch.float64)
                st["ar1"] = st["ar1"] * (1.0 + sensitivity_eps * noise.to(st["ar1"].device))
                return st
            return dataclasses.replace(sp, state=None, make_state=make)

        bp = Batch(n, precision="fp64", device=dev)
        for k, (sp, log) in enumerate(zip(specs, logs)):
            bp.add(perturbed(sp, k), dt_log=log, dt_mode="replay")
        bp.run(warmup + steps + 2)
        torch.cuda.synchronize()
        l1p = [density_l1(bp.slots[k]["q"], batches["fp64"].slots[k]["q"]) for k in range(n)]
        bp.close()
        order = sorted(range(n), key=lambda k: -l1[k])[:4]
        sensitivity = {"relative_perturbation": sensitivity_eps,
                       "density_l1_fp64_perturbed_vs_fp64_max": max(l1p),
                       "density_l1_fp64_perturbed_vs_fp64_median": float(sorted(l1p)[len(l1p) // 2]),
                       "largest_fp32_errors_with_their_fp64_sensitivity":
                           [{"solve": k, "grid": f"{specs[k].nx}x{specs[k].ny}", "fp32_vs_fp64": l1[k],
                             "fp64_perturbed_vs_fp64": l1p[k]} for k in order]}
    for b in batches.values():
        b.close()
    del batches
    torch.cuda.empty_cache()
    # serial plain binary64: each solve alone through the per-solve path, same step count
    total_ms = 0.0
    for sp in specs:
        p = wavemp.SolverParams(dx=sp.dx, dy=sp.dy, gamma1=sp.gamma1, pinf1=sp.pinf1, bc=sp.bc,
                                recon="mp5c6", variant="sc", cfl=0.4)
        s = wavemp.Solver(p, sp.nx, sp.ny, device=dev)
        q = sp.make_state()
        old = wavemp.alloc_state(sp.nx, sp.ny, names=wavemp.FIELDS, device=dev)
        s.initialize(q)
        s.init_dt(q)
        for _ in range(min(warmup, 2)):
            s.step(q, old, None, sync=False)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            s.step(q, old, None, sync=False)
        e1.record(stream)
        torch.cuda.synchronize()
        total_ms += e0.elapsed_time(e1)
        s.close()
    serial = cells * 3 * steps / (total_ms * 1e-3) / 1e6
    summary = {
        "workload": f"{n} shock-droplet solves, grids log-uniform 128x64..1024x512 (seed 0), "
                    f"{cells} cells in all; {steps} steps timed after {warmup} warm-up",
        "batched_fp64": out["fp64"], "batched_fp32": out["fp32"],
        "batched_fp32_switches32": out["fp32_switches32"],
        "serial_plain_fp64": {"value": round(serial, 3), "unit": "Mcell-stage/s",
                              "ms_per_step": round(total_ms / steps, 3)},
        "speedup_fp32_vs_serial_plain": round(out["fp32"]["value"] / serial, 3),
        "speedup_fp64_vs_serial_plain": round(out["fp64"]["value"] / serial, 3),
        "density_l1_fp32_vs_fp64_max_over_solves": worst,
        "density_l1_fp32_vs_fp64_median": float(sorted(l1)[len(l1) // 2]),
        "solves_within_1e-5": sum(v <= 1e-5 for v in l1),
        "error_note": "the binary32 batch replays the binary64 batch's dt sequence",
    }
    if sensitivity is not None:
        summary["conditioning"] = sensitivity
    return summary, shapes32


def served_form(dev, nreq, shapes=None, capacity=16, chunk_steps=10, budget_gb=150.0, tight_gb=1.0):
    """Serving form on the serving workload (Poisson arrivals at 20/s, seed 0, grids log-uniform
    64x32 to 2048x1024, step counts U[50, 2000], binary32 form): p50/p99 latency (arrival to result
    on the host) and cell-stage/s with the 150 GB admission budget, again with a budget small enough
    that memory rather than the slots limits admission, and -- measured on the same clock -- the same
    requests served one at a time in arrival order by the plain binary64 per-solve path."""
    import torch

    from wavemp.serve import Server, poisson_requests, serve_serial

    out = {"workload": f"{nreq} requests, Poisson 20/s (seed 0), grids 64x32..2048x1024, "
                       f"steps U[50,2000], binary32 form"}
    for key, budget in (("served_fp32", budget_gb), ("served_fp32_budget_bound", tight_gb)):
        reqs = poisson_requests(nreq, rate=20.0, seed=0, device=dev)
        srv = Server(capacity=capacity, budget_bytes=budget * 1e9, precision="fp32",
                     chunk_steps=chunk_steps, shapes=shapes, keep_results=False, device=dev)
        res = srv.run(reqs)
        res.update({"slots": capacity, "chunk_steps": chunk_steps, "budget_gb": budget,
                    "peak_admitted_gb": round(srv.admission.peak_bytes / 1e9, 3), "launches": srv.launches,
                    "rounds_waiting_for_slot": srv.admission.blocked_by_slots,
                    "rounds_waiting_for_budget": srv.admission.blocked_by_budget})
        srv.close()
        torch.cuda.empty_cache()
        out[key] = res
    reqs = poisson_requests(nreq, rate=20.0, seed=0, device=dev)
    serial = serve_serial(reqs, precision="fp64", device=dev)
    serial["how"] = "measured: one request at a time through the per-solve plain binary64 path"
    torch.cuda.empty_cache()
    served = out["served_fp32"]
    out["serial_plain_fp64"] = serial
    out["speedup_vs_serial_plain"] = round(served["value"] / serial["value"], 3)
    out["p50_ratio_serial_over_served"] = round(serial["p50_s"] / served["p50_s"], 3)
    out["p99_ratio_serial_over_served"] = round(serial["p99_s"] / served["p99_s"], 3)
    return out


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# --------------------------------------------------------------------------- replicas --------
def max_over_ranks(x, world, device="cpu"):
    """Largest value of x over the ranks (the slowest replica sets the whole job's time)."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(cells_per_rank, steps, world, ms):
    """Mcell-stage/s of all replicas together: every rank advances its own solve `steps` steps of
    three stages each, and the job takes the slowest rank's `ms`."""
    return cells_per_rank * 3 * steps * world / (ms * 1e-3) / 1e6


# ------------------------------------------------------------------------------ clocks ------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.gpu = gpu_index
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons)}


# ------------------------------------------------------------------------- CPU oracle -------
def cpu_oracle_rate(nx, ny, steps=None, seconds=12.0, warmup=1):
    """Mcell-stage/s of the CPU oracle (all host cores) on the same problem at nx x ny: `warmup`
    untimed steps (page-in, thread start), then `steps` timed steps, or as many as fit in
    `seconds` when steps is None."""
    import numpy as np

    import wavemp
    from oracle import oracle as orc

    st = wavemp.ic.triple_point(nx, ny, device="cpu")
    P = orc.make_params(7.0 / nx, 3.0 / ny, 1.5, 0.0, 1.4, 0.0, variant=orc.SC, recon=orc.MP5C6,
                        bc=[orc.SLIP] * 4, cfl=0.4)
    o = orc.PackedOracle(nx, ny, P)
    for c, k in enumerate(orc.ALL10):
        o.fields[c][...] = st[k].numpy()
    del st
    o.init_sequence()
    dt = o.get_dt()
    for _ in range(max(warmup, 1)):
        dt = o.steps(1, dt)
    done, t0 = 0, time.perf_counter()
    while True:
        dt = o.steps(1, dt)
        done += 1
        el = time.perf_counter() - t0
        if (steps is not None and done >= steps) or (steps is None and el >= seconds):
            break
    assert np.isfinite(dt)
    return nx * ny * 3 * done / el / 1e6, done, el


def run_reference(args):
    """The reference arm: the CPU implementation of the path (the oracle, a C restatement of the
    reference's kernels pinned bit-exact to their source) on the benchmark's own 7168 x 3072 grid,
    every host core, W untimed then K timed SSP-RK3 steps."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import oracle as orc

    orc.build()
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    warm = max(args.warmup, 1)
    rate, steps, el = cpu_oracle_rate(NX, NY, steps=args.steps, warmup=warm)
    sample = f"the whole {NX}x{NY} grid, {steps} SSP-RK3 steps after {warm} warm-up"
    line = {
        "impl": "reference", "metric": "Mcell-stage/s", "value": round(rate, 3),
        "unit": "Mcell-stage/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(el / steps * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "nx": NX, "ny": NY,
                   "scheme": "SC, MP5 + THINC + central-6", "form": "plain binary64",
                   "step": "one SSP-RK3 step (3 RHS stages)"},
        "cpu_baseline": {"value": round(rate, 3), "unit": "Mcell-stage/s", "cores": int(os.environ["OMP_NUM_THREADS"]),
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(rate, 3), "unit": "Mcell-stage/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "the reference's own path is NVIDIA Warp (not installable offline); the CPU oracle "
                "restates its kernels and is pinned bit-exact to the reference's kernel source",
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------------------ GPU ---------
def run_ours(args):
    import torch
    import torch.distributed as dist

    import wavemp

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    def barrier():
        if world > 1:
            dist.barrier()

    if args.form in ("batched", "serve", "m10"):
        if args.form == "m10":
            res = precision_m10(dev, args.m10_steps)
            value = res["fp32"]["value"]
        elif args.form == "batched":
            res, _ = batched_form(dev, args.batch_steps, args.warmup, sensitivity_eps=args.batch_sensitivity)
            value = res["batched_fp32"]["value"]
        else:
            res = served_form(dev, args.serve_requests, capacity=args.serve_slots, chunk_steps=args.serve_chunk)
            value = res["served_fp32"]["value"]
        if rank == 0:
            print(json.dumps({"metric": "Mcell-stage/s", "value": value, "unit": "Mcell-stage/s",
                              "form": args.form, **res}), flush=True)
        return 0
    if args.form == "fp32":
        ms32, prof32, finite32 = time_form("fp32", args.steps, args.warmup, dev)
        v32 = NX * NY * 3 * args.steps / (ms32 * 1e-3) / 1e6
        if rank == 0:
            print(json.dumps({"metric": "Mcell-stage/s", "value": round(v32, 3), "unit": "Mcell-stage/s",
                              "form": "precision_fp32", "workload": WORKLOAD, "finite": finite32,
                              "kernels": {g: [round(t, 3), n] for g, (t, n) in prof32.items()}}), flush=True)
        return 0
    fp64_peak = wavemp.probe_fp64_flops()
    s = wavemp.Solver(params(), NX, NY)
    if LIMITER_IN_PLACE is not None:
        s.set_limiter_sweeps(LIMITER_IN_PLACE)
    q = wavemp.ic.triple_point(NX, NY, device=dev)
    old = wavemp.alloc_state(NX, NY, names=wavemp.FIELDS, device=dev)
    s.initialize(q)
    s.init_dt(q)
    for _ in range(args.warmup):
        s.step(q, old, None, sync=False)
    torch.cuda.synchronize()

    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    time.sleep(0.4)
    s.profile(True)
    s.profile_read(reset=True)
    barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        s.step(q, old, None, sync=False)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    prof = s.profile_read(reset=True)
    s.profile(False)
    clk = clocks.stop()
    dt_now = s.get_dt(q)
    finite = all(bool(torch.isfinite(q[k]).all()) for k in wavemp.FIELDS) and dt_now > 0
    ms = max_over_ranks(ms, world, dev)
    cells = NX * NY
    value = whole_job_rate(cells, args.steps, world, ms)
    ms_step = ms / args.steps
    launches = sum(n for _, n in prof.values())

    # ---- end to end through the C ABI with host buffers ----
    # The caller holds the conserved state (the six cell arrays the scheme advances) in one pinned
    # host buffer. Every step copies it to the device (one copy: the six arrays are contiguous in the
    # device state block, alloc_state's layout), rebuilds the primitives there (update_prims, as
    # every step does at its end), runs the step and copies the new conserved state back. The
    # copies are the library's own (copy_state: the SMs read and write the pinned buffer in place).
    nf = len(wavemp.FIELDS)
    qb = wavemp.alloc_state(NX, NY, device=dev)
    for k in wavemp.ALL:
        qb[k].copy_(q[k])
    nxg, nyg = NX + 2 * G, NY + 2 * G
    blk = torch.as_strided(qb["ar1"], (nf, nxg, nyg), (nxg * nyg, nyg, 1))
    assert all(blk[c].data_ptr() == qb[k].data_ptr() for c, k in enumerate(wavemp.FIELDS))
    host = torch.empty((nf, NX + 2 * G, NY + 2 * G), dtype=torch.float64, pin_memory=True)
    host.copy_(blk)
    del q
    q = qb
    torch.cuda.synchronize()
    ke = max(3, args.steps)
    h2d = host.numel() * 8
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(ke):
        wavemp.copy_state(blk, host)
        s.update_prims(q)
        s.step(q, old, None, sync=False)
        wavemp.copy_state(host, blk)
    f1.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ms_e2e = max(f0.elapsed_time(f1), wall * 1e3)
    ms_e2e = max_over_ranks(ms_e2e, world, dev)
    e2e_value = whole_job_rate(cells, ke, world, ms_e2e)

    # ---- roofline and FP64 rate ----
    hbm, hbm_kind = measured_peaks()
    stage_ms = ms_step / 3.0
    achieved = ALG_BYTES_PER_CELL_STAGE * cells / (stage_ms * 1e-3) / 1e9
    face_ms, face_n = prof["faces"]
    face_ms_per_launch = face_ms / max(face_n, 1)
    faces_per_stage = (NX + 1) * NY + NX * (NY + 1)
    fp64 = {"peak": round(fp64_peak / 1e12, 4), "unit": "TFLOP/s", "peak_kind": "measured (DFMA loop)",
            "face_sweep_ms_per_stage": round(face_ms / max(face_n / 2, 1), 3)}
    if FP64_FLOP_PER_FACE:
        fl = FP64_FLOP_PER_FACE * faces_per_stage / (face_ms / max(face_n / 2, 1) * 1e-3)
        fp64.update({"achieved": round(fl / 1e12, 4), "frac": round(fl / fp64_peak, 4)})
    roof = {"bound": "hbm", "achieved": round(achieved, 2), "peak": hbm, "unit": "GB/s",
            "frac": round(achieved / hbm, 5), "peak_kind": hbm_kind,
            "traffic": (round(DRAM_BYTES_PER_CELL_STAGE * cells / 1e9, 3) if DRAM_BYTES_PER_CELL_STAGE else None),
            "unit_of_work": "one RHS stage over all cells (128 B algorithmic per cell-stage)",
            "stage_ms": round(stage_ms, 3)}

    kernels = {g: {"ms_per_launch": round(t / max(n, 1), 4), "launches": n,
                   "share": round(t / max(sum(v[0] for v in prof.values()), 1e-9), 4)}
               for g, (t, n) in prof.items()}
    line = {
        "metric": "Mcell-stage/s", "value": round(value, 3), "unit": "Mcell-stage/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "nx": NX, "ny": NY, "ghost": G,
                   "scheme": "SC, MP5 + THINC + central-6", "form": "plain binary64",
                   "bc": "slip walls on four sides", "step": "one SSP-RK3 step (3 RHS stages)",
                   "l2": "state of 1.8 GB is larger than L2; no flush", "parallelism": "replicas"},
        "roofline": roof, "fp64": fp64,
        "e2e": {"value": round(e2e_value, 3), "unit": "Mcell-stage/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": h2d, "steps": ke},
        "gpu_launches": launches, "kernels": kernels, "clocks": clk, "finite": finite,
    }
    # ---- precision form (binary32 face sweep, binary64 recovery / bound solves / accumulation) ----
    del q, old, host, s
    torch.cuda.empty_cache()
    if args.form == "plain":
        if rank == 0:
            print(json.dumps(line), flush=True)
        return 0
    ms32, prof32, finite32 = time_form("fp32", args.steps, args.warmup, dev)
    ms32 = max_over_ranks(ms32, world, dev)
    v32 = whole_job_rate(cells, args.steps, world, ms32)
    err_steps = 10
    line["forms"] = {"precision_fp32": {
        "value": round(v32, 3), "unit": "Mcell-stage/s", "ms_per_step": round(ms32 / args.steps, 3),
        "speedup_vs_plain": round(v32 / value, 3), "finite": finite32,
        "kernels": {g: {"ms_per_launch": round(t / max(n, 1), 4), "launches": n} for g, (t, n) in prof32.items()},
        "error_vs_fp64": {"steps": err_steps, "dt": "fixed, CFL 0.4 of the initial state",
                          "fields": precision_errors(err_steps, dev)},
        "roofline": {"bound": "hbm", "achieved": round(ALG_BYTES_PER_CELL_STAGE * cells / (ms32 / args.steps / 3 * 1e-3) / 1e9, 2),
                     "peak": hbm, "unit": "GB/s",
                     "traffic": round(DRAM_BYTES_PER_CELL_STAGE_FP32 * cells / 1e9, 3),
                     "frac": round(ALG_BYTES_PER_CELL_STAGE * cells / (ms32 / args.steps / 3 * 1e-3) / 1e9 / hbm, 5)},
    }}
    batched, shapes32 = batched_form(dev, args.batch_steps, args.warmup)
    line["forms"]["batched"] = batched
    line["forms"]["served"] = served_form(dev, args.serve_requests, shapes=shapes32,
                                          capacity=args.serve_slots, chunk_steps=args.serve_chunk)
    ms32s, _, finite32s = time_form("fp32", args.steps, args.warmup, dev, fp64_switches=False)
    ms32s = max_over_ranks(ms32s, world, dev)
    v32s = whole_job_rate(cells, args.steps, world, ms32s)
    line["forms"]["precision_fp32_switches32"] = {
        "value": round(v32s, 3), "unit": "Mcell-stage/s", "speedup_vs_plain": round(v32s / value, 3),
        "finite": finite32s,
        "note": "the precision form with its THINC indicator and Ducros sensor in binary32 (faster; "
                "round-off can move a switch decision: not the default)"}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        os.environ.setdefault("OMP_NUM_THREADS", str(cores))
        rate, steps, el = cpu_oracle_rate(NX, NY, seconds=12.0)
        line["cpu_baseline"] = {"value": round(rate, 3), "unit": "Mcell-stage/s",
                                "cores": int(os.environ["OMP_NUM_THREADS"]), "kind": "port",
                                "sample": f"the whole {NX}x{NY} grid, {steps} SSP-RK3 steps in "
                                          f"{el:.1f} s after one warm-up step"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--grid", default=None,
                    help="NXxNY: a smaller case of the same problem (profiling captures only)")
    ap.add_argument("--form", choices=("both", "plain", "fp32", "batched", "serve", "m10"), default="both",
                    help="time one form alone (profiling captures, full-length batched/served runs)")
    ap.add_argument("--batch-steps", type=int, default=300,
                    help="steps of the 64-solve batched workload (the workload is 300 steps)")
    ap.add_argument("--serve-requests", type=int, default=48, help="requests of the serving workload")
    ap.add_argument("--batch-sensitivity", type=float, default=0.0,
                    help="also run the binary64 batch from initial states perturbed by this relative amount")
    ap.add_argument("--m10-steps", type=int, default=500, help="steps of the Mach-10 precision run")
    ap.add_argument("--limiter", choices=("default", "in-place", "deferred"), default="default",
                    help="per-solve fused stage: blend sweeps in place or rebuilt in registers")
    ap.add_argument("--serve-slots", type=int, default=16, help="slots of the serving batch")
    ap.add_argument("--serve-chunk", type=int, default=10, help="steps per serving launch")
    args = ap.parse_args()
    if args.grid:
        global NX, NY, WORKLOAD
        NX, NY = (int(v) for v in args.grid.lower().split("x"))
        WORKLOAD = f"triple_point_{NX}x{NY}"
    global LIMITER_IN_PLACE
    LIMITER_IN_PLACE = None if args.limiter == "default" else args.limiter == "in-place"
    if args.warmup < 3:
        print("note: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
