"""Serving form: a request loop with continuous batching over the slots of one ``Batch``.

Requests are independent shock-droplet solves that arrive over time. The server keeps every
admitted solve's state on the device and advances all of them together, ``chunk_steps`` SSP-RK3
steps per persistent-kernel launch (a replayed CUDA graph). Between launches it

* retires the solves that reached their step budget: their ten cell arrays are copied to host
  memory (the request's latency ends when that copy is complete) and their slot and device
  memory are released;
* admits waiting requests in arrival order while a slot is free and the device-memory budget
  (cell arrays, step-start arrays and workspace of every admitted solve) has room for the head of
  the queue; an admitted solve runs the reference's start-up sequence (SC:1998-2007) and gets its
  first dt on the device, then joins the next launch.

A request that arrives while others are on the GPU is therefore admitted as soon as a slot and
memory free up, and its steps overlap with theirs inside the same launches. Every solve's arithmetic
is independent of the others in the launch (each cell of each solve is computed by the same code
from that solve's own arrays, and each solve's dt comes from its own CFL reduction), so a result
is the same alone and in the mix.

``poisson_requests`` makes the serving workload: arrivals of a Poisson process (rate 20/s,
``numpy.random.default_rng(seed)``), grids log-uniform between 64x32 and 2048x1024 (aspect 2:1, nx a
multiple of 8), step counts U[50, 2000], droplet and shock parameters drawn as in the batched
workload (``batch.config3_solves``).

``serve_serial`` serves the same requests one at a time in arrival order through the per-solve
path (``Solver``, one solve on the device at a time, the plain binary64 form by default): the
comparison the serving measurement reports, measured on the same clock as the served run.
``serial_schedule`` gives those latencies from per-request service times instead (a model, for
the host-side tests).
"""
from __future__ import annotations

import collections
import dataclasses
import math
import time

import numpy as np

from .batch import Batch, SolveSpec


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float  # seconds after the start of the serving run
    spec: SolveSpec
    admitted: float | None = None
    finished: float | None = None
    steps_done: int = 0
    result: dict | None = None  # host copies of the ten cell arrays

    @property
    def latency(self) -> float:
        return self.finished - self.arrival

    @property
    def cell_stages(self) -> int:
        return 3 * self.spec.nx * self.spec.ny * self.spec.max_steps


def poisson_requests(n, rate=20.0, seed=0, min_nx=64, max_nx=2048, min_steps=50, max_steps=2000,
                     device="cuda") -> list[Request]:
    """`n` requests; per request the generator draws, in this order: the inter-arrival time
    (exponential, mean 1/rate), nx (log-uniform, rounded to a multiple of 8, ny = nx/2), the droplet
    radius U[0.05, 0.15], its centre U[0.25, 0.4] x U[0.2, 0.3], the shock Mach number U[1.5, 6] and
    the step count U{min_steps..max_steps}. The shock sits at min(0.15, xc - R - 3 dx)."""
    from . import ic

    rng = np.random.default_rng(seed)
    out, t = [], 0.0
    for k in range(n):
        t += float(rng.exponential(1.0 / rate))
        nx = int(round(math.exp(rng.uniform(math.log(min_nx), math.log(max_nx))) / 8.0)) * 8
        nx = min(max(nx, min_nx), max_nx)
        ny = nx // 2
        radius = float(rng.uniform(0.05, 0.15))
        xc, yc = float(rng.uniform(0.25, 0.4)), float(rng.uniform(0.2, 0.3))
        mach = float(rng.uniform(1.5, 6.0))
        steps = int(rng.integers(min_steps, max_steps + 1))
        dx = 1.0 / nx
        x_shock = min(0.15, xc - radius - 3.0 * dx)

        def make(nx=nx, ny=ny, xc=xc, yc=yc, r=radius, m=mach, xs=x_shock):
            return ic.shock_droplet(nx, ny, 1.0, 0.5, mach=m, xc=xc, yc=yc, radius=r, x_shock=xs,
                                    device=device)

        spec = SolveSpec(nx=nx, ny=ny, dx=dx, dy=0.5 / ny, max_steps=steps, make_state=make)
        out.append(Request(rid=k, arrival=t, spec=spec))
    return out


class Admission:
    """First-come-first-served admission by free slots and a device-memory budget in bytes."""

    def __init__(self, slots: int, budget_bytes: float):
        self.slots = int(slots)
        self.budget = float(budget_bytes)
        self.in_use = 0
        self.bytes = 0
        self.peak_bytes = 0
        self.blocked_by_slots = 0   # launch rounds in which the head of the queue waited for a slot
        self.blocked_by_budget = 0  # ... had a free slot but waited for budget

    def note_refusal(self, nbytes: int):
        """Count why the head of the queue was not admitted (slots take precedence)."""
        if self.in_use >= self.slots:
            self.blocked_by_slots += 1
        elif self.bytes + nbytes > self.budget:
            self.blocked_by_budget += 1

    def fits_at_all(self, nbytes: int) -> bool:
        return nbytes <= self.budget

    def can_admit(self, nbytes: int) -> bool:
        return self.in_use < self.slots and self.bytes + nbytes <= self.budget

    def admit(self, nbytes: int):
        if not self.can_admit(nbytes):
            raise RuntimeError("admission over the slot count or the memory budget")
        self.in_use += 1
        self.bytes += nbytes
        self.peak_bytes = max(self.peak_bytes, self.bytes)

    def release(self, nbytes: int):
        self.in_use -= 1
        self.bytes -= nbytes


def serial_schedule(arrivals, service) -> list[float]:
    """Finish times of requests served one at a time in arrival order: f_k = max(a_k, f_{k-1}) + s_k."""
    out, f = [], -math.inf
    for a, s in zip(arrivals, service):
        f = max(a, f) + s
        out.append(f)
    return out


def percentile(values, q) -> float:
    return float(np.percentile(np.asarray(values, dtype=np.float64), q))


class Server:
    """Continuous batching over the slots of one Batch (see the module docstring)."""

    def __init__(self, capacity=32, budget_bytes=150e9, precision="fp32", chunk_steps=10,
                 shapes=None, keep_results=True, device=None, batch=None, **scheme):
        self.batch = batch if batch is not None else Batch(capacity, precision=precision, device=device, **scheme)
        for cls, sh in (shapes or {}).items():
            self.batch.set_shape(int(cls), int(sh))
        self.admission = Admission(capacity, budget_bytes)
        self.chunk_steps = int(chunk_steps)
        self.keep_results = keep_results
        self.launches = 0

    def close(self):
        self.batch.close()

    def run(self, requests, clock=time.perf_counter, sleep=time.sleep) -> dict:
        """Serve `requests` (arrival times relative to the start of this call) to completion and
        return the run's summary; each request gets its admission and finish times and result."""
        for r in requests:
            if r.spec.max_steps < 1:
                raise ValueError("a served solve needs a step budget")
            if not self.admission.fits_at_all(self.batch.bytes_for(r.spec.nx, r.spec.ny)):
                raise ValueError(f"request {r.rid} needs more memory than the whole budget")
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        waiting = collections.deque()
        active = {}  # slot -> (request, bytes)
        t0 = clock()
        busy = 0.0
        while pending or waiting or active:
            now = clock() - t0
            while pending and pending[0].arrival <= now:
                waiting.append(pending.popleft())
            while waiting:
                nbytes = self.batch.bytes_for(waiting[0].spec.nx, waiting[0].spec.ny)
                if not self.admission.can_admit(nbytes):
                    self.admission.note_refusal(nbytes)
                    break
                r = waiting.popleft()
                slot = self.batch.add(r.spec)
                self.admission.admit(nbytes)
                r.admitted = clock() - t0
                active[slot] = (r, nbytes)
            if not active:
                if pending:
                    sleep(max(0.0, pending[0].arrival - (clock() - t0)))
                continue
            c0 = clock()
            self.batch.run(self.chunk_steps)
            st = self.batch.status()  # waits for the launch
            busy += clock() - c0
            self.launches += 1
            for slot in [s for s in active if st[s]["done"]]:
                r, nbytes = active.pop(slot)
                entry = self.batch.remove(slot)
                host = {k: v.to("cpu") for k, v in entry["q"].items()}  # blocking device->host copies
                r.finished = clock() - t0
                r.steps_done = st[slot]["steps"]
                r.result = host if self.keep_results else None
                self.admission.release(nbytes)
                del entry
        return summarize(requests, busy)


def serve_serial(requests, precision="fp64", keep_results=False, device=None, clock=time.perf_counter,
                 sleep=time.sleep, variant="sc", recon="mp5c6", cfl=0.4) -> dict:
    """Serve `requests` one at a time in arrival order through the per-solve path: for each, wait
    for its arrival if the GPU is idle, allocate a Solver and its state, run the start-up sequence
    and its step budget with the dt on the device, copy the ten cell arrays to host memory (the
    request's latency ends there) and free the device memory. Returns the run's summary."""
    import torch

    from .params import SolverParams
    from .solver import FIELDS, Solver, alloc_state

    t0 = clock()
    for r in sorted(requests, key=lambda r: r.arrival):
        wait = r.arrival - (clock() - t0)
        if wait > 0:
            sleep(wait)
        sp = r.spec
        p = SolverParams(dx=sp.dx, dy=sp.dy, gamma1=sp.gamma1, pinf1=sp.pinf1, gamma2=sp.gamma2,
                         pinf2=sp.pinf2, bc=tuple(sp.bc), variant=variant, recon=recon, cfl=cfl,
                         precision=precision)
        r.admitted = clock() - t0
        s = Solver(p, sp.nx, sp.ny, device=device)
        src = sp.state if sp.state is not None else sp.make_state()
        q = alloc_state(sp.nx, sp.ny, device=s.device)
        for k in q:
            q[k].copy_(src[k])
        old = alloc_state(sp.nx, sp.ny, device=s.device, names=FIELDS)
        s.initialize(q)
        s.init_dt(q)
        for _ in range(sp.max_steps):
            s.step(q, old, None, sync=False)
        host = {k: v.to("cpu") for k, v in q.items()}  # blocking device->host copies
        r.finished = clock() - t0
        r.steps_done = sp.max_steps
        r.result = host if keep_results else None
        s.close()
        del s, q, old, src
    torch.cuda.synchronize()
    return summarize(requests)


def summarize(requests, busy_s=None) -> dict:
    lat = [r.latency for r in requests]
    first = min(r.arrival for r in requests)
    last = max(r.finished for r in requests)
    work = sum(3 * r.spec.nx * r.spec.ny * r.steps_done for r in requests)
    out = {"requests": len(requests), "p50_s": round(percentile(lat, 50), 4),
           "p99_s": round(percentile(lat, 99), 4), "mean_s": round(float(np.mean(lat)), 4),
           "makespan_s": round(last - first, 4),
           "value": round(work / (last - first) / 1e6, 3), "unit": "Mcell-stage/s",
           "cell_stages": int(work)}
    if busy_s is not None:
        out["gpu_busy_s"] = round(busy_s, 4)
    return out
