"""Batched form: many independent solves of uneven grid sizes in one persistent launch.

``Batch`` owns the device memory of its slots (cell arrays, step-start arrays, workspace), drives
``wm_batch_*`` of the C ABI, and carries the tile-shape autotuner. A solve enters a slot with its
initial state (the reference's start-up sequence is run on it, SC:1998-2007) and its own end time
and/or step budget; ``run(n)`` advances every unfinished solve by up to n SSP-RK3 steps in one
persistent kernel launch replayed from a CUDA graph, each solve with its own device-resident dt.

``config3_solves`` generates the benchmark's batched workload: 64 shock-droplet solves on grids
log-uniform between 128x64 and 1024x512 (aspect 2:1, nx a multiple of 8), droplet radius
U[0.05, 0.15], centre U[0.25, 0.4] x U[0.2, 0.3], shock Mach U[1.5, 6], water/air as configuration 0
(seed 0; the shock sits at min(0.15, xc - R - 3 dx) so that it never starts inside the droplet).
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
import time

import numpy as np
import torch

from . import _lib, ic
from .params import SolverParams
from .solver import FIELDS, Solver, _stream, alloc_state

SHAPES = ((1, 128), (2, 64), (4, 32), (8, 16))  # tile rows x columns, 128 cells each


def size_class(nx: int, ny: int) -> int:
    return int(math.floor(math.log2(nx * ny)))


@dataclasses.dataclass
class SolveSpec:
    """One solve of a batch: grid, physics, stopping rule and (optional) initial state."""

    nx: int
    ny: int
    dx: float
    dy: float
    gamma1: float = 4.4
    pinf1: float = 6.0e8
    gamma2: float = 1.4
    pinf2: float = 0.0
    bc: tuple = ("transmissive",) * 4
    t_end: float = 0.0
    max_steps: int = 0
    state: dict | None = None  # ten (nx+2g, ny+2g) float64 tensors; made by `make_state` if None
    make_state: object = None


class Batch:
    def __init__(self, capacity: int, variant="sc", recon="mp5c6", precision="fp64",
                 emergency_repair=True, cfl=0.4, g=5, tile_shape=-1, device=None, fp64_switches=True,
                 spin_limit: int = 0):
        self.L = _lib.load()
        self.g = g
        self.capacity = capacity
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.scheme = dict(variant=variant, recon=recon, precision=precision,
                           emergency_repair=emergency_repair, cfl=cfl, fp64_switches=fp64_switches)
        p = _lib.WmBatchParams()
        p.variant, p.recon = _lib.VARIANT[variant], _lib.RECON[recon]
        p.precision, p.emergency_repair = _lib.PRECISION[precision], int(bool(emergency_repair))
        p.g, p.cfl, p.tile_shape = g, cfl, tile_shape
        p.fp64_switches = int(bool(fp64_switches))
        p.spin_limit = int(spin_limit)  # grid-barrier wait limit (0: the library's default)
        self._p = p
        h = ctypes.c_void_p()
        _lib.check(self.L.wm_batch_create(ctypes.byref(p), capacity, ctypes.byref(h)), "wm_batch_create")
        self._h = h
        self.slots: list[dict | None] = [None] * capacity
        self.tuned: dict[int, int] = {}

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self.L.wm_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- memory ---------------------------------------------------------------------------------
    def bytes_for(self, nx: int, ny: int) -> int:
        """Device bytes one solve of this size occupies (cell arrays + step-start + workspace)."""
        params = SolverParams(dx=1.0, dy=1.0, **self._solver_kw())
        ws = Solver.workspace_bytes(params, nx, ny, self.g)
        return ws + 16 * (nx + 2 * self.g) * (ny + 2 * self.g) * 8

    def _solver_kw(self):
        s = self.scheme
        return dict(variant=s["variant"], recon=s["recon"], precision=s["precision"],
                    emergency_repair=s["emergency_repair"], cfl=s["cfl"], fp64_switches=s["fp64_switches"])

    # -- slots ----------------------------------------------------------------------------------
    def free_slot(self) -> int | None:
        for k, v in enumerate(self.slots):
            if v is None:
                return k
        return None

    def add(self, spec: SolveSpec, slot: int | None = None, dt_log=None, dt_mode: str = "") -> int:
        """Place a solve in a free slot: allocate its memory, run the start-up sequence on its
        state, compute its first dt on the device, and register it with the batch. dt_log: a
        float64 device tensor that records (dt_mode "record") or supplies (dt_mode "replay") the
        dt of every step."""
        if slot is None:
            slot = self.free_slot()
        if slot is None or self.slots[slot] is not None:
            raise RuntimeError("no free slot")
        g = self.g
        params = SolverParams(dx=spec.dx, dy=spec.dy, gamma1=spec.gamma1, pinf1=spec.pinf1,
                              gamma2=spec.gamma2, pinf2=spec.pinf2, bc=tuple(spec.bc), **self._solver_kw())
        nbytes = Solver.workspace_bytes(params, spec.nx, spec.ny, g)
        ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        q = alloc_state(spec.nx, spec.ny, g, device=self.device)
        src = spec.state if spec.state is not None else spec.make_state()
        for k in q:
            q[k].copy_(src[k])
        old = alloc_state(spec.nx, spec.ny, g, device=self.device, names=FIELDS)
        s = Solver(params, spec.nx, spec.ny, g, device=self.device, workspace=ws)
        s.initialize(q)
        s.close()
        d = _lib.WmSolveDesc()
        d.nx, d.ny, d.dx, d.dy = spec.nx, spec.ny, spec.dx, spec.dy
        d.gamma1, d.pinf1, d.gamma2, d.pinf2 = spec.gamma1, spec.pinf1, spec.gamma2, spec.pinf2
        for k, side in enumerate(spec.bc):
            d.bc[k] = _lib.BC[side]
        d.t_end, d.max_steps = float(spec.t_end), int(spec.max_steps)
        d.q = s._fields(q)
        d.q_old = s._fields(old, need_prims=False)
        _lib.check(self.L.wm_batch_set(self._h, slot, ctypes.byref(d), ctypes.c_void_p(ws.data_ptr()), nbytes),
                   "wm_batch_set")
        if dt_mode:
            mode = {"record": 1, "replay": 2}[dt_mode]
            if dt_log is None or dt_log.dtype != torch.float64 or not dt_log.is_cuda:
                raise ValueError("dt_log must be a float64 device tensor")
            _lib.check(self.L.wm_batch_dt_log(self._h, slot, ctypes.c_void_p(dt_log.data_ptr()), dt_log.numel(), mode),
                       "wm_batch_dt_log")
        _lib.check(self.L.wm_batch_init_dt(self._h, slot, _stream()), "wm_batch_init_dt")
        self.slots[slot] = {"spec": spec, "q": q, "old": old, "ws": ws, "dt_log": dt_log}
        return slot

    def remove(self, slot: int) -> dict:
        """Clear a slot; returns its arrays (the caller may keep the final state)."""
        entry = self.slots[slot]
        _lib.check(self.L.wm_batch_clear(self._h, slot), "wm_batch_clear")
        self.slots[slot] = None
        return entry

    # -- running --------------------------------------------------------------------------------
    def run(self, nsteps: int):
        _lib.check(self.L.wm_batch_run(self._h, int(nsteps), _stream()), "wm_batch_run")

    def status(self) -> list[dict]:
        st = (_lib.WmSolveStatus * self.capacity)()
        _lib.check(self.L.wm_batch_query(self._h, st, _stream()), "wm_batch_query")
        return [{"used": bool(x.used), "done": bool(x.done), "t": x.t, "dt": x.dt, "steps": x.steps}
                for x in st]

    def info(self) -> dict:
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _lib.check(self.L.wm_batch_info(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)), "wm_batch_info")
        return {"tiles": a.value, "grid": b.value, "graph": bool(c.value)}

    def profile(self, enable: bool = True):
        """Per-phase device timing of later runs (block 0's clock between grid barriers)."""
        _lib.check(self.L.wm_batch_profile(self._h, int(bool(enable))), "wm_batch_profile")

    def profile_read(self, reset: bool = True) -> dict:
        ms = (ctypes.c_double * len(_lib.BATCH_PHASES))()
        _lib.check(self.L.wm_batch_profile_read(self._h, ctypes.byref(ms), int(reset), _stream()),
                   "wm_batch_profile_read")
        return dict(zip(_lib.BATCH_PHASES, list(ms)))

    def set_spin_limit(self, limit: int = 0):
        """Grid-barrier wait limit of later runs (0: the library's default). A run whose barrier
        wait runs out stops part-way; the next status() raises WavempError (WM_ERR_STATE) and
        clears the condition."""
        _lib.check(self.L.wm_batch_spin_limit(self._h, int(limit)), "wm_batch_spin_limit")

    def set_shape(self, cls: int, shape: int):
        _lib.check(self.L.wm_batch_tile_shape(self._h, int(cls), int(shape)), "wm_batch_tile_shape")

    # -- autotuner ------------------------------------------------------------------------------
    def _snapshot(self):
        scal = (ctypes.c_ubyte * (self.capacity * 40))()
        _lib.check(self.L.wm_batch_scalars(self._h, scal, 0, _stream()), "wm_batch_scalars")
        fields = {k: ({n: t.clone() for n, t in e["q"].items()}, {n: t.clone() for n, t in e["old"].items()})
                  for k, e in enumerate(self.slots) if e is not None}
        return scal, fields

    def _restore(self, snap):
        scal, fields = snap
        for k, (q, old) in fields.items():
            for n, t in q.items():
                self.slots[k]["q"][n].copy_(t)
            for n, t in old.items():
                self.slots[k]["old"][n].copy_(t)
        torch.cuda.synchronize()
        _lib.check(self.L.wm_batch_scalars(self._h, scal, 1, _stream()), "wm_batch_scalars")

    def autotune(self, steps: int = 1, repeats: int = 2) -> dict:
        """Pick, per grid-size class of the occupied slots, the tile shape with the shortest
        measured step of the whole batch (coordinate descent over classes; every measurement is
        undone, so the solves' state is unchanged). Returns {class: (shape, [ms per shape])}."""
        classes = sorted({size_class(e["spec"].nx, e["spec"].ny) for e in self.slots if e is not None})
        for c in classes:
            self.set_shape(c, 2)
        snap = self._snapshot()
        report = {}
        stream = torch.cuda.current_stream()
        for c in classes:
            times = []
            for shape in range(len(SHAPES)):
                self.set_shape(c, shape)
                self.run(steps)  # capture / warm up
                torch.cuda.synchronize()
                self._restore(snap)
                best = float("inf")
                for _ in range(repeats):
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    self.run(steps)
                    e1.record(stream)
                    torch.cuda.synchronize()
                    best = min(best, e0.elapsed_time(e1))
                    self._restore(snap)
                times.append(best)
            pick = int(np.argmin(times))
            self.set_shape(c, pick)
            self.tuned[c] = pick
            report[c] = (pick, times)
        self._restore(snap)
        return report

    def cells(self) -> int:
        return sum(e["spec"].nx * e["spec"].ny for e in self.slots if e is not None)


def config3_solves(n=64, seed=0, min_nx=128, max_nx=1024, steps=300, device="cuda") -> list[SolveSpec]:
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(n):
        nx = int(round(math.exp(rng.uniform(math.log(min_nx), math.log(max_nx))) / 8.0)) * 8
        nx = min(max(nx, min_nx), max_nx)
        ny = nx // 2
        radius = rng.uniform(0.05, 0.15)
        xc, yc = rng.uniform(0.25, 0.4), rng.uniform(0.2, 0.3)
        mach = rng.uniform(1.5, 6.0)
        dx = 1.0 / nx
        x_shock = min(0.15, xc - radius - 3.0 * dx)

        def make(nx=nx, ny=ny, xc=xc, yc=yc, r=radius, m=mach, xs=x_shock):
            return ic.shock_droplet(nx, ny, 1.0, 0.5, mach=m, xc=xc, yc=yc, radius=r, x_shock=xs,
                                    device=device)

        specs.append(SolveSpec(nx=nx, ny=ny, dx=dx, dy=0.5 / ny, max_steps=steps, make_state=make))
    return specs
