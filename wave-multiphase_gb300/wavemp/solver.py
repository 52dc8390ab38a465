"""Python front end of the GB300 RHS: the reference's closures over torch float64 CUDA tensors.

The reference keeps 47 module-level Warp arrays and drives them with closures inside ``main()``
(SC:1839-1995). ``Solver`` owns the workspace those closures need (fluxes, limiter factors,
sensors) and exposes each closure as a method with the reference's name and argument meaning.
The state is a dict of the ten per-cell arrays ``ar1, ar2, ru, rv, E, al, u_p, v_p, p_p, al_prim``
(SC:1839-1841), each a ``torch.float64`` CUDA tensor of shape ``(nx + 2g, ny + 2g)``, x first,
y contiguous -- the reference's layout. Every call is enqueued on torch's current CUDA stream.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .params import SolverParams

FIELDS = ("ar1", "ar2", "ru", "rv", "E", "al")
PRIMS = ("u_p", "v_p", "p_p")
ALL = FIELDS + PRIMS + ("al_prim",)


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def alloc_state(nx: int, ny: int, g: int = 5, device="cuda", names=ALL) -> dict:
    """Zeroed state arrays, one contiguous (10, nx+2g, ny+2g) block viewed per field."""
    block = torch.zeros((len(names), nx + 2 * g, ny + 2 * g), dtype=torch.float64, device=device)
    return {k: block[c] for c, k in enumerate(names)}


class Solver:
    """Per-stage RHS of the 2-D five-equation stiffened-gas model on one GPU.

    ``Solver(params, nx, ny, g=5)`` allocates its workspace with torch on the current CUDA
    device. Methods mirror the reference's closures (``apply_bc``, ``compute_fluxes``,
    ``compute_low_fluxes``, ``limit_fluxes``, ``rk3_update``, ``enforce_admissible``,
    ``update_prims``, ``copy_old``, ``get_dt``) and add the fused ``rhs_stage`` and ``step``.
    """

    def __init__(self, params: SolverParams, nx: int, ny: int, g: int = 5, device=None,
                 workspace: torch.Tensor | None = None):
        if not torch.cuda.is_available():
            raise _lib.WavempError("wavemp needs a CUDA device (there is no CPU path)")
        self.L = _lib.load()
        self.params = params
        self.nx, self.ny, self.g = nx, ny, g
        self.nxg, self.nyg = nx + 2 * g, ny + 2 * g
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self._cp = params.to_c()
        nbytes = self.L.wm_workspace_bytes(ctypes.byref(self._cp), nx, ny, g)
        if nbytes == 0:
            raise ValueError("invalid solver parameters or grid size")
        with torch.cuda.device(self.device):
            if workspace is not None:
                if workspace.numel() * workspace.element_size() < nbytes or workspace.data_ptr() % 256:
                    raise ValueError("workspace too small or not 256-byte aligned")
                self._ws = workspace
            else:
                self._ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
            h = ctypes.c_void_p()
            _lib.check(self.L.wm_create(ctypes.byref(self._cp), nx, ny, g,
                                        ctypes.c_void_p(self._ws.data_ptr()), nbytes,
                                        ctypes.byref(h)), "wm_create")
        self._h = h
        self._dt_host = ctypes.c_double(0.0)

    @staticmethod
    def workspace_bytes(params: SolverParams, nx: int, ny: int, g: int = 5) -> int:
        L = _lib.load()
        cp = params.to_c()
        return int(L.wm_workspace_bytes(ctypes.byref(cp), nx, ny, g))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self.L.wm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- argument marshalling ------------------------------------------------------------------
    def _fields(self, q: dict, need_prims: bool = True) -> _lib.WmFields:
        f = _lib.WmFields()
        pitch = None
        for k in ALL:
            t = q.get(k)
            if t is None:
                if need_prims or k in FIELDS:
                    raise ValueError(f"state is missing field {k!r}")
                continue
            if t.dtype != torch.float64 or not t.is_cuda or t.dim() != 2:
                raise ValueError(f"{k}: expected a 2-D torch.float64 CUDA tensor")
            if tuple(t.shape) != (self.nxg, self.nyg) or t.stride(1) != 1:
                raise ValueError(f"{k}: expected shape {(self.nxg, self.nyg)} with contiguous rows")
            if pitch is None:
                pitch = t.stride(0)
            elif t.stride(0) != pitch:
                raise ValueError("all fields must share one row pitch")
            setattr(f, k, t.data_ptr())
        f.pitch = pitch
        return f

    # -- the reference's closures (SC:1894-1995) ------------------------------------------------
    def apply_bc(self, q):
        _lib.check(self.L.wm_apply_bc(self._h, ctypes.byref(self._fields(q)), _stream()), "apply_bc")

    def compute_fluxes(self, q):
        _lib.check(self.L.wm_compute_fluxes(self._h, ctypes.byref(self._fields(q)), _stream()),
                   "compute_fluxes")

    def compute_low_fluxes(self, q):
        _lib.check(self.L.wm_compute_low_fluxes(self._h, ctypes.byref(self._fields(q)), _stream()),
                   "compute_low_fluxes")

    def limit_fluxes(self, q, dt: float):
        _lib.check(self.L.wm_limit_fluxes(self._h, ctypes.byref(self._fields(q)), float(dt),
                                          _stream()), "limit_fluxes")

    def rk3_update(self, q, q_old, alpha: float, beta: float, dt: float):
        old = self._fields(q_old, need_prims=False) if q_old is not None else None
        _lib.check(self.L.wm_rk3_update(self._h, ctypes.byref(self._fields(q)),
                                        ctypes.byref(old) if old is not None else None,
                                        float(alpha), float(beta), float(dt), _stream()),
                   "rk3_update")

    def enforce_admissible(self, q):
        _lib.check(self.L.wm_enforce_admissible(self._h, ctypes.byref(self._fields(q)), _stream()),
                   "enforce_admissible")

    def update_prims(self, q):
        _lib.check(self.L.wm_update_prims(self._h, ctypes.byref(self._fields(q)), _stream()),
                   "update_prims")

    def copy_old(self, q, q_old):
        _lib.check(self.L.wm_copy_old(self._h, ctypes.byref(self._fields(q, need_prims=False)),
                                      ctypes.byref(self._fields(q_old, need_prims=False)),
                                      _stream()), "copy_old")

    def get_dt(self, q) -> float:
        _lib.check(self.L.wm_get_dt(self._h, ctypes.byref(self._fields(q)),
                                    ctypes.byref(self._dt_host), _stream()), "get_dt")
        return self._dt_host.value

    def initialize(self, q):
        """The reference's start-up sequence (SC:1998-2007 minus I/O): enforce_admissible,
        apply_bc, update_prims, apply_bc."""
        self.enforce_admissible(q)
        self.apply_bc(q)
        self.update_prims(q)
        self.apply_bc(q)

    # -- fused forms ----------------------------------------------------------------------------
    def rhs_stage(self, q, q_old, dt: float, alpha: float, beta: float):
        """One SSP-RK3 stage (SC:2030-2055 body); updates q in place."""
        old = self._fields(q_old, need_prims=False) if q_old is not None else None
        _lib.check(self.L.wm_rhs_stage(self._h, ctypes.byref(self._fields(q)),
                                       ctypes.byref(old) if old is not None else None,
                                       float(dt), float(alpha), float(beta), _stream()),
                   "rhs_stage")

    def init_dt(self, q):
        """Compute the next step's dt on the device (no host wait)."""
        _lib.check(self.L.wm_init_dt(self._h, ctypes.byref(self._fields(q)), _stream()), "init_dt")

    def step(self, q, q_old, dt: float | None = None, sync: bool = True):
        """One SSP-RK3 step (SC:2033-2059). dt=None uses the device-resident dt of the previous
        step (or of init_dt). Returns the next dt as a float when sync, else None."""
        out = ctypes.byref(self._dt_host) if sync else None
        _lib.check(self.L.wm_step(self._h, ctypes.byref(self._fields(q)),
                                  ctypes.byref(self._fields(q_old, need_prims=False)),
                                  float(dt) if dt is not None else 0.0, out, _stream()), "step")
        return self._dt_host.value if sync else None

    def run(self, q, q_old, t_end: float, save_times=(), t: float = 0.0, step: int = 0,
            on_save=None, max_steps: int | None = None):
        """The reference's time loop (SC:2009-2073) with its steps on the device (wm_run): dt
        clamped to the save times and to t_end, one host wait per save time. on_save(q, step, t, k)
        is called when save time k is reached (the reference writes its npz there). Returns
        (t, step); the schedule of the last call is kept in ``self.schedule``."""
        times = [float(v) for v in save_times]
        if len(times) > _lib.MAX_SAVES:
            raise ValueError(f"at most {_lib.MAX_SAVES} save times")
        sch = _lib.WmSchedule()
        sch.t, sch.t_end, sch.step, sch.nsaves = float(t), float(t_end), int(step), len(times)
        for k, ts in enumerate(times):
            sch.save_times[k] = ts
            sch.saved[k] = int(t >= ts - 1.0e-14)
        limit = (1 << 62) if max_steps is None else int(max_steps)
        fq, fo = self._fields(q), self._fields(q_old, need_prims=False)
        done = 0
        while done < limit:
            before = sch.step
            _lib.check(self.L.wm_run(self._h, ctypes.byref(fq), ctypes.byref(fo), ctypes.byref(sch),
                                     min(limit - done, 1 << 40), _stream()), "run")
            done += sch.step - before
            if sch.hit >= 0 and on_save is not None:
                on_save(q, sch.step, sch.t, sch.hit)
            if sch.finished or sch.step == before:
                break
        self.schedule = sch
        return sch.t, sch.step

    def verify_limiter_precheck(self, q, dt: float) -> tuple[int, int]:
        """Precision form diagnostic (after compute_fluxes / compute_low_fluxes; does the work of
        limit_fluxes): (cells whose bound pass the binary32 pre-check decided, cells where the
        binary64 solve disagreed -- 0 when its margins hold)."""
        a, b = ctypes.c_longlong(), ctypes.c_longlong()
        _lib.check(self.L.wm_verify_limiter_precheck(self._h, ctypes.byref(self._fields(q)), float(dt),
                                                     ctypes.byref(a), ctypes.byref(b), _stream()),
                   "verify_limiter_precheck")
        return a.value, b.value

    def verify_switch_precheck(self, q) -> tuple[int, int, int]:
        """Diagnostic of the THINC switch pre-check on state q: (stencils checked, settled by the
        binary32 pre-check, settled differently from the binary64 decision -- 0 when its error
        bound holds)."""
        a, b, c = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        _lib.check(self.L.wm_verify_switch_precheck(self._h, ctypes.byref(self._fields(q, need_prims=True)),
                                                    ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                                    _stream()), "verify_switch_precheck")
        return a.value, b.value, c.value

    def verify_ducros_precheck(self, q) -> tuple[int, int, int]:
        """Diagnostic of the Ducros sensor pre-check on state q: (direction stencils checked, settled
        by the binary32 pre-check, settled differently from the binary64 sigma < 0.01 -- 0 when its
        error bound holds)."""
        a, b, c = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        _lib.check(self.L.wm_verify_ducros_precheck(self._h, ctypes.byref(self._fields(q, need_prims=True)),
                                                    ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                                    _stream()), "verify_ducros_precheck")
        return a.value, b.value, c.value

    def set_prechecks(self, on: bool):
        """Binary32 pre-checks that skip binary64 tests they decide -- the limiter's bound solves,
        the combine's admissibility tests, the THINC switch of binary64 sensors (default on; the
        results are the same bits either way)."""
        _lib.check(self.L.wm_set_prechecks(self._h, int(bool(on))), "set_prechecks")

    def set_limiter_sweeps(self, in_place: bool):
        """Fused stage: blend sweeps in place (the reference's form; default of the binary64
        form) or rebuilt in registers by the next pass and the combine (bit-identical; default of
        the binary32 form)."""
        _lib.check(self.L.wm_set_limiter_sweeps(self._h, int(bool(in_place))), "set_limiter_sweeps")

    def run_uses_graph(self) -> bool:
        return bool(self.L.wm_run_uses_graph(self._h))

    # -- diagnostics ----------------------------------------------------------------------------
    def workspace(self, which: int) -> torch.Tensor:
        out = torch.empty((self.nxg, self.nyg), dtype=torch.float64, device=self.device)
        _lib.check(self.L.wm_read_workspace(self._h, int(which), ctypes.c_void_p(out.data_ptr()),
                                            _stream()), "read_workspace")
        return out

    def fluxes(self, which: str = "high") -> tuple[list, list]:
        """The x and y face arrays of the workspace: "high" the high-order (after a limiter,
        blended) fluxes, "low" the first-order ones of the last compute_low_fluxes -- a binary64
        fused stage with blends in place forms those where the limiter reads them and stores none."""
        base_x, base_y = (_lib.WS_FX, _lib.WS_GY) if which == "high" else (_lib.WS_FXL, _lib.WS_GYL)
        return ([self.workspace(base_x + c) for c in range(7)],
                [self.workspace(base_y + c) for c in range(7)])

    def profile(self, enable: bool = True):
        """Record CUDA events around each kernel group of every stage (see profile_read)."""
        _lib.check(self.L.wm_profile(self._h, int(bool(enable))), "profile")

    def profile_read(self, reset: bool = True) -> dict:
        """{group: (milliseconds, launches)} summed since the last reset."""
        ms = (ctypes.c_double * 5)()
        n = (ctypes.c_longlong * 5)()
        _lib.check(self.L.wm_profile_read(self._h, ctypes.byref(ms), ctypes.byref(n), int(reset)),
                   "profile_read")
        return {g: (ms[i], n[i]) for i, g in enumerate(_lib.PROF_GROUPS)}

    def status(self, reset: bool = False) -> dict:
        st = _lib.WmStats()
        _lib.check(self.L.wm_status(self._h, ctypes.byref(st), int(reset), _stream()), "status")
        return {k: getattr(st, k) for k, _ in _lib.WmStats._fields_}


def copy_state(dst: torch.Tensor, src: torch.Tensor):
    """dst <- src by the SMs (wm_copy_state): contiguous tensors of the same size in bytes, each on
    the device or in page-locked host memory (pin_memory), asynchronous on the current stream."""
    if not (dst.is_contiguous() and src.is_contiguous()):
        raise ValueError("copy_state needs contiguous tensors")
    nbytes = dst.numel() * dst.element_size()
    if src.numel() * src.element_size() != nbytes:
        raise ValueError("copy_state: sizes differ")
    L = _lib.load()
    _lib.check(L.wm_copy_state(ctypes.c_void_p(dst.data_ptr()), ctypes.c_void_p(src.data_ptr()), nbytes,
                               _stream()), "copy_state")


def probe_fp64_flops() -> float:
    L = _lib.load()
    v = ctypes.c_double()
    _lib.check(L.wm_probe_fp64_flops(ctypes.byref(v), _stream()), "probe_fp64_flops")
    return v.value
