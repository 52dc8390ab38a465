"""ctypes front end of the CPU oracle (``liboracle.so``, built from ``wavemp_oracle.c``).

TEST INFRASTRUCTURE ONLY: used by ``tests/`` as the checker, by ``__graft_entry__.smoke()`` and by
``bench.py``'s CPU-baseline / reference arm. The product (``wavemp``) never imports this module.

``OracleSolver`` owns numpy arrays laid out like the reference's ``main()`` (SC:1839-1866): every
field is a ``(nx+2g, ny+2g)`` C-order float64 array, x first, y contiguous. Its methods are the
reference's closures (SC:1894-1995): ``copy_old``, ``apply_bc``, ``compute_fluxes``,
``compute_low_fluxes``, ``limit_fluxes``, ``rk3_update``, ``enforce_admissible``,
``update_prims``, ``get_dt``, plus ``stage`` / ``step`` that run them in the reference's order.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

FIELDS = ("ar1", "ar2", "ru", "rv", "E", "al")
PRIMS = ("u_p", "v_p", "p_p")
ALL10 = FIELDS + PRIMS + ("al_prim",)

SC, M10 = 0, 1
SHIPPED, MP5C6 = 0, 1
TRANSMISSIVE, SLIP = 0, 1
FN = {name: i for i, name in enumerate(
    ("mp5_ul", "mp5_ur", "central6", "muscl_ul", "muscl_ur", "thinc_ul", "thinc_ur", "cator2",
     "mm4", "mm2", "eos", "hllc_x", "hllc_y", "eigen", "pplim", "theta"))}


class OrcParams(ctypes.Structure):
    _fields_ = [("g1", ctypes.c_double), ("p1", ctypes.c_double), ("g2", ctypes.c_double),
                ("p2", ctypes.c_double), ("dx", ctypes.c_double), ("dy", ctypes.c_double),
                ("cfl", ctypes.c_double), ("variant", ctypes.c_int), ("recon", ctypes.c_int),
                ("bc", ctypes.c_int * 4), ("repair", ctypes.c_int)]


def build(force: bool = False) -> str:
    """Compile liboracle.so in place with the recipe in oracle/Makefile."""
    src = os.path.join(HERE, "wavemp_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE, "-B" if force else "liboracle.so"], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER(OrcParams)
        vp = ctypes.c_void_p
        i = ctypes.c_int
        d = ctypes.c_double
        L.orc_cons_to_prim.argtypes = [P, i, i] + [vp] * 9
        L.orc_ducros.argtypes = [i, i] + [vp] * 5
        L.orc_enforce_admissible.argtypes = [P, i, i] + [vp] * 6
        L.orc_face_flux.argtypes = [P, i, i, i, i, vp, vp, vp]
        L.orc_face_flux_low.argtypes = [P, i, i, i, i, vp, vp]
        L.orc_cell_theta.argtypes = [P, i, i, i, vp, vp, vp, vp, vp, vp, vp, d, i]
        L.orc_blend.argtypes = [i, i, i, i, vp, vp, vp]
        L.orc_rk3.argtypes = [P, i, i, i, vp, vp, vp, vp, vp, d, d, d]
        L.orc_apply_bc.argtypes = [ctypes.POINTER(ctypes.c_int), i, i, i, vp]
        L.orc_get_dt.argtypes = [P, i, i, i] + [vp] * 6
        L.orc_get_dt.restype = d
        L.orc_workspace_doubles.argtypes = [i, i, i]
        L.orc_workspace_doubles.restype = ctypes.c_size_t
        L.orc_stage.argtypes = [P, i, i, i, vp, vp, vp, d, d, d]
        L.orc_steps.argtypes = [P, i, i, i, vp, vp, i, ctypes.POINTER(d)]
        L.orc_init_sequence.argtypes = [P, i, i, i, vp]
        L.orc_unit.argtypes = [P, i, ctypes.c_long, vp, i, vp, i]
        L.orc_unit.restype = i
        _lib = L
    return _lib


def _ptrs(arrays):
    for a in arrays:
        assert a.dtype == np.float64 and a.flags.c_contiguous
    arr = (ctypes.c_void_p * len(arrays))(*[a.ctypes.data for a in arrays])
    return arr


def make_params(dx, dy, g1=4.4, p1=6.0e8, g2=1.4, p2=0.0, variant=SC, recon=SHIPPED,
                bc=(TRANSMISSIVE, TRANSMISSIVE, SLIP, SLIP), cfl=0.4, repair=True) -> OrcParams:
    P = OrcParams()
    P.g1, P.p1, P.g2, P.p2 = g1, p1, g2, p2
    P.dx, P.dy, P.cfl = dx, dy, cfl
    P.variant, P.recon = int(variant), int(recon)
    for k in range(4):
        P.bc[k] = int(bc[k])
    P.repair = int(bool(repair))
    return P


class OracleSolver:
    def __init__(self, nx, ny, params: OrcParams, g=5):
        self.nx, self.ny, self.g = nx, ny, g
        self.nxg, self.nyg = nx + 2 * g, ny + 2 * g
        self.P = params
        z = lambda: np.zeros((self.nxg, self.nyg))  # noqa: E731
        self.f = {k: z() for k in ALL10}
        self.old = {k: z() for k in FIELDS}
        self.fh = [z() for _ in range(7)]
        self.gh = [z() for _ in range(7)]
        self.fl = [z() for _ in range(7)]
        self.gl = [z() for _ in range(7)]
        self.theta = z()
        self.sigma_x, self.sigma_y = z(), z()
        self.L = lib()

    # -- state in / out ------------------------------------------------------------------------
    def load(self, arrays: dict):
        for k, v in arrays.items():
            if k in self.f:
                self.f[k][...] = v

    def state(self) -> dict:
        return {k: v.copy() for k, v in self.f.items()}

    # -- reference closures --------------------------------------------------------------------
    def copy_old(self):
        for k in FIELDS:
            self.old[k][...] = self.f[k]

    def apply_bc(self):
        bc = (ctypes.c_int * 4)(*self.P.bc)
        self.L.orc_apply_bc(bc, self.nx, self.ny, self.g, _ptrs([self.f[k] for k in FIELDS + PRIMS]))

    def enforce_admissible(self):
        if self.P.repair:
            self.L.orc_enforce_admissible(ctypes.byref(self.P), self.nxg, self.nyg,
                                          *[self.f[k].ctypes.data for k in FIELDS])

    def update_prims(self):
        self.L.orc_cons_to_prim(ctypes.byref(self.P), self.nxg, self.nyg,
                                *[self.f[k].ctypes.data for k in FIELDS + PRIMS])
        self.f["al_prim"][...] = self.f["al"]

    def _cells(self):
        f = self.f
        return _ptrs([f["ar1"], f["ar2"], f["ru"], f["rv"], f["p_p"], f["al"]])

    def compute_fluxes(self):
        f = self.f
        if self.P.variant == SC:
            self.L.orc_ducros(self.nxg, self.nyg, f["u_p"].ctypes.data, f["v_p"].ctypes.data,
                              f["p_p"].ctypes.data, self.sigma_x.ctypes.data,
                              self.sigma_y.ctypes.data)
        cells = self._cells()
        self.L.orc_face_flux(ctypes.byref(self.P), 0, self.nx, self.ny, self.g, cells,
                             self.sigma_x.ctypes.data, _ptrs(self.fh))
        self.L.orc_face_flux(ctypes.byref(self.P), 1, self.nx, self.ny, self.g, cells,
                             self.sigma_y.ctypes.data, _ptrs(self.gh))

    def compute_low_fluxes(self):
        cells = self._cells()
        self.L.orc_face_flux_low(ctypes.byref(self.P), 0, self.nx, self.ny, self.g, cells,
                                 _ptrs(self.fl))
        self.L.orc_face_flux_low(ctypes.byref(self.P), 1, self.nx, self.ny, self.g, cells,
                                 _ptrs(self.gl))

    def limit_fluxes(self, dt, record=None):
        q = _ptrs([self.f[k] for k in FIELDS])
        for stage in range(3):
            self.L.orc_cell_theta(ctypes.byref(self.P), self.nx, self.ny, self.g, q,
                                  self.f["al_prim"].ctypes.data, _ptrs(self.fh), _ptrs(self.gh),
                                  _ptrs(self.fl), _ptrs(self.gl), self.theta.ctypes.data,
                                  float(dt), stage)
            if record is not None:
                record[f"theta{stage}"] = self.theta.copy()
            self.L.orc_blend(0, self.nx, self.ny, self.g, _ptrs(self.fh), _ptrs(self.fl),
                             self.theta.ctypes.data)
            self.L.orc_blend(1, self.nx, self.ny, self.g, _ptrs(self.gh), _ptrs(self.gl),
                             self.theta.ctypes.data)

    def rk3_update(self, alpha, beta, dt):
        self.L.orc_rk3(ctypes.byref(self.P), self.nx, self.ny, self.g,
                       _ptrs([self.old[k] for k in FIELDS]), _ptrs([self.f[k] for k in FIELDS]),
                       self.f["al_prim"].ctypes.data, _ptrs(self.fh), _ptrs(self.gh),
                       float(dt), float(alpha), float(beta))

    def get_dt(self):
        f = self.f
        return self.L.orc_get_dt(ctypes.byref(self.P), self.nx, self.ny, self.g,
                                 *[f[k].ctypes.data for k in ("ar1", "ar2", "u_p", "v_p", "p_p", "al")])

    def init_sequence(self):
        self.enforce_admissible()
        self.apply_bc()
        self.update_prims()
        self.apply_bc()

    def stage(self, alpha, beta, dt, record=None):
        self.apply_bc()
        self.compute_fluxes()
        if record is not None:
            record["sigma_x"], record["sigma_y"] = self.sigma_x.copy(), self.sigma_y.copy()
            record["high_fx"] = [a.copy() for a in self.fh]
            record["high_gy"] = [a.copy() for a in self.gh]
        self.compute_low_fluxes()
        if record is not None:
            record["low_fx"] = [a.copy() for a in self.fl]
            record["low_gy"] = [a.copy() for a in self.gl]
        self.limit_fluxes(dt, record)
        if record is not None:
            record["lim_fx"] = [a.copy() for a in self.fh]
            record["lim_gy"] = [a.copy() for a in self.gh]
        self.rk3_update(alpha, beta, dt)
        if record is not None:
            record["rk3"] = {k: self.f[k].copy() for k in FIELDS}
        self.enforce_admissible()
        if record is not None:
            record["adm"] = {k: self.f[k].copy() for k in FIELDS}
        self.update_prims()

    def step(self, dt):
        self.copy_old()
        self.stage(0.0, 1.0, dt)
        self.stage(0.75, 0.25, dt)
        self.stage(1.0 / 3.0, 2.0 / 3.0, dt)
        return self.get_dt()


class PackedOracle:
    """Whole steps in C (no Python between kernels): the CPU baseline's timed loop."""

    def __init__(self, nx, ny, params: OrcParams, g=5):
        self.nx, self.ny, self.g, self.P = nx, ny, g, params
        n = (nx + 2 * g) * (ny + 2 * g)
        self.L = lib()
        self.fields = np.zeros((10, nx + 2 * g, ny + 2 * g))
        self.ws = np.zeros(self.L.orc_workspace_doubles(nx, ny, g))
        assert self.ws.size == 37 * n
        self._f = _ptrs(list(self.fields))

    def init_sequence(self):
        self.L.orc_init_sequence(ctypes.byref(self.P), self.nx, self.ny, self.g, self._f)

    def get_dt(self):
        f = self.fields
        return self.L.orc_get_dt(ctypes.byref(self.P), self.nx, self.ny, self.g,
                                 f[0].ctypes.data, f[1].ctypes.data, f[6].ctypes.data,
                                 f[7].ctypes.data, f[8].ctypes.data, f[5].ctypes.data)

    def steps(self, n, dt):
        d = ctypes.c_double(dt)
        self.L.orc_steps(ctypes.byref(self.P), self.nx, self.ny, self.g, self._f,
                         self.ws.ctypes.data, int(n), ctypes.byref(d))
        return d.value


def unit(fn: str, params: OrcParams, inputs: np.ndarray, nout: int) -> np.ndarray:
    inputs = np.ascontiguousarray(inputs, dtype=np.float64)
    n, k = inputs.shape
    out = np.zeros((n, nout))
    rc = lib().orc_unit(ctypes.byref(params), FN[fn], n, inputs.ctypes.data, k, out.ctypes.data, nout)
    assert rc == 0
    return out
