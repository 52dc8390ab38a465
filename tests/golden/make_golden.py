"""Generate golden vectors by executing the reference's own Warp kernels on the CPU.

Test infrastructure only; it is run by hand in a checkout that has the reference scripts
(``sainath_SC_it_works.py`` "SC" and ``Sainath_M10.py`` "M10") and writes small ``.npz`` fixtures
next to this file. Those fixtures, not the reference, are what the test-suite reads.

How the reference is executed
-----------------------------
* ``warp_shim.py`` stands in for ``import warp``: every ``@wp.func`` / ``@wp.kernel`` of the
  reference runs as Python on numpy float64 scalars, one thread index at a time.
* The physical constants that the configurations change (``WG1, WP1, WG2, WP2`` at SC:40-43) are
  module globals read at call time, so they are overridden on the loaded module.
* The ``mp5c6`` reconstruction named by the hot-path specification (MP5 where the shipped code
  calls MUSCL, the sixth-order central average where it calls the fourth-order one) exists in the
  reference only as unused functions (``mp5_ul`` / ``mp5_ur`` SC:353-405, ``central6_avg``
  SC:407-412). It is produced here by an AST substitution of the call sites inside ``fx_kernel`` /
  ``gy_kernel`` (SC:1062-1082, SC:1229-1250) at generation time; nothing of it is kept.
* ``RefRunner`` replays the order of operations of the reference's ``main()`` (SC:1894-2059):
  ``copy_old``, then per stage ``apply_bc``, ``compute_fluxes``, ``compute_low_fluxes``,
  ``limit_fluxes``, ``rk3_update``, ``enforce_admissible``, ``update_prims``; ``get_dt`` after the
  third stage.

Usage: ``python tests/golden/make_golden.py --ref-dir DIR [--only CASE ...]`` (or the environment
variable ``WAVEMP_REFERENCE_DIR`` in place of ``--ref-dir``)
"""
from __future__ import annotations

import argparse
import ast
import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import warp_shim  # noqa: E402

G = 5
FIELDS = ("ar1", "ar2", "ru", "rv", "E", "al")
PRIMS = ("u_p", "v_p", "p_p")


# ----------------------------------------------------------------------------------------------
# Loading the reference under the shim
# ----------------------------------------------------------------------------------------------
class _Mp5C6(ast.NodeTransformer):
    """Replace MUSCL / central-4 call sites in the face-flux kernels by MP5 / central-6."""

    KERNELS = ("fx_kernel", "gy_kernel")

    def __init__(self):
        self.in_kernel = False
        self.count = {"ul": 0, "ur": 0, "c6": 0}

    def visit_FunctionDef(self, node):
        if node.name in self.KERNELS:
            self.in_kernel = True
            self.generic_visit(node)
            self.in_kernel = False
            return node
        return node

    @staticmethod
    def _attr(var, field):
        return ast.Attribute(value=ast.Name(id=var, ctx=ast.Load()), attr=field, ctx=ast.Load())

    def visit_Call(self, node):
        self.generic_visit(node)
        if not self.in_kernel or not isinstance(node.func, ast.Name):
            return node
        name = node.func.id
        if name in ("muscl_char_ul", "muscl_char_ur"):
            got = [(a.value.id, a.attr) for a in node.args]
            field = got[0][1]
            assert got == [("wm1", field), ("w0", field), ("w1", field), ("w2", field)], got
            if name == "muscl_char_ul":
                stencil = ("wm2", "wm1", "w0", "w1", "w2")
                self.count["ul"] += 1
                new = "mp5_ul"
            else:
                stencil = ("wm1", "w0", "w1", "w2", "w3")
                self.count["ur"] += 1
                new = "mp5_ur"
            return ast.Call(func=ast.Name(id=new, ctx=ast.Load()),
                            args=[self._attr(v, field) for v in stencil], keywords=[])
        return node

    def visit_Assign(self, node):
        self.generic_visit(node)
        if (self.in_kernel and len(node.targets) == 1 and isinstance(node.targets[0], ast.Name)
                and node.targets[0].id == "iph_v3"):
            self.count["c6"] += 1
            node.value = ast.Call(
                func=ast.Name(id="central6_avg", ctx=ast.Load()),
                args=[self._attr(v, "v3") for v in ("wm2", "wm1", "w0", "w1", "w2", "w3")],
                keywords=[])
        return node


def load_reference(path: str, recon: str = "shipped") -> types.ModuleType:
    src = open(path, encoding="utf-8").read()
    tree = ast.parse(src, filename=path)
    if recon == "mp5c6":
        tr = _Mp5C6()
        tree = tr.visit(tree)
        ast.fix_missing_locations(tree)
        assert tr.count["ul"] == 12 and tr.count["ur"] == 12, tr.count
    code = compile(tree, path, "exec")

    fake_mpl = types.ModuleType("matplotlib")
    fake_mpl.use = lambda *a, **k: None
    fake_plt = types.ModuleType("matplotlib.pyplot")
    fake_mpl.pyplot = fake_plt
    saved = {k: sys.modules.get(k) for k in ("warp", "matplotlib", "matplotlib.pyplot")}
    saved_argv = sys.argv
    sys.modules["warp"] = warp_shim
    sys.modules["matplotlib"] = fake_mpl
    sys.modules["matplotlib.pyplot"] = fake_plt
    sys.argv = [path]
    try:
        mod = types.ModuleType("reference_" + os.path.basename(path).replace(".py", ""))
        mod.__file__ = path
        exec(code, mod.__dict__)
    finally:
        sys.argv = saved_argv
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    return mod


def set_eos(mod, g1, p1, g2, p2):
    mod.WG1, mod.WP1, mod.WG2, mod.WP2 = (np.float64(g1), np.float64(p1),
                                          np.float64(g2), np.float64(p2))


# ----------------------------------------------------------------------------------------------
# Harness replaying main()'s closures (SC:1894-1995; M10 has no Ducros sensor)
# ----------------------------------------------------------------------------------------------
class RefRunner:
    def __init__(self, mod, nx, ny, dx, dy, has_ducros, cfl=0.4):
        self.m, self.nx, self.ny, self.dx, self.dy = mod, nx, ny, dx, dy
        self.nxg, self.nyg = nx + 2 * G, ny + 2 * G
        self.has_ducros, self.cfl = has_ducros, cfl
        z = lambda: np.zeros((self.nxg, self.nyg))  # noqa: E731
        self.a = {k: z() for k in FIELDS + PRIMS + ("al_prim",)}
        for k in FIELDS:
            self.a[k + "_old"] = z()
        for pre in ("fx", "gy", "fxl", "gyl"):
            for c in range(6):
                self.a[f"{pre}{c}"] = z()
        for k in ("srcx", "srcy", "srcxl", "srcyl", "theta_cell", "sigma_x", "sigma_y"):
            self.a[k] = z()

    def L(self, kern, dim, inputs):
        warp_shim.launch(kern, dim, inputs)

    def q(self):
        return [self.a[k] for k in FIELDS]

    def q9(self):
        return [self.a[k] for k in FIELDS + PRIMS]

    def copy_old(self):
        for k in FIELDS:
            self.a[k + "_old"][...] = self.a[k]

    def apply_bc(self):
        self.L(self.m.bc_x_kernel, (G, self.nyg), self.q9() + [G, self.nx, self.ny])
        self.L(self.m.bc_y_kernel, (self.nxg, G), self.q9() + [G, self.ny])

    def enforce_admissible(self):
        self.L(self.m.enforce_admissible_kernel, (self.nxg, self.nyg), self.q())

    def update_prims(self):
        self.L(self.m.cons_to_prim_kernel, (self.nxg, self.nyg), self.q9())
        self.a["al_prim"][...] = self.a["al"]

    def _face_args(self, pre, src):
        return [self.a[f"{pre}{c}"] for c in range(6)] + [self.a[src]]

    def compute_fluxes(self):
        a = self.a
        base = [a["ar1"], a["ar2"], a["ru"], a["rv"], a["p_p"], a["al"]]
        if self.has_ducros:
            self.L(self.m.ducros_kernel, (self.nxg, self.nyg),
                   [a["u_p"], a["v_p"], a["p_p"], a["sigma_x"], a["sigma_y"], self.nxg, self.nyg])
            sx, sy = [a["sigma_x"]], [a["sigma_y"]]
        else:
            sx, sy = [], []
        self.L(self.m.fx_kernel, (self.nx + 1, self.ny),
               base + sx + self._face_args("fx", "srcx") + [G - 1, G])
        self.L(self.m.gy_kernel, (self.nx, self.ny + 1),
               base + sy + self._face_args("gy", "srcy") + [G, G - 1])

    def compute_low_fluxes(self):
        a = self.a
        base = [a["ar1"], a["ar2"], a["ru"], a["rv"], a["p_p"], a["al"]]
        self.L(self.m.fx_low_kernel, (self.nx + 1, self.ny),
               base + self._face_args("fxl", "srcxl") + [G - 1, G])
        self.L(self.m.gy_low_kernel, (self.nx, self.ny + 1),
               base + self._face_args("gyl", "srcyl") + [G, G - 1])

    def limit_fluxes(self, dt, record=None):
        a = self.a
        f64 = np.float64
        for stage in range(3):
            self.L(self.m.pp_cell_theta_kernel, (self.nx, self.ny),
                   self.q() + [a["al_prim"]] + self._face_args("fx", "srcx")
                   + self._face_args("gy", "srcy") + self._face_args("fxl", "srcxl")
                   + self._face_args("gyl", "srcyl")
                   + [a["theta_cell"], f64(self.dx), f64(self.dy), f64(dt), G, G, stage])
            if record is not None:
                record[f"theta{stage}"] = a["theta_cell"].copy()
            self.L(self.m.pp_blend_x_flux_kernel, (self.nx + 1, self.ny),
                   self._face_args("fx", "srcx") + self._face_args("fxl", "srcxl")
                   + [a["theta_cell"], G - 1, G, G, self.nx])
            self.L(self.m.pp_blend_y_flux_kernel, (self.nx, self.ny + 1),
                   self._face_args("gy", "srcy") + self._face_args("gyl", "srcyl")
                   + [a["theta_cell"], G, G - 1, G, self.ny])

    def rk3_update(self, alpha, beta, dt):
        a = self.a
        f64 = np.float64
        self.L(self.m.rk3_kernel, (self.nx, self.ny),
               [a[k + "_old"] for k in FIELDS] + self.q() + [a["al_prim"]]
               + self._face_args("fx", "srcx") + self._face_args("gy", "srcy")
               + [f64(self.dx), f64(self.dy), f64(dt), f64(alpha), f64(beta), G, G])

    def get_dt(self):
        a = self.a
        buf = np.array([1.0e30])
        self.L(self.m.timestep_kernel, (self.nx, self.ny),
               [a["ar1"], a["ar2"], a["u_p"], a["v_p"], a["p_p"], a["al"],
                np.float64(self.dx), np.float64(self.dy), buf, G, G])
        return self.cfl * buf[0]

    def init_sequence(self):
        # SC:1998-2007 (minus I/O)
        self.enforce_admissible()
        self.apply_bc()
        self.update_prims()
        self.apply_bc()

    def stage(self, alpha, beta, dt, record=None):
        self.apply_bc()
        if record is not None:
            for k in FIELDS + PRIMS:
                record["bc_" + k] = self.a[k].copy()
        self.compute_fluxes()
        if record is not None:
            if self.has_ducros:
                record["sigma_x"] = self.a["sigma_x"].copy()
                record["sigma_y"] = self.a["sigma_y"].copy()
            for k in [f"fx{c}" for c in range(6)] + ["srcx"] + [f"gy{c}" for c in range(6)] + ["srcy"]:
                record["high_" + k] = self.a[k].copy()
        self.compute_low_fluxes()
        if record is not None:
            for k in [f"fxl{c}" for c in range(6)] + ["srcxl"] + [f"gyl{c}" for c in range(6)] + ["srcyl"]:
                record["low_" + k] = self.a[k].copy()
        self.limit_fluxes(dt, record)
        if record is not None:
            for k in [f"fx{c}" for c in range(6)] + ["srcx"] + [f"gy{c}" for c in range(6)] + ["srcy"]:
                record["lim_" + k] = self.a[k].copy()
        self.rk3_update(alpha, beta, dt)
        if record is not None:
            for k in FIELDS:
                record["rk3_" + k] = self.a[k].copy()
        self.enforce_admissible()
        if record is not None:
            for k in FIELDS:
                record["adm_" + k] = self.a[k].copy()
        self.update_prims()
        if record is not None:
            for k in FIELDS + PRIMS + ("al_prim",):
                record["out_" + k] = self.a[k].copy()

    def step(self, dt, record=None):
        self.copy_old()
        self.stage(0.0, 1.0, dt, record)
        self.stage(0.75, 0.25, dt)
        self.stage(1.0 / 3.0, 2.0 / 3.0, dt)
        return self.get_dt()

    def snapshot(self, prefix):
        return {prefix + k: self.a[k].copy() for k in FIELDS + PRIMS + ("al_prim",)}


# ----------------------------------------------------------------------------------------------
# Initial states
# ----------------------------------------------------------------------------------------------
def centres(nx, ny, x0, x1, y0, y1):
    dx, dy = (x1 - x0) / nx, (y1 - y0) / ny
    x = np.array([x0 + (i - G + 0.5) * dx for i in range(nx + 2 * G)])
    y = np.array([y0 + (j - G + 0.5) * dy for j in range(ny + 2 * G)])
    return x, y, dx, dy


def reference_ic(runner, mod, x, y):
    a = runner.a
    warp_shim.launch(mod.ic_kernel2, (runner.nxg, runner.nyg),
                     [a[k] for k in FIELDS + PRIMS] + [x, y])


def rankine_hugoniot(ms, gamma, p1, rho1):
    p2 = p1 * (1.0 + 2.0 * gamma / (gamma + 1.0) * (ms * ms - 1.0))
    rho2 = rho1 * (gamma + 1.0) * ms * ms / ((gamma - 1.0) * ms * ms + 2.0)
    c1 = np.sqrt(gamma * p1 / rho1)
    u2 = ms * c1 * (1.0 - rho1 / rho2)
    return p2, rho2, u2


def droplet_ic(runner, x, y, dx, g1, p1, g2, p2, ms, xc=0.3, yc=0.25, r=0.1, x_shock=0.15,
               eps=1e-6, rho_w=1000.0, rho_a=1.2, p_a=1.0e5):
    """Water disk in air with a planar air shock (tanh interface, width parameter 2 dx)."""
    ps, rs, us = rankine_hugoniot(ms, g2, p_a, rho_a)
    X, Y = np.meshgrid(x, y, indexing="ij")
    rr = np.sqrt((X - xc) ** 2 + (Y - yc) ** 2)
    al = eps + (1.0 - 2.0 * eps) * 0.5 * (1.0 - np.tanh((rr - r) / (2.0 * dx)))
    shock = X < x_shock
    rho_air = np.where(shock, rs, rho_a)
    u = np.where(shock, us, 0.0)
    p = np.where(shock, ps, p_a)
    ar1 = al * rho_w
    ar2 = (1.0 - al) * rho_air
    rho = ar1 + ar2
    gb = al / (g1 - 1.0) + (1.0 - al) / (g2 - 1.0)
    pb = al * g1 * p1 / (g1 - 1.0) + (1.0 - al) * g2 * p2 / (g2 - 1.0)
    a = runner.a
    a["ar1"][...] = ar1
    a["ar2"][...] = ar2
    a["ru"][...] = rho * u
    a["rv"][...] = 0.0
    a["E"][...] = gb * p + pb + 0.5 * rho * u * u
    a["al"][...] = al
    a["u_p"][...] = u
    a["v_p"][...] = 0.0
    a["p_p"][...] = p


def perturb(runner, rng, g1, p1, g2, p2, amp=0.05):
    """Multiplicative noise on a valid state, then consistent energies (exercises every switch)."""
    a = runner.a
    al = np.clip(a["al"] * (1.0 + amp * rng.standard_normal(a["al"].shape)), 1e-8, 1 - 1e-8)
    ar1 = a["ar1"] * (1.0 + amp * rng.standard_normal(al.shape))
    ar2 = a["ar2"] * (1.0 + amp * rng.standard_normal(al.shape))
    ar1 = np.abs(ar1) + 1e-9
    ar2 = np.abs(ar2) + 1e-9
    rho = ar1 + ar2
    cscale = np.sqrt(1.4e5 / 1.2)
    u = a["u_p"] + amp * cscale * rng.standard_normal(al.shape)
    v = a["v_p"] + amp * cscale * rng.standard_normal(al.shape)
    p = a["p_p"] * (1.0 + amp * rng.standard_normal(al.shape))
    gb = al / (g1 - 1.0) + (1.0 - al) / (g2 - 1.0)
    pb = al * g1 * p1 / (g1 - 1.0) + (1.0 - al) * g2 * p2 / (g2 - 1.0)
    a["ar1"][...], a["ar2"][...], a["al"][...] = ar1, ar2, al
    a["ru"][...], a["rv"][...] = rho * u, rho * v
    a["E"][...] = gb * p + pb + 0.5 * rho * (u * u + v * v)
    a["u_p"][...], a["v_p"][...], a["p_p"][...] = u, v, p


def stress_ic(runner, rng, g1, p1, g2, p2, vel, pmin, margin, flip_frac=0.3, ar1_exp=(-13, -7)):
    """Near-vacuum, rough state that drives all three Wong limiter passes and the repairs.

    Fluid-1 partial density 10^ar1_exp (default 1e-13..1e-7), alpha within 1e-6 of 0 or 1, random velocities and
    pressures; cells that are mostly fluid 1 get a pressure close to -pinf_1 (small rho c~^2).
    """
    a = runner.a
    sh = a["al"].shape
    ar1 = 10 ** rng.uniform(ar1_exp[0], ar1_exp[1], sh)
    ar2 = np.abs(1.2 * (1 + 0.3 * rng.standard_normal(sh))) + 0.05
    al = 10 ** rng.uniform(-9.5, -6, sh)
    flip = rng.uniform(size=sh) < flip_frac
    al = np.where(flip, 1 - al, al)
    u = vel * rng.standard_normal(sh)
    v = vel * rng.standard_normal(sh)
    p = 10 ** rng.uniform(pmin, 5, sh)
    p = np.where(flip, p - margin * p1, p)
    rho = ar1 + ar2
    gb = al / (g1 - 1) + (1 - al) / (g2 - 1)
    pb = al * g1 * p1 / (g1 - 1) + (1 - al) * g2 * p2 / (g2 - 1)
    a["ar1"][...], a["ar2"][...], a["al"][...] = ar1, ar2, al
    a["ru"][...], a["rv"][...] = rho * u, rho * v
    a["E"][...] = gb * p + pb + 0.5 * rho * (u * u + v * v)
    a["u_p"][...], a["v_p"][...], a["p_p"][...] = u, v, p


def triple_point_ic(runner, x, y, eps=1e-6):
    """Gas-gas triple point on [0,7]x[0,3]; fluid 1 gamma=1.5, fluid 2 gamma=1.4 (both pi=0)."""
    X, Y = np.meshgrid(x, y, indexing="ij")
    left = X < 1.0
    top = (~left) & (Y >= 1.5)
    bottom = (~left) & (Y < 1.5)
    al = np.where(bottom, eps, 1.0 - eps)
    rho = np.where(left, 1.0, np.where(top, 0.125, 1.0))
    p = np.where(left, 1.0, 0.1)
    a = runner.a
    a["ar1"][...] = al * rho
    a["ar2"][...] = (1.0 - al) * rho
    a["ru"][...] = 0.0
    a["rv"][...] = 0.0
    gb = al / 0.5 + (1.0 - al) / 0.4
    a["E"][...] = gb * p
    a["al"][...] = al
    a["u_p"][...] = 0.0
    a["v_p"][...] = 0.0
    a["p_p"][...] = p


# ----------------------------------------------------------------------------------------------
# Cases
# ----------------------------------------------------------------------------------------------
def run_case(name, ref_dir, out_dir):
    sc = os.path.join(ref_dir, "sainath_SC_it_works.py")
    m10 = os.path.join(ref_dir, "Sainath_M10.py")
    rec = {}
    t0 = time.time()
    if name == "sc_ref_ic":
        # The SC script as shipped: its constants, its IC (SC:779-837), its domain.
        mod = load_reference(sc)
        nx, ny = 24, 16
        x, y, dx, dy = centres(nx, ny, 0.0, 0.111, 0.0, 0.074)
        r = RefRunner(mod, nx, ny, dx, dy, has_ducros=True)
        reference_ic(r, mod, x, y)
        meta = dict(variant="sc", recon="shipped", g1=6.12, p1=3.43e8, g2=1.4, p2=0.0, steps=2)
    elif name == "m10_ref_ic":
        mod = load_reference(m10)
        nx, ny = 24, 16
        x, y, dx, dy = centres(nx, ny, 0.0, 0.030, 0.0, 0.020)
        r = RefRunner(mod, nx, ny, dx, dy, has_ducros=False)
        reference_ic(r, mod, x, y)
        meta = dict(variant="m10", recon="shipped", g1=6.12, p1=3.43e8, g2=1.4, p2=0.0, steps=2)
    elif name in ("sc_cfg0", "sc_mp5c6_cfg0", "sc_mp5c6_rand", "m10_cfg2", "m10_mp5c6_rand"):
        variant = "m10" if name.startswith("m10") else "sc"
        recon = "mp5c6" if "mp5c6" in name else "shipped"
        mod = load_reference(m10 if variant == "m10" else sc, recon)
        g1, p1, g2, p2 = 4.4, 6.0e8, 1.4, 0.0
        set_eos(mod, g1, p1, g2, p2)
        nx, ny = (20, 10) if name.endswith("rand") else (32, 16)
        x, y, dx, dy = centres(nx, ny, 0.0, 1.0, 0.0, 0.5)
        r = RefRunner(mod, nx, ny, dx, dy, has_ducros=(variant == "sc"))
        ms = 10.0 if name == "m10_cfg2" else 2.4
        droplet_ic(r, x, y, dx, g1, p1, g2, p2, ms)
        if name.endswith("rand"):
            perturb(r, np.random.default_rng(7), g1, p1, g2, p2)
        meta = dict(variant=variant, recon=recon, g1=g1, p1=p1, g2=g2, p2=p2,
                    steps=1 if name.endswith("rand") else 2)
    elif name in ("sc_mp5c6_stress", "m10_stress"):
        # m10_stress is not part of the fixture set: M10's staged limiter switches hard at
        # partial densities of 1e-11 (SC:233-237) and such near-vacuum states flip those
        # switches under 1e-15 input noise, so the reference's own output is not reproducible
        # to round-off there. It stays generable for inspection.
        variant = "m10" if name.startswith("m10") else "sc"
        recon = "mp5c6" if "mp5c6" in name else "shipped"
        mod = load_reference(m10 if variant == "m10" else sc, recon)
        g1, p1, g2, p2 = 4.4, 6.0e8, 1.4, 0.0
        set_eos(mod, g1, p1, g2, p2)
        nx, ny = 16, 10
        x, y, dx, dy = centres(nx, ny, 0.0, 0.8, 0.0, 0.5)
        r = RefRunner(mod, nx, ny, dx, dy, has_ducros=(variant == "sc"))
        if variant == "sc":
            stress_ic(r, np.random.default_rng(11), g1, p1, g2, p2, 30.0, 3.0, 0.5)
        else:
            stress_ic(r, np.random.default_rng(5), g1, p1, g2, p2, 100.0, 3.0, 0.9)
        meta = dict(variant=variant, recon=recon, g1=g1, p1=p1, g2=g2, p2=p2, steps=1)
    elif name == "sc_mp5c6_triple":
        mod = load_reference(sc, "mp5c6")
        set_eos(mod, 1.5, 0.0, 1.4, 0.0)
        nx, ny = 28, 12
        x, y, dx, dy = centres(nx, ny, 0.0, 7.0, 0.0, 3.0)
        r = RefRunner(mod, nx, ny, dx, dy, has_ducros=True)
        triple_point_ic(r, x, y)
        meta = dict(variant="sc", recon="mp5c6", g1=1.5, p1=0.0, g2=1.4, p2=0.0, steps=2)
    else:
        raise ValueError(name)

    rec.update({"ic_" + k: r.a[k].copy() for k in FIELDS + PRIMS})
    r.init_sequence()
    rec.update(r.snapshot("in_"))
    dt0 = r.get_dt()
    rec["dt0"] = np.float64(dt0)
    stage_rec = {}
    r.copy_old()
    r.stage(0.0, 1.0, dt0, stage_rec)
    rec.update({"s1_" + k: v for k, v in stage_rec.items()})
    r.stage(0.75, 0.25, dt0)
    rec.update(r.snapshot("s2_"))
    r.stage(1.0 / 3.0, 2.0 / 3.0, dt0)
    rec.update(r.snapshot("step1_"))
    dt1 = r.get_dt()
    rec["dt1"] = np.float64(dt1)
    for s in range(1, meta["steps"]):
        dt1 = r.step(dt1)
    rec.update(r.snapshot("final_"))
    rec["dt_final"] = np.float64(dt1)
    for k, v in meta.items():
        rec["meta_" + k] = np.array(v)
    rec["meta_nx"], rec["meta_ny"], rec["meta_g"] = np.array(nx), np.array(ny), np.array(G)
    rec["meta_dx"], rec["meta_dy"] = np.float64(dx), np.float64(dy)
    path = os.path.join(out_dir, f"{name}.npz")
    np.savez_compressed(path, **rec)
    print(f"{name}: {time.time() - t0:.1f}s -> {path} ({os.path.getsize(path) // 1024} KB)")


UNIT_CASES = 400


def run_units(ref_dir, out_dir):
    """Known-answer vectors for single reference device functions on seeded random inputs."""
    mod = load_reference(os.path.join(ref_dir, "sainath_SC_it_works.py"))
    set_eos(mod, 4.4, 6.0e8, 1.4, 0.0)
    rng = np.random.default_rng(11)
    out = {}
    n = UNIT_CASES
    f = np.float64

    # 5-point stencils with a mix of smooth, monotone, extremal and flat data
    st = rng.standard_normal((n, 6))
    st[: n // 4] = np.cumsum(np.abs(st[: n // 4]), axis=1)              # monotone
    st[n // 4: n // 3] = 1.0                                              # flat
    st[n // 3: n // 2] = np.sign(st[n // 3: n // 2]) * 1e-3               # +-tiny jumps
    out["stencil"] = st
    out["mp5_ul"] = np.array([mod.mp5_ul(*map(f, s[:5])) for s in st])
    out["mp5_ur"] = np.array([mod.mp5_ur(*map(f, s[:5])) for s in st])
    out["central6"] = np.array([mod.central6_avg(*map(f, s)) for s in st])
    out["muscl_ul"] = np.array([mod.muscl_char_ul(*map(f, s[:4])) for s in st])
    out["muscl_ur"] = np.array([mod.muscl_char_ur(*map(f, s[:4])) for s in st])
    out["thinc_ul"] = np.array([mod.thinc_ul(*map(f, s[:3])) for s in st])
    out["thinc_ur"] = np.array([mod.thinc_ur(*map(f, s[:3])) for s in st])
    out["cator2"] = np.array([mod.cator2_val(*map(f, s[:5])) for s in st])
    out["mm4"] = np.array([mod.mm4(*map(f, s[:4])) for s in st])
    out["mm2"] = np.array([mod.mm2(*map(f, s[:2])) for s in st])

    # EOS
    a1 = np.concatenate([rng.uniform(0, 1, n - 4), [0.0, 1.0, 1e-10, 1 - 1e-10]])
    out["eos_a1"] = a1
    gp = [mod.mix_gamma_pinf(f(a)) for a in a1]
    out["eos_g"] = np.array([g for g, _ in gp])
    out["eos_pinf"] = np.array([p for _, p in gp])

    # HLLC left/right primitive states covering all four branches
    def prim_state(k):
        alv = rng.uniform(1e-6, 1 - 1e-6, k)
        rho1 = rng.uniform(500, 1500, k)
        rho2 = rng.uniform(0.5, 5, k)
        u = rng.uniform(-3000, 3000, k)
        v = rng.uniform(-300, 300, k)
        p = 10 ** rng.uniform(4, 8, k)
        return np.stack([alv * rho1, (1 - alv) * rho2, u, v, p, alv], axis=1)

    L, R = prim_state(n), prim_state(n)
    out["hllc_L"], out["hllc_R"] = L, R
    hx, hy, sx, sy = [], [], [], []
    for l, rr in zip(L, R):
        l = [f(v) for v in l]
        rr = [f(v) for v in rr]
        fx = mod.hllc_x(*l, *rr)
        fy = mod.hllc_y(*l, *rr)
        hx.append([fx.v0, fx.v1, fx.v2, fx.v3, fx.v4, fx.v5])
        hy.append([fy.v0, fy.v1, fy.v2, fy.v3, fy.v4, fy.v5])
        sx.append(mod.hllc_x_src(l[0], l[1], l[2], l[4], l[5], rr[0], rr[1], rr[2], rr[4], rr[5]))
        sy.append(mod.hllc_y_src(l[0], l[1], l[3], l[4], l[5], rr[0], rr[1], rr[3], rr[4], rr[5]))
    out["hllc_x"], out["hllc_y"] = np.array(hx), np.array(hy)
    out["hllc_x_src"], out["hllc_y_src"] = np.array(sx), np.array(sy)

    # Eigen projections (x and y) and a round trip
    U = prim_state(n)
    U[:, 2] *= U[:, 0] + U[:, 1]
    U[:, 3] *= U[:, 0] + U[:, 1]
    avg = prim_state(n)
    cx, px, cy, py = [], [], [], []
    for u, a in zip(U, avg):
        rho = f(a[0] + a[1])
        c = mod.sound_speed(rho, f(a[4]), f(a[5]))
        args = [f(v) for v in u] + [c, rho, f(a[0]), f(a[1]), f(a[2]), f(a[3])]
        w = mod.to_char_x(*args)
        cx.append([w.v0, w.v1, w.v2, w.v3, w.v4, w.v5])
        b = mod.to_phys_x(w, c, rho, f(a[0]), f(a[1]), f(a[2]), f(a[3]))
        px.append([b.v0, b.v1, b.v2, b.v3, b.v4, b.v5])
        w = mod.to_char_y(*args)
        cy.append([w.v0, w.v1, w.v2, w.v3, w.v4, w.v5])
        b = mod.to_phys_y(w, c, rho, f(a[0]), f(a[1]), f(a[2]), f(a[3]))
        py.append([b.v0, b.v1, b.v2, b.v3, b.v4, b.v5])
    out["eig_U"], out["eig_avg"] = U, avg
    out["to_char_x"], out["to_phys_x"] = np.array(cx), np.array(px)
    out["to_char_y"], out["to_phys_y"] = np.array(cy), np.array(py)

    # Positivity helpers: reconstructed-state limiter (M10's staged Wong limiter) and theta solves
    hi = prim_state(n)
    hi[:, 0] *= rng.choice([1.0, -1.0, 1e-12], n)
    hi[:, 4] *= rng.choice([1.0, -1.0], n, p=[0.7, 0.3])
    hi[:, 5] = rng.uniform(-0.2, 1.2, n)
    base = prim_state(n)
    lim = []
    for h, b in zip(hi, base):
        s_h, s_b = mod.S6(), mod.S6()
        for k in range(6):
            setattr(s_h, f"v{k}", f(h[k]))
            setattr(s_b, f"v{k}", f(b[k]))
        s = mod.pp_limit_reconstructed_state(s_h, s_b)
        lim.append([s.v0, s.v1, s.v2, s.v3, s.v4, s.v5])
    out["pplim_high"], out["pplim_base"], out["pplim_out"] = hi, base, np.array(lim)
    th = []
    lq = rng.standard_normal((n, 6)) * [1, 1, 1e3, 1e3, 1e9, 0.5] + [1e-3, 1e-3, 0, 0, 1e9, 0.5]
    hq = lq * (1 + 0.5 * rng.standard_normal((n, 6)))
    for l, h in zip(lq, hq):
        th.append([mod.theta_cons_stage(*map(f, l), *map(f, h), s) for s in range(3)])
    out["theta_l"], out["theta_h"], out["theta_out"] = lq, hq, np.array(th)
    path = os.path.join(out_dir, "units.npz")
    np.savez_compressed(path, **out)
    print(f"units -> {path} ({os.path.getsize(path) // 1024} KB)")


class _Arrays:
    def __init__(self, nx, ny):
        self.a = {k: np.zeros((nx + 2 * G, ny + 2 * G)) for k in FIELDS + PRIMS}


def run_checkpoint(ref_dir, out_dir):
    """The reference's output and restart functions -- ``save_npz`` (SC:1714-1726),
    ``load_restart_host`` (SC:1779-1821) and ``infer_restart_step`` (SC:1773-1776) -- on a small
    perturbed droplet state with the script's own water EOS (6.12, 3.43e8), plus a restart file
    whose alpha1 leaves [0, 1] (the loader clips it to [1e-8, 1 - 1e-8])."""
    import tempfile

    mod = load_reference(os.path.join(ref_dir, "sainath_SC_it_works.py"))
    nx, ny = 24, 12
    mod.NX, mod.NY, mod.NXG, mod.NYG = nx, ny, nx + 2 * G, ny + 2 * G
    x, y, dx, dy = centres(nx, ny, 0.0, 1.0, 0.0, 0.5)
    st = _Arrays(nx, ny)
    g1, p1, g2, p2 = 6.12, 3.43e8, 1.4, 0.0
    droplet_ic(st, x, y, dx, g1, p1, g2, p2, 2.4)
    perturb(st, np.random.default_rng(5), g1, p1, g2, p2)
    a = st.a
    out = {f"in_{k}": a[k] for k in FIELDS + PRIMS}
    out.update(in_x=x, in_y=y, in_step=np.int64(137), in_time=np.float64(1.25e-5))
    rng = np.random.default_rng(6)
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        os.chdir(d)
        try:
            mod.save_npz(a["ar1"], a["ar2"], a["u_p"], a["v_p"], a["p_p"], a["al"], x, y, 137, 1.25e-5)
            name = "mp5_000137.npz"
            with np.load(name) as f:
                for k in f.files:
                    out["saved_" + k] = f[k]
            res = mod.load_restart_host(os.path.join(d, name), x, y)
            out["restart_step"] = np.int64(mod.infer_restart_step(os.path.join(d, name)))
            edge = {k: out["saved_" + k].copy() for k in ("ar1", "ar2", "u", "v", "p", "alpha1")}
            edge["alpha1"] = rng.uniform(-0.2, 1.2, size=(nx, ny))
            edge["alpha1"][0, :4] = [0.0, 1.0, 1e-9, 1.0 - 1e-9]
            np.savez(os.path.join(d, "edge.npz"), **edge)  # no time key: restart time 0
            res_edge = mod.load_restart_host(os.path.join(d, "edge.npz"), x, y)
        finally:
            os.chdir(cwd)
    names = ("ar1", "ar2", "ru", "rv", "E", "al", "u_p", "v_p", "p_p")
    for k, v in zip(names, res[:9]):
        out["restart_" + k] = v
    out["restart_time"] = np.float64(res[9])
    for k, v in edge.items():
        out["edge_in_" + k] = v
    for k, v in zip(names, res_edge[:9]):
        out["edge_restart_" + k] = v
    out["edge_restart_time"] = np.float64(res_edge[9])
    path = os.path.join(out_dir, "checkpoint.npz")
    np.savez_compressed(path, **out)
    print(f"checkpoint -> {path} ({os.path.getsize(path) // 1024} KB)")


ALL_CASES = ("sc_ref_ic", "m10_ref_ic", "sc_cfg0", "sc_mp5c6_cfg0", "sc_mp5c6_rand",
             "m10_cfg2", "m10_mp5c6_rand", "sc_mp5c6_triple", "sc_mp5c6_stress")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-dir", default=os.environ.get("WAVEMP_REFERENCE_DIR"),
                    required="WAVEMP_REFERENCE_DIR" not in os.environ,
                    help="directory holding the reference's two scripts (or set WAVEMP_REFERENCE_DIR)")
    ap.add_argument("--out-dir", default=HERE)
    ap.add_argument("--only", nargs="*", default=None)
    args = ap.parse_args()
    todo = args.only if args.only else list(ALL_CASES) + ["units", "checkpoint"]
    for name in todo:
        if name == "units":
            run_units(args.ref_dir, args.out_dir)
        elif name == "checkpoint":
            run_checkpoint(args.ref_dir, args.out_dir)
        else:
            run_case(name, args.ref_dir, args.out_dir)


if __name__ == "__main__":
    main()
