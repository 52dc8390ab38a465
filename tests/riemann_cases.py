"""Shock-tube problems with exact solutions, shared by the oracle and device Riemann tests.

Each case is a 1-D Riemann problem on [0, 1] laid along x (nx cells, one row) or along y (the
transposed grid, (u, v) swapped): the five-equation state of the left and right gases with the
volume fraction alpha1 = 1 - eps for fluid 1 and eps for fluid 2 (eps = 1e-6, the value of the
benchmark initial states; binary32 cannot hold 1 - 1e-8 apart from 1), run to t_end with the scheme's
CFL time step clamped to t_end, and compared with the exact stiffened-gas solution
(riemann_exact) by the relative L1 error of the mixture density, sum |rho - rho_exact| / sum rho_exact.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

import riemann_exact as rx

EPS = 1.0e-6
G = 5


@dataclass(frozen=True)
class Case:
    name: str
    g1: float
    p1: float
    g2: float
    p2: float
    left: tuple     # (rho, u, p, fluid) with fluid 1 or 2
    right: tuple
    x0: float
    t_end: float

    def sides(self):
        out = []
        for rho, u, p, fl in (self.left, self.right):
            g, pi = (self.g1, self.p1) if fl == 1 else (self.g2, self.p2)
            out.append(rx.Side(rho, u, p, g, pi))
        return out


# Sod's problem (Toro's test 1) in Pa and kg/m^3, so the speeds are sqrt(1e5) times Toro's.
_SOD_T = 0.2 / np.sqrt(1.0e5)
CASES = {
    "sod_fluid1": Case("sod_fluid1", 1.4, 0.0, 1.6, 0.0, (1.0, 0.0, 1.0e5, 1), (0.125, 0.0, 1.0e4, 1),
                       0.5, _SOD_T),
    "sod_fluid2": Case("sod_fluid2", 1.4, 0.0, 1.6, 0.0, (1.0, 0.0, 1.0e5, 2), (0.125, 0.0, 1.0e4, 2),
                       0.5, _SOD_T),
    # stiffened-gas water, 1 GPa against 1 bar: a rarefaction into the high-pressure water and a
    # strong shock into the low-pressure water
    "water_tube": Case("water_tube", 4.4, 6.0e8, 1.4, 0.0, (1000.0, 0.0, 1.0e9, 1),
                       (1000.0, 0.0, 1.0e5, 1), 0.5, 1.5e-4),
    # water at 1 GPa against air at 1 bar, interface at x = 0.7 (the classic two-fluid shock tube)
    "water_air": Case("water_air", 4.4, 6.0e8, 1.4, 0.0, (1000.0, 0.0, 1.0e9, 1), (50.0, 0.0, 1.0e5, 2),
                      0.7, 2.4e-4),
}


def centres(n: int) -> np.ndarray:
    return (np.arange(n) + 0.5) / n


def initial_line(case: Case, n: int, g: int = G) -> dict:
    """The ten padded fields along one line of n interior cells (ghosts included), as 1-D arrays."""
    x = (np.arange(n + 2 * g) - g + 0.5) / n
    left = x < case.x0
    vals = {}
    for key, idx in (("rho", 0), ("u", 1), ("p", 2)):
        vals[key] = np.where(left, case.left[idx], case.right[idx])
    fluid1 = np.where(left, case.left[3] == 1, case.right[3] == 1)
    al = np.where(fluid1, 1.0 - EPS, EPS)
    rho, u, p = vals["rho"], vals["u"], vals["p"]
    g1, p1, g2, p2 = case.g1, case.p1, case.g2, case.p2
    gb = al / (g1 - 1.0) + (1.0 - al) / (g2 - 1.0)
    pb = al * g1 * p1 / (g1 - 1.0) + (1.0 - al) * g2 * p2 / (g2 - 1.0)
    E = gb * p + pb + 0.5 * rho * u * u
    return {"ar1": al * rho, "ar2": (1.0 - al) * rho, "ru": rho * u, "rv": np.zeros_like(rho), "E": E,
            "al": al, "u_p": u, "v_p": np.zeros_like(rho), "p_p": p, "al_prim": al.copy()}


def initial_grid(case: Case, n: int, along: str, width: int = 1, g: int = G) -> dict:
    """Padded (nxg, nyg) fields of the tube laid along x or y, `width` cells across."""
    line = initial_line(case, n, g)
    out = {}
    for k, v in line.items():
        if along == "x":
            out[k] = np.ascontiguousarray(np.repeat(v[:, None], width + 2 * g, axis=1))
        else:
            out[k] = np.ascontiguousarray(np.repeat(v[None, :], width + 2 * g, axis=0))
    if along == "y":  # the normal velocity of the tube is v
        out["ru"], out["rv"] = out["rv"], out["ru"]
        out["u_p"], out["v_p"] = out["v_p"], out["u_p"]
    return out


def density_line(fields: dict, n: int, along: str, g: int = G) -> np.ndarray:
    rho = np.asarray(fields["ar1"]) + np.asarray(fields["ar2"])
    return rho[g:g + n, g] if along == "x" else rho[g, g:g + n]


def l1_error(case: Case, rho: np.ndarray) -> float:
    L, R = case.sides()
    exact, _, _, _ = rx.solve(L, R, centres(rho.size), case.x0, case.t_end)
    return float(np.abs(rho - exact).sum() / np.abs(exact).sum())


def run_oracle(case: Case, n: int, variant: str = "sc", recon: str = "shipped", along: str = "x") -> dict:
    """The oracle's solve of the tube (n cells, transmissive sides) to case.t_end; padded fields."""
    from oracle import oracle as orc

    nx, ny = (n, 1) if along == "x" else (1, n)
    P = orc.make_params(1.0 / nx, 1.0 / ny, case.g1, case.p1, case.g2, case.p2,
                        variant=orc.M10 if variant == "m10" else orc.SC,
                        recon=orc.MP5C6 if recon == "mp5c6" else orc.SHIPPED, bc=(orc.TRANSMISSIVE,) * 4)
    s = orc.PackedOracle(nx, ny, P)
    init = initial_grid(case, n, along)
    for c, k in enumerate(orc.ALL10):
        s.fields[c][...] = init[k]
    s.init_sequence()
    time_loop(lambda dt: s.steps(1, dt), s.get_dt(), case.t_end)
    return {k: s.fields[c].copy() for c, k in enumerate(orc.ALL10)}


def time_loop(step, dt: float, t_end: float) -> int:
    """The reference's time loop (SC:2009-2073) without save times: while t < t_end - 1e-14, clamp
    dt to t_end, step (step(dt) returns the next CFL dt). Returns the number of steps."""
    t, n = 0.0, 0
    while t < t_end - 1.0e-14:
        if t + dt > t_end:
            dt = t_end - t
        dt_next = step(dt)
        t += dt
        n += 1
        dt = dt_next
    return n
