"""Exact solution of the 1-D Riemann problem for two stiffened gases (test infrastructure).

Each side K has its own EOS p = (gamma_K - 1) rho e - gamma_K p_inf_K, sound speed
c^2 = gamma_K (p + p_inf_K) / rho. The solution follows the exact Riemann solver of Toro, "Riemann
Solvers and Numerical Methods for Fluid Dynamics" (3rd ed., ch. 4), with the pressure of each side
shifted by its p_inf: in the shock and rarefaction relations p becomes p + p_inf_K (the form used for
stiffened-gas shock tubes, e.g. Ivings, Causon & Toro, Int. J. Numer. Meth. Fluids 28 (1998)). The
contact separates the two gases, so a gas-water tube is solved with the gas EOS left of it and the
water EOS right of it (or the reverse).

The star pressure is the root of f_L(p) + f_R(p) + u_R - u_L by Newton's method from Toro's
primitive-variable estimate, kept above -min(p_inf_L, p_inf_R).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class Side:
    rho: float
    u: float
    p: float
    gamma: float
    pinf: float = 0.0

    @property
    def c(self) -> float:
        return math.sqrt(self.gamma * (self.p + self.pinf) / self.rho)


def _f(p: float, s: Side) -> tuple[float, float]:
    """Toro's f_K and its derivative for side s (shifted pressures)."""
    g, pi = s.gamma, s.pinf
    ps, pk = p + pi, s.p + pi
    if p > s.p:  # shock
        A = 2.0 / ((g + 1.0) * s.rho)
        B = (g - 1.0) / (g + 1.0) * pk
        q = math.sqrt(A / (ps + B))
        return (p - s.p) * q, q * (1.0 - 0.5 * (p - s.p) / (B + ps))
    r = ps / pk  # rarefaction
    c = s.c
    return (2.0 * c / (g - 1.0) * (r ** ((g - 1.0) / (2.0 * g)) - 1.0),
            1.0 / (s.rho * c) * r ** (-(g + 1.0) / (2.0 * g)))


def star_state(L: Side, R: Side, tol: float = 1.0e-14, maxit: int = 200) -> tuple[float, float]:
    """(p*, u*) of the Riemann problem."""
    floor = -min(L.pinf, R.pinf) + 1.0e-12 * max(1.0, L.p + L.pinf, R.p + R.pinf)
    # primitive-variable (linearised) estimate
    p = max(0.5 * (L.p + R.p) - 0.125 * (R.u - L.u) * (L.rho + R.rho) * (L.c + R.c), floor)
    for _ in range(maxit):
        fl, dl = _f(p, L)
        fr, dr = _f(p, R)
        step = (fl + fr + R.u - L.u) / (dl + dr)
        p_new = p - step
        if p_new <= floor:
            p_new = 0.5 * (p + floor)
        if abs(p_new - p) <= tol * 0.5 * (abs(p_new) + abs(p)):
            p = p_new
            break
        p = p_new
    else:
        raise RuntimeError("star pressure did not converge")
    fl, _ = _f(p, L)
    fr, _ = _f(p, R)
    return p, 0.5 * (L.u + R.u) + 0.5 * (fr - fl)


def _sample_side(S: float, s: Side, p_star: float, u_star: float, sign: float):
    """(rho, u, p) at speed S = (x - x0) / t on the side of s (sign -1 left, +1 right)."""
    g, pi = s.gamma, s.pinf
    c = s.c
    ratio = (p_star + pi) / (s.p + pi)
    gm = (g - 1.0) / (g + 1.0)
    if p_star > s.p:  # shock
        rho_star = s.rho * (ratio + gm) / (gm * ratio + 1.0)
        speed = s.u + sign * c * math.sqrt((g + 1.0) / (2.0 * g) * ratio + (g - 1.0) / (2.0 * g))
        outside = S < speed if sign < 0 else S > speed
        return (s.rho, s.u, s.p) if outside else (rho_star, u_star, p_star)
    rho_star = s.rho * ratio ** (1.0 / g)
    c_star = c * ratio ** ((g - 1.0) / (2.0 * g))
    head = s.u + sign * c
    tail = u_star + sign * c_star
    if (S < head) if sign < 0 else (S > head):
        return s.rho, s.u, s.p
    if (S > tail) if sign < 0 else (S < tail):
        return rho_star, u_star, p_star
    # inside the fan
    k = 2.0 / (g + 1.0)
    u = k * (-sign * c + 0.5 * (g - 1.0) * s.u + S)
    cf = k * (c - sign * 0.5 * (g - 1.0) * (s.u - S))
    rho = s.rho * (cf / c) ** (2.0 / (g - 1.0))
    p = (s.p + pi) * (cf / c) ** (2.0 * g / (g - 1.0)) - pi
    return rho, u, p


def solve(L: Side, R: Side, x: np.ndarray, x0: float, t: float):
    """(rho, u, p, left) at positions x and time t > 0 for the discontinuity at x0; `left` is True
    where the gas of the left side is found (left of the contact)."""
    p_star, u_star = star_state(L, R)
    out = np.zeros((4, x.size))
    for k, xv in enumerate(np.asarray(x, dtype=np.float64)):
        S = (xv - x0) / t
        if S <= u_star:
            rho, u, p = _sample_side(S, L, p_star, u_star, -1.0)
            out[:, k] = (rho, u, p, 1.0)
        else:
            rho, u, p = _sample_side(S, R, p_star, u_star, +1.0)
            out[:, k] = (rho, u, p, 0.0)
    return out[0], out[1], out[2], out[3] > 0.5
