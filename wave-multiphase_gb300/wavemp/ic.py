"""Initial states of the benchmark configurations, generated on the device with torch.

The reference writes its initial state with ``ic_kernel2`` (SC:779-837, M10:736-790): partial
densities, momenta, total energy from the mixture EOS (SC:105-110), alpha1 and the primitives, over
the whole padded grid (ghost cells included). These generators produce the same ten arrays for the
configurations of the benchmark; ``Solver.initialize`` then runs the reference's start-up
sequence (SC:1998-2007).

* ``shock_droplet``: water disk in air hit by a planar air shock whose post-shock state follows
  from the Rankine-Hugoniot relations (configurations 0, 2, 3, 4). The volume fraction is a tanh
  profile alpha1 = eps + (1-2 eps) * (1 - tanh((r - R) / (2 dx))) / 2.
* ``triple_point``: the gas-gas triple-point problem on [0,7] x [0,3] (configuration 1), sharp
  interfaces at cell centres.
* ``random_valid``: a seeded droplet state with multiplicative noise, for parity tests.
"""
from __future__ import annotations

import math

import numpy as np
import torch

G = 5


def _centres(n, lo, hi, g, device):
    d = (hi - lo) / n
    return lo + (torch.arange(n + 2 * g, dtype=torch.float64, device=device) - g + 0.5) * d, d


def _pack(ar1, ar2, u, v, p, al, g1, p1, g2, p2):
    rho = ar1 + ar2
    gb = al / (g1 - 1.0) + (1.0 - al) / (g2 - 1.0)
    pb = al * g1 * p1 / (g1 - 1.0) + (1.0 - al) * g2 * p2 / (g2 - 1.0)
    E = gb * p + pb + 0.5 * rho * (u * u + v * v)
    out = {"ar1": ar1, "ar2": ar2, "ru": rho * u, "rv": rho * v, "E": E, "al": al,
           "u_p": u, "v_p": v, "p_p": p, "al_prim": al.clone()}
    return {k: t.contiguous() for k, t in out.items()}


def rankine_hugoniot(mach, gamma=1.4, p1=1.0e5, rho1=1.2):
    """Post-shock (p, rho, u) behind a normal shock of Mach `mach` moving into gas at rest."""
    p2 = p1 * (1.0 + 2.0 * gamma / (gamma + 1.0) * (mach * mach - 1.0))
    rho2 = rho1 * (gamma + 1.0) * mach * mach / ((gamma - 1.0) * mach * mach + 2.0)
    u2 = mach * math.sqrt(gamma * p1 / rho1) * (1.0 - rho1 / rho2)
    return p2, rho2, u2


def shock_droplet(nx, ny, lx=1.0, ly=0.5, mach=2.4, xc=0.3, yc=0.25, radius=0.1, x_shock=0.15,
                  eps=1.0e-6, rho_w=1000.0, rho_a=1.2, p_a=1.0e5, g1=4.4, p1=6.0e8, g2=1.4,
                  p2=0.0, g=G, device="cuda") -> dict:
    x, dx = _centres(nx, 0.0, lx, g, device)
    y, _ = _centres(ny, 0.0, ly, g, device)
    X, Y = torch.meshgrid(x, y, indexing="ij")
    r = torch.sqrt((X - xc) ** 2 + (Y - yc) ** 2)
    al = eps + (1.0 - 2.0 * eps) * 0.5 * (1.0 - torch.tanh((r - radius) / (2.0 * dx)))
    ps, rs, us = rankine_hugoniot(mach, g2, p_a, rho_a)
    post = X < x_shock
    rho_air = torch.where(post, torch.full_like(X, rs), torch.full_like(X, rho_a))
    u = torch.where(post, torch.full_like(X, us), torch.zeros_like(X))
    p = torch.where(post, torch.full_like(X, ps), torch.full_like(X, p_a))
    return _pack(al * rho_w, (1.0 - al) * rho_air, u, torch.zeros_like(X), p, al, g1, p1, g2, p2)


def triple_point(nx, ny, eps=1.0e-6, g=G, device="cuda") -> dict:
    """Fluid 1 (gamma 1.5) for x < 1 and for x >= 1, y >= 1.5; fluid 2 (gamma 1.4) for x >= 1,
    y < 1.5. Left: rho 1, p 1. Right bottom: rho 1, p 0.1. Right top: rho 0.125, p 0.1."""
    x, _ = _centres(nx, 0.0, 7.0, g, device)
    y, _ = _centres(ny, 0.0, 3.0, g, device)
    X, Y = torch.meshgrid(x, y, indexing="ij")
    left = X < 1.0
    top = (~left) & (Y >= 1.5)
    bottom = (~left) & (Y < 1.5)
    one = torch.ones_like(X)
    al = torch.where(bottom, eps * one, (1.0 - eps) * one)
    rho = torch.where(top, 0.125 * one, one)
    p = torch.where(left, one, 0.1 * one)
    z = torch.zeros_like(X)
    return _pack(al * rho, (1.0 - al) * rho, z, z.clone(), p, al, 1.5, 0.0, 1.4, 0.0)


def random_valid(nx, ny, rng: np.random.Generator, amp=0.05, g1=4.4, p1=6.0e8, g2=1.4, p2=0.0,
                 g=G, device="cuda") -> dict:
    """A droplet state with seeded multiplicative noise on every primitive (all cells valid)."""
    base = shock_droplet(max(nx, 8), max(ny, 8), 1.0, 0.5, 2.4, g=g, device="cpu", g1=g1, p1=p1,
                         g2=g2, p2=p2)
    sh = (nx + 2 * g, ny + 2 * g)
    pick = {k: v[: sh[0], : sh[1]].numpy() for k, v in base.items()}
    n = lambda: rng.standard_normal(sh)  # noqa: E731
    al = np.clip(pick["al"] * (1 + amp * n()), 1e-8, 1 - 1e-8)
    ar1 = np.abs(pick["ar1"] * (1 + amp * n())) + 1e-9
    ar2 = np.abs(pick["ar2"] * (1 + amp * n())) + 1e-9
    c = math.sqrt(1.4e5 / 1.2)
    u = pick["u_p"] + amp * c * n()
    v = pick["v_p"] + amp * c * n()
    p = pick["p_p"] * (1 + amp * n())
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device)  # noqa: E731
    return _pack(t(ar1), t(ar2), t(u), t(v), t(p), t(al), g1, p1, g2, p2)
