"""Checkpoint output and restart in the reference's ``.npz`` schema.

* ``save_npz`` follows ``save_npz`` (SC:1714-1726): a compressed ``{prefix}_{step:06d}.npz`` with
  ``time`` (float64 scalar), the interior cell centres ``x`` (nx) and ``y`` (ny), and the interior
  (nx, ny) float64 arrays ``rho`` = ar1 + ar2, ``ar1``, ``ar2``, ``u``, ``v``, ``p`` and ``alpha1``
  (the conserved volume fraction ``al``, not ``al_prim``).
* ``load_restart`` follows ``load_restart_host`` (SC:1779-1821) and ``infer_restart_step``
  (SC:1773-1776): it needs ``ar1 ar2 u v p alpha1`` (KeyError otherwise) of shape (nx, ny)
  (ValueError otherwise), clips alpha1 to [1e-8, 1 - 1e-8], rebuilds rho u, rho v and E from the
  primitives, zeroes the ghost cells (and ``al_prim``), and takes the time from ``time`` (0 when
  absent) and the step from the last ``_`` field of the file name (0 when not a number). The
  caller then runs the start-up sequence (``Solver.initialize``), as the reference does
  (SC:1998-2005).

One deliberate difference: the reference rebuilds E with its hard-coded water EOS (gamma 6.12,
p_inf 3.43e8, gas p_inf 0; SC:1811-1813) whatever the run's constants; here E uses the run's own
EOS from ``SolverParams``. With the reference's constants the arithmetic is the reference's, term
for term, and the result is bit-identical; the gas-2 stiffness term is added only when p_inf2 != 0.
The rebuild runs on the device (torch element-wise operations, which do not fuse multiply-adds;
divisions by the EOS constants are divisions by tensors, which CUDA rounds as IEEE division).
"""
from __future__ import annotations

import os

import numpy as np
import torch

from .params import SolverParams
from .solver import ALL

RESTART_KEYS = ("ar1", "ar2", "u", "v", "p", "alpha1")


def cell_centres(n: int, lo: float, hi: float, g: int = 5) -> np.ndarray:
    """Padded cell-centre coordinates lo + (i - g + 0.5) * d, d = (hi - lo) / n (SC:1831-1832)."""
    d = (hi - lo) / n
    return np.array([lo + (i - g + 0.5) * d for i in range(n + 2 * g)], dtype=np.float64)


def checkpoint_name(step: int, prefix: str = "mp5") -> str:
    return f"{prefix}_{step:06d}.npz"


def save_npz(q: dict, x, y, step: int, t: float, directory: str = ".", prefix: str = "mp5",
             g: int = 5) -> str:
    """Write the checkpoint of state `q` (ten padded arrays, on any device) at `step`, time `t`;
    `x`, `y` are the padded cell centres. Returns the file's path."""
    nxg, nyg = q["ar1"].shape
    nx, ny = nxg - 2 * g, nyg - 2 * g
    inner = (slice(g, g + nx), slice(g, g + ny))
    host = {k: q[k][inner].to("cpu").numpy() for k in ("ar1", "ar2", "u_p", "v_p", "p_p", "al")}
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    path = os.path.join(directory, checkpoint_name(step, prefix))
    np.savez_compressed(path, time=np.float64(t), x=x[g:g + nx], y=y[g:g + ny],
                        rho=host["ar1"] + host["ar2"], ar1=host["ar1"], ar2=host["ar2"],
                        u=host["u_p"], v=host["v_p"], p=host["p_p"], alpha1=host["al"])
    return path


def infer_restart_step(path: str) -> int:
    stem = os.path.splitext(os.path.basename(path))[0]
    tail = stem.split("_")[-1]
    return int(tail) if tail.isdigit() else 0


def load_restart(path: str, params: SolverParams, nx: int, ny: int, g: int = 5, device="cuda",
                 time: float | None = None, step: int | None = None):
    """Read a checkpoint into a new padded state. Returns (q, time, step)."""
    with np.load(path) as data:
        for key in RESTART_KEYS:
            if key not in data:
                raise KeyError(f"Restart file {path} is missing '{key}'")
        arr = {k: np.asarray(data[k], dtype=np.float64) for k in RESTART_KEYS}
        t_file = float(data["time"]) if "time" in data else 0.0
    if arr["ar1"].shape != (nx, ny):
        raise ValueError(f"Restart shape {arr['ar1'].shape} does not match {(nx, ny)}")
    dev = torch.device(device)
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in arr.items()}
    al = torch.clamp(d["alpha1"], 1.0e-8, 1.0 - 1.0e-8)
    ar1, ar2, u, v, p = d["ar1"], d["ar2"], d["u"], d["v"], d["p"]
    rho = ar1 + ar2
    g1, p1, g2, p2 = params.gamma1, params.pinf1, params.gamma2, params.pinf2

    def div(a, c):  # a true division (torch's CUDA kernels multiply by 1/c for a Python scalar c)
        return a / torch.full_like(a, c)

    gb = div(al, g1 - 1.0) + div(1.0 - al, g2 - 1.0)
    pb = div(al * g1 * p1, g1 - 1.0)
    if p2 != 0.0:
        pb = pb + div((1.0 - al) * g2 * p2, g2 - 1.0)
    E = gb * p + pb + 0.5 * rho * (u * u + v * v)
    interior = {"ar1": ar1, "ar2": ar2, "ru": rho * u, "rv": rho * v, "E": E, "al": al,
                "u_p": u, "v_p": v, "p_p": p}
    q = {k: torch.zeros((nx + 2 * g, ny + 2 * g), dtype=torch.float64, device=dev) for k in ALL}
    for k, val in interior.items():
        q[k][g:g + nx, g:g + ny] = val
    t = t_file if time is None else float(time)
    n = infer_restart_step(path) if step is None else int(step)
    return q, t, n
