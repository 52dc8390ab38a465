"""Shared helpers of the GPU parity tests (tolerances, fixture loading, state transfer)."""
from __future__ import annotations

import glob
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
               if not p.endswith(("units.npz", "checkpoint.npz")))
FIELDS = ("ar1", "ar2", "ru", "rv", "E", "al")
PRIMS = ("u_p", "v_p", "p_p")
ALL = FIELDS + PRIMS + ("al_prim",)

# FP64 parity tolerance of the hot-path specification: 1e-10 relative, measured in the units in
# which the reference's own result is determined (see natural_scales):
#  * cell arrays, element-wise: |a - b| <= 1e-10 (|b| + 1e-4 S_k). S_k is the largest magnitude of
#    array k, except: momenta use rho_max w and velocities use w, with w = max(|u| + |v| + c) the
#    largest wave speed (in a fluid at rest they are round-off of that size); pressure is compared
#    as p + p_inf(alpha), because a stiffened-gas pressure recovered from the total energy
#    (p = (E - Pi - kin) / Gamma) is only determined to round-off of E ~ p_inf.
#  * face fluxes, norm-wise: max |a - b| <= 1e-10 S_c with the natural scale of component c:
#    partial density x w for the mass fluxes, rho_max w^2 for momentum, (|E|+|p|)_max w for energy,
#    w for the volume-fraction flux and the interface velocity. A flux is a sum of terms of that
#    size and may be far smaller (a fluid at rest, a gas near its p_inf bound); with fused
#    multiply-add the cancellations end at round-off of S_c instead of exact zero.
RTOL_FP64 = 1e-10
FLOOR = 1e-4


def _scale(arrs):
    m = 0.0
    for b in arrs:
        b = np.asarray(b, dtype=np.float64)
        fin = np.isfinite(b)
        if fin.any():
            m = max(m, float(np.abs(b[fin]).max()))
    return m


def natural_scales(state: dict, g1, p1, g2, p2, g=5) -> dict:
    """Scales of `state`: w, rho_max, flux scales, and p_inf of every cell."""
    al_all = np.asarray(state["al"], dtype=np.float64)
    gb_all = al_all / (g1 - 1.0) + (1.0 - al_all) / (g2 - 1.0)
    pb_all = al_all * g1 * p1 / (g1 - 1.0) + (1.0 - al_all) * g2 * p2 / (g2 - 1.0)
    gam_all = 1.0 / gb_all + 1.0
    pinf_all = (gam_all - 1.0) * pb_all / gam_all
    sl = (slice(g, -g), slice(g, -g))
    ar1, ar2 = np.asarray(state["ar1"])[sl], np.asarray(state["ar2"])[sl]
    p = np.asarray(state["p_p"])[sl]
    u, v, E = np.asarray(state["u_p"])[sl], np.asarray(state["v_p"])[sl], np.asarray(state["E"])[sl]
    rho = ar1 + ar2
    c = np.sqrt(np.maximum(gam_all[sl] * (p + pinf_all[sl]) / rho, 1e-20))
    w = float(np.nanmax(np.abs(u) + np.abs(v) + c))
    rmax = float(np.nanmax(rho))
    flux = [float(np.nanmax(np.abs(ar1))) * w, float(np.nanmax(np.abs(ar2))) * w, rmax * w * w,
            rmax * w * w, float(np.nanmax(np.abs(E)) + np.nanmax(np.abs(p))) * w,
            float(np.nanmax(np.abs(al_all[sl]))) * w, w]
    return {"w": w, "rho_max": rmax, "flux": flux, "pinf": np.abs(pinf_all)}


def case_scales(d) -> dict:
    return natural_scales({k: d["in_" + k] for k in ALL}, float(d["meta_g1"]), float(d["meta_p1"]),
                          float(d["meta_g2"]), float(d["meta_p2"]), int(d["meta_g"]))


def _err(a, b, den):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    err = np.where(np.isnan(a) & np.isnan(b), 0.0, np.abs(a - b) / (den + 1e-300))
    err = np.where(np.isnan(err), np.inf, err)
    return float(err.max()) if err.size else 0.0


def rel_err(a, b, floor=FLOOR, scale=None):
    b = np.asarray(b, dtype=np.float64)
    if scale is None:
        scale = _scale([b])
    return _err(a, b, np.abs(b) + floor * scale)


def assert_close(a, b, what, rtol=RTOL_FP64, floor=FLOOR, scale=None):
    e = rel_err(a, b, floor, scale)
    assert e <= rtol, f"{what}: max relative error {e:.3e} > {rtol:.1e}"


def cell_err(got: dict, ref: dict, key: str, sc: dict) -> float:
    """Element-wise error of cell array `key` in its natural units (see the header)."""
    b = np.asarray(ref[key], dtype=np.float64)
    if key == "p_p":
        den = np.abs(b) + sc["pinf"] + FLOOR * _scale([b])
    elif key in ("ru", "rv"):
        den = np.abs(b) + FLOOR * sc["rho_max"] * sc["w"]
    elif key in ("u_p", "v_p"):
        den = np.abs(b) + FLOOR * sc["w"]
    else:
        den = np.abs(b) + FLOOR * _scale([b])
    return _err(got[key], b, den)


def assert_cells(got: dict, ref: dict, keys, sc: dict, what, rtol=RTOL_FP64):
    for k in keys:
        e = cell_err(got, ref, k, sc)
        assert e <= rtol, f"{what} {k}: max relative error {e:.3e} > {rtol:.1e}"


def flux_err(ax, ay, bx, by, scale) -> float:
    """Norm-wise error of one flux component over its x and y face arrays, relative to `scale`."""
    d = 0.0
    for a, b in ((ax, bx), (ay, by)):
        a, b = np.asarray(a), np.asarray(b)
        dd = np.abs(a - b)
        dd = np.where(np.isnan(a) & np.isnan(b), 0.0, dd)
        dd = np.where(np.isnan(dd), np.inf, dd)
        d = max(d, float(dd.max()))
    return d / (scale + 1e-300)


def assert_fluxes(ax, ay, bx, by, scales, what, rtol=RTOL_FP64):
    for c in range(len(bx)):
        e = flux_err(ax[c], ay[c], bx[c], by[c], scales[c])
        assert e <= rtol, f"{what} component {c}: norm-wise relative error {e:.3e} > {rtol:.1e}"


def assert_abs(a, b, what, atol):
    a, b = np.asarray(a), np.asarray(b)
    d = np.abs(a - b)
    d = np.where(np.isnan(a) & np.isnan(b), 0.0, d)
    d = np.where(np.isnan(d), np.inf, d)
    assert d.max() <= atol, f"{what}: max abs error {d.max():.3e} > {atol:.1e}"


def load_case(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def params_from(d, **over):
    import wavemp

    kw = dict(dx=float(d["meta_dx"]), dy=float(d["meta_dy"]), gamma1=float(d["meta_g1"]),
              pinf1=float(d["meta_p1"]), gamma2=float(d["meta_g2"]), pinf2=float(d["meta_p2"]),
              variant=str(d["meta_variant"]), recon=str(d["meta_recon"]))
    kw.update(over)
    return wavemp.SolverParams(**kw)


def to_device(d, prefix, names=ALL):
    import torch

    from wavemp import alloc_state

    nxg, nyg = d[prefix + names[0]].shape
    q = alloc_state(nxg - 10, nyg - 10, 5, names=names) if nxg > 10 else None
    for k in names:
        q[k].copy_(torch.from_numpy(np.ascontiguousarray(d[prefix + k])))
    return q


def host(t):
    return t.detach().cpu().numpy()
