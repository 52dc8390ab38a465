"""Pin the CPU oracle against golden vectors produced by the reference's own kernel source.

The fixtures in tests/golden/ come from tests/golden/make_golden.py, which executes the Warp
functions and kernels of sainath_SC_it_works.py / Sainath_M10.py on the CPU. The oracle is a C
restatement compiled without fused multiply-add, so every intermediate array of a stage, the state
after a full SSP-RK3 step and the time step must agree BIT FOR BIT (x86-64; on other hosts libm's
pow/tanh may differ in the last bit, so there the comparison allows 1e-13 relative).
"""
import glob
import os
import platform
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
from oracle import oracle as orc  # noqa: E402
sys.path.insert(0, os.path.join(ROOT, "tests"))

GOLDEN = os.path.join(ROOT, "tests", "golden")
CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
               if not p.endswith(("units.npz", "checkpoint.npz")))
EXACT = platform.machine() in ("x86_64", "AMD64")
FIELDS, PRIMS = orc.FIELDS, orc.PRIMS


def same(a, b, what):
    a, b = np.asarray(a), np.asarray(b)
    if EXACT:
        bad = ~((a == b) | (np.isnan(a) & np.isnan(b)))
        assert not bad.any(), f"{what}: {bad.sum()} entries differ, max |d|={np.nanmax(np.abs(a - b))}"
    else:
        np.testing.assert_allclose(a, b, rtol=1e-13, atol=1e-300, err_msg=what)


def solver_for(d):
    variant = orc.M10 if str(d["meta_variant"]) == "m10" else orc.SC
    recon = orc.MP5C6 if str(d["meta_recon"]) == "mp5c6" else orc.SHIPPED
    P = orc.make_params(float(d["meta_dx"]), float(d["meta_dy"]), float(d["meta_g1"]),
                        float(d["meta_p1"]), float(d["meta_g2"]), float(d["meta_p2"]),
                        variant=variant, recon=recon)
    return orc.OracleSolver(int(d["meta_nx"]), int(d["meta_ny"]), P, g=int(d["meta_g"]))


@pytest.fixture(scope="module", params=CASES)
def case(request):
    return request.param, np.load(os.path.join(GOLDEN, request.param + ".npz"))


def test_cases_present():
    assert len(CASES) >= 8


def test_init_sequence(case):
    name, d = case
    s = solver_for(d)
    s.load({k: d["ic_" + k] for k in FIELDS + PRIMS})
    s.init_sequence()
    for k in orc.ALL10:
        same(s.f[k], d["in_" + k], f"{name} init {k}")
    same(s.get_dt(), d["dt0"], f"{name} dt0")


def test_stage_intermediates(case):
    name, d = case
    s = solver_for(d)
    s.load({k: d["in_" + k] for k in orc.ALL10})
    dt = float(d["dt0"])
    s.copy_old()
    rec = {}
    s.apply_bc()
    for k in FIELDS + PRIMS:
        same(s.f[k], d["s1_bc_" + k], f"{name} bc {k}")
    s.compute_fluxes()
    if "s1_sigma_x" in d.files:
        same(s.sigma_x, d["s1_sigma_x"], f"{name} sigma_x")
        same(s.sigma_y, d["s1_sigma_y"], f"{name} sigma_y")
    names_x = [f"fx{c}" for c in range(6)] + ["srcx"]
    names_y = [f"gy{c}" for c in range(6)] + ["srcy"]
    for c in range(7):
        same(s.fh[c], d["s1_high_" + names_x[c]], f"{name} high {names_x[c]}")
        same(s.gh[c], d["s1_high_" + names_y[c]], f"{name} high {names_y[c]}")
    s.compute_low_fluxes()
    lx = [f"fxl{c}" for c in range(6)] + ["srcxl"]
    ly = [f"gyl{c}" for c in range(6)] + ["srcyl"]
    for c in range(7):
        same(s.fl[c], d["s1_low_" + lx[c]], f"{name} low {lx[c]}")
        same(s.gl[c], d["s1_low_" + ly[c]], f"{name} low {ly[c]}")
    s.limit_fluxes(dt, rec)
    for st in range(3):
        same(rec[f"theta{st}"], d[f"s1_theta{st}"], f"{name} theta{st}")
    for c in range(7):
        same(s.fh[c], d["s1_lim_" + names_x[c]], f"{name} lim {names_x[c]}")
        same(s.gh[c], d["s1_lim_" + names_y[c]], f"{name} lim {names_y[c]}")
    s.rk3_update(0.0, 1.0, dt)
    for k in FIELDS:
        same(s.f[k], d["s1_rk3_" + k], f"{name} rk3 {k}")
    s.enforce_admissible()
    for k in FIELDS:
        same(s.f[k], d["s1_adm_" + k], f"{name} admissible {k}")
    s.update_prims()
    for k in orc.ALL10:
        same(s.f[k], d["s1_out_" + k], f"{name} prims {k}")


def test_full_steps(case):
    name, d = case
    s = solver_for(d)
    s.load({k: d["in_" + k] for k in orc.ALL10})
    dt = s.step(float(d["dt0"]))
    for k in orc.ALL10:
        same(s.f[k], d["step1_" + k], f"{name} step1 {k}")
    same(dt, d["dt1"], f"{name} dt1")
    for _ in range(1, int(d["meta_steps"])):
        dt = s.step(dt)
    for k in orc.ALL10:
        same(s.f[k], d["final_" + k], f"{name} final {k}")
    same(dt, d["dt_final"], f"{name} dt_final")


def test_packed_steps_match_closures(case):
    """The all-C step loop (CPU baseline) equals the closure-by-closure path."""
    name, d = case
    s = solver_for(d)
    p = orc.PackedOracle(s.nx, s.ny, s.P, g=s.g)
    for c, k in enumerate(orc.ALL10):
        p.fields[c][...] = d["in_" + k]
    dt = p.steps(int(d["meta_steps"]), float(d["dt0"]))
    for c, k in enumerate(orc.ALL10):
        same(p.fields[c], d["final_" + k], f"{name} packed final {k}")
    same(dt, d["dt_final"], f"{name} packed dt")


@pytest.fixture(scope="module")
def units():
    return np.load(os.path.join(GOLDEN, "units.npz"))


def test_unit_functions(units):
    u = units
    P = orc.make_params(1.0, 1.0, 4.4, 6.0e8, 1.4, 0.0)
    st = u["stencil"]
    for fn, key, k in (("mp5_ul", "mp5_ul", 5), ("mp5_ur", "mp5_ur", 5), ("central6", "central6", 6),
                       ("muscl_ul", "muscl_ul", 4), ("muscl_ur", "muscl_ur", 4),
                       ("thinc_ul", "thinc_ul", 3), ("thinc_ur", "thinc_ur", 3),
                       ("cator2", "cator2", 5), ("mm4", "mm4", 4), ("mm2", "mm2", 2)):
        same(orc.unit(fn, P, st[:, :k], 1)[:, 0], u[key], fn)
    eos = orc.unit("eos", P, u["eos_a1"][:, None], 2)
    same(eos[:, 0], u["eos_g"], "eos g")
    same(eos[:, 1], u["eos_pinf"], "eos pinf")
    lr = np.concatenate([u["hllc_L"], u["hllc_R"]], axis=1)
    hx = orc.unit("hllc_x", P, lr, 7)
    hy = orc.unit("hllc_y", P, lr, 7)
    same(hx[:, :6], u["hllc_x"], "hllc_x")
    same(hy[:, :6], u["hllc_y"], "hllc_y")
    same(hx[:, 6], u["hllc_x_src"], "hllc_x_src")
    same(hy[:, 6], u["hllc_y_src"], "hllc_y_src")
    eig = orc.unit("eigen", P, np.concatenate([u["eig_U"], u["eig_avg"]], axis=1), 24)
    same(eig[:, 0:6], u["to_char_x"], "to_char_x")
    same(eig[:, 6:12], u["to_phys_x"], "to_phys_x")
    same(eig[:, 12:18], u["to_char_y"], "to_char_y")
    same(eig[:, 18:24], u["to_phys_y"], "to_phys_y")
    lim = orc.unit("pplim", P, np.concatenate([u["pplim_high"], u["pplim_base"]], axis=1), 6)
    same(lim, u["pplim_out"], "pp_limit_reconstructed_state")
    th = orc.unit("theta", P, np.concatenate([u["theta_l"], u["theta_h"]], axis=1), 3)
    same(th, u["theta_out"], "theta_cons_stage")


def test_hllc_branch_coverage(units):
    """The HLLC vectors exercise all four wave-pattern branches (SL>0, star-L, star-R, SR<0)."""
    u = units
    P = orc.make_params(1.0, 1.0, 4.4, 6.0e8, 1.4, 0.0)
    L, R = u["hllc_L"], u["hllc_R"]
    seen = set()
    for l, r in zip(L, R):
        rl, rr = l[0] + l[1], r[0] + r[1]
        eos = orc.unit("eos", P, np.array([[l[5]], [r[5]]]), 2)
        cl = np.sqrt(max(eos[0, 0] * (l[4] + eos[0, 1]) / rl, 1e-20))
        cr = np.sqrt(max(eos[1, 0] * (r[4] + eos[1, 1]) / rr, 1e-20))
        sl = min(l[2] - cl, 0.5 * (l[2] + r[2]) - 0.5 * (cl + cr))
        sr = max(r[2] + cr, 0.5 * (l[2] + r[2]) + 0.5 * (cl + cr))
        den = rl * (sl - l[2]) - rr * (sr - r[2])
        sp = (r[4] - l[4] + rl * l[2] * (sl - l[2]) - rr * r[2] * (sr - r[2])) / den
        seen.add(0 if sl > 0 else 1 if sp > 0 else 2 if sr >= 0 else 3)
    assert seen == {0, 1, 2, 3}


def test_cases_are_well_conditioned(case):
    """Every fixture is reproducible to round-off: the oracle on inputs perturbed by 1e-15 relative
    noise stays within a tenth of the GPU parity tolerances (parity_util), so a GPU result that
    differs from the fixture by more than the tolerance differs in arithmetic, not in round-off
    amplified by the problem. (Near-vacuum states of the M10 staged limiter fail this and are
    not fixtures.)"""
    import parity_util as pu

    name, d = case
    sc = pu.case_scales(d)
    nx_ = [f"fx{c}" for c in range(6)] + ["srcx"]
    ny_ = [f"gy{c}" for c in range(6)] + ["srcy"]
    rng = np.random.default_rng(1)
    s = solver_for(d)
    s.load({k: d["in_" + k] * (1 + 1e-15 * rng.standard_normal(d["in_" + k].shape)) for k in orc.ALL10})
    s.copy_old()
    rec = {}
    s.stage(0.0, 1.0, float(d["dt0"]), rec)
    for c in range(7):
        assert pu.flux_err(rec["lim_fx"][c], rec["lim_gy"][c], d["s1_lim_" + nx_[c]],
                           d["s1_lim_" + ny_[c]], sc["flux"][c]) <= 1e-11, (name, c)
    got = {k: s.f[k] for k in orc.ALL10}
    ref = {k: d["s1_out_" + k] for k in orc.ALL10}
    for k in orc.ALL10:
        assert pu.cell_err(got, ref, k, sc) <= 1e-11, (name, k)
    s2 = solver_for(d)
    s2.load({k: d["in_" + k] * (1 + 1e-15 * rng.standard_normal(d["in_" + k].shape)) for k in orc.ALL10})
    dt = float(d["dt0"])
    for _ in range(int(d["meta_steps"])):
        dt = s2.step(dt)
    got = {k: s2.f[k] for k in orc.ALL10}
    ref = {k: d["final_" + k] for k in orc.ALL10}
    for k in orc.ALL10:
        assert pu.cell_err(got, ref, k, sc) <= 1e-10, (name, k)
