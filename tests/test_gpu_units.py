"""The binary64 face sweep's device functions, one at a time, against the reference's own outputs.

tests/golden/units.npz holds the reference's device functions (SC:83-771) evaluated on seeded
inputs: MP5 (left and right), central-6, MUSCL, THINC, cator2, minmod-2/4, the mixture EOS, HLLC in x
and y with the interface velocity (the vectors cover all four wave-pattern branches), the
characteristic projections and back-projections, M10's staged limiter on reconstructed states and
the three limiter bound solves. A test-only library (tests/csrc/wm_units.cu) runs the CUDA device
functions of csrc/wm_device.cuh on the same rows, in the forms the sweep uses (MP5 in difference
form, refined reciprocals and roots, integer-pipe minmods and sign selection).

Tolerances: the minmods are bit-identical (they select, they do not round); every other value is
within 1e-12 of its natural scale (the component's largest magnitude over the vectors, or the
stencil's, or 1 for limiter factors) -- the sweep contracts multiply-adds and refines reciprocals,
so values differ from the no-FMA reference by a few units in the last place. The interface
velocity at SP = +-0 agrees with the oracle's (which the oracle tests pin to the reference) within
round-off of the wave speeds, and the sign selection behind it (Warp's sign(0) = +1 picks the left
state) is bit-identical to the reference's products.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import units_lib as ul  # noqa: E402
from oracle import oracle as orc  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-12


@pytest.fixture(scope="module")
def u():
    return np.load(os.path.join(GOLDEN, "units.npz"))


def normwise(got, ref, what, scale=None, tol=TOL):
    got, ref = np.atleast_2d(np.asarray(got).T).T, np.atleast_2d(np.asarray(ref).T).T
    for c in range(ref.shape[1]):
        s = float(np.abs(ref[:, c]).max()) if scale is None else scale
        d = float(np.abs(got[:, c] - ref[:, c]).max())
        assert np.isfinite(d) and d <= tol * max(s, 1e-300), f"{what}[{c}]: {d:.3e} vs scale {s:.3e}"


def test_stencil_functions(u):
    st = u["stencil"]
    for fn, k in (("mp5_ul", 5), ("mp5_ur", 5), ("central6", 6), ("muscl_ul", 4), ("muscl_ur", 4),
                  ("thinc_ul", 3), ("thinc_ur", 3), ("cator2", 5)):
        got = ul.unit(fn, st[:, :k], 1)[:, 0]
        ref = u[fn]
        scale = np.maximum(np.abs(st[:, :k]).max(axis=1), np.abs(ref))
        d = np.abs(got - ref) / np.maximum(scale, 1e-300)
        assert d.max() <= TOL, f"{fn}: row {int(d.argmax())} differs by {d.max():.3e} of its scale"


def test_minmods_are_bit_identical(u):
    st = u["stencil"]
    for fn, k in (("mm4", 4), ("mm2", 2)):
        got = ul.unit(fn, st[:, :k], 1)[:, 0]
        assert np.array_equal(got.view(np.int64), u[fn].view(np.int64)), fn


def test_mixture_eos(u):
    got = ul.unit("eos", u["eos_a1"][:, None], 2)
    normwise(got[:, 0:1], u["eos_g"][:, None], "eos gamma", tol=1e-15)
    normwise(got[:, 1:2], u["eos_pinf"][:, None], "eos p_inf", tol=1e-15)


def test_hllc_all_branches(u):
    lr = np.concatenate([u["hllc_L"], u["hllc_R"]], axis=1)
    for d, key in ((0, "hllc_x"), (1, "hllc_y")):
        got = ul.unit(key, lr, 7)
        normwise(got[:, :6], u[key], key)
        normwise(got[:, 6:7], u[key + "_src"][:, None], key + " interface velocity")


def interface_cases():
    """States whose contact speed SP is exactly +-0 (equal pressures at rest, with equal or
    different densities and volume fractions) and symmetric collisions, where SP is round-off."""
    rows = []
    for rho1, rho2, a in ((1000.0, 1.2, 0.5), (2.0, 0.5, 1e-6), (800.0, 3.0, 1 - 1e-6)):
        L = [a * rho1, (1 - a) * rho2, 0.0, 0.0, 1.0e5, a]
        rows.append(L + L)
        R = [0.3 * rho1, 0.7 * rho2, 0.0, 25.0, 1.0e5, 0.3]
        rows.append(L + R)
        rows.append([a * rho1, (1 - a) * rho2, 100.0, 0.0, 1.0e5, a] +
                    [a * rho1, (1 - a) * rho2, -100.0, 0.0, 1.0e5, a])
        rows.append([a * rho1, (1 - a) * rho2, 0.0, 100.0, 1.0e5, a] +
                    [a * rho1, (1 - a) * rho2, 0.0, -100.0, 1.0e5, a])
    return np.array(rows)


def test_interface_velocity_at_zero_contact_speed():
    """At SP = +-0 both sides' interface velocities are 0 up to round-off of the wave speeds (the
    star-state ratio is 1 in exact arithmetic), so u* agrees with the reference's within round-off
    of the largest wave speed, and the fluxes within their scale."""
    rows = interface_cases()
    P = orc.make_params(1.0, 1.0, 4.4, 6.0e8, 1.4, 0.0)
    w = 1.0e4  # bounds |u| + c of these states
    rho = float((rows[:, 0] + rows[:, 1]).max())
    # natural flux scales (mass, momentum, energy, volume fraction): the fluxes of a fluid at rest
    # are round-off of these, not of their own (zero) values
    scales = (rho * w, rho * w, rho * w * w, rho * w * w, 1.0e9 * w, w)
    for key in ("hllc_x", "hllc_y"):
        got = ul.unit(key, rows, 7)
        ref = orc.unit(key, P, rows, 7)
        d = np.abs(got[:, 6] - ref[:, 6]).max()
        assert d <= 1e-14 * w, f"{key} u* differs by {d:.3e}"
        for c in range(6):
            normwise(got[:, c], ref[:, c], f"{key} flux {c} at SP = 0", scale=scales[c])


def test_sign_selection_is_warps_bit_for_bit():
    """u* = 0.5 (1 + s) left + 0.5 (1 - s) right with s = wp.sign(SP) (SC:686, 770; Warp: -1 for
    SP < 0, +1 otherwise, so SP = -0 and NaN pick the left side): the sweep's integer-pipe
    selection against the reference's products in IEEE binary64, zeros' signs, infinities and NaN
    included."""
    specials = [0.0, -0.0, 5e-324, -5e-324, 1.0, -1.0, 1e300, -1e300, np.inf, -np.inf, np.nan]
    rng = np.random.default_rng(4)
    rows = [[sp, a, b] for sp in specials for a in specials + [2.5] for b in specials + [-7.0]]
    rows += list(rng.standard_normal((2000, 3)))
    rows = np.array(rows, dtype=np.float64)
    got = ul.unit("sign_select", rows, 1)[:, 0]
    with np.errstate(invalid="ignore", over="ignore"):
        s = np.where(rows[:, 0] < 0, -1.0, 1.0)
        ref = 0.5 * (1.0 + s) * rows[:, 1] + 0.5 * (1.0 - s) * rows[:, 2]
    same = (got.view(np.int64) == ref.view(np.int64)) | (np.isnan(got) & np.isnan(ref))
    assert same.all(), rows[~same][:5]


def test_projections(u):
    rows = np.concatenate([u["eig_U"], u["eig_avg"], u["to_char_x"], u["to_char_y"]], axis=1)
    got = ul.unit("eigen", rows, 24)
    normwise(got[:, 0:6], u["to_char_x"], "to_char_x")
    normwise(got[:, 6:12], u["to_phys_x"], "to_phys_x")
    normwise(got[:, 12:18], u["to_char_y"], "to_char_y")
    normwise(got[:, 18:24], u["to_phys_y"], "to_phys_y")


def test_staged_limiter_and_bound_solves(u):
    got = ul.unit("pplim", np.concatenate([u["pplim_high"], u["pplim_base"]], axis=1), 6)
    normwise(got, u["pplim_out"], "pp_limit_reconstructed_state")
    got = ul.unit("theta", np.concatenate([u["theta_l"], u["theta_h"]], axis=1), 3)
    normwise(got, u["theta_out"], "theta_cons_stage", scale=1.0)


def test_ratio_precheck_series_within_their_bound():
    """log1p_pc and expm1_pc (the ratio pre-check's log1p and expm1: the fifth-order series for
    |x| <= 2^-5, CUDA's log1pf / expm1f beyond) within 2^-22.9 of the exact values on binary32
    arguments over the range the pre-check admits (|x| <= 0.5), the series' edge included."""
    rng = np.random.default_rng(9)
    x = np.concatenate([rng.uniform(-0.5, 0.5, 400_000),
                        np.sign(rng.standard_normal(400_000)) * 10.0 ** rng.uniform(-38, -1.5, 400_000),
                        np.array([0.0, -0.0, 0.03125, -0.03125, 0.0312500037, -0.0312500037, 2.0 ** -126,
                                  1e-45, 0.5, -0.5])]).astype(np.float32).astype(np.float64)
    for fn, ref in (("log1p_pc", np.log1p), ("expm1_pc", np.expm1)):
        got = ul.unit(fn, x[:, None], 1)[:, 0]
        exact = ref(x)
        tiny = np.abs(exact) < 2.0 ** -126  # binary32 subnormal results: absolute 2^-149
        rel = np.abs(got - exact) / np.where(tiny, 1.0, np.abs(exact))
        bound = np.where(tiny, 2.0 ** -148, 2.0 ** -22.9)
        assert (rel <= bound).all(), (fn, x[rel > bound][:4], got[rel > bound][:4])
