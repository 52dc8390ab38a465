"""The first-order HLLC's finiteness proof (hllc_surely_finite in csrc/wm_device.cuh), restated in
numpy binary64 and checked against HLLC's own outputs.

The binary64 fused stage's face sweep forms only the first-order HLLC's wave speeds (fx_low_kernel,
SC:1303-1347, through hllc_x / hllc_y, SC:594-752) and writes one byte per face: 1 when the seven
first-order values are finite. Where every side value (ar1, ar2, rho, u_n, u_t, p, alpha, c, E of
both cells) is finite and at most 2^60 in magnitude, and S_L - u_L, S_R - u_R, S_L - S_P and
S_R - S_P are each at least 2^-60 in magnitude, the byte is 1 without forming the values: every
quotient and product HLLC forms is then bounded (|S_P| < 2^251, star ratios < 2^122, star
energies < 2^563, fluxes and u* < 2^750). Here: seeded side states of every magnitude from 2^-80
to 2^62 and of both signs, states whose contact speed sits within 2^-70 .. 2^-40 of a wave speed,
and states far outside the bounds. Wherever the test says finite, every output of both sides'
supersonic and star fluxes and both parts of u* must be finite and below those bounds; outside it
the outputs are formed and tested, so the test need only be sound.
"""
import numpy as np

TINY = 1.0e-20
FIELDS = ("ar1", "ar2", "rho", "un", "ut", "p", "a", "c", "E")


def side(rng, n, lo, hi):
    """Seeded side states: each value of magnitude 2^U(lo, hi), random sign (c >= 0)."""
    def mag():
        return np.exp2(rng.uniform(lo, hi, n))

    def signed():
        return mag() * rng.choice([-1.0, 1.0], n)

    s = {"ar1": mag(), "ar2": mag(), "un": signed(), "ut": signed(), "p": signed(), "a": rng.random(n),
         "c": mag(), "E": signed()}
    s["rho"] = s["ar1"] + s["ar2"]
    return s


def speeds(L, R):
    """hllc_speeds: S_L, S_R and the contact speed S_P, its divisor clamped (SC:594-612)."""
    n_avg = 0.5 * (L["un"] + R["un"])
    c_avg = 0.5 * (L["c"] + R["c"])
    SL = np.minimum(L["un"] - L["c"], n_avg - c_avg)
    SR = np.maximum(R["un"] + R["c"], n_avg + c_avg)
    denom = L["rho"] * (SL - L["un"]) - R["rho"] * (SR - R["un"])
    denom = np.where(np.abs(denom) < TINY, TINY, denom)
    SP = (R["p"] - L["p"] + L["rho"] * L["un"] * (SL - L["un"]) - R["rho"] * R["un"] * (SR - R["un"])) / denom
    return SL, SR, SP


def surely_finite(L, R, SL, SR, SP):
    """hllc_surely_finite: the 18 side values at most 2^60, the four divisors at least 2^-60."""
    ok = np.ones(SL.shape, bool)
    for K in (L, R):
        for f in FIELDS:
            ok &= np.abs(K[f]) <= 2.0 ** 60
    for d in (SL - L["un"], SR - R["un"], SL - SP, SR - SP):
        ok &= (np.abs(d) >= 2.0 ** -60) & np.isfinite(d)
    return ok


def outputs(L, R, SL, SR, SP):
    """Every value HLLC can form from either side: supersonic and star fluxes of both sides, both
    parts of u*, the star ratios and energies (SC:594-662 and the u* of hllc_x_src)."""
    out = {"SP": [SP]}
    ratio = {"L": (SL - L["un"]) / (SL - SP), "R": (SR - R["un"]) / (SR - SP)}
    out["ratio"] = list(ratio.values())
    out["E_star"], out["flux"] = [], []
    for K, S, key in ((L, SL, "L"), (R, SR, "R")):
        r = ratio[key]
        ar1, ar2, rho, un, ut, p, a, E = (K[f] for f in ("ar1", "ar2", "rho", "un", "ut", "p", "a", "E"))
        E_star = E + (SP - un) * (SP * rho + p / (S - un))
        out["E_star"].append(E_star)
        sup = [ar1 * un, ar2 * un, rho * un * un + p, rho * un * ut, (E + p) * un, a * un]
        star = [sup[0] + S * (ar1 * r - ar1), sup[1] + S * (ar2 * r - ar2),
                sup[2] + S * (rho * SP * r - rho * un), sup[3] + S * (rho * ut * r - rho * ut),
                sup[4] + S * (E_star * r - E), sup[5] + S * (a * r - a)]
        out["flux"] += sup + star
    out["flux"].append(L["un"] + np.minimum(0.0, SL) * (ratio["L"] - 1.0))
    out["flux"].append(R["un"] + np.maximum(0.0, SR) * (ratio["R"] - 1.0))
    return out


BOUNDS = {"SP": 251, "ratio": 122, "E_star": 563, "flux": 750}


def check(L, R):
    with np.errstate(all="ignore"):
        SL, SR, SP = speeds(L, R)
        ok = surely_finite(L, R, SL, SR, SP)
        out = outputs(L, R, SL, SR, SP)
        fin = np.ones(SL.shape, bool)
        for name, vals in out.items():
            for v in vals:
                fin &= np.isfinite(v)
                assert not (ok & ~(np.abs(v) < 2.0 ** BOUNDS[name])).any(), name
    assert not (ok & ~fin).any()
    return ok, fin


def test_random_states_of_every_magnitude():
    rng = np.random.default_rng(11)
    n = 200000
    for lo, hi in ((-80, 62), (-10, 30), (40, 62), (-80, -40)):
        ok, fin = check(side(rng, n, lo, hi), side(rng, n, lo, hi))
        if (lo, hi) == (-10, 30):
            assert ok.mean() > 0.99  # ordinary states: nearly every face proved


def test_contact_speed_next_to_a_wave_speed():
    # R.p chosen so that S_P lands within delta of S_L or S_R: the star ratios' divisors near zero
    rng = np.random.default_rng(12)
    n = 100000
    proved = 0
    for lo, hi in ((-5, 20), (30, 58)):
        L, R = side(rng, n, lo, hi), side(rng, n, lo, hi)
        with np.errstate(all="ignore"):
            SL, SR, _ = speeds(L, R)
            denom = L["rho"] * (SL - L["un"]) - R["rho"] * (SR - R["un"])
            denom = np.where(np.abs(denom) < TINY, TINY, denom)
            target = np.where(rng.random(n) < 0.5, SL, SR)
            delta = np.exp2(rng.uniform(-70, -40, n)) * rng.choice([-1.0, 1.0], n) * np.maximum(1.0, np.abs(target))
            R["p"] = (target + delta) * denom + L["p"] - L["rho"] * L["un"] * (SL - L["un"]) + \
                R["rho"] * R["un"] * (SR - R["un"])
        ok, _ = check(L, R)
        proved += int(ok.sum())
    assert proved > 0


def test_outside_the_bounds_is_left_to_the_values():
    # huge states and degenerate speeds: the test must not claim these, some of which overflow
    rng = np.random.default_rng(13)
    n = 100000
    L, R = side(rng, n, 300, 700), side(rng, n, 300, 700)
    ok, fin = check(L, R)
    assert not ok.any() and not fin.all()
    L, R = side(rng, n, -5, 5), side(rng, n, -5, 5)
    for f in FIELDS:
        R[f] = L[f].copy()
    R["c"] = np.zeros(n)
    L["c"] = np.zeros(n)  # S_L = u_L: the star energies' divisor is zero
    ok, _ = check(L, R)
    assert not ok.any()


def test_specials():
    n = 4
    rng = np.random.default_rng(14)
    for bad in (np.nan, np.inf, -np.inf, 2.0 ** 61):
        for f in FIELDS:
            L, R = side(rng, n, -3, 3), side(rng, n, -3, 3)
            L[f] = np.full(n, bad)
            ok, _ = check(L, R)
            assert not ok.any(), (f, bad)


def test_bit_thresholds_are_the_stated_powers():
    # mag_at_most_2p60 / mag_at_least_2m60 (csrc/wm_device.cuh) compare the magnitude's bits with
    # these two patterns and with the exponent field of infinity
    assert np.float64(2.0 ** 60).view(np.uint64) == 0x43B0000000000000
    assert np.float64(2.0 ** -60).view(np.uint64) == 0x3C30000000000000
    assert np.float64(np.inf).view(np.uint64) == 0x7FF0000000000000
