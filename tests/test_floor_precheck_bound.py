"""The binary32 pre-check of the first-order state's pressure floor (below_floor in
csrc/wm_bodies.cuh), restated in numpy binary32 and checked against the binary64 test it replaces.

The binary32 form's preparation pass floors the first-order pressure where
((1 + Gamma) p + Pi) Gamma < 1e-8 (1 + Gamma) (fx_low_kernel's pressure floor, SC:1309-1327, written
with the mixture's Gamma and Pi). The pre-check decides from the binary32 roundings where the two
products are more than 2^-20 apart and leaves the rest to binary64. Here: seeded operands placed on
the threshold to within 1e-3 .. 1e-16, negative and huge numerators, and the guarded ranges of
Gamma. Wherever it decides, the decision must be binary64's.
"""
import numpy as np

F = np.float32
CTILDE = 1.0e-8


def precheck(num, gb, gp1):
    with np.errstate(all="ignore"):
        g, h = gb.astype(F), gp1.astype(F)
        ok = (g >= F(2.0 ** -100)) & (g <= F(2.0 ** 100)) & (h <= F(2.0 ** 100))
        lhs, rhs = num.astype(F) * g, F(CTILDE) * h
        above = ok & (lhs > rhs * F(1.0 + 2.0 ** -20))
        below = ok & ~above & (lhs < rhs * F(1.0 - 2.0 ** -20))
    return np.where(above, 0, np.where(below, 1, -1))


def check(num, gb, gp1):
    with np.errstate(all="ignore"):
        exact = (num * gb < CTILDE * gp1).astype(np.int64)
    got = precheck(num, gb, gp1)
    bad = (got >= 0) & (got != exact)
    assert not bad.any(), (num[bad][:3], gb[bad][:3])
    return float((got >= 0).mean())


def test_floor_precheck_on_and_off_the_threshold():
    rng = np.random.default_rng(7)
    n = 200000
    for gam in (0.29, 2.5, 1.0 / 0.5, 1.0e-3, 40.0):
        gb = gam * (1.0 + 0.1 * rng.random(n))
        gp1 = 1.0 + gb
        thr = CTILDE * gp1 / gb
        for rel in (1e-3, 1e-6, 1e-9, 1e-12, 1e-16):
            num = thr * (1.0 + rel * rng.standard_normal(n))
            frac = check(num, gb, gp1)
            if rel >= 1e-3:
                assert frac > 0.99
        # ordinary states far from the floor: p from 1 Pa to 1e9 Pa
        num = gp1 * 10.0 ** rng.uniform(0, 9, n) + 6e8 * gb
        assert check(num, gb, gp1) == 1.0
        # the stiffened gas near p = -p_inf: numerators of both signs around zero
        num = 1e-6 * rng.standard_normal(n)
        check(num, gb, gp1)


def test_floor_precheck_specials():
    n = 7
    gb = np.full(n, 2.5)
    gp1 = 1.0 + gb
    num = np.array([np.nan, np.inf, -np.inf, 1e300, -1e300, 0.0, -0.0])
    got = precheck(num, gb, gp1)
    assert got[0] == -1  # NaN: binary64 decides
    check(num[1:], gb[1:], gp1[1:])
    for g in (2.0 ** -110, 2.0 ** 110, 0.0, np.nan):
        gbx = np.full(3, g)
        assert (precheck(np.array([1.0, -1.0, 1e-8]), gbx, 1.0 + gbx) == -1).all()
