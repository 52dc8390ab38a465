"""The integer pre-test of MP5's limiter condition in the binary64 sweep (mp5_diff in
csrc/wm_device.cuh), checked on the CPU.

MP5 (SC:353-377) applies its limiter when (VOR - v0)(VOR - VMP) >= 1e-20. With D = VOR - v0 and
m = VMP - v0 = mm2(d0, 4 dm1), the sweep writes the test as D (D - m) >= 1e-20 and first settles it
from the bit patterns of D and m alone: the test cannot pass when D is +-0, or when D and m have the
same sign bit and |m| > |D| as magnitudes (D - m is then nonzero with D's opposite sign, so the
product is negative; an infinite or NaN m makes it negative or NaN). Here that bit rule is restated
and compared with IEEE binary64 evaluation of D (D - m) >= 1e-20 on edge operands: both zeros, equal
magnitudes of either sign, neighbours one unit apart, subnormals, the largest finite values,
infinities, NaN of both signs, the +0 that mm2 returns for opposite signs, and random pairs. The
rule must never skip a case in which the test passes (it may leave undecided cases to the binary64
evaluation, which is the test itself).
"""
import math
import random
import struct

MASK = 0x7FFFFFFFFFFFFFFF


def bits(x: float) -> int:
    return struct.unpack("<q", struct.pack("<d", x))[0]


def pretest_skips(D: float, m: float) -> bool:
    """mp5_diff's bit rule: True when the limiter test is known to fail without evaluating it."""
    bD, bm = bits(D), bits(m)
    aD, am = bD & MASK, bm & MASK
    return aD == 0 or ((bD ^ bm) >= 0 and am > aD)


def limiter_test_passes(D: float, m: float) -> bool:
    """The limiter condition as the sweep evaluates it: IEEE binary64, D (D - m) >= 1e-20 (false
    for NaN)."""
    try:
        prod = D * (D - m)
    except OverflowError:  # Python raises where IEEE gives infinity
        prod = math.copysign(math.inf, D) * math.copysign(1.0, D - m)
    return prod >= 1e-20


def mm2(x: float, y: float) -> float:
    """The reference's minmod-2 (SC:295-297) with Warp's sign (x < 0 ? -1 : 1)."""
    sx = -1.0 if x < 0 else 1.0
    sy = -1.0 if y < 0 else 1.0
    a, b = abs(x), abs(y)
    return 0.5 * (sx + sy) * (a if a < b else b)


def edge_values():
    tiny = 5e-324
    vals = [0.0, -0.0, tiny, -tiny, 2.2250738585072014e-308, -2.2250738585072014e-308,
            1e-10, -1e-10, 1e-20, -1e-20, 1.0, -1.0, math.nextafter(1.0, 2.0), math.nextafter(1.0, 0.0),
            -math.nextafter(1.0, 2.0), 1.7976931348623157e308, -1.7976931348623157e308, math.inf,
            -math.inf, math.nan, -math.nan, 3.0, -3.0, 1e150, -1e150, 1e-160, -1e-160]
    return vals


def check(D, m):
    if pretest_skips(D, m):
        assert not limiter_test_passes(D, m), f"pre-test skips a passing case D={D!r} m={m!r}"


def test_edge_pairs():
    vals = edge_values()
    for D in vals:
        for m in vals:
            check(D, m)


def test_mm2_zeros_and_equal_magnitudes():
    vals = edge_values()
    for a in vals:
        for b in vals:
            m = mm2(a, b)  # +0 for opposite signs, NaN for inf * 0
            for D in (a, -a, b, -b, 0.0, -0.0, 1e-10, -1e-10):
                check(D, m)
    for D in (1.0, -1.0, 1e-12, -1e-12):
        check(D, D)              # equal: D - m = 0, product 0
        check(D, -D)             # opposite: not skipped by the rule
        check(D, math.nextafter(D, math.copysign(math.inf, D)))  # |m| one unit above |D|
        check(D, math.nextafter(D, 0.0))                          # |m| one unit below |D|


def test_random_pairs_and_what_the_rule_settles():
    rng = random.Random(7)
    skipped = passed = 0
    for _ in range(200000):
        D = math.ldexp(rng.uniform(1, 2), rng.randint(-80, 5)) * rng.choice((-1.0, 1.0))
        m = D * rng.choice((rng.uniform(-3, 3), rng.uniform(0.9, 1.1), 0.0, -0.0))
        check(D, m)
        skipped += pretest_skips(D, m)
        passed += limiter_test_passes(D, m)
    # the rule settles a large share of the failing cases, and only failing ones
    assert skipped > 0.2 * (200000 - passed)
