"""The error bounds of the binary64 face sweep's refined reciprocal, quotient, paired quotients and
square root (rcp_nr, div_nr, div2_nr, sqrt_nr in csrc/wm_device.cuh), checked on the CPU in exact
arithmetic: each fused multiply-add is the exact rational a b + c rounded once to binary64
(Python's int / int division rounds correctly), each product likewise, and the seeds are taken at
the worst relative errors the binary32 stage can leave (|1 - y s| up to 2^-19.8 for the reciprocal,
|1 - x h^2| up to 2^-19 for the root, both signs) as well as inside them. The GPU self-check
(tests/test_gpu_conversions.py) compares the CUDA code itself with the hardware operations; this
test shows the bounds hold for every seed the hardware may give, not only for the ones it gave."""
import math
import random
from fractions import Fraction

E_RCP = 2.0 ** -19.8   # |1 - y s| of the reciprocal seed (truncation 2^-20 + rcp.approx 2^-23)
E_SQRT = 2.0 ** -19.0  # |1 - x h^2| of the root seed (rsqrt.approx of a truncated operand)


def rnd(q: Fraction) -> float:
    return q.numerator / q.denominator  # correctly rounded to binary64


def fma(a, b, c):
    return rnd(Fraction(a) * Fraction(b) + Fraction(c))


def mul(a, b):
    return rnd(Fraction(a) * Fraction(b))


def ulps(got: float, exact: Fraction) -> float:
    """|got - exact| in units in the last place of the correctly rounded exact value."""
    return float(abs(Fraction(got) - exact) / Fraction(math.ulp(rnd(exact))))


def seed(exact: Fraction, rel: float) -> float:
    return rnd(exact * (1 + Fraction(rel)))


def rcp_refine(y, s):
    e = fma(-y, s, 1.0)
    return fma(s, fma(e, e, e), s)


def operands(rng, n, lo, hi):
    for _ in range(n):
        m = rng.uniform(1.0, 2.0)
        yield math.ldexp(m, rng.randint(lo, hi)) * rng.choice((-1.0, 1.0))


def seeds_rel(rng, bound):
    return (bound, -bound, bound * 0.999, -bound * 0.999, rng.uniform(-bound, bound))


def test_reciprocal_within_one_ulp():
    rng = random.Random(5)
    worst = 0.0
    for y in operands(rng, 3000, -125, 124):
        exact = 1 / Fraction(y)
        # the seed's error bound is on e = 1 - y s, i.e. s = (1/y)(1 - e)
        for rel in seeds_rel(rng, E_RCP):
            worst = max(worst, ulps(rcp_refine(y, seed(exact, -rel)), exact))
    assert worst <= 1.0, worst


def test_quotient_within_one_ulp():
    rng = random.Random(6)
    worst = 0.0
    ys = list(operands(rng, 1500, -125, 124))
    xs = list(operands(rng, 1500, -896, 896))
    for x, y in zip(xs, ys):
        exact = Fraction(x) / Fraction(y)
        for rel in seeds_rel(rng, E_RCP):
            s = rcp_refine(y, seed(1 / Fraction(y), -rel))
            q0 = mul(x, s)
            q = fma(fma(-y, q0, x), s, q0)
            worst = max(worst, ulps(q, exact))
    assert worst <= 1.0, worst


def test_paired_quotients_within_four_ulps():
    rng = random.Random(7)
    worst = 0.0
    for _ in range(1500):
        b, d = (math.ldexp(rng.uniform(1, 2), rng.randint(-60, 60)) * rng.choice((-1, 1)) for _ in range(2))
        a, c = (math.ldexp(rng.uniform(1, 2), rng.randint(-300, 300)) * rng.choice((-1, 1)) for _ in range(2))
        bd = mul(b, d)
        if not (2.0 ** -125 <= abs(bd) < 2.0 ** 125):
            continue  # the seeded range; outside it the two quotients are taken separately
        for rel in seeds_rel(rng, E_RCP):
            r = rcp_refine(bd, seed(1 / Fraction(bd), -rel))
            q1, q2 = mul(a, mul(d, r)), mul(c, mul(b, r))
            worst = max(worst, ulps(q1, Fraction(a) / Fraction(b)), ulps(q2, Fraction(c) / Fraction(d)))
    assert worst <= 4.0, worst


def test_square_root_within_one_ulp():
    rng = random.Random(8)
    worst = 0.0
    for x in operands(rng, 3000, -125, 124):
        x = abs(x)
        ref = math.sqrt(x)  # correctly rounded
        for rel in seeds_rel(rng, E_SQRT):
            # h with 1 - x h^2 = rel: h = (1 - rel)^(1/2) / sqrt(x), to well below an ulp
            h = (1.0 - rel) ** 0.5 / ref
            h = rnd(Fraction(h))
            hh = h / 2  # exact
            z = mul(x, h)
            z = fma(fma(-z, z, x), hh, z)
            z = fma(fma(-z, z, x), hh, z)
            worst = max(worst, abs(z - ref) / math.ulp(ref))
    assert worst <= 1.0, worst
