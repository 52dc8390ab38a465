"""The integer-pipe conversions (to_f32 / to_f64) equal the hardware binary64 <-> binary32
conversions bit for bit, on random bit patterns and on every boundary the rounding code
distinguishes: ties to even, carries into the exponent, the edges of binary32's normal range
(subnormal results, overflow to infinity), zeros, infinities, NaN. The integer binary64 compares
(dlt, dneg and the wmin / wmax / wsign built on them) equal the hardware compares on the same
inputs and on every pair of special values."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

from wavemp import _lib  # noqa: E402
from wavemp.solver import _stream  # noqa: E402


def check(values_u64: np.ndarray):
    L = _lib.load()
    t = torch.from_numpy(values_u64.view(np.int64)).cuda()
    a, b, c = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
    _lib.check(L.wm_check_conversions(ctypes.c_void_p(t.data_ptr()), t.numel(), ctypes.byref(a),
                                      ctypes.byref(b), ctypes.byref(c), _stream()), "wm_check_conversions")
    return a.value, b.value, c.value


def test_random_bit_patterns():
    rng = np.random.default_rng(0)
    bits = rng.integers(0, 2**63, size=4_000_000, dtype=np.uint64) * np.uint64(2)
    bits |= rng.integers(0, 2, size=bits.size, dtype=np.uint64)
    assert check(bits) == (0, 0, 0)


def test_values_in_binary32_range_and_boundaries():
    rng = np.random.default_rng(1)
    x = np.concatenate([
        rng.standard_normal(1_000_000) * 10.0 ** rng.uniform(-45, 39, 1_000_000),
        np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, -1.0, 3.4028234663852886e38,
                  3.4028235677973366e38, 3.402823567797337e38, 1.1754943508222875e-38,
                  1.1754942106924411e-38, 1.401298464324817e-45, 7.006492321624085e-46,
                  2.0 ** -149, 2.0 ** -150, 2.0 ** 128, 6.0e8, 1e-10, 1e-13, 1.0 - 1e-10]),
    ])
    bits = x.view(np.uint64).copy()
    # exact ties and their neighbours at the rounding bit, odd and even significands
    base = rng.standard_normal(200_000).view(np.uint64) & ~np.uint64(0x1FFFFFFF)
    ties = np.concatenate([base | np.uint64(0x10000000), base | np.uint64(0x0FFFFFFF),
                           base | np.uint64(0x10000001), base | np.uint64(0x1FFFFFFF)])
    # the largest binary32 significand: rounding carries into the exponent
    carry = (rng.standard_normal(100_000).view(np.uint64) | np.uint64(0x000FFFFFF0000000))
    assert check(np.concatenate([bits, ties, carry])) == (0, 0, 0)


def test_compares_on_special_pairs():
    """Every pair of special values (both zeros, infinities, NaNs of both signs, the smallest and
    largest magnitudes, equal values) in both orders, via neighbouring inputs."""
    sp = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, -np.nan, 5e-324, -5e-324,
                   1.7976931348623157e308, -1.7976931348623157e308, 2.0, 1.0000000000000002,
                   0.9999999999999999, -2.0])
    nan_payload = np.array([0x7FF0000000000001, 0xFFF8000000000123], dtype=np.uint64).view(np.float64)
    sp = np.concatenate([sp, nan_payload])
    pairs = [np.array([a, b]) for a in sp for b in sp]
    assert check(np.concatenate(pairs).view(np.uint64)) == (0, 0, 0)


def check_arith(values_u64: np.ndarray):
    L = _lib.load()
    t = torch.from_numpy(values_u64.view(np.int64)).cuda()
    counts = (ctypes.c_longlong * 11)()
    _lib.check(L.wm_check_sweep_arith(ctypes.c_void_p(t.data_ptr()), t.numel(), counts, _stream()),
               "wm_check_sweep_arith")
    return list(counts)


def test_sweep_arithmetic_within_one_ulp():
    """The face sweep's binary64 reciprocal, quotient and square root (binary32 seed refined by fused
    multiply-adds) are within one unit in the last place of IEEE 1/y, x/y and sqrt(x), and its pairs
    of quotients from one shared reciprocal within four, on random
    bit patterns, on values of every magnitude the fast path takes, and at the edges of its operand
    ranges; special values (zeros, subnormals, infinities, NaN, out-of-range operands) give the
    IEEE results bit for bit."""
    rng = np.random.default_rng(2)
    bits = rng.integers(0, 2**63, size=2_000_000, dtype=np.uint64) * np.uint64(2)
    bits |= rng.integers(0, 2, size=bits.size, dtype=np.uint64)
    vals = rng.standard_normal(2_000_000) * 10.0 ** rng.uniform(-40, 40, 2_000_000)
    edges = []
    for k in (-126, -125, -124, 124, 125, 126, -897, -896, -895, 896, 897, 898):
        for m in (1.0, 1.0 - 2.0 ** -53, 1.0 + 2.0 ** -52, 1.5, 1.9999999999999998):
            edges += [m * 2.0 ** k, -m * 2.0 ** k]
    special = [0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 2.2250738585072014e-308,
               1.7976931348623157e308, 1.0, -1.0, 3.0, 6e8, 1e-20, 1.0 + 2.0 ** -52]
    # significands just below and above a binary32 truncation boundary (the seed's 20 fraction bits)
    base = (rng.standard_normal(200_000).view(np.uint64) & ~np.uint64(0xFFFFFFFF))
    trunc = np.concatenate([base | np.uint64(0xFFFFFFFF), base, base | np.uint64(1)])
    allv = np.concatenate([bits, vals.view(np.uint64), np.array(edges + special).view(np.uint64), trunc])
    c = check_arith(allv)
    assert c[:3] == [0, 0, 0], c
    # the refinement is not a different rounding rule: most results are the IEEE ones exactly
    assert max(c[3:6]) < 0.05 * allv.size, c
    assert c[6:] == [0, 0, 0, 0, 0], c


def test_minmods_equal_the_sign_sum_products():
    """mm2 / mm4 on the integer pipe equal 0.5 (sign x + sign y) min|.| and
    0.125 s |(sa + sc)(sa + sd)| min|.| on the hardware operations bit for bit, and so do the halving
    and the sign selection of the interface velocity: every sign pattern of zeros of both signs,
    infinities, NaN, the smallest normals and finite values, in all orders."""
    sp = np.array([0.0, -0.0, 1.0, -1.0, 2.5, -2.5, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 1e300,
                   2.2250738585072014e-308, -4.450147717014403e-308])
    quads = np.array(np.meshgrid(sp, sp, sp, sp)).reshape(4, -1).T.copy()
    rng = np.random.default_rng(3)
    rnd = rng.standard_normal(400_000) * 10.0 ** rng.uniform(-5, 5, 400_000)
    c = check_arith(np.concatenate([quads.ravel(), rnd]).view(np.uint64))
    assert c[6:] == [0, 0, 0, 0, 0], c
