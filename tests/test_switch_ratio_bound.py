"""The entropy-ratio pre-check of the THINC switch (thinc_side_delta in csrc/wm_bodies.cuh),
restated in numpy binary32 on the CPU and checked against the binary64 decision it must reproduce.

The switch is cator2 < 0.35 over the five cell entropies of a stencil (SC:318-325, 1028-1032). The
pre-check works with the entropies' ratios to the centre's, d_k = e_k / e_0 - 1 =
expm1(log1p(dp/p0) - g_k log1p(dr/r0) - dg ln r0), the differences from binary32 pairs hi + lo of
the binary64 values (split32) and the rest in binary32, and decides only when its interval bound
clears the threshold. Here the same steps run
in numpy (binary32 arrays, IEEE operations, the fifth-order series of log1p and expm1 for small
arguments, the C library's log1pf / logf / expm1f, each within an ulp as CUDA's are, beyond) on a million seeded stencils: smooth one-fluid flow at SI and dimensionless
scales with fluctuations from 1e-15 to 1e-2, gradients, mixtures with varying gamma, and stencils
placed on the threshold. Wherever it decides, the decision must equal the binary64 one (p / rho^g
with binary64 pow, cator2 in binary64); and it must decide most smooth stencils.
"""
import numpy as np

F = np.float32
YUXIN = 0.9 * 0.35 * 1.0e-2 / (1.0 - 0.9 * 0.35)
K13 = F(13.0 / 12.0)


def binary64_side(p, r, g):
    """cator2 < 0.35 of the binary64 entropies (1: at or above, 0: below), rows of 5 cells."""
    e = p / np.power(r, g)
    em2, em1, e0, ep1, ep2 = (e[:, k] for k in range(5))
    aa = 0.25 * np.abs(em2 - 4.0 * em1 + 3.0 * e0) + (13.0 / 12.0) * np.abs(e0 - 2.0 * em1 + em2)
    bb = 0.25 * np.abs(3.0 * e0 - 4.0 * ep1 + ep2) + (13.0 / 12.0) * np.abs(e0 - 2.0 * ep1 + ep2)
    c = (2.0 * aa * bb + YUXIN) / (aa * aa + bb * bb + YUXIN)
    return np.where(c < 0.35, 0, 1), e[:, 2]


def fmaf(x, y, z):
    return (x.astype(np.float64) * np.float64(y) + np.float64(z)).astype(F)


def log1p_pc(x):
    """log1p_pc: the fifth-order series for |x| <= 2^-5, else the library's log1pf."""
    t = fmaf(x, 0.2, -0.25)
    t = fmaf(x, t, F(0.33333334))
    t = fmaf(x, t, -0.5)
    t = fmaf(x, t, 1.0)
    with np.errstate(all="ignore"):
        return np.where(np.abs(x) <= F(0.03125), (x * t).astype(F), np.log1p(x).astype(F))


def expm1_pc(x):
    """expm1_pc: the fifth-order series for |x| <= 2^-5, else the library's expm1f."""
    t = fmaf(x, F(0.008333334), F(0.041666668))
    t = fmaf(x, t, F(0.16666667))
    t = fmaf(x, t, 0.5)
    t = fmaf(x, t, 1.0)
    with np.errstate(all="ignore"):
        return np.where(np.abs(x) <= F(0.03125), (x * t).astype(F), np.expm1(x).astype(F))


def split32(x):
    """split32: x as binary32 hi + lo (hi = x rounded, lo = (x - hi) rounded)."""
    with np.errstate(all="ignore"):
        hi = x.astype(F)
        return hi, (x - hi.astype(np.float64)).astype(F)


def ratio_precheck(p, r, g, e0):
    """thinc_side_delta restated: 0 / 1 where it decides, -1 where it does not."""
    n = p.shape[0]
    out = np.full(n, -1, dtype=np.int64)
    ok = np.ones(n, dtype=bool)
    ae0 = np.abs(F(e0))
    ok &= (ae0 > 0) & (ae0 <= F(3e38))
    ph, pl = split32(p)
    rh, rl = split32(r)
    gh, gl_ = split32(g)
    p0, r0, g0 = ph[:, 2], rh[:, 2], gh[:, 2]
    ok &= (np.abs(p0) >= F(8.67361738e-19)) & (np.abs(p0) <= F(3e38)) & (r0 >= F(8.67361738e-19)) & (r0 <= F(3e38))
    with np.errstate(all="ignore"):
        lnr0 = np.log(r0).astype(F)
        ip0, ir0 = (F(1) / p0).astype(F), (F(1) / r0).astype(F)
        w0 = F(1) + np.abs(lnr0)
        d = np.zeros((n, 5), dtype=F)
        D = np.zeros((n, 5), dtype=F)
        for k in (0, 1, 3, 4):
            dp = (ph[:, k] - p0) + (pl[:, k] - pl[:, 2])
            dr = (rh[:, k] - r0) + (rl[:, k] - rl[:, 2])
            dg = (gh[:, k] - g0) + (gl_[:, k] - gl_[:, 2])
            xp, xr = (dp * ip0).astype(F), (dr * ir0).astype(F)
            ok &= (np.abs(xp) <= F(0.5)) & (np.abs(xr) <= F(0.5))
            gk = gh[:, k]
            ok &= (gk > 0) & (gk <= F(64)) & (g0 > 0) & (g0 <= F(64)) & (np.abs(dg) <= F(64))
            lp = log1p_pc(xp)
            gl = (gk * log1p_pc(xr)).astype(F)
            dl = (dg * lnr0).astype(F)
            L = ((lp - gl) - dl).astype(F)
            ok &= np.abs(L) <= F(0.5)
            dL = F(1.9073486e-06) * (np.abs(lp) + np.abs(gl) + np.abs(dg) * w0) + \
                F(2.0 ** -43) * (F(1) + gk + (gk + g0) * np.abs(lnr0))
            d[:, k] = expm1_pc(L)
            D[:, k] = F(2.3841858e-07) * np.abs(d[:, k]) + F(1.7) * dL
        A = F(0.25) * np.abs(d[:, 0] - F(4) * d[:, 1]) + K13 * np.abs(d[:, 0] - F(2) * d[:, 1])
        B = F(0.25) * np.abs(d[:, 4] - F(4) * d[:, 3]) + K13 * np.abs(d[:, 4] - F(2) * d[:, 3])
        MA = F(0.25) * (np.abs(d[:, 0]) + F(4) * np.abs(d[:, 1])) + K13 * (np.abs(d[:, 0]) + F(2) * np.abs(d[:, 1]))
        MB = F(0.25) * (np.abs(d[:, 4]) + F(4) * np.abs(d[:, 3])) + K13 * (np.abs(d[:, 4]) + F(2) * np.abs(d[:, 3]))
        wA = F(0.25) * (D[:, 0] + F(4) * D[:, 1]) + K13 * (D[:, 0] + F(2) * D[:, 1]) + F(4.7683716e-07) * MA + \
            F(5.6843419e-14) * (F(6.4) + MA)
        wB = F(0.25) * (D[:, 4] + F(4) * D[:, 3]) + K13 * (D[:, 4] + F(2) * D[:, 3]) + F(4.7683716e-07) * MB + \
            F(5.6843419e-14) * (F(6.4) + MB)
        big = ae0 > F(1e17)
        Y = (F(0.65) * F(YUXIN)) / (ae0 * ae0)
        Ylo = np.where(big, F(0), Y * F(1 - 2.4414062e-04)).astype(F)
        Yhi = np.where(big, F(1e-36), Y * F(1 + 2.4414062e-04)).astype(F)
        Alo, Ahi = np.maximum(A - wA, F(0)), A + wA
        Blo, Bhi = np.maximum(B - wB, F(0)), B + wB
        fmin = F(2) * Alo * Blo - F(0.35) * (Ahi * Ahi + Bhi * Bhi) + Ylo
        fmax = F(2) * Ahi * Bhi - F(0.35) * (Alo * Alo + Blo * Blo) + Yhi
        m = F(3.8146973e-06) * (F(2) * Ahi * Bhi + F(0.35) * (Ahi * Ahi + Bhi * Bhi) + Yhi)
        fin = np.isfinite(A) & np.isfinite(B) & np.isfinite(wA) & np.isfinite(wB)
        ok &= fin
        one = (fmin > m) | (np.isinf(Ylo) & np.isfinite(Ahi) & np.isfinite(Bhi))
        zero = fmax < -m
    out[ok & one] = 1
    out[ok & ~one & zero] = 0
    return out


def gamma_of(al, g1=4.4, g2=1.4):
    """The mixture gamma of alpha1 (1 / Gamma + 1), binary64."""
    gb = al / (g1 - 1.0) + (1.0 - al) / (g2 - 1.0)
    return 1.0 / gb + 1.0


def stencils(rng, n, p0, r0, al0, sigma, slope, mixed=False):
    x = np.arange(5) - 2.0
    p = p0 * (1.0 + slope * x + 0.3 * slope * slope * x * x) * (1.0 + sigma * rng.standard_normal((n, 5)))
    r = r0 * (1.0 + 0.7 * slope * x) * (1.0 + sigma * rng.standard_normal((n, 5)))
    al = np.full((n, 5), al0)
    if mixed:
        al = np.clip(al0 + sigma * rng.standard_normal((n, 5)), 1e-8, 1 - 1e-8)
    return p, r, gamma_of(al)


def check(p, r, g):
    side64, e0_64 = binary64_side(p, r, g)
    e0 = e0_64.astype(F)  # stands for the binary32 entropy, within its 2^-14 bound
    dec = ratio_precheck(p, r, g, e0)
    bad = (dec >= 0) & (dec != side64)
    assert not bad.any(), (p[bad][:2], r[bad][:2], g[bad][:2])
    return int((dec >= 0).sum()), p.shape[0]


def test_smooth_one_fluid_stencils_are_settled_correctly():
    rng = np.random.default_rng(3)
    settled = total = 0
    for p0, r0, al0 in ((1.0e5, 1.2, 1e-6), (1.0e5, 1000.0, 1 - 1e-6), (1.165e7, 6.857, 1e-6),
                        (1.0, 1.0, 1 - 1e-6), (0.1, 0.125, 1 - 1e-6), (3.0e5, 500.0, 0.5)):
        for sigma in (0.0, 1e-15, 1e-12, 1e-9, 1e-6, 1e-4, 1e-2):  # 1e-15: differences in the lo parts only
            for slope in (0.0, 1e-4, 1e-2, 1e-1):
                s, t = check(*stencils(rng, 4000, p0, r0, al0, sigma, slope))
                settled += s
                total += t
    assert settled >= 0.98 * total, (settled, total)


def test_mixtures_and_the_threshold():
    """Varying gamma across the stencil, and stencils tuned so cator2 is near 0.35 (one side's
    second difference about 0.2 and 5 times the other's): decisions there must still be right."""
    rng = np.random.default_rng(4)
    for p0, r0, al0 in ((1.0e5, 1.2, 1e-6), (1.0e5, 300.0, 0.3), (1.0, 1.0, 0.5)):
        for sigma in (1e-6, 1e-3, 3e-2):
            check(*stencils(rng, 20000, p0, r0, al0, sigma, 1e-2, mixed=True))
    n = 200000
    x = np.arange(5) - 2.0
    a = rng.uniform(0.0, 1.0, (n, 1))
    base = 1.0 + 1e-3 * np.where(x < 0, a * x * x, (a * rng.uniform(0.15, 0.3, (n, 1))) * x * x)
    for scale in (1.0, 8e4, 1e-8):
        p = scale * base * (1.0 + 1e-9 * rng.standard_normal((n, 5)))
        r = np.ones((n, 5))
        g = np.full((n, 5), 1.4)
        s, t = check(p, r, g)
        assert s > 0
