"""The binary32 pre-check of the Ducros sensor (ducros_pre in csrc/wm_bodies.cuh), restated in numpy
binary32 on the CPU and checked against the binary64 decision it must reproduce.

The face sweep uses the Ducros sensor (ducros_kernel, SC:875-916) only through sigma < 0.01. The
pre-check bounds the binary64 a, b (the pressure stencil's fourth difference and sum) and
D = div^2 / (div^2 + curl^2 + 1e-30) from the binary32 roundings of u, v and p, and decides only
when the whole interval of sigma = (a / (b + 1e-30)) D lies on one side of 0.01. Here the same
steps run in numpy (binary32 arrays, IEEE operations; fmaf through binary64, which rounds within
the same bound) on seeded stencils: smooth and shocked flow at SI and dimensionless scales, stencils
placed on the threshold to within 1e-3 .. 1e-14, pressures of mixed sign, magnitudes at the edges of
the guarded ranges, subnormal velocity differences and NaN. Wherever it decides, the decision must
equal the binary64 one; and it must decide nearly all stencils that are not on the threshold.
"""
import numpy as np

F = np.float32


def binary64_sigma(u, v, p):
    """sigma_x, sigma_y of ducros_kernel in binary64, rows of stencil values:
    u, v: (n, 4) at (i-1, j), (i+1, j), (i, j-1), (i, j+1); p: (n, 9) = p0, x -2 -1 +1 +2, y -2 -1 +1 +2."""
    with np.errstate(all="ignore"):
        der_ux = 0.5 * (-u[:, 0] + u[:, 1])
        der_vx = 0.5 * (-v[:, 0] + v[:, 1])
        der_uy = 0.5 * (-u[:, 2] + u[:, 3])
        der_vy = 0.5 * (-v[:, 2] + v[:, 3])
        div = der_ux + der_vy
        curl = der_vx - der_uy
        ducros = div * div / (div * div + curl * curl + 1.0e-30)
        out = []
        for o in (1, 5):
            pm2, pm1, pp1, pp2 = p[:, o], p[:, o + 1], p[:, o + 2], p[:, o + 3]
            p0 = p[:, 0]
            aa = np.abs(-pm2 + 16.0 * pm1 - 30.0 * p0 + 16.0 * pp1 - pp2)
            bb = np.abs(pm2 + 16.0 * pm1 + 30.0 * p0 + 16.0 * pp1 + pp2)
            out.append((aa / (bb + 1.0e-30)) * ducros)
    return out


def side(s):
    return np.where(s < 0.01, 0, np.where(np.isnan(s), -2, 1))


def fmaf(x, y, z):
    return (x.astype(np.float64) * np.float64(y) + np.float64(z)).astype(F)


def ducros_precheck(u, v, p):
    """ducros_pre restated: per direction 0 / 1 where it decides, -1 where it does not."""
    with np.errstate(all="ignore"):
        uf, vf, pf = u.astype(F), v.astype(F), p.astype(F)
        h = F(0.5)
        div = h * (-uf[:, 0] + uf[:, 1]) + h * (-vf[:, 2] + vf[:, 3])
        curl = h * (-vf[:, 0] + vf[:, 1]) - h * (-uf[:, 2] + uf[:, 3])
        Mu = h * (np.abs(uf[:, 0]) + np.abs(uf[:, 1]) + np.abs(vf[:, 2]) + np.abs(vf[:, 3]))
        Mc = h * (np.abs(vf[:, 0]) + np.abs(vf[:, 1]) + np.abs(uf[:, 2]) + np.abs(uf[:, 3]))
        Ed, Ec = fmaf(Mu, 2.0 ** -21, 2.0 ** -140), fmaf(Mc, 2.0 ** -21, 2.0 ** -140)
        dlo, dhi = np.maximum(np.abs(div) - Ed, F(0)), np.abs(div) + Ed
        clo, chi = np.maximum(np.abs(curl) - Ec, F(0)), np.abs(curl) + Ec
        dlo2, dhi2 = dlo * dlo, dhi * dhi
        Dlo = np.maximum(fmaf(dlo2 / (dlo2 + chi * chi + F(1e-30)), 1.0 - 2.0 ** -20, -2.0 ** -48), F(0))
        Dhi = fmaf(dhi2 / (dhi2 + clo * clo + F(1e-30)), 1.0 + 2.0 ** -20, 2.0 ** -48)
        okv = (Mu <= F(2.0 ** 60)) & (Mc <= F(2.0 ** 60))
        out = []
        for o in (1, 5):
            pm2, pm1, p0, pp1, pp2 = pf[:, o], pf[:, o + 1], pf[:, 0], pf[:, o + 2], pf[:, o + 3]
            a = np.abs(-pm2 + F(16) * pm1 - F(30) * p0 + F(16) * pp1 - pp2)
            b = np.abs(pm2 + F(16) * pm1 + F(30) * p0 + F(16) * pp1 + pp2)
            M = np.abs(pm2) + F(16) * np.abs(pm1) + F(30) * np.abs(p0) + F(16) * np.abs(pp1) + np.abs(pp2)
            E = F(2.0 ** -20) * M
            alo, ahi, blo, bhi = np.maximum(a - E, F(0)), a + E, b - E, b + E
            ok = okv & (M >= F(2.0 ** -90)) & (M <= F(2.0 ** 100))
            zero = ok & (blo >= F(2.0 ** -100)) & (ahi * Dhi < F(0.009999962) * blo)
            one = ok & ~zero & (alo * Dlo > F(0.010000038) * (bhi + F(1e-30)))
            out.append(np.where(zero, 0, np.where(one, 1, -1)))
    return out


def stencils(rng, n, pscale, uscale, pnoise, unoise):
    p = pscale * (1.0 + pnoise * rng.standard_normal((n, 9)))
    u = uscale * (rng.standard_normal((n, 1)) + unoise * rng.standard_normal((n, 4)))
    v = uscale * (rng.standard_normal((n, 1)) + unoise * rng.standard_normal((n, 4)))
    return u, v, p


def on_threshold(rng, n, rel):
    """Stencils whose sigma_x is 0.01 (1 + rel * N(0, 1)): the pressure deviations are scaled by the
    factor that puts sigma_x on the threshold (a is linear in it; b nearly constant)."""
    u, v, p = stencils(rng, n, 1.0e5, 30.0, 0.0, 0.3)
    u[:, 0] -= 5.0  # a compression, so D is not small
    dev = rng.standard_normal((n, 9))
    dev[:, 0] = 0.0
    base = 1.0e5 + 0.0 * dev
    sx, _ = binary64_sigma(u, v, base + dev)
    target = 0.01 * (1.0 + rel * rng.standard_normal(n))
    s = np.ones(n)
    for _ in range(6):  # sigma_x(s) is a / b D with a = s |.|, b nearly fixed: fixed-point iterations
        sx, _ = binary64_sigma(u, v, base + s[:, None] * dev)
        s = s * target / np.where(sx > 0, sx, 1.0)
    return u, v, base + s[:, None] * dev


def check(u, v, p, label, min_decided=None):
    ref = binary64_sigma(u, v, p)
    pre = ducros_precheck(u, v, p)
    decided = 0
    for d, (r, c) in enumerate(zip(ref, pre)):
        exact = side(r)
        bad = (c >= 0) & (c != exact)
        assert not bad.any(), f"{label} dir {d}: decided {c[bad][:4]} vs binary64 {exact[bad][:4]} at {np.flatnonzero(bad)[:4]}"
        decided += int((c >= 0).sum())
    frac = decided / (2 * len(p))
    if min_decided is not None:
        assert frac >= min_decided, f"{label}: decided only {frac:.4f}"
    return frac


def test_smooth_and_shocked_flow_at_several_scales():
    rng = np.random.default_rng(11)
    for pscale, uscale in ((1.0e5, 100.0), (1.0, 1.0), (6.0e8, 1.0e3), (1.0e-3, 1.0e-4)):
        for pnoise in (1e-10, 1e-6, 1e-3, 1e-1, 1.0):
            for unoise in (0.0, 1e-12, 1e-6, 1e-2, 1.0):
                u, v, p = stencils(rng, 4000, pscale, uscale, pnoise, unoise)
                # smooth stencils are far from the threshold; the rough ones straddle it
                check(u, v, p, f"p {pscale} u {uscale} noise {pnoise}/{unoise}",
                      0.99 if pnoise <= 1e-6 else None)


def test_stencils_on_the_threshold():
    rng = np.random.default_rng(12)
    for rel in (1e-3, 1e-5, 1e-7, 1e-9, 1e-12, 1e-14):
        u, v, p = on_threshold(rng, 20000, rel)
        frac = check(u, v, p, f"threshold rel {rel}")
        if rel >= 1e-3:
            assert frac > 0.9  # the y direction and most x stencils are decided
    # exactly at binary64's 0.01 boundary: sigma_x within an ulp or two of 0.01
    u, v, p = on_threshold(rng, 20000, 1e-15)
    check(u, v, p, "threshold ulp")


def test_mixed_signs_ranges_and_specials():
    rng = np.random.default_rng(13)
    n = 20000
    # pressures of both signs (tension), b near zero
    u, v, p = stencils(rng, n, 1.0, 1.0, 0.0, 0.5)
    p = rng.standard_normal((n, 9))
    check(u, v, p, "mixed-sign pressures")
    p[:, 5:9] = -p[:, 0:1] * np.array([1.0, 16.0, 16.0, 1.0]) / 34.0 * 30.0 / 30.0
    check(u, v, p, "b cancelled")
    # magnitudes around the guards
    for ps in (2.0 ** -95, 2.0 ** -88, 2.0 ** -80, 2.0 ** 90, 2.0 ** 96, 2.0 ** 120, 1e300):
        u, v, p = stencils(rng, 4000, ps / 64.0, 1.0, 0.3, 0.3)
        check(u, v, p, f"pressure scale {ps:.3g}")
    for us in (1e-45, 2.0 ** -140, 1e-38, 1e-20, 1e-15, 2.0 ** 59, 2.0 ** 61, 1e300):
        u, v, p = stencils(rng, 4000, 1.0, us, 0.05, 0.5)
        check(u, v, p, f"velocity scale {us:.3g}")
    # uniform velocity (D = 0 exactly: the binary32 interval of div is still 2^-21 |u| wide, so
    # only a / b below 0.01 decides), uniform pressure (a = 0 exactly: decided)
    u, v, p = stencils(rng, 4000, 1.0e5, 50.0, 0.1, 0.0)
    check(u, v, p, "uniform velocity")
    u, v, p = stencils(rng, 4000, 1.0e5, 50.0, 0.0, 0.5)
    assert check(u, v, p, "uniform pressure") > 0.99
    # NaN and infinities: never decided
    u, v, p = stencils(rng, 3000, 1.0, 1.0, 0.3, 0.3)
    u[:1000, 1] = np.nan
    p[1000:2000, 6] = np.inf
    v[2000:, 3] = -np.inf
    pre = ducros_precheck(u, v, p)
    assert (pre[0][:1000] < 0).all() and (pre[1][:1000] < 0).all()
    assert (pre[1][1000:2000] < 0).all()
    assert (pre[0][2000:] < 0).all() and (pre[1][2000:] < 0).all()
