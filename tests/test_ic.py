"""Known-answer tests of the initial-state generators (CPU; torch on the host).

The post-shock air state of every shock-droplet configuration comes from
``wavemp.ic.rankine_hugoniot``. The reference writes its post-shock states as literal tables:
M10's Mach-10 air (rho 6.8571, u 2817.9, p 1.165e7 behind a shock into 1e5 Pa, 1.2 kg/m^3;
Sainath_M10.py:770-772) and SC's Mach ~2.4 air (rho 3.7579, u 574.57, p 6.6189e5 behind a shock
into 101312.5 Pa, 1.17 kg/m^3; sainath_SC_it_works.py:812-814).
"""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from wavemp import ic  # noqa: E402


def rel(a, b):
    return abs(a - b) / abs(b)


def test_mach10_matches_the_m10_table():
    """M10:770-772 prints five significant digits; the relations reproduce them to rounding."""
    p2, rho2, u2 = ic.rankine_hugoniot(10.0, gamma=1.4, p1=1.0e5, rho1=1.2)
    assert rel(rho2, 6.8571) <= 0.5e-4
    assert rel(u2, 2817.9) <= 0.5e-4
    assert rel(p2, 1.165e7) <= 1e-12  # 1e5 (1 + 2.8 / 2.4 * 99) is 1.165e7 exactly in decimal
    # the exact fractions behind the table: rho2 = 1.2 * 240 / 42, p2 = 1e5 * 116.5
    assert rel(rho2, 1.2 * 240.0 / 42.0) <= 1e-15


def test_mach2p4_matches_the_stated_values():
    """Mach 2.4 into air at 1e5 Pa and 1.2 kg/m^3: p2 ~ 6.55e5 Pa, rho2 ~ 3.85, u2 ~ 565 m/s
    (three significant digits)."""
    p2, rho2, u2 = ic.rankine_hugoniot(2.4)
    assert rel(p2, 6.55e5) <= 1e-3
    assert rel(rho2, 3.85) <= 2e-3
    assert rel(u2, 565.0) <= 2e-3
    # closed forms at M^2 = 5.76
    assert rel(p2, 1e5 * (1 + 2.8 / 2.4 * 4.76)) <= 1e-15
    assert rel(rho2, 1.2 * 2.4 * 5.76 / (0.4 * 5.76 + 2.0)) <= 1e-15


def test_sc_table_is_the_same_relations():
    """SC's table (SC:812-814) is a Mach ~2.4 shock into 101312.5 Pa, 1.17 kg/m^3 air: the Mach
    number that gives its pressure ratio gives its density and velocity to the table's rounding
    (the table carries about three significant digits of the Mach number)."""
    ratio = 6.6189e5 / 101312.5
    mach = math.sqrt(1.0 + (ratio - 1.0) * 2.4 / 2.8)
    assert abs(mach - 2.4) < 5e-3
    p2, rho2, u2 = ic.rankine_hugoniot(mach, gamma=1.4, p1=101312.5, rho1=1.17)
    assert rel(p2, 6.6189e5) <= 1e-12
    assert rel(rho2, 3.7579) <= 2e-3
    assert rel(u2, 574.57) <= 2e-3


def test_jump_conditions_hold_exactly():
    """Mass, momentum and energy fluxes across the shock are continuous in the shock frame."""
    g, p1, r1 = 1.4, 1.0e5, 1.2
    for mach in (1.5, 2.4, 4.0, 6.0, 10.0):
        p2, r2, u2 = ic.rankine_hugoniot(mach, g, p1, r1)
        s = mach * math.sqrt(g * p1 / r1)          # shock speed into gas at rest
        w1, w2 = s, s - u2                          # velocities relative to the shock
        assert rel(r1 * w1, r2 * w2) <= 1e-13
        assert rel(r1 * w1 * w1 + p1, r2 * w2 * w2 + p2) <= 1e-13
        h1 = g / (g - 1) * p1 / r1 + 0.5 * w1 * w1
        h2 = g / (g - 1) * p2 / r2 + 0.5 * w2 * w2
        assert rel(h1, h2) <= 1e-13


@pytest.mark.parametrize("mach", [2.4, 10.0])
def test_shock_droplet_post_shock_cells(mach):
    """Cells behind the shock carry the Rankine-Hugoniot air state; cells ahead are at rest."""
    nx, ny = 64, 32
    st = ic.shock_droplet(nx, ny, 1.0, 0.5, mach=mach, device="cpu")
    p2, rho2, u2 = ic.rankine_hugoniot(mach)
    x = (np.arange(nx + 10) - 5 + 0.5) / nx
    post, pre = int(np.argmax(x > 0.05)), int(np.argmax(x > 0.9))
    j = 5  # first interior row, far from the droplet
    for i, (p, r, u) in ((post, (p2, rho2, u2)), (pre, (1.0e5, 1.2, 0.0))):
        al = float(st["al"][i, j])
        assert al < 2e-6  # air
        assert rel(float(st["ar2"][i, j]), (1.0 - al) * r) <= 1e-15
        assert float(st["p_p"][i, j]) == p
        assert float(st["u_p"][i, j]) == u
        assert float(st["v_p"][i, j]) == 0.0
        rho = float(st["ar1"][i, j] + st["ar2"][i, j])
        assert rel(float(st["ru"][i, j]) + 1e-300, rho * u + 1e-300) <= 1e-15
