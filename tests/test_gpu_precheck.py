"""The binary32 limiter pre-checks (precision form from its binary32 copies, plain form from
binary32 roundings of its binary64 state and fluxes) never decide a cell the binary64 bound solve
would limit (wm_verify_limiter_precheck runs both): on the golden fixtures (the near-vacuum stress
state included), and on seeded states pushed onto every bound's floor -- partial densities near
1e-10, volume fractions near 1e-10 and 1 - 1e-10, energies near the rho c~^2 floor -- with time
steps up to 4x the CFL step so that many high-order states cross the floors."""
import numpy as np
import pytest

import parity_util as pu

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import wavemp  # noqa: E402
from wavemp import Solver, alloc_state, ic  # noqa: E402


def load_state(d):
    nx, ny, g = int(d["meta_nx"]), int(d["meta_ny"]), int(d["meta_g"])
    q = alloc_state(nx, ny, g)
    for k in pu.ALL:
        q[k].copy_(torch.from_numpy(np.ascontiguousarray(d["in_" + k])))
    return q


def verify(s, q, dt):
    s.apply_bc(q)
    s.compute_fluxes(q)
    s.compute_low_fluxes(q)
    return s.verify_limiter_precheck(q, dt)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("case", pu.CASES)
def test_precheck_on_fixtures(case, precision):
    d = pu.load_case(case)
    nx, ny = int(d["meta_nx"]), int(d["meta_ny"])
    s = Solver(pu.params_from(d, precision=precision), nx, ny)
    for scale in (1.0, 4.0):
        decided, disagreed = verify(s, load_state(d), scale * float(d["dt0"]))
        assert disagreed == 0, (case, scale, decided)
        assert decided > 0


def near_floor_state(nx, ny, seed):
    rng = np.random.default_rng(seed)
    q = ic.random_valid(nx, ny, rng)
    g = 5
    inner = (slice(g, g + nx), slice(g, g + ny))
    shape = (nx, ny)
    pick = lambda frac: torch.from_numpy(rng.random(shape) < frac).cuda()  # noqa: E731
    rel = lambda: torch.from_numpy(1.0 + 1e-6 * rng.standard_normal(shape)).cuda()  # noqa: E731
    ar1, ar2, al = q["ar1"][inner], q["ar2"][inner], q["al"][inner]
    m = pick(0.15)
    ar1[m] = (1e-10 * rel())[m]
    m = pick(0.15)
    ar2[m] = (1e-10 * rel())[m]
    m = pick(0.1)
    al[m] = (1e-10 * rel())[m]
    m = pick(0.1)
    al[m] = (1.0 - 1e-10 * rel())[m]
    q["al_prim"].copy_(q["al"])
    # energies just above the rho c~^2 floor: E = kin + p_inf + 1e-8 (1 + noise)
    p = wavemp.SolverParams(dx=1.0 / nx, dy=0.5 / ny, gamma1=4.4, pinf1=6e8, precision="fp32")
    a = al.clamp(1e-10, 1 - 1e-10)
    gb = a / (p.gamma1 - 1) + (1 - a) / (p.gamma2 - 1)
    pb = a * p.gamma1 * p.pinf1 / (p.gamma1 - 1) + (1 - a) * p.gamma2 * p.pinf2 / (p.gamma2 - 1)
    rho = ar1 + ar2
    kin = 0.5 * (q["ru"][inner] ** 2 + q["rv"][inner] ** 2) / rho
    m = pick(0.1)
    q["E"][inner][m] = (kin + pb / (1 + gb) + 1e-8 * rel())[m]
    return p, q


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_precheck_near_the_floors(seed, precision):
    nx, ny = 96, 48
    p, q = near_floor_state(nx, ny, seed)
    p.precision = precision
    s = Solver(p, nx, ny)
    s.initialize(q)
    dt = s.get_dt(q)
    total_decided = 0
    for scale in (0.5, 1.0, 4.0):
        decided, disagreed = verify(s, {k: v.clone() for k, v in q.items()}, scale * dt)
        assert disagreed == 0, (seed, scale, decided)
        total_decided += decided
    assert 0 < total_decided < 3 * 3 * 3 * nx * ny  # some cells decided, not all


def run_steps(p, q0, nx, ny, prechecks, steps=3):
    s = Solver(p, nx, ny)
    s.set_prechecks(prechecks)
    q = {k: v.clone() for k, v in q0.items()}
    old = alloc_state(nx, ny, names=wavemp.FIELDS)
    s.initialize(q)
    s.init_dt(q)
    for _ in range(steps):
        s.step(q, old, None, sync=False)
    torch.cuda.synchronize()
    return {k: pu.host(v) for k, v in q.items()}, s.status()


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("seed", [4, 5])
def test_prechecks_do_not_change_bits(seed, precision):
    """Steps with the binary32 pre-checks (limiter and combine) equal steps without them, bit for
    bit, on states at the floors (repairs and limiting happen) and on the golden fixtures."""
    nx, ny = 96, 48
    p, q0 = near_floor_state(nx, ny, seed)
    p.precision = precision
    a, sa = run_steps(p, q0, nx, ny, True)
    b, sb = run_steps(p, q0, nx, ny, False)
    for k in pu.ALL:
        assert np.array_equal(a[k], b[k], equal_nan=True), k
    assert sa["repaired_cells"] == sb["repaired_cells"] and sa["limited_cells"] == sb["limited_cells"]
    assert sa["limited_cells"] > 0
    for case in ("sc_mp5c6_stress", "m10_cfg2", "sc_mp5c6_triple"):
        d = pu.load_case(case)
        nxc, nyc = int(d["meta_nx"]), int(d["meta_ny"])
        pc = pu.params_from(d, precision=precision)
        qc = load_state(d)
        a, _ = run_steps(pc, qc, nxc, nyc, True, steps=2)
        b, _ = run_steps(pc, qc, nxc, nyc, False, steps=2)
        for k in pu.ALL:
            assert np.array_equal(a[k], b[k], equal_nan=True), (case, k)


# ---- the THINC switch pre-checks (binary32 entropies, then entropy ratios, with error bounds) -----
@pytest.mark.parametrize("case", pu.CASES)
def test_switch_precheck_on_fixtures(case):
    d = pu.load_case(case)
    nx, ny = int(d["meta_nx"]), int(d["meta_ny"])
    s = Solver(pu.params_from(d), nx, ny)
    checked, decided, disagreed = s.verify_switch_precheck(load_state(d))
    assert disagreed == 0, (case, checked, decided)
    assert checked > 0


def switch_states(seed, nx=128, ny=64):
    """Seeded states whose entropy stencils put cator2 near its 0.35 threshold: entropies
    s0 (1 + N(0, sigma)) with sigma spread over decades (the switch turns where the stencil
    differences reach sqrt(eps) ~ 0.07 of the entropy scale), pressures and densities scaled over
    1e-6 .. 1e6, both fluids and mixtures."""
    rng = np.random.default_rng(seed)
    g = 5
    shape = (nx + 2 * g, ny + 2 * g)
    for p_scale in (1e-6, 1e-2, 1.0, 1e2, 1e5, 1e9):
        for sigma in (1e-4, 3e-3, 3e-2, 0.3):
            al = np.clip(rng.random(shape), 1e-8, 1 - 1e-8)
            al[rng.random(shape) < 0.3] = 1 - 1e-8
            al[rng.random(shape) < 0.3] = 1e-8
            rho = np.exp(rng.uniform(-2, 2)) * (1.0 + 0.1 * rng.random(shape))
            p = p_scale * (1.0 + sigma * rng.standard_normal(shape))
            q = {k: torch.zeros(shape, dtype=torch.float64, device="cuda") for k in pu.ALL}
            q["ar1"].copy_(torch.from_numpy(al * rho))
            q["ar2"].copy_(torch.from_numpy((1 - al) * rho))
            q["al"].copy_(torch.from_numpy(al))
            q["al_prim"].copy_(torch.from_numpy(al))
            q["p_p"].copy_(torch.from_numpy(p))
            yield p_scale, sigma, q


def smooth_states(seed, nx=128, ny=64):
    """Seeded smooth states of one fluid (air or water, alpha uniform) at SI scales -- entropies
    p / rho^gamma from 1e-9 to 1e9 -- with relative fluctuations from 1e-9 to 1e-2 and smooth
    gradients, so that cator2 sits near its threshold while the binary32 entropies' bound is far too
    wide to settle it: the ratio pre-check's domain."""
    rng = np.random.default_rng(seed)
    g = 5
    shape = (nx + 2 * g, ny + 2 * g)
    x = np.linspace(0.0, 1.0, shape[0])[:, None] + np.zeros(shape)
    for al_v, p0, rho0 in ((1e-6, 1.0e5, 1.2), (1 - 1e-6, 1.0e5, 1000.0), (1e-6, 1.0e7, 6.0), (0.5, 3.0e5, 500.0)):
        for sigma in (1e-9, 1e-6, 1e-4, 1e-2):
            for slope in (0.0, 1e-3, 1e-1):
                al = np.full(shape, al_v)
                rho = rho0 * (1.0 + slope * x) * (1.0 + sigma * rng.standard_normal(shape))
                p = p0 * (1.0 + 0.5 * slope * x * x) * (1.0 + sigma * rng.standard_normal(shape))
                q = {k: torch.zeros(shape, dtype=torch.float64, device="cuda") for k in pu.ALL}
                q["ar1"].copy_(torch.from_numpy(al * rho))
                q["ar2"].copy_(torch.from_numpy((1 - al) * rho))
                q["al"].copy_(torch.from_numpy(al))
                q["al_prim"].copy_(torch.from_numpy(al))
                q["p_p"].copy_(torch.from_numpy(p))
                yield (al_v, p0, sigma, slope), q


@pytest.mark.parametrize("seed", [21, 22])
def test_ratio_precheck_on_smooth_si_states(seed):
    """The entropy-ratio pre-check (thinc_side_delta) never contradicts the binary64 decision on
    smooth one-fluid states at SI scales, and settles nearly all of them."""
    nx, ny = 128, 64
    params = wavemp.SolverParams(dx=1.0 / nx, dy=0.5 / ny, gamma1=4.4, pinf1=6e8, recon="mp5c6")
    s = Solver(params, nx, ny)
    total = settled = 0
    for what, q in smooth_states(seed, nx, ny):
        checked, decided, disagreed = s.verify_switch_precheck(q)
        assert disagreed == 0, (what, checked, decided)
        total += checked
        settled += decided
    assert settled >= 0.99 * total, (settled, total)


def test_switch_precheck_settles_the_droplet():
    """On the Mach-2.4 water-cylinder state (air at 1 bar in SI units, entropies about 8e4) the two
    pre-checks together settle nearly every stencil, so the binary64 pow is rare."""
    nx, ny = 400, 200
    params = wavemp.SolverParams(dx=1.0 / nx, dy=0.5 / ny, gamma1=4.4, pinf1=6e8, recon="mp5c6",
                                 bc=("transmissive",) * 4)
    q = ic.shock_droplet(nx, ny, 1.0, 0.5, mach=2.4)
    s = Solver(params, nx, ny)
    s.initialize(q)
    old = alloc_state(nx, ny, names=wavemp.FIELDS)
    s.init_dt(q)
    for _ in range(20):
        s.step(q, old, None, sync=False)
    checked, decided, disagreed = s.verify_switch_precheck(q)
    assert disagreed == 0
    assert decided >= 0.99 * checked, (checked, decided)


@pytest.mark.parametrize("seed", [11, 12])
def test_switch_precheck_near_the_threshold(seed):
    nx, ny = 128, 64
    params = wavemp.SolverParams(dx=1.0 / nx, dy=0.5 / ny, gamma1=4.4, pinf1=6e8, recon="mp5c6")
    s = Solver(params, nx, ny)
    undecided = 0
    for p_scale, sigma, q in switch_states(seed, nx, ny):
        checked, decided, disagreed = s.verify_switch_precheck(q)
        assert disagreed == 0, (p_scale, sigma, checked, decided)
        undecided += checked - decided
    assert undecided > 0  # the bound is exercised: some stencils are left to binary64


def test_switch_precheck_settles_the_triple_point():
    """On the dimensionless triple point nearly every stencil is settled in binary32."""
    nx, ny = 448, 192
    q = ic.triple_point(nx, ny)
    s = Solver(wavemp.SolverParams(dx=7.0 / nx, dy=3.0 / ny, gamma1=1.5, pinf1=0.0, gamma2=1.4, pinf2=0.0,
                                   recon="mp5c6", bc=("slip",) * 4), nx, ny)
    s.initialize(q)
    old = alloc_state(nx, ny, names=wavemp.FIELDS)
    s.init_dt(q)
    for _ in range(20):
        s.step(q, old, None, sync=False)
    checked, decided, disagreed = s.verify_switch_precheck(q)
    assert disagreed == 0
    assert decided >= 0.99 * checked, (checked, decided)


@pytest.mark.parametrize("case", ["sc_mp5c6_triple", "sc_cfg0", "m10_cfg2"])
def test_switch_precheck_does_not_change_bits(case):
    """Steps with the switch pre-check equal steps without it, bit for bit, in the plain form and
    in the precision form with binary64 switches."""
    d = pu.load_case(case)
    nxc, nyc = int(d["meta_nx"]), int(d["meta_ny"])
    for precision, sw in (("fp64", False), ("fp32", True)):
        pc = pu.params_from(d, precision=precision)
        pc.fp64_switches = sw
        qc = load_state(d)
        a, _ = run_steps(pc, qc, nxc, nyc, True, steps=3)
        b, _ = run_steps(pc, qc, nxc, nyc, False, steps=3)
        for k in pu.ALL:
            assert np.array_equal(a[k], b[k], equal_nan=True), (case, precision, k)


def stepped(params, q, nx, ny, steps):
    s = Solver(params, nx, ny)
    s.initialize(q)
    old = alloc_state(nx, ny, names=wavemp.FIELDS)
    s.init_dt(q)
    for _ in range(steps):
        s.step(q, old, None, sync=False)
    return s


def test_ducros_precheck_settles_the_droplet_and_the_triple_point():
    """The binary32 Ducros pre-check (ducros_pre) never contradicts the binary64 sigma < 0.01 and
    settles nearly every stencil of the Mach-2.4 water cylinder (SI units) and the triple point
    after 20 steps, shocks, interfaces and vortices included."""
    nx, ny = 400, 200
    q = ic.shock_droplet(nx, ny, 1.0, 0.5, mach=2.4)
    s = stepped(wavemp.SolverParams(dx=1.0 / nx, dy=0.5 / ny, gamma1=4.4, pinf1=6e8, recon="mp5c6",
                                    bc=("transmissive",) * 4), q, nx, ny, 20)
    checked, decided, disagreed = s.verify_ducros_precheck(q)
    assert checked == 2 * (nx + 6) * (ny + 6)
    assert disagreed == 0
    assert decided >= 0.99 * checked, (checked, decided)
    nx, ny = 448, 192
    q = ic.triple_point(nx, ny)
    s = stepped(wavemp.SolverParams(dx=7.0 / nx, dy=3.0 / ny, gamma1=1.5, pinf1=0.0, gamma2=1.4, pinf2=0.0,
                                    recon="mp5c6", bc=("slip",) * 4), q, nx, ny, 20)
    checked, decided, disagreed = s.verify_ducros_precheck(q)
    assert disagreed == 0
    assert decided >= 0.99 * checked, (checked, decided)


@pytest.mark.parametrize("seed", [31, 32])
def test_ducros_precheck_on_noisy_states(seed):
    """Seeded states whose pressure noise puts the Ducros sigma around 0.01 (relative noise 0.03:
    a / b about 0.6 of it) and on either side, with noisy velocities, at SI scales: no stencil is
    decided against the binary64 decision."""
    nx, ny = 512, 256
    rng = np.random.default_rng(seed)
    params = wavemp.SolverParams(dx=1.0 / nx, dy=0.5 / ny, gamma1=4.4, pinf1=6e8, recon="mp5c6")
    s = Solver(params, nx, ny)
    total = settled = 0
    for amp in (1e-4, 3e-3, 0.03, 0.3):
        q = ic.random_valid(nx, ny, rng, amp=amp)
        shape = tuple(q["p_p"].shape)
        noise = torch.from_numpy(1.0 + amp * rng.standard_normal(shape)).cuda()
        q["p_p"].mul_(noise)
        for k in ("u_p", "v_p"):
            q[k].add_(torch.from_numpy(100.0 * amp * rng.standard_normal(shape)).cuda())
        checked, decided, disagreed = s.verify_ducros_precheck(q)
        assert disagreed == 0, (amp, checked, decided)
        total += checked
        settled += decided
    assert settled >= 0.99 * total, (settled, total)


@pytest.mark.parametrize("case", pu.CASES)
def test_ducros_precheck_on_fixtures(case):
    d = pu.load_case(case)
    nx, ny = int(d["meta_nx"]), int(d["meta_ny"])
    s = Solver(pu.params_from(d), nx, ny)
    checked, decided, disagreed = s.verify_ducros_precheck(load_state(d))
    assert disagreed == 0, (case, checked, decided)
    assert decided > 0
