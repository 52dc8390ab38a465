"""GPU vs the CPU oracle at the benchmark configurations' own sizes and step counts.

* Shock-water cylinder, 400 x 200, SC with MP5 + THINC + central-6, transmissive sides, Mach 2.4:
  the full 100 SSP-RK3 steps at CFL 0.4, each side on its own dt sequence (reference loop
  SC:2009-2063).
* Gas-gas triple point, 7168 x 3072, slip walls, MP5 + THINC + central-6: every intermediate of the
  first stage (ghost fill, high- and first-order face fluxes, the limiter factor of each pass, the
  limited fluxes, the combine, the repair, the primitives; SC:2030-2055), then two whole steps.
* Mach-10 shock-water cylinder, 4096 x 2048, M10 as shipped: five steps.

Tolerances are the parity tests' own (natural units, tests/parity_util.py): 1e-10 per closure,
1e-9 per whole-step result, and dt within 1e-10 relative. The oracle runs on every host core, so
each case costs seconds of CPU time at these sizes; the 7168 x 3072 oracle holds ~8.5 GB of host
memory.
"""
import gc

import numpy as np
import pytest

import parity_util as pu

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import wavemp  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from wavemp import Solver, SolverParams, alloc_state  # noqa: E402
from wavemp import ic  # noqa: E402

BCS = {"transmissive": orc.TRANSMISSIVE, "slip": orc.SLIP}
RTOL_STEPS = 1e-9


def oracle_for(params: SolverParams, nx, ny, state):
    P = orc.make_params(params.dx, params.dy, params.gamma1, params.pinf1, params.gamma2,
                        params.pinf2, variant=orc.M10 if params.variant == "m10" else orc.SC,
                        recon=orc.MP5C6 if params.recon == "mp5c6" else orc.SHIPPED,
                        bc=[BCS[b] for b in params.bc], cfl=params.cfl,
                        repair=params.emergency_repair)
    o = orc.OracleSolver(nx, ny, P)
    o.load(state)
    o.init_sequence()
    return o


def gpu_state_from(o, nx, ny):
    q = alloc_state(nx, ny)
    for k in pu.ALL:
        q[k].copy_(torch.from_numpy(o.f[k]))
    return q


def state_err(q, o, params):
    """Largest natural-unit error over the ten cell arrays, and the array it occurs in."""
    ref = {k: o.f[k] for k in pu.ALL}
    sc = pu.natural_scales(ref, params.gamma1, params.pinf1, params.gamma2, params.pinf2)
    errs = {k: pu.cell_err({k: pu.host(q[k])}, ref, k, sc) for k in pu.ALL}
    worst = max(errs, key=errs.get)
    return errs[worst], worst


def release():
    """Return the host and device memory of the arrays a test has dropped."""
    gc.collect()
    torch.cuda.empty_cache()


def test_cfg0_droplet_100_steps_vs_oracle():
    """Configuration 0 exactly as stated: 400 x 200, 100 steps, each side on its own dt."""
    nx, ny = 400, 200
    params = SolverParams(dx=1.0 / nx, dy=0.5 / ny, gamma1=4.4, pinf1=6e8, variant="sc",
                          recon="mp5c6", bc=("transmissive",) * 4)
    st = {k: v.numpy() for k, v in ic.shock_droplet(nx, ny, 1.0, 0.5, mach=2.4, device="cpu").items()}
    o = oracle_for(params, nx, ny, st)
    s = Solver(params, nx, ny)
    q = gpu_state_from(o, nx, ny)
    old = alloc_state(nx, ny, names=pu.FIELDS)
    dt_o = dt_g = o.get_dt()
    history = []
    for n in range(1, 101):
        dt_o = o.step(dt_o)
        dt_g = s.step(q, old, dt_g)
        if n in (1, 10, 25, 50, 75, 100):
            e, k = state_err(q, o, params)
            history.append((n, e, k, abs(dt_g - dt_o) / dt_o))
    print("cfg0 400x200 error after n steps (natural units):",
          ", ".join(f"{n}: {e:.2e} ({k}), dt {d:.1e}" for n, e, k, d in history))
    for n, e, k, d in history:
        assert e <= RTOL_STEPS, f"step {n}: {k} differs by {e:.3e} > {RTOL_STEPS:.0e}"
        assert d <= 1e-10, f"step {n}: dt differs by {d:.3e}"


@pytest.fixture(scope="module")
def triple_full():
    nx, ny = 7168, 3072
    params = SolverParams(dx=7.0 / nx, dy=3.0 / ny, gamma1=1.5, pinf1=0.0, gamma2=1.4, pinf2=0.0,
                          variant="sc", recon="mp5c6", bc=("slip",) * 4)
    st = {k: v.numpy() for k, v in ic.triple_point(nx, ny, device="cpu").items()}
    return nx, ny, params, st


def test_cfg1_triple_point_first_stage_intermediates(triple_full):
    """Every closure of the first stage of configuration 1 at 7168 x 3072 against the oracle."""
    nx, ny, params, st = triple_full
    o = oracle_for(params, nx, ny, st)
    s = Solver(params, nx, ny)
    q = gpu_state_from(o, nx, ny)
    old = alloc_state(nx, ny, names=pu.FIELDS)
    dt = o.get_dt()
    assert abs(s.get_dt(q) - dt) <= 1e-10 * dt
    o.copy_old()
    s.copy_old(q, old)
    ref0 = {k: o.f[k] for k in pu.ALL}
    sc = pu.natural_scales(ref0, params.gamma1, params.pinf1, params.gamma2, params.pinf2)
    fsc = sc["flux"]

    o.apply_bc()
    s.apply_bc(q)
    for k in pu.FIELDS + pu.PRIMS:
        assert np.array_equal(pu.host(q[k]), o.f[k]), f"apply_bc {k}"

    o.compute_fluxes()
    s.compute_fluxes(q)
    fx, gy = s.fluxes("high")
    pu.assert_fluxes([pu.host(a) for a in fx], [pu.host(a) for a in gy], o.fh, o.gh, fsc,
                     "cfg1 high-order flux")
    del fx, gy
    o.compute_low_fluxes()
    s.compute_low_fluxes(q)
    fx, gy = s.fluxes("low")
    pu.assert_fluxes([pu.host(a) for a in fx], [pu.host(a) for a in gy], o.fl, o.gl, fsc,
                     "cfg1 first-order flux")
    del fx, gy
    thetas = {}
    o.limit_fluxes(dt, record=thetas)
    s.limit_fluxes(q, dt)
    for p in range(3):
        pu.assert_abs(pu.host(s.workspace(wavemp._lib.WS_THETA + p)), thetas[f"theta{p}"],
                      f"cfg1 theta pass {p}", 1e-9)
    del thetas
    fx, gy = s.fluxes("high")
    pu.assert_fluxes([pu.host(a) for a in fx], [pu.host(a) for a in gy], o.fh, o.gh, fsc,
                     "cfg1 limited flux")
    del fx, gy
    o.rk3_update(0.0, 1.0, dt)
    s.rk3_update(q, old, 0.0, 1.0, dt)
    pu.assert_cells({k: pu.host(q[k]) for k in pu.FIELDS}, o.f, pu.FIELDS, sc, "cfg1 rk3")
    o.enforce_admissible()
    s.enforce_admissible(q)
    pu.assert_cells({k: pu.host(q[k]) for k in pu.FIELDS}, o.f, pu.FIELDS, sc, "cfg1 admissible")
    o.update_prims()
    s.update_prims(q)
    pu.assert_cells({k: pu.host(q[k]) for k in pu.ALL}, o.f, pu.ALL, sc, "cfg1 update_prims")
    del o, s, q, old
    release()


def test_cfg1_triple_point_two_steps(triple_full):
    """Two whole SSP-RK3 steps of configuration 1 at 7168 x 3072 (fused stage) against the oracle."""
    nx, ny, params, st = triple_full
    o = oracle_for(params, nx, ny, st)
    s = Solver(params, nx, ny)
    q = gpu_state_from(o, nx, ny)
    old = alloc_state(nx, ny, names=pu.FIELDS)
    dt_o = dt_g = o.get_dt()
    for n in (1, 2):
        dt_o = o.step(dt_o)
        dt_g = s.step(q, old, dt_g)
        e, k = state_err(q, o, params)
        print(f"cfg1 7168x3072 step {n}: {e:.2e} ({k}), dt {abs(dt_g - dt_o) / dt_o:.1e}")
        assert e <= RTOL_STEPS, f"step {n}: {k} differs by {e:.3e}"
        assert abs(dt_g - dt_o) <= 1e-10 * dt_o
    del o, s, q, old
    release()


def test_cfg2_mach10_five_steps():
    """Configuration 2: 4096 x 2048 Mach-10 cylinder, M10 as shipped, five steps."""
    nx, ny = 4096, 2048
    params = SolverParams(dx=1.0 / nx, dy=0.5 / ny, gamma1=4.4, pinf1=6e8, variant="m10",
                          recon="shipped", bc=("transmissive",) * 4)
    st = {k: v.numpy() for k, v in ic.shock_droplet(nx, ny, 1.0, 0.5, mach=10.0, device="cpu").items()}
    o = oracle_for(params, nx, ny, st)
    s = Solver(params, nx, ny)
    q = gpu_state_from(o, nx, ny)
    old = alloc_state(nx, ny, names=pu.FIELDS)
    dt_o = dt_g = o.get_dt()
    for n in range(1, 6):
        dt_o = o.step(dt_o)
        dt_g = s.step(q, old, dt_g)
        e, k = state_err(q, o, params)
        print(f"cfg2 4096x2048 step {n}: {e:.2e} ({k}), dt {abs(dt_g - dt_o) / dt_o:.1e}")
        assert e <= RTOL_STEPS, f"step {n}: {k} differs by {e:.3e}"
        assert abs(dt_g - dt_o) <= 1e-10 * dt_o
    del o, s, q, old
    release()
