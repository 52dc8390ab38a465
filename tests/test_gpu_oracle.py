"""GPU vs the CPU oracle on larger seeded states, every scheme variant and boundary rule, plus the
size-independent properties checked at the headline workload's size (7168 x 3072)."""
import numpy as np
import pytest

import parity_util as pu

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

from oracle import oracle as orc  # noqa: E402
from wavemp import Solver, SolverParams, alloc_state  # noqa: E402
from wavemp import ic  # noqa: E402

BCS = {"transmissive": orc.TRANSMISSIVE, "slip": orc.SLIP}


def run_both(state, nx, ny, params: SolverParams, steps, dt=None):
    """Run `steps` SSP-RK3 steps on GPU and oracle from the same state; return both states."""
    P = orc.make_params(params.dx, params.dy, params.gamma1, params.pinf1, params.gamma2,
                        params.pinf2, variant=orc.M10 if params.variant == "m10" else orc.SC,
                        recon=orc.MP5C6 if params.recon == "mp5c6" else orc.SHIPPED,
                        bc=[BCS[b if b != "reflective" else "slip"] for b in params.bc],
                        cfl=params.cfl, repair=params.emergency_repair)
    o = orc.OracleSolver(nx, ny, P)
    o.load(state)
    o.init_sequence()
    s = Solver(params, nx, ny)
    q = alloc_state(nx, ny)
    for k in pu.ALL:
        q[k].copy_(torch.from_numpy(o.f[k]))
    old = alloc_state(nx, ny, names=pu.FIELDS)
    dt_o = o.get_dt() if dt is None else dt
    dt_g = dt_o
    for _ in range(steps):
        dt_o = o.step(dt_o)
        dt_g = s.step(q, old, dt_g)
    return o, q, dt_o, dt_g


def assert_state(q, o, params, what, rtol=1e-9):
    """GPU state vs oracle state after several steps (natural units, parity_util)."""
    ref = {k: o.f[k] for k in pu.ALL}
    sc = pu.natural_scales(ref, params.gamma1, params.pinf1, params.gamma2, params.pinf2)
    pu.assert_cells({k: pu.host(q[k]) for k in pu.ALL}, ref, pu.ALL, sc, what, rtol=rtol)


@pytest.mark.parametrize("variant,recon", [("sc", "shipped"), ("sc", "mp5c6"), ("m10", "shipped"),
                                           ("m10", "mp5c6")])
def test_droplet_vs_oracle(variant, recon):
    nx, ny = 160, 80
    params = SolverParams(dx=1.0 / nx, dy=0.5 / ny, gamma1=4.4, pinf1=6e8, variant=variant,
                          recon=recon, bc=("transmissive",) * 4)
    st = ic.shock_droplet(nx, ny, 1.0, 0.5, mach=2.4 if variant == "sc" else 10.0, device="cpu")
    st = {k: v.numpy() for k, v in st.items()}
    o, q, dt_o, dt_g = run_both(st, nx, ny, params, steps=3)
    assert_state(q, o, params, f"{variant}/{recon}")
    assert abs(dt_g - dt_o) <= 1e-10 * dt_o


@pytest.mark.parametrize("bc", [("slip",) * 4, ("transmissive",) * 4,
                                ("slip", "transmissive", "transmissive", "slip")])
def test_boundary_rules_vs_oracle(bc):
    nx, ny = 56, 24
    params = SolverParams(dx=7.0 / nx, dy=3.0 / ny, gamma1=1.5, pinf1=0.0, gamma2=1.4, pinf2=0.0,
                          recon="mp5c6", bc=bc)
    st = {k: v.numpy() for k, v in ic.triple_point(nx, ny, device="cpu").items()}
    o, q, dt_o, dt_g = run_both(st, nx, ny, params, steps=4)
    assert_state(q, o, params, f"bc={bc}")


@pytest.mark.parametrize("nx,ny", [(1, 1), (1, 7), (9, 1), (3, 5), (33, 17)])
def test_ragged_tiny_grids_vs_oracle(nx, ny):
    """Grids smaller than a warp or a block, odd sizes, a single cell."""
    params = SolverParams(dx=0.1, dy=0.07, gamma1=4.4, pinf1=6e8, recon="mp5c6")
    rng = np.random.default_rng(nx * 100 + ny)
    st = {k: v.numpy() for k, v in ic.random_valid(nx, ny, rng, device="cpu").items()}
    o, q, _, _ = run_both(st, nx, ny, params, steps=2)
    assert_state(q, o, params, f"{nx}x{ny}")


def oracle_self_sensitivity(state, nx, ny, params, steps):
    """Largest natural-unit change of the oracle's result when its input gets 1e-15 relative noise."""
    P = orc.make_params(params.dx, params.dy, params.gamma1, params.pinf1, params.gamma2,
                        params.pinf2)
    outs = []
    for seed in (None, 1, 2):
        o = orc.OracleSolver(nx, ny, P)
        if seed is None:
            o.load(state)
        else:
            r = np.random.default_rng(seed)
            o.load({k: v * (1 + 1e-15 * r.standard_normal(v.shape)) for k, v in state.items()})
        o.init_sequence()
        dt = o.get_dt()
        for _ in range(steps):
            dt = o.step(dt)
        outs.append({k: o.f[k].copy() for k in pu.ALL})
    sc = pu.natural_scales(outs[0], params.gamma1, params.pinf1, params.gamma2, params.pinf2)
    return max(pu.cell_err(x, outs[0], k, sc) for x in outs[1:] for k in pu.ALL)


def test_poisoned_cells_are_repaired_like_the_reference():
    """NaN in the input state: the reference's isnan guards and the emergency repair decide the
    outcome; the GPU must make the same decisions as the oracle. A repaired cell sits at the
    pressure floor (rho c~^2 = 1e-8, sound speed ~0), which makes its neighbours' Riemann problems
    nearly singular: the oracle's own result moves by ~2e-9 under 1e-15 input noise here, so the
    tolerance is ten times that measured sensitivity (at least 1e-9)."""
    nx, ny = 24, 16
    params = SolverParams(dx=0.01, dy=0.01, gamma1=4.4, pinf1=6e8)
    rng = np.random.default_rng(3)
    st = {k: v.numpy().copy() for k, v in ic.random_valid(nx, ny, rng, device="cpu").items()}
    st["E"][12, 9] = np.nan
    st["ar2"][14, 12] = np.nan
    st["ru"][8, 15] = np.nan
    tol = max(1e-9, 10.0 * oracle_self_sensitivity(st, nx, ny, params, steps=1))
    assert tol < 1e-7
    o, q, _, _ = run_both(st, nx, ny, params, steps=1)
    for k in pu.ALL:
        a, b = pu.host(q[k]), o.f[k]
        assert np.array_equal(np.isnan(a), np.isnan(b)), f"NaN pattern {k}"
    assert_state(q, o, params, "poisoned", rtol=tol)


# ---------------------------------------------------------------- properties at full size -----
FULL = (7168, 3072)


def test_full_size_uniform_state_stays_uniform():
    nx, ny = FULL
    params = SolverParams(dx=7.0 / nx, dy=3.0 / ny, gamma1=1.5, pinf1=0.0, recon="mp5c6",
                          bc=("slip",) * 4)
    s = Solver(params, nx, ny)
    q = alloc_state(nx, ny)
    q["ar1"].fill_(0.6)
    q["ar2"].fill_(0.4)
    q["al"].fill_(0.6)
    q["E"].fill_(2.5)
    s.update_prims(q)
    old = alloc_state(nx, ny, names=pu.FIELDS)
    e0 = q["E"][5, 5].item()
    s.step(q, old, 1e-3)
    for k in pu.FIELDS:
        t = q[k][5:-5, 5:-5]
        assert torch.equal(t, t[0, 0].expand_as(t)), f"uniformity lost in {k}"
    assert abs(q["E"][5, 5].item() - e0) <= 4e-16 * abs(e0)
    del s, q, old
    torch.cuda.empty_cache()


def test_full_size_conservation_with_walls():
    """Slip walls on all four sides: partial masses and energy are conserved to round-off."""
    nx, ny = FULL
    params = SolverParams(dx=7.0 / nx, dy=3.0 / ny, gamma1=1.5, pinf1=0.0, recon="mp5c6",
                          bc=("slip",) * 4)
    s = Solver(params, nx, ny)
    q = ic.triple_point(nx, ny)
    old = alloc_state(nx, ny, names=pu.FIELDS)
    s.update_prims(q)
    tot0 = {k: q[k][5:-5, 5:-5].sum().item() for k in ("ar1", "ar2", "E")}
    dt = s.get_dt(q)
    for _ in range(2):
        dt = s.step(q, old, dt)
    for k, v in tot0.items():
        v1 = q[k][5:-5, 5:-5].sum().item()
        assert abs(v1 - v) <= 1e-12 * abs(v), f"{k}: {v} -> {v1}"
    assert s.status()["repaired_cells"] == 0
    del s, q, old
    torch.cuda.empty_cache()


def test_mirror_symmetry_full_size():
    """The y sweep on a state equals the x sweep on its transpose with u and v exchanged."""
    nx, ny = 2048, 1024
    pa = SolverParams(dx=1.0 / nx, dy=0.5 / ny, gamma1=4.4, pinf1=6e8, recon="mp5c6",
                      bc=("transmissive",) * 4)
    pb = SolverParams(dx=0.5 / ny, dy=1.0 / nx, gamma1=4.4, pinf1=6e8, recon="mp5c6",
                      bc=("transmissive",) * 4)
    qa = ic.shock_droplet(nx, ny, 1.0, 0.5, mach=2.4)
    qb = {}
    swap = {"ru": "rv", "rv": "ru", "u_p": "v_p", "v_p": "u_p"}
    for k, v in qa.items():
        qb[swap.get(k, k)] = v.t().contiguous()
    sa, sb = Solver(pa, nx, ny), Solver(pb, ny, nx)
    sa.update_prims(qa)
    sb.update_prims(qb)
    oa, ob = alloc_state(nx, ny, names=pu.FIELDS), alloc_state(ny, nx, names=pu.FIELDS)
    dt = min(sa.get_dt(qa), sb.get_dt(qb))
    sa.step(qa, oa, dt)
    sb.step(qb, ob, dt)
    got = {k: pu.host(qa[k]) for k in pu.ALL}
    ref = {k: pu.host(qb[swap.get(k, k)]).T for k in pu.ALL}
    sc = pu.natural_scales(ref, 4.4, 6e8, 1.4, 0.0)
    pu.assert_cells(got, ref, pu.ALL, sc, "mirror", rtol=1e-10)
