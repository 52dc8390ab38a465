"""Shock tubes with exact solutions through the device solver (Solver.run, the device time loop).

Four 1-D Riemann problems (Sod in either fluid, a stiffened-water tube, the water-air tube; see
tests/riemann_cases.py) on 400 cells laid along x and along y, with every scheme of the reference:
* binary64: the density profile equals the oracle's solve of the same tube to round-off
  (max |rho - rho_oracle| <= 1e-9 max rho after 200-640 steps), so the density L1 error against the
  exact solution is the oracle's, below the bound the oracle tests pin;
* the tube along y gives the tube along x (the y sweeps are the x sweeps with u and v exchanged);
* the precision form (binary32 reconstruction and fluxes) stays within the same bound against the
  exact solution, and its distance to the binary64 density (L1) is below a tenth of the binary64
  error against the exact solution (measured: 4e-8 .. 5.5e-6, against 7e-4 .. 3.5e-3): binary32
  moves knife-edge decisions of the scheme (the THINC and MP5 switches) at a few faces, which costs
  far less than the discretisation does;
* volume fraction in [1e-8, 1 - 1e-8] and partial densities at or above the floor after the run.
"""
import numpy as np
import pytest

import riemann_cases as rc

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import wavemp  # noqa: E402
from wavemp import Solver, SolverParams, alloc_state  # noqa: E402

N = 400
BOUND_400 = {"sod_fluid1": 2.8e-3, "sod_fluid2": 3.0e-3, "water_tube": 1.7e-3, "water_air": 5.0e-3}
SCHEMES = [("sc", "shipped"), ("sc", "mp5c6"), ("m10", "shipped")]


def run_device(case, variant, recon, along="x", precision="fp64"):
    nx, ny = (N, 1) if along == "x" else (1, N)
    p = SolverParams(dx=1.0 / nx, dy=1.0 / ny, gamma1=case.g1, pinf1=case.p1, gamma2=case.g2,
                     pinf2=case.p2, variant=variant, recon=recon, bc=("transmissive",) * 4,
                     precision=precision)
    s = Solver(p, nx, ny)
    q = {k: torch.from_numpy(v).cuda() for k, v in rc.initial_grid(case, N, along).items()}
    old = alloc_state(nx, ny, names=wavemp.FIELDS)
    s.initialize(q)
    t, steps = s.run(q, old, case.t_end)
    torch.cuda.synchronize()
    assert abs(t - case.t_end) <= 1e-12 * case.t_end and steps > 0
    out = {k: v.cpu().numpy() for k, v in q.items()}
    s.close()
    return out


def check_bounds(f, along):
    inner = (slice(rc.G, rc.G + N), slice(rc.G, rc.G + 1)) if along == "x" else \
        (slice(rc.G, rc.G + 1), slice(rc.G, rc.G + N))
    assert f["al"][inner].min() >= 1.0e-8 and f["al"][inner].max() <= 1.0 - 1.0e-8
    assert min(f["ar1"][inner].min(), f["ar2"][inner].min()) >= 1.0e-10


@pytest.mark.parametrize("variant,recon", SCHEMES)
@pytest.mark.parametrize("name", sorted(rc.CASES))
def test_shock_tube_fp64(name, variant, recon):
    case = rc.CASES[name]
    ref = rc.density_line(rc.run_oracle(case, N, variant, recon), N, "x")
    fx = run_device(case, variant, recon, "x")
    fy = run_device(case, variant, recon, "y")
    for f, along in ((fx, "x"), (fy, "y")):
        rho = rc.density_line(f, N, along)
        assert np.isfinite(rho).all()
        assert np.abs(rho - ref).max() <= 1e-9 * np.abs(ref).max(), f"{along}: device vs oracle"
        err = rc.l1_error(case, rho)
        assert err <= BOUND_400[name], f"{name} {variant}/{recon} along {along}: L1 {err:.3e}"
        check_bounds(f, along)


@pytest.mark.parametrize("variant,recon", SCHEMES)
@pytest.mark.parametrize("name", sorted(rc.CASES))
def test_shock_tube_precision_form(name, variant, recon):
    case = rc.CASES[name]
    ref = rc.density_line(run_device(case, variant, recon, "x"), N, "x")
    discretisation = rc.l1_error(case, ref)
    for along in ("x", "y"):
        f = run_device(case, variant, recon, along, precision="fp32")
        rho = rc.density_line(f, N, along)
        assert np.isfinite(rho).all()
        l1 = np.abs(rho - ref).sum() / np.abs(ref).sum()
        assert l1 <= 0.1 * discretisation, \
            f"{name} {variant}/{recon} along {along}: fp32 vs fp64 L1 {l1:.3e}, fp64 vs exact {discretisation:.3e}"
        assert rc.l1_error(case, rho) <= BOUND_400[name]
        check_bounds(f, along)
