"""The batched droplet solve that the precision form leaves above the 1e-5 density-L1 bar (solve 63
of the 64 seeded shock-droplet solves: 168 x 84, Mach 5.6) is a knife edge of the reference's own
algorithm, not of this build's arithmetic.

The oracle (the CPU restatement of the reference's stage, SC:1899-1995, binary64 throughout) steps
the solve 300 times on its own CFL time steps. The same run with the conserved state multiplied by
1 + 1e-8 N(0, 1) after every step (a sixth of a binary32 rounding; the time steps replayed) ends more
than 1e-5 away in density L1, while an ordinary solve of the same workload (solve 11, 176 x 88)
moves by less than 1e-6 under the same noise. The noiseless run repeats bit for bit.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import oracle as O  # noqa: E402
from wavemp.batch import config3_solves  # noqa: E402

ALL10 = ("ar1", "ar2", "ru", "rv", "E", "al", "u_p", "v_p", "p_p", "al_prim")
STEPS = 300


def density_l1(a, b, g=5):
    ra, rb = (a[0] + a[1])[g:-g, g:-g], (b[0] + b[1])[g:-g, g:-g]
    return float(np.abs(ra - rb).sum() / np.abs(rb).sum())


def run(spec, state, eps=0.0, seed=0, dts=None):
    """STEPS steps of the oracle; after each, the six conserved fields times 1 + eps N(0, 1) (seeded)
    and the primitives rebuilt. dts: the time steps to replay (else the run's own CFL steps)."""
    P = O.make_params(spec.dx, spec.dy, variant=O.SC, recon=O.MP5C6, bc=(O.TRANSMISSIVE,) * 4, cfl=0.4,
                      repair=True)
    po = O.PackedOracle(spec.nx, spec.ny, P)
    for c, k in enumerate(ALL10):
        po.fields[c] = state[k].numpy()
    po.init_sequence()
    dt = po.get_dt()
    rng = np.random.default_rng(seed)
    used = []
    for s in range(STEPS):
        d = dts[s] if dts is not None else dt
        used.append(d)
        po.steps(1, d)
        if eps:
            for c in range(6):
                po.fields[c] *= 1.0 + eps * rng.standard_normal(po.fields[c].shape)
        po.init_sequence()
        dt = po.get_dt()
    return po.fields.copy(), used


@pytest.fixture(scope="module")
def solves():
    return config3_solves(n=64, seed=0, steps=STEPS, device="cpu")


def test_solve_63_moves_past_the_bar_under_sub_rounding_noise(solves):
    sp = solves[63]
    assert (sp.nx, sp.ny) == (168, 84)
    st = sp.make_state()
    base, dts = run(sp, st)
    again, _ = run(sp, st, dts=dts)
    assert density_l1(again, base) == 0.0
    for seed in (1, 2):
        moved, _ = run(sp, st, eps=1e-8, seed=seed, dts=dts)
        assert density_l1(moved, base) > 1e-5, seed


def test_an_ordinary_solve_stays_well_inside_it(solves):
    sp = solves[11]
    st = sp.make_state()
    base, dts = run(sp, st)
    moved, _ = run(sp, st, eps=1e-8, seed=1, dts=dts)
    assert density_l1(moved, base) < 1e-6
