"""The time loop on the device (wm_run, Solver.run) against the reference's loop (SC:2009-2073)
driven from the host step by step with host-side dt clamps: the same save steps and times, and the
same state at every save and at the end, bit for bit (the same kernels on the same dt values).
Also: the per-call step limit, a restart from a written checkpoint, and the graph form in use."""
import numpy as np
import pytest

import parity_util as pu

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import wavemp  # noqa: E402
from wavemp import Solver, SolverParams, alloc_state, ic  # noqa: E402
from wavemp.checkpoint import cell_centres, load_restart, save_npz  # noqa: E402

NX, NY = 64, 32


def make(precision="fp64"):
    p = SolverParams(dx=1.0 / NX, dy=0.5 / NY, gamma1=4.4, pinf1=6e8, bc=("transmissive",) * 4,
                     recon="mp5c6", precision=precision)
    s = Solver(p, NX, NY)
    q = ic.shock_droplet(NX, NY, 1.0, 0.5, mach=2.4)
    old = alloc_state(NX, NY, names=wavemp.FIELDS)
    s.initialize(q)
    return p, s, q, old


def host_loop(s, q, old, t_end, saves, t=0.0, step=0):
    """SC:2013-2073 as the reference writes it, one host step at a time."""
    flags = [t >= ts - 1.0e-14 for ts in saves]
    dt = s.get_dt(q)
    hits = []
    while t < t_end - 1.0e-14:
        for k, ts in enumerate(saves):
            if not flags[k] and t + dt > ts:
                dt = ts - t
        if t + dt > t_end:
            dt = t_end - t
        dt_next = s.step(q, old, dt)
        t += dt
        step += 1
        dt = dt_next
        for k, ts in enumerate(saves):
            if not flags[k] and abs(t - ts) < 0.5 * dt:
                if not any(h[0] == step for h in hits):
                    hits.append((step, t, {n: pu.host(v) for n, v in q.items()}))
                flags[k] = True
    return t, step, hits


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_device_loop_equals_host_loop(precision):
    _, s1, q1, old1 = make(precision)
    dt0 = s1.get_dt(q1)
    t_end, saves = 23.37 * dt0, [5.5 * dt0, 5.9 * dt0, 14.25 * dt0, 23.37 * dt0]
    t_h, n_h, hits_h = host_loop(s1, q1, old1, t_end, saves)
    _, s2, q2, old2 = make(precision)
    hits_d = []
    t_d, n_d = s2.run(q2, old2, t_end, saves,
                      on_save=lambda q, n, t, k: hits_d.append((n, t, {m: pu.host(v) for m, v in q.items()})))
    assert s2.run_uses_graph()
    assert (t_d, n_d) == (t_h, n_h)
    assert [(n, t) for n, t, _ in hits_d] == [(n, t) for n, t, _ in hits_h]
    for (_, _, a), (_, _, b) in zip(hits_d, hits_h):
        for k in wavemp.ALL:
            assert np.array_equal(a[k], b[k], equal_nan=True), k
    for k in wavemp.ALL:
        assert np.array_equal(pu.host(q1[k]), pu.host(q2[k]), equal_nan=True), k


def test_step_limit_and_continuation():
    _, s1, q1, old1 = make()
    dt0 = s1.get_dt(q1)
    t, n = s1.run(q1, old1, 1.0, max_steps=3)  # far end time: the limit stops it
    assert n == 3 and not s1.schedule.finished
    t, n = s1.run(q1, old1, 1.0, t=t, step=n, max_steps=4)
    assert n == 7
    _, s2, q2, old2 = make()
    s2.run(q2, old2, 1.0, max_steps=7)
    for k in wavemp.ALL:
        assert np.array_equal(pu.host(q1[k]), pu.host(q2[k]), equal_nan=True), k
    assert dt0 > 0


def test_restart_from_checkpoint_continues_the_run(tmp_path):
    p, s1, q1, old1 = make()
    dt0 = s1.get_dt(q1)
    t_end, mid = 12.0 * dt0, 5.0 * dt0
    x, y = cell_centres(NX, 0.0, 1.0), cell_centres(NY, 0.0, 0.5)
    files = []
    s1.run(q1, old1, t_end, [mid], on_save=lambda q, n, t, k: files.append(save_npz(q, x, y, n, t, str(tmp_path))))
    assert len(files) == 1
    q2, t2, n2 = load_restart(files[0], p, NX, NY)
    s2 = Solver(p, NX, NY)
    old2 = alloc_state(NX, NY, names=wavemp.FIELDS)
    s2.initialize(q2)
    t_fin, n_fin = s2.run(q2, old2, t_end, [mid], t=t2, step=n2)
    assert n_fin == s1.schedule.step and abs(t_fin - t_end) <= 1e-12 * t_end
    sc = pu.natural_scales({k: pu.host(v) for k, v in q1.items()}, 4.4, 6e8, 1.4, 0.0)
    pu.assert_cells({k: pu.host(v) for k, v in q2.items()}, {k: pu.host(v) for k, v in q1.items()},
                    pu.FIELDS, sc, "restarted run", rtol=1e-9)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_step_from_conserved_state_alone(precision):
    """A caller that keeps only the six conserved arrays (bench.py's end-to-end loop) copies them
    in, rebuilds the primitives with update_prims and steps: the same bits as stepping the
    device-resident state, whose primitives the previous step left."""
    p, s, q, old = make(precision)
    dt = s.get_dt(q)
    s.step(q, old, dt)  # primitives now those the step leaves
    q2 = alloc_state(NX, NY)
    for k in wavemp.FIELDS:
        q2[k].copy_(q[k])
    for k in ("u_p", "v_p", "p_p", "al_prim"):
        q2[k].fill_(float("nan"))
    s2 = Solver(p, NX, NY)
    old2 = alloc_state(NX, NY, names=wavemp.FIELDS)
    s2.update_prims(q2)
    for k in wavemp.ALL:
        assert torch.equal(q2[k], q[k]), k
    s.step(q, old, dt)
    s2.step(q2, old2, dt)
    for k in wavemp.ALL:
        assert torch.equal(q2[k], q[k]), k
