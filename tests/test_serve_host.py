"""Host logic of the serving form, without a GPU: the request generator, admission by slots and
memory budget, the serial comparison schedule, and the continuous-batching loop driven through a
stand-in batch that advances step counters instead of launching kernels."""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from wavemp.serve import Admission, Request, Server, percentile, poisson_requests, serial_schedule  # noqa: E402
from wavemp.batch import SolveSpec  # noqa: E402


def test_poisson_requests_are_seeded_and_in_range():
    a = poisson_requests(400, device="cpu")
    b = poisson_requests(400, device="cpu")
    assert [(r.arrival, r.spec.nx, r.spec.max_steps) for r in a] == [(r.arrival, r.spec.nx, r.spec.max_steps) for r in b]
    gaps = np.diff([0.0] + [r.arrival for r in a])
    assert np.all(gaps > 0)
    assert abs(gaps.mean() - 1.0 / 20.0) < 0.15 / 20.0  # rate 20/s
    for r in a:
        assert 64 <= r.spec.nx <= 2048 and r.spec.nx % 8 == 0 and r.spec.ny * 2 == r.spec.nx
        assert 50 <= r.spec.max_steps <= 2000
        assert math.isclose(r.spec.dx, 1.0 / r.spec.nx) and math.isclose(r.spec.dy, 0.5 / r.spec.ny)
    logs = np.log([r.spec.nx for r in a])
    assert logs.min() < math.log(100) and logs.max() > math.log(1500)  # spans the range
    c = poisson_requests(5, seed=1, device="cpu")
    assert [r.spec.nx for r in c] != [r.spec.nx for r in a[:5]]


def test_admission_by_slots_and_budget():
    adm = Admission(slots=2, budget_bytes=100)
    assert adm.can_admit(60)
    adm.admit(60)
    assert not adm.can_admit(50)  # over the budget
    assert adm.can_admit(40)
    adm.admit(40)
    assert not adm.can_admit(0)  # no slot
    with pytest.raises(RuntimeError):
        adm.admit(0)
    adm.release(60)
    assert adm.can_admit(60) and adm.peak_bytes == 100
    assert not adm.fits_at_all(101)


def test_serial_schedule_and_percentiles():
    f = serial_schedule([0.0, 1.0, 1.5, 10.0], [2.0, 1.0, 3.0, 1.0])
    assert f == [2.0, 3.0, 6.0, 11.0]
    assert percentile([1, 2, 3, 4, 5], 50) == 3.0
    assert math.isclose(percentile(list(range(101)), 99), 99.0)


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, d):
        self.t += d


class FakeBatch:
    """Slots with step counters; one step of the batch takes 1 ms of the fake clock."""

    def __init__(self, capacity, clock):
        self.slots = [None] * capacity
        self.clock = clock
        self.log = []

    def bytes_for(self, nx, ny):
        return nx * ny

    def set_shape(self, cls, shape):
        pass

    def close(self):
        pass

    def add(self, spec):
        slot = self.slots.index(None)
        self.slots[slot] = {"spec": spec, "steps": 0, "q": {"ar1": torch.zeros(2)}}
        self.log.append(("add", self.clock.t, spec.nx))
        return slot

    def run(self, n):
        for e in self.slots:
            if e is not None:
                e["steps"] = min(e["steps"] + n, e["spec"].max_steps)
        self.clock.t += 1e-3 * n

    def status(self):
        return [{"used": e is not None, "done": e is None or e["steps"] >= e["spec"].max_steps,
                 "steps": 0 if e is None else e["steps"]} for e in self.slots]

    def remove(self, slot):
        e = self.slots[slot]
        self.slots[slot] = None
        self.log.append(("remove", self.clock.t, e["spec"].nx))
        return e


def reqs(specs):
    return [Request(rid=k, arrival=a, spec=SolveSpec(nx=nx, ny=nx // 2, dx=1.0 / nx, dy=1.0 / nx, max_steps=s))
            for k, (a, nx, s) in enumerate(specs)]


def test_continuous_batching_loop():
    clock = FakeClock()
    fb = FakeBatch(2, clock)
    srv = Server(capacity=2, budget_bytes=10_000, chunk_steps=5, batch=fb)
    rs = reqs([(0.0, 64, 20), (0.001, 64, 50), (0.002, 64, 10), (0.5, 64, 5)])
    out = srv.run(rs, clock=clock, sleep=clock.sleep)
    assert all(r.steps_done == r.spec.max_steps for r in rs)
    # the third request waits for a slot, joins while the second is still running
    assert rs[2].admitted >= rs[0].finished and rs[2].admitted < rs[1].finished
    # the fourth arrives after the others are done: the loop idles until it arrives
    assert rs[3].admitted >= 0.5
    assert all(r.latency >= 0 for r in rs)
    assert out["requests"] == 4 and out["cell_stages"] == sum(3 * 64 * 32 * s for s in (20, 50, 10, 5))
    assert srv.admission.in_use == 0 and srv.admission.bytes == 0


def test_budget_bounds_memory_in_flight():
    clock = FakeClock()
    fb = FakeBatch(8, clock)
    srv = Server(capacity=8, budget_bytes=3 * 128 * 64, chunk_steps=3, batch=fb)
    rs = reqs([(0.0, 128, 9), (0.0, 128, 9), (0.0, 128, 9), (0.0, 128, 9), (0.0, 64, 3)])
    srv.run(rs, clock=clock, sleep=clock.sleep)
    assert srv.admission.peak_bytes <= 3 * 128 * 64
    live = peak = 0
    for kind, _, _ in fb.log:
        live += 1 if kind == "add" else -1
        peak = max(peak, live)
    assert peak <= 3
    with pytest.raises(ValueError):
        Server(capacity=2, budget_bytes=100, batch=FakeBatch(2, clock)).run(reqs([(0.0, 64, 3)]), clock=clock)
