"""Serving form on the device: every request's result is the same when it is served in a mix with
others (joining and leaving a running batch, other tile shapes, another launch length) as when it
is served alone. Tolerance: none -- the results are compared bit for bit, since no solve's
arithmetic depends on the other solves in the launch, on the tile shape or on the launch length.
The memory budget bounds what is in flight."""
import dataclasses

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import wavemp  # noqa: E402
from wavemp.batch import size_class  # noqa: E402
from wavemp.serve import Server, poisson_requests  # noqa: E402


def small_requests(n=6, seed=3):
    return poisson_requests(n, rate=200.0, seed=seed, min_nx=64, max_nx=192, min_steps=6, max_steps=22)


def fresh(r):
    return dataclasses.replace(r, arrival=0.0, admitted=None, finished=None, steps_done=0, result=None)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_served_result_same_alone_and_in_the_mix(precision):
    rs = small_requests()
    srv = Server(capacity=3, precision=precision, chunk_steps=4)
    out = srv.run(rs)
    srv.close()
    assert out["requests"] == len(rs)
    assert max(r.admitted for r in rs) > min(r.finished for r in rs)  # someone joined a running batch
    for r in rs:
        assert r.steps_done == r.spec.max_steps
        shapes = {size_class(r.spec.nx, r.spec.ny): 0}
        alone = Server(capacity=1, precision=precision, chunk_steps=7, shapes=shapes)
        ra = fresh(r)
        alone.run([ra])
        alone.close()
        for k in wavemp.ALL:
            a, b = r.result[k].numpy(), ra.result[k].numpy()
            assert np.array_equal(a, b, equal_nan=True), f"request {r.rid} {r.spec.nx}x{r.spec.ny} {k}"
        assert all(np.isfinite(r.result[k].numpy()).all() for k in wavemp.FIELDS)


def test_budget_bounds_what_is_in_flight():
    rs = small_requests(5, seed=4)
    probe = Server(capacity=1, precision="fp32")
    sizes = [probe.batch.bytes_for(r.spec.nx, r.spec.ny) for r in rs]
    probe.close()
    budget = max(sizes) + min(sizes)  # at most two solves at a time, sometimes one
    srv = Server(capacity=5, budget_bytes=budget, precision="fp32", chunk_steps=5, keep_results=False)
    srv.run(rs)
    srv.close()
    assert srv.admission.peak_bytes <= budget
    assert all(r.steps_done == r.spec.max_steps for r in rs)
