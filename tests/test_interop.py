"""The CUDA Array Interface adapter (``wavemp.from_cuda_array`` / ``from_warp``).

CPU: the validation of an interface description (type, rank, strides, pointer, read-only flag)
rejects every layout the solver cannot use before anything touches device memory. GPU: arrays
handed over through the interface alone (a holder object that is not a torch tensor, as a Warp
array is not) give the same step, bit for bit, as the solver's own tensors, and the step writes
into the producer's memory.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import parity_util as pu  # noqa: E402
import wavemp  # noqa: E402
from wavemp import interop  # noqa: E402


class Holder:
    """A device array known only through its CUDA Array Interface."""

    def __init__(self, **cai):
        base = dict(shape=(12, 9), typestr="<f8", data=(0x7f0000000000, False), version=3,
                    strides=None)
        base.update(cai)
        self.__cuda_array_interface__ = base


def test_accepts_contiguous_and_pitched_rows():
    assert interop.check_cuda_array(Holder()) == (0x7f0000000000, (12, 9), 9)
    assert interop.check_cuda_array(Holder(strides=(9 * 8, 8))) == (0x7f0000000000, (12, 9), 9)
    assert interop.check_cuda_array(Holder(strides=(16 * 8, 8)))[2] == 16
    assert interop.check_cuda_array(Holder(), shape=(12, 9))[1] == (12, 9)


@pytest.mark.parametrize("cai,msg", [
    (dict(typestr="<f4"), "float64"),
    (dict(shape=(12,)), "2-D"),
    (dict(shape=(2, 3, 4)), "2-D"),
    (dict(strides=(8, 12 * 8)), "contiguous"),
    (dict(strides=(4 * 8, 8)), "row stride"),
    (dict(strides=(9 * 8 + 4, 8)), "row stride"),
    (dict(data=(0x7f0000000004, False)), "aligned"),
    (dict(data=(0, False)), "null"),
    (dict(data=(0x7f0000000000, True)), "read-only"),
])
def test_rejects_unusable_layouts(cai, msg):
    with pytest.raises(ValueError, match=msg):
        interop.check_cuda_array(Holder(**cai))


def test_rejects_wrong_shape_and_non_producers():
    with pytest.raises(ValueError, match="shape"):
        interop.check_cuda_array(Holder(), shape=(12, 10))
    with pytest.raises(TypeError):
        interop.check_cuda_array(np.zeros((3, 3)))
    with pytest.raises(ValueError, match="missing field"):
        interop.state_from_cuda_arrays({"ar1": Holder()})


class Foreign:
    """Hides a torch tensor behind its CUDA Array Interface (the way a Warp array presents)."""

    def __init__(self, t):
        self._t = t
        self.__cuda_array_interface__ = t.__cuda_array_interface__


@pytest.mark.gpu
def test_foreign_arrays_step_like_the_solvers_own():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    nx, ny = 64, 32
    params = wavemp.SolverParams(dx=1.0 / nx, dy=0.5 / ny, gamma1=4.4, pinf1=6e8, recon="mp5c6",
                                 bc=("transmissive",) * 4)
    st = wavemp.ic.shock_droplet(nx, ny, 1.0, 0.5, mach=2.4)
    # one separate allocation per field, as the reference's alloc2d() makes them
    own = {k: v.clone() for k, v in st.items()}
    raw = {k: v.clone() for k, v in st.items()}
    foreign = {k: Foreign(v) for k, v in raw.items()}
    olds = {k: Foreign(torch.zeros_like(st[k])) for k in wavemp.FIELDS}
    q = wavemp.from_warp(foreign["ar1"])
    assert q.data_ptr() == raw["ar1"].data_ptr()
    q = wavemp.state_from_cuda_arrays(foreign)
    q_old = wavemp.state_from_cuda_arrays(olds, names=wavemp.FIELDS)
    s = wavemp.Solver(params, nx, ny)
    s.initialize(q)
    s.initialize(own)
    own_old = {k: torch.zeros_like(v) for k, v in own.items() if k in wavemp.FIELDS}
    dt = s.get_dt(own)
    for _ in range(2):
        s.step(q, q_old, dt)
        s.step(own, own_old, dt)
    for k in pu.ALL:
        # the producer's own memory holds the result
        assert torch.equal(raw[k], own[k]), k
