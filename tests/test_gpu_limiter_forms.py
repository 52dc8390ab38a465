"""The fused stage's two limiter forms give the same bits: blend sweeps in place (the reference's
pp_blend_x/y_flux_kernel, SC:1479-1548) and blends rebuilt in registers by the next pass and the
combine. Both precisions, both variants, a case that limits (the near-vacuum stress fixture) and
whole steps with the device dt."""
import numpy as np
import pytest

import parity_util as pu

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import wavemp  # noqa: E402
from wavemp import Solver, alloc_state  # noqa: E402

CASES = ["sc_mp5c6_stress", "m10_cfg2", "sc_mp5c6_triple", "m10_mp5c6_rand"]


def load_state(d):
    nx, ny, g = int(d["meta_nx"]), int(d["meta_ny"]), int(d["meta_g"])
    q = alloc_state(nx, ny, g)
    for k in pu.ALL:
        q[k].copy_(torch.from_numpy(np.ascontiguousarray(d["in_" + k])))
    return q


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("case", CASES)
def test_deferred_blends_equal_in_place(case, precision):
    if precision == "fp32" and "stress" in case:
        pytest.skip("near-vacuum states are outside the binary32 form")
    d = pu.load_case(case)
    nx, ny = int(d["meta_nx"]), int(d["meta_ny"])
    out = []
    limited = []
    for in_place in (True, False):
        s = Solver(pu.params_from(d, precision=precision), nx, ny)
        s.set_limiter_sweeps(in_place)
        q = load_state(d)
        old = alloc_state(nx, ny, names=wavemp.FIELDS)
        s.init_dt(q)
        for _ in range(3):
            s.step(q, old, None, sync=False)
        torch.cuda.synchronize()
        out.append({k: pu.host(v) for k, v in q.items()})
        limited.append(s.status()["limited_cells"])
    for k in pu.ALL:
        assert np.array_equal(out[0][k], out[1][k], equal_nan=True), f"{case} {precision} {k}"
    assert limited[0] == limited[1]
    if "stress" in case:
        assert limited[0] > 0  # the case exercises the limiter


@pytest.mark.parametrize("case", ["sc_mp5c6_stress", "sc_mp5c6_triple"])
def test_faces_outside_the_finiteness_bound(case):
    """A block of cells at total energy 1e20 (pressure far above 2^60): the binary64 sweep cannot
    prove those faces' first-order values finite from the wave speeds, forms them and tests them.
    The in-place form (values formed on demand, byte from the proof or the values) and the deferred
    form (values stored, byte from the values) must still give the same bits."""
    d = pu.load_case(case)
    nx, ny, g = int(d["meta_nx"]), int(d["meta_ny"]), int(d["meta_g"])
    out = []
    for in_place in (True, False):
        s = Solver(pu.params_from(d, precision="fp64"), nx, ny)
        s.set_limiter_sweeps(in_place)
        q = load_state(d)
        i0, j0 = g + nx // 2 - 2, g + ny // 2 - 2
        q["E"][i0:i0 + 4, j0:j0 + 4] = 1.0e20
        s.update_prims(q)
        assert float(q["p_p"][i0:i0 + 4, j0:j0 + 4].abs().min()) > 2.0 ** 60
        old = alloc_state(nx, ny, names=wavemp.FIELDS)
        s.init_dt(q)
        for _ in range(2):
            s.step(q, old, None, sync=False)
        torch.cuda.synchronize()
        out.append({k: pu.host(v) for k, v in q.items()})
    for k in pu.ALL:
        assert np.array_equal(out[0][k], out[1][k], equal_nan=True), f"{case} {k}"
