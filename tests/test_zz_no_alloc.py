"""wm_rhs_stage_static: one RHS stage for callers that cannot allocate device memory.

Such callers (a host application that serves all device memory from its own pool and forbids
libraries to call cudaMalloc, or a loop that must not wait on the allocator) get a stage whose
workspace is a device array inside the library, for grids up to 32768 padded cells, in the plain
binary64 form. These tests call it through the C ABI and check that two calls in a row give the
same state as the handle-based wm_rhs_stage, bit for bit (the same kernels run the same
arithmetic), for both scheme variants, both reconstructions, both boundary rules and with the
emergency repair on and off; that a call allocates no device memory; and that a grid above the
limit is refused with a clear message. This file is collected last so that, if it fails, a run
that stops at the first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import wavemp  # noqa: E402
from wavemp import _lib  # noqa: E402


def c_fields(q):
    f = _lib.WmFields()
    for k in wavemp.ALL:
        if k in q:
            setattr(f, k, q[k].data_ptr())
    f.pitch = q["ar1"].stride(0)
    return f


def clone(q):
    block = torch.stack([q[k] for k in q]).clone()
    return {k: block[c] for c, k in enumerate(q)}


CASES = [
    ("sc", "mp5c6", ("transmissive",) * 4, True),
    ("sc", "shipped", ("transmissive", "transmissive", "slip", "slip"), True),
    ("m10", "shipped", ("transmissive",) * 4, True),
    ("m10", "mp5c6", ("slip",) * 4, False),
    ("sc", "mp5c6", ("slip",) * 4, False),
]


@pytest.mark.parametrize("variant,recon,bc,repair", CASES)
def test_static_stage_equals_handle_stage_twice(variant, recon, bc, repair):
    nx, ny, g = 64, 32, 5
    assert (nx + 2 * g) * (ny + 2 * g) <= _lib.STATIC_MAX_CELLS
    params = wavemp.SolverParams(dx=1.0 / nx, dy=0.5 / ny, gamma1=4.4, pinf1=6e8, variant=variant,
                                 recon=recon, bc=bc, emergency_repair=repair)
    s = wavemp.Solver(params, nx, ny, g)
    q_ref = wavemp.ic.shock_droplet(nx, ny, 1.0, 0.5, mach=2.4 if variant == "sc" else 10.0)
    s.initialize(q_ref)
    q_new = clone(q_ref)
    old = clone({k: q_ref[k] for k in wavemp.FIELDS})
    dt = s.get_dt(q_ref)
    L = _lib.load()
    cp = params.to_c()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call, (alpha, beta) in enumerate(((0.0, 1.0), (0.75, 0.25))):
        s.rhs_stage(q_ref, old, dt, alpha, beta)
        f_new, f_old = c_fields(q_new), c_fields(old)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = L.wm_rhs_stage_static(ctypes.byref(cp), nx, ny, g, ctypes.byref(f_new),
                                   ctypes.byref(f_old), dt, alpha, beta, stream)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        assert rc == _lib.WM_OK, L.wm_last_error().decode()
        if call == 1:  # the first call may load the library's device code; later ones allocate nothing
            assert free_after == free_before
        for k in wavemp.ALL:
            a, b = q_new[k].cpu().numpy(), q_ref[k].cpu().numpy()
            assert np.array_equal(a, b, equal_nan=True), f"static stage call {call + 1}: {k}"


def test_static_stage_rejects_grids_above_the_limit():
    L = _lib.load()
    nx = ny = 200  # 210 x 210 padded cells > 32768
    params = wavemp.SolverParams(dx=0.01, dy=0.01)
    empty = _lib.WmFields()
    rc = L.wm_rhs_stage_static(ctypes.byref(params.to_c()), nx, ny, 5, ctypes.byref(empty), None,
                               1e-6, 0.0, 1.0, None)
    assert rc == -1
    assert b"exceeds the static scratch limit" in L.wm_last_error()
