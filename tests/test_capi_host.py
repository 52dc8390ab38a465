"""The C ABI's host-side logic without a GPU: workspace sizes (the layout's bytes per padded cell
for both forms, the batch's per-solve size within the handle's, so that wavemp.batch.Batch.add
gives wm_batch_set enough), argument validation (every rejected parameter returns 0 bytes and
WM_ERR_INVALID from wm_create, before any CUDA call), a caller workspace that is too small or
misaligned (WM_ERR_NOMEM, before the library touches it), wm_copy_state's argument checks, and the
Python parameter checks. No kernel is launched and no device memory is allocated."""
import ctypes
import math
import os
import shutil

import pytest

pytestmark = pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                                reason="needs nvcc to build the library")

WM_ERR_INVALID, WM_ERR_CUDA, WM_ERR_NOMEM = -1, -2, -3


@pytest.fixture(scope="module")
def lib():
    from wavemp import _lib

    return _lib.load()


def params(**kw):
    from wavemp import SolverParams

    base = dict(dx=1.0 / 64, dy=1.0 / 64, gamma1=4.4, pinf1=6e8, recon="mp5c6", bc=("transmissive",) * 4)
    base.update(kw)
    return SolverParams(**base).to_c()


def bytes_for(lib, p, nx, ny, g=5):
    return lib.wm_workspace_bytes(ctypes.byref(p), nx, ny, g)


@pytest.mark.parametrize("precision, per_cell", [("fp64", 42 * 8 + 5 * 4 + 2), ("fp32", 54 * 4 + 8 + 2)])
def test_workspace_bytes_per_padded_cell(lib, precision, per_cell):
    """Plain form: 42 binary64 arrays and five binary32 arrays per padded cell (the switch
    pre-check's entropy and four of its pair arrays: 336 + 20 B); precision form: 54 binary32 arrays
    (three of them pair arrays) and one binary64 array (224 B); both: two bytes of first-order
    finiteness (x and y faces); each array 256-byte aligned."""
    p = params(precision=precision)
    prev = 0
    for nx, ny in ((1, 1), (33, 17), (400, 200), (1024, 512), (7168, 3072)):
        cells = (nx + 10) * (ny + 10)
        n = bytes_for(lib, p, nx, ny)
        assert per_cell * cells <= n <= per_cell * cells + 60 * 256 + 65536, (nx, ny, n)
        assert n > prev
        prev = n


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_solve_workspace_fits_in_the_handle_size(lib, precision):
    from wavemp import _lib

    p = params(precision=precision)
    bp = _lib.WmBatchParams()
    bp.variant, bp.recon, bp.precision = _lib.VARIANT["sc"], _lib.RECON["mp5c6"], _lib.PRECISION[precision]
    bp.emergency_repair, bp.g, bp.cfl, bp.tile_shape = 1, 5, 0.4, -1
    for nx, ny in ((64, 32), (136, 68), (1024, 512), (2048, 1024)):
        need = lib.wm_solve_workspace_bytes(ctypes.byref(bp), nx, ny)
        assert 0 < need <= bytes_for(lib, p, nx, ny), (nx, ny)
    assert lib.wm_solve_workspace_bytes(ctypes.byref(bp), 0, 8) == 0


def bad_params():
    yield "gamma1 = 1", params(gamma1=1.0)
    yield "gamma2 < 1", params(gamma2=0.5)
    yield "dx = 0", params(dx=0.0)
    yield "dy < 0", params(dy=-1.0)
    yield "pinf infinite", params(pinf1=math.inf)
    yield "pinf NaN", params(pinf2=math.nan)
    yield "cfl = 0", params(cfl=0.0)
    p = params()
    p.variant = 7
    yield "variant", p
    p = params()
    p.recon = 9
    yield "recon", p
    p = params()
    p.precision = 5
    yield "precision", p
    p = params()
    p.bc[2] = 3
    yield "bc", p


def test_invalid_parameters_are_rejected(lib):
    for what, p in bad_params():
        assert bytes_for(lib, p, 64, 64) == 0, what
        h = ctypes.c_void_p(123)
        assert lib.wm_create(ctypes.byref(p), 64, 64, 5, None, 0, ctypes.byref(h)) == WM_ERR_INVALID, what
        assert h.value is None, what


def test_invalid_sizes_are_rejected(lib):
    p = params()
    for nx, ny, g in ((0, 8, 5), (8, 0, 5), (-3, 8, 5), (8, 8, 3), (8, 8, 65), (70000, 70000, 5)):
        assert bytes_for(lib, p, nx, ny, g) == 0, (nx, ny, g)
        h = ctypes.c_void_p()
        assert lib.wm_create(ctypes.byref(p), nx, ny, g, None, 0, ctypes.byref(h)) == WM_ERR_INVALID
    assert lib.wm_create(ctypes.byref(p), 8, 8, 5, None, 0, None) == WM_ERR_INVALID


def test_caller_workspace_too_small_or_misaligned(lib):
    """wm_create checks a caller's buffer before it uses it: the pointers below are never read."""
    p = params()
    need = bytes_for(lib, p, 64, 32)
    h = ctypes.c_void_p()
    assert lib.wm_create(ctypes.byref(p), 64, 32, 5, ctypes.c_void_p(1 << 20), need - 1,
                         ctypes.byref(h)) == WM_ERR_NOMEM
    assert lib.wm_create(ctypes.byref(p), 64, 32, 5, ctypes.c_void_p((1 << 20) + 8), need,
                         ctypes.byref(h)) == WM_ERR_NOMEM
    assert h.value is None


def test_python_parameters_reject_unknown_values():
    from wavemp import SolverParams

    for kw in (dict(variant="sc2"), dict(recon="weno"), dict(precision="fp16"), dict(bc=("wall",) * 4)):
        with pytest.raises(ValueError):
            SolverParams(dx=0.1, dy=0.1, **kw).to_c()
    with pytest.raises(ValueError):
        SolverParams(dx=0.1, dy=0.1, bc=("slip",) * 3).to_c()


def test_static_stage_refuses_the_precision_form_and_large_grids(lib):
    """wm_rhs_stage_static (the no-allocation stage) carries only the binary64 form's workspace:
    a WM_PREC_FP32 parameter set, a grid above WM_STATIC_MAX_CELLS padded cells and invalid
    parameters are refused with their own messages before any CUDA call (the field pointers below
    are never read)."""
    from wavemp import _lib

    empty = _lib.WmFields()
    p = params(precision="fp32")
    assert lib.wm_rhs_stage_static(ctypes.byref(p), 16, 16, 5, ctypes.byref(empty), None,
                                   1e-6, 0.0, 1.0, None) == WM_ERR_INVALID
    assert b"binary64 form only" in lib.wm_last_error()
    p = params()
    assert lib.wm_rhs_stage_static(ctypes.byref(p), 200, 200, 5, ctypes.byref(empty), None,
                                   1e-6, 0.0, 1.0, None) == WM_ERR_INVALID
    assert b"exceeds the static scratch limit" in lib.wm_last_error()
    for what, bad in bad_params():
        assert lib.wm_rhs_stage_static(ctypes.byref(bad), 16, 16, 5, ctypes.byref(empty), None,
                                       1e-6, 0.0, 1.0, None) == WM_ERR_INVALID, what
        assert b"invalid parameters" in lib.wm_last_error(), what
    assert lib.wm_rhs_stage_static(ctypes.byref(p), 16, 16, 5, ctypes.byref(empty), None,
                                   1e-6, 0.0, 1.0, None) == WM_ERR_INVALID
    assert b"invalid field pointers" in lib.wm_last_error()


def test_copy_state_argument_checks(lib):
    """wm_copy_state refuses null or unaligned addresses, sizes that are not a multiple of 16 and
    negative sizes before any CUDA call, and does nothing for 0 bytes; without a device even an
    aligned copy returns an error before any launch."""
    import numpy as np
    import torch

    buf = np.zeros(128, dtype=np.float64)
    a = buf.ctypes.data
    a16 = a + (-a) % 16  # 16-byte aligned, inside buf with 512 bytes after it
    vp = ctypes.c_void_p
    assert lib.wm_copy_state(vp(a16), vp(a16 + 256), 24, None) == WM_ERR_INVALID
    assert lib.wm_copy_state(vp(a16 + 8), vp(a16 + 256), 16, None) == WM_ERR_INVALID
    assert lib.wm_copy_state(vp(a16), vp(a16 + 264), 16, None) == WM_ERR_INVALID
    assert lib.wm_copy_state(vp(a16), vp(a16 + 256), -16, None) == WM_ERR_INVALID
    assert lib.wm_copy_state(None, vp(a16), 16, None) == WM_ERR_INVALID
    assert lib.wm_copy_state(vp(a16), vp(a16 + 256), 0, None) == 0
    if not torch.cuda.is_available():
        assert lib.wm_copy_state(vp(a16), vp(a16 + 256), 64, None) == WM_ERR_CUDA
