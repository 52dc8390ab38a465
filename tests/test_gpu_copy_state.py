"""wm_copy_state / wavemp.copy_state: the SM-driven copy of a state block between page-locked host
memory and the device (the caller's host <-> device transfers, which the reference makes with
wp.copy of wp.array(host), SC:1877-1886, and .numpy(), SC:2004-2007), and its argument checks."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import wavemp  # noqa: E402
from wavemp import _lib  # noqa: E402

INVALID = -1  # WM_ERR_INVALID


def test_round_trip_pinned_host_and_device():
    n = (1 << 20) + 6  # binary64 words: 8 MiB + 48 B
    src = torch.randn(n, dtype=torch.float64).pin_memory()
    dev = torch.empty(n, dtype=torch.float64, device="cuda")
    back = torch.zeros(n, dtype=torch.float64).pin_memory()
    wavemp.copy_state(dev, src)
    wavemp.copy_state(back, dev)
    torch.cuda.synchronize()
    assert torch.equal(dev.cpu(), src)
    assert torch.equal(back, src)


@pytest.mark.parametrize("n", [2, 6, 1024, 3 * 4096 * 256 + 2])
def test_device_to_device_every_tail(n):
    a = torch.randn(n, dtype=torch.float64, device="cuda")
    b = torch.zeros_like(a)
    wavemp.copy_state(b, a)
    torch.cuda.synchronize()
    assert torch.equal(a, b)


def test_argument_checks():
    L = _lib.load()
    a = torch.zeros(64, dtype=torch.float64, device="cuda")
    b = torch.zeros(64, dtype=torch.float64, device="cuda")
    pa, pb = a.data_ptr(), b.data_ptr()
    vp = ctypes.c_void_p
    assert L.wm_copy_state(vp(pa), vp(pb), 24, None) == INVALID      # not a multiple of 16
    assert L.wm_copy_state(vp(pa + 8), vp(pb), 16, None) == INVALID  # misaligned
    assert L.wm_copy_state(vp(pa), vp(pb), -16, None) == INVALID
    assert L.wm_copy_state(vp(pa), vp(pb), 0, None) == _lib.WM_OK
    with pytest.raises(ValueError):
        wavemp.copy_state(a, b[:32])
