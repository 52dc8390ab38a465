"""The C ABI without a GPU: libwavemp.so builds (nvcc cross-compiles for sm_103a) and loads, and it
exports every function include/wavemp.h declares -- the names the Python front end binds and the
ones a caller of the C header links against. No kernel is launched."""
import ctypes
import os
import re
import shutil

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "wavemp.h")


def declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)  # comments mention names too
    return sorted(set(re.findall(r"^[A-Za-z][\w \*]*?\b(wm_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_bound_names():
    from wavemp import _lib

    names = declared()
    assert len(names) >= 40
    assert set(names) == set(_lib.EXPORTS)


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="needs nvcc to build the library")
def test_library_loads_and_exports_every_declared_symbol():
    from wavemp import _lib

    L = _lib.load()
    missing = [n for n in declared() if not hasattr(L, n)]
    assert not missing, missing
    L.wm_version.restype = ctypes.c_char_p
    L.wm_last_error.restype = ctypes.c_char_p
    assert L.wm_version()
    assert isinstance(L.wm_last_error(), bytes)
