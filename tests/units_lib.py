"""Loader of the test-only unit library (tests/csrc/wm_units.cu): the binary64 face sweep's device
functions on rows of inputs, for comparison with the reference's known-answer vectors. Built with
nvcc for sm_103a next to its source on first use (or by __graft_entry__.build())."""
from __future__ import annotations

import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc", "wm_units.cu")
LIB = os.path.join(HERE, "csrc", "libwm_units.so")
INC = os.path.join(os.path.dirname(HERE), "wave-multiphase_gb300", "csrc")
FN = {name: k for k, name in enumerate(
    ("mp5_ul", "mp5_ur", "central6", "muscl_ul", "muscl_ur", "thinc_ul", "thinc_ur", "cator2", "mm4",
     "mm2", "eos", "hllc_x", "hllc_y", "eigen", "pplim", "theta", "sign_select", "log1p_pc", "expm1_pc"))}


def build(force: bool = False) -> str:
    deps = [SRC, os.path.join(INC, "wm_device.cuh")]
    if force or not os.path.exists(LIB) or any(os.path.getmtime(d) > os.path.getmtime(LIB) for d in deps):
        from wavemp import _build

        cmd = [_build.nvcc(), *_build.ARCH, *_build.FLAGS, "-I", INC, "-shared", "-o", LIB, SRC]
        subprocess.run(cmd, check=True, capture_output=True)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build())
        vp, i, ll = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong
        L.wmt_unit.argtypes = [i, ll, vp, i, vp, i, vp, vp]
        L.wmt_unit.restype = i
        _lib = L
    return _lib


def unit(fn: str, rows, n_out: int, eos=(4.4, 6.0e8, 1.4, 0.0)):
    """Apply device function `fn` to every row of `rows` (a 2-D float64 array) on the GPU."""
    import numpy as np
    import torch

    rows = np.ascontiguousarray(rows, dtype=np.float64)
    x = torch.from_numpy(rows).cuda()
    y = torch.full((rows.shape[0], n_out), float("nan"), dtype=torch.float64, device="cuda")
    e = (ctypes.c_double * 4)(*eos)
    rc = load().wmt_unit(FN[fn], rows.shape[0], x.data_ptr(), rows.shape[1], y.data_ptr(), n_out, e,
                         torch.cuda.current_stream().cuda_stream)
    assert rc == 0, f"wmt_unit({fn}) returned {rc}"
    torch.cuda.synchronize()
    return y.cpu().numpy()
