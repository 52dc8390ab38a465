"""Post-processing on the device: the schlieren and volume-fraction figure of the reference
(``save_png``, SC:1728-1771) as arrays and a headless image, without a plotting library.

``schlieren`` returns |grad rho| over the interior, computed by ``wm_schlieren`` with
numpy.gradient's rule on the cell-centre coordinates (bit-identical to the reference's
``np.gradient(rho, xg, axis=0)`` / ``axis=1`` and ``np.sqrt(drhodx**2 + drhody**2)``), and
optionally an RGB image of two panels: the schlieren on a blue ramp over [1, 2400] with the
alpha1 = 0.5 level in red, and alpha1 in inverted grey. ``save_schlieren`` writes both as
``{prefix}_{step:06d}_schlieren.npz`` (grad, alpha1, x, y, time) and a binary PPM image.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np
import torch

from . import _lib
from .solver import _stream


def _fields(q, g):
    f = _lib.WmFields()
    for name in ("ar1", "ar2", "ru", "rv", "E", "al", "u_p", "v_p", "p_p", "al_prim"):
        t = q[name]
        if t.dtype != torch.float64 or not t.is_cuda or not t.is_contiguous():
            raise ValueError(f"{name}: a contiguous float64 CUDA tensor is required")
        setattr(f, name, ctypes.c_void_p(t.data_ptr()))
    f.pitch = q["ar1"].shape[1]
    return f


def _axis(coords, device):
    h = np.diff(np.asarray(coords, dtype=np.float64))
    if (h == h[0]).all():  # numpy.gradient's uniform branch
        return None, float(h[0])
    return torch.from_numpy(h).to(device), 0.0


def schlieren(q: dict, x, y, g: int = 5, image: bool = True):
    """(grad, rgb): grad a (nx, ny) float64 device tensor, rgb a (ny, 2 nx, 3) uint8 device tensor
    or None. `x`, `y` are the padded cell centres."""
    L = _lib.load()
    nxg, nyg = q["ar1"].shape
    nx, ny = nxg - 2 * g, nyg - 2 * g
    dev = q["ar1"].device
    hx, hx0 = _axis(np.asarray(x)[g:g + nx], dev)
    hy, hy0 = _axis(np.asarray(y)[g:g + ny], dev)
    rho = torch.empty((nx, ny), dtype=torch.float64, device=dev)
    grad = torch.empty((nx, ny), dtype=torch.float64, device=dev)
    rgb = torch.empty((ny, 2 * nx, 3), dtype=torch.uint8, device=dev) if image else None
    ptr = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
    _lib.check(L.wm_schlieren(ctypes.byref(_fields(q, g)), nx, ny, g, ptr(hx), ptr(hy), hx0, hy0,
                              ptr(rho), ptr(grad), ptr(rgb), _stream()), "wm_schlieren")
    return grad, rgb


def write_ppm(path: str, rgb) -> str:
    a = rgb.to("cpu").numpy() if isinstance(rgb, torch.Tensor) else np.asarray(rgb)
    h, w, _ = a.shape
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (w, h))
        f.write(np.ascontiguousarray(a, dtype=np.uint8).tobytes())
    return path


def save_schlieren(q: dict, x, y, step: int, t: float, directory: str = ".", prefix: str = "mp5",
                   g: int = 5) -> tuple[str, str]:
    grad, rgb = schlieren(q, x, y, g)
    nxg, nyg = q["ar1"].shape
    nx, ny = nxg - 2 * g, nyg - 2 * g
    base = os.path.join(directory, f"{prefix}_{step:06d}_schlieren")
    np.savez_compressed(base + ".npz", time=np.float64(t), x=np.asarray(x)[g:g + nx],
                        y=np.asarray(y)[g:g + ny], grad=grad.to("cpu").numpy(),
                        alpha1=q["al"][g:g + nx, g:g + ny].to("cpu").numpy())
    return base + ".npz", write_ppm(base + ".ppm", rgb)
