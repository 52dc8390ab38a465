"""Zero-copy views of device arrays made by other libraries.

The reference keeps its state in Warp arrays, ``wp.zeros((NXG, NYG), dtype=wp.float64)`` allocated
one per field in ``main()`` (SC:1839-1866). Warp arrays (like CuPy, Numba and torch arrays) publish
the CUDA Array Interface, ``__cuda_array_interface__``: a device pointer, a shape, a type string and
optional strides. ``from_cuda_array`` wraps such an object as a torch tensor over the same device
memory, so the reference's buffers can be handed to ``wavemp.Solver`` as they are, and the solver's
in-place updates are seen by the script that owns them. No data is copied, and the wrapped
object must outlive the tensor.
"""
from __future__ import annotations

from typing import Any, Mapping

import torch

from .solver import ALL

_F64 = ("<f8", "=f8")


def _interface(obj: Any) -> dict:
    cai = getattr(obj, "__cuda_array_interface__", None)
    if not isinstance(cai, dict):
        raise TypeError(f"{type(obj).__name__} does not expose __cuda_array_interface__")
    return cai


def check_cuda_array(obj: Any, shape: tuple | None = None) -> tuple:
    """Validate that ``obj`` describes a 2-D float64 device array whose second (y) index is
    contiguous, as the solver's fields are; return its (pointer, shape, row stride in elements).
    Raises ValueError naming the first property that does not hold."""
    cai = _interface(obj)
    typestr = cai.get("typestr")
    if typestr not in _F64:
        raise ValueError(f"expected float64 data ('<f8'), got typestr {typestr!r}")
    shp = tuple(int(n) for n in cai.get("shape", ()))
    if len(shp) != 2:
        raise ValueError(f"expected a 2-D array, got shape {shp}")
    if shape is not None and shp != tuple(shape):
        raise ValueError(f"expected shape {tuple(shape)}, got {shp}")
    strides = cai.get("strides")
    if strides is None:
        row = shp[1]
    else:
        sx, sy = (int(s) for s in strides)
        if sy != 8 and shp[1] > 1:
            raise ValueError(f"the y index must be contiguous (stride 8 bytes), got {sy}")
        if sx % 8 or sx < 8 * shp[1]:
            raise ValueError(f"row stride {sx} bytes is not a whole number of rows of {shp[1]}")
        row = sx // 8
    ptr, read_only = cai.get("data", (0, False))
    if read_only:
        raise ValueError("the array is read-only; the solver updates its fields in place")
    if shp[0] * shp[1] and (not ptr or ptr % 8):
        raise ValueError(f"device pointer {ptr:#x} is null or not 8-byte aligned")
    return int(ptr), shp, row


def from_cuda_array(obj: Any, shape: tuple | None = None) -> torch.Tensor:
    """A torch float64 CUDA tensor over the device memory of ``obj`` (no copy).

    ``obj`` is any producer of the CUDA Array Interface -- a Warp ``wp.array2d(dtype=wp.float64)``
    as the reference allocates, or a CuPy / Numba / torch array -- holding a 2-D float64 array with
    a contiguous second index. ``shape`` optionally pins the expected (nx + 2g, ny + 2g)."""
    ptr, shp, row = check_cuda_array(obj, shape)
    if isinstance(obj, torch.Tensor):
        t = obj
    else:
        t = torch.as_tensor(obj, device="cuda")
    if t.dtype != torch.float64 or tuple(t.shape) != shp or (shp[0] * shp[1] and t.data_ptr() != ptr):
        raise ValueError("the CUDA Array Interface view did not map to the same device memory")
    if shp[0] > 1 and t.stride(0) != row:
        raise ValueError("the CUDA Array Interface view has a different row stride")
    return t


def state_from_cuda_arrays(arrays: Mapping[str, Any], names=ALL) -> dict:
    """The solver's state dict from the reference's arrays by name (``ar1 ar2 ru rv E al u_p v_p
    p_p al_prim``, SC:1842-1845; or the six conserved names for a step-start state), each wrapped by
    ``from_cuda_array``. All must have the same shape."""
    missing = [k for k in names if k not in arrays]
    if missing:
        raise ValueError(f"missing field {missing[0]!r}")
    shape = check_cuda_array(arrays[names[0]])[1]
    for k in names:
        check_cuda_array(arrays[k], shape)
    out = {}
    for k in names:
        t = from_cuda_array(arrays[k], shape)
        shape = tuple(t.shape)
        out[k] = t
    return out
