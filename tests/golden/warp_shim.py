"""CPU stand-in for the small part of the NVIDIA Warp API that the reference scripts use.

Test infrastructure only. It lets ``make_golden.py`` execute the reference's own ``@wp.func`` /
``@wp.kernel`` source as plain Python, one "thread" at a time, so that golden vectors come from
the reference code itself rather than from a restatement of it.

Semantics follow Warp's documented builtins for ``float64``:

* ``wp.min(a, b)`` is ``a < b ? a : b`` and ``wp.max(a, b)`` is ``a > b ? a : b`` (only differs from
  other conventions when an operand is NaN).
* ``wp.sign(x)`` is ``-1`` for ``x < 0`` and ``+1`` otherwise (so ``sign(0) == +1``).
* ``wp.sqrt``, ``wp.pow``, ``wp.tanh`` call the C library (``libm``) directly, as Warp's CPU backend
  does, so results are those of glibc and not of a vectorised numpy implementation.
* Arithmetic is IEEE binary64 with no fused multiply-add (numpy float64 scalars), and division by
  zero yields inf/NaN instead of raising.
* ``@wp.struct`` values have value semantics across ``@wp.func`` calls: arguments and results are
  copied, as in the C++ Warp generates, so a callee that mutates a struct argument never changes
  the caller's copy.
"""
from __future__ import annotations

import ctypes
import ctypes.util
import itertools
import math
import types

import numpy as np

np.seterr(all="ignore")

_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
for _name, _nargs in (("pow", 2), ("tanh", 1), ("sqrt", 1)):
    _f = getattr(_libm, _name)
    _f.restype = ctypes.c_double
    _f.argtypes = [ctypes.c_double] * _nargs

float64 = np.float64
float32 = np.float32
int32 = np.int32
_F = np.float64


def init():
    return None


def synchronize():
    return None


def constant(value):
    return value


def array2d(dtype=None, **_kw):
    return ("array2d", dtype)


def array(*_a, dtype=None, **_kw):
    return ("array", dtype)


def _copy(value):
    if isinstance(value, _StructBase):
        return value._copy()
    if isinstance(value, tuple):
        return tuple(_copy(v) for v in value)
    return value


class _StructBase:
    __slots__ = ()

    def _copy(self):
        other = object.__new__(type(self))
        for name in self.__slots__:
            setattr(other, name, getattr(self, name))
        return other


def struct(cls):
    names = tuple(cls.__dict__.get("__annotations__", {}))

    def __init__(self):
        for name in names:
            setattr(self, name, _F(0.0))

    return type(cls.__name__, (_StructBase,), {"__slots__": names, "__init__": __init__})


def func(fn):
    def wrapper(*args):
        return _copy(fn(*[_copy(a) for a in args]))

    wrapper.__name__ = fn.__name__
    wrapper.__wrapped__ = fn
    return wrapper


class Kernel:
    def __init__(self, fn):
        self.fn = fn
        self.__name__ = fn.__name__


def kernel(fn):
    return Kernel(fn)


_TID = None


def tid():
    return _TID


def launch(kern, dim, inputs, device=None):
    """Run ``kern`` once per index of ``dim`` in row-major order (one CPU 'thread' at a time)."""
    global _TID
    fn = kern.fn
    if isinstance(dim, int):
        dim = (dim,)
    for idx in itertools.product(*[range(d) for d in dim]):
        _TID = idx if len(dim) > 1 else idx[0]
        fn(*inputs)
    _TID = None


def min(a, b):  # noqa: A001 - mirrors wp.min
    return a if a < b else b


def max(a, b):  # noqa: A001 - mirrors wp.max
    return a if a > b else b


def abs(x):  # noqa: A001 - mirrors wp.abs
    return _F(math.fabs(x))


def sign(x):
    return _F(-1.0) if x < 0 else _F(1.0)


def isnan(x):
    return math.isnan(x)


def sqrt(x):
    return _F(_libm.sqrt(float(x)))


def pow(a, b):  # noqa: A001 - mirrors wp.pow
    return _F(_libm.pow(float(a), float(b)))


def tanh(x):
    return _F(_libm.tanh(float(x)))


def atomic_min(arr, index, value):
    if value < arr[index]:
        arr[index] = value


def make_module() -> types.ModuleType:
    """Return this shim as a module object suitable for ``sys.modules['warp']``."""
    import sys

    return sys.modules[__name__]
