"""wavemp: GB300-native per-stage RHS of the 2-D five-equation stiffened-gas solver of
aschamarthi/Wave-Multiphase (hand-written sm_103a CUDA behind a C ABI, driven with torch tensors).
"""
from . import ic
from ._lib import WavempError
from .params import SolverParams
from .solver import ALL, FIELDS, PRIMS, Solver, alloc_state, probe_fp64_flops

__all__ = ["Solver", "SolverParams", "WavempError", "alloc_state", "probe_fp64_flops",
           "FIELDS", "PRIMS", "ALL"]
