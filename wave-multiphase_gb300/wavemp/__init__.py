"""wavemp: GB300-native per-stage RHS of the 2-D five-equation stiffened-gas solver of
aschamarthi/Wave-Multiphase (hand-written sm_103a CUDA behind a C ABI, driven with torch tensors).
"""
from . import ic
from ._lib import WavempError
from .interop import from_cuda_array, state_from_cuda_arrays
from .params import SolverParams
from .solver import ALL, FIELDS, PRIMS, Solver, alloc_state, copy_state, probe_fp64_flops

# the reference's buffers are Warp arrays (SC:1839-1866): wrap them without a copy
from_warp = from_cuda_array

__all__ = ["Solver", "SolverParams", "WavempError", "alloc_state", "copy_state", "probe_fp64_flops",
           "from_cuda_array", "from_warp", "state_from_cuda_arrays", "FIELDS", "PRIMS", "ALL"]
