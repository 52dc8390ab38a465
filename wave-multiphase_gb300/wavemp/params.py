"""Solver parameters (the reference's module constants, SC:26-70, made per-run)."""
from __future__ import annotations

import dataclasses

from . import _lib


@dataclasses.dataclass
class SolverParams:
    """Physics and scheme parameters of one solve.

    Defaults are the shipped SC script: water (gamma 6.12, p_inf 3.43e8, SC:40-41) as fluid 1, air
    (1.4, 0) as fluid 2, CFL 0.4 (SC:33), transmissive x sides and slip-wall y sides
    (SC:1616-1682), emergency repair on (SC:37), MUSCL + central-4 reconstruction.
    """

    dx: float
    dy: float
    gamma1: float = 6.12
    pinf1: float = 3.43e8
    gamma2: float = 1.4
    pinf2: float = 0.0
    cfl: float = 0.4
    variant: str = "sc"          # "sc" (SC script) or "m10" (M10 script)
    recon: str = "shipped"       # "shipped" (MUSCL + central-4) or "mp5c6" (MP5 + central-6)
    bc: tuple = ("transmissive", "transmissive", "slip", "slip")  # x-lo, x-hi, y-lo, y-hi
    emergency_repair: bool = True
    precision: str = "fp64"
    # precision form: the THINC / Ducros switch decisions from binary64 sensors (default). False
    # takes them from binary32 sensors -- faster, but the THINC indicator's second differences of
    # cell entropies (about 8e4 for air at 1 bar in SI units) then cancel below binary32's
    # resolution, so round-off can move a switch in smooth flow.
    fp64_switches: bool = True

    def to_c(self) -> _lib.WmParams:
        p = _lib.WmParams()
        p.gamma1, p.pinf1, p.gamma2, p.pinf2 = self.gamma1, self.pinf1, self.gamma2, self.pinf2
        p.dx, p.dy, p.cfl = self.dx, self.dy, self.cfl
        try:
            p.variant = _lib.VARIANT[self.variant]
            p.recon = _lib.RECON[self.recon]
            for k, side in enumerate(self.bc):
                p.bc[k] = _lib.BC[side]
            p.precision = _lib.PRECISION[self.precision]
        except KeyError as exc:
            raise ValueError(f"unknown parameter value {exc}") from None
        if len(self.bc) != 4:
            raise ValueError("bc needs four sides (x-lo, x-hi, y-lo, y-hi)")
        p.emergency_repair = int(bool(self.emergency_repair))
        p.fp64_switches = int(bool(self.fp64_switches))
        return p
