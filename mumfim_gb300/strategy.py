"""Per-RVE solution strategy (MicroSolutionStrategyExplicit, MicroFOParams.h:82-95)."""
from __future__ import annotations

from dataclasses import dataclass

from ._abi import MFG_MODE_RAMP, MFG_MODE_RELAX


@dataclass
class SolutionStrategy:
    """Knobs of one RVE's explicit solve.

    visc_damp_coeff         mass-proportional damping c ("Viscous Damping Factor")
    crit_time_scale_factor  dt = factor * l_min / sqrt(E/rho); the reference's batched
                            kernel always uses 0.8 (TeamOuterLoop.h:312)
    residual_tol            relaxation stops when the free-node residual <= tol (1e-6 in
                            the reference, TeamOuterLoop.h:371)
    max_steps               RELAX: step cap (0 = none, as the reference); RAMP: step count
    mode                    MFG_MODE_RELAX (reference algorithm) or MFG_MODE_RAMP
    """

    visc_damp_coeff: float = 0.5
    crit_time_scale_factor: float = 0.8
    residual_tol: float = 1e-6
    max_steps: int = 0
    mode: int = MFG_MODE_RELAX

    @classmethod
    def ramp(cls, steps: int, visc_damp_coeff: float = 0.5, crit_time_scale_factor: float = 0.8):
        return cls(visc_damp_coeff, crit_time_scale_factor, 0.0, int(steps), MFG_MODE_RAMP)
