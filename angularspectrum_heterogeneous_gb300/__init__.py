"""GB300-native angular-spectrum march (drop-in for angular_spectrum_solver's solver API).

    from angularspectrum_heterogeneous_gb300 import SolverParams, angular_spectrum_solve
"""
from ._lib import SubcycleCapError  # noqa: F401
from .solver import (ASGError, Batch, Plan, SolverParams, StabilityError,  # noqa: F401
                     angular_spectrum_solve, release_cached_plan, solve_batch)
from .sources import (CompactPlane, generate_phase_screen, make_bowl_source,  # noqa: F401
                      make_bowl_source_planes, skull_to_phase_screens)

__all__ = ["SolverParams", "angular_spectrum_solve", "solve_batch", "release_cached_plan", "Plan",
           "Batch", "ASGError",
           "StabilityError", "SubcycleCapError",
           "make_bowl_source", "make_bowl_source_planes", "CompactPlane", "generate_phase_screen",
           "skull_to_phase_screens"]
