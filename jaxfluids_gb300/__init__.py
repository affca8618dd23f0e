"""GB300-native (sm_103a, FP64) single-phase finite-volume right-hand side of JAX-Fluids.

Public objects:

* ``CaseConfig`` -- the case / numerical setup, readable from JAX-Fluids
  setup dictionaries (``CaseConfig.from_setups``);
* ``SpaceSolver``, ``HaloManager``, ``EquationManager``, ``TimeIntegrator``,
  ``TimeStepSize`` -- drop-ins for the reference's per-stage calls on halo
  buffers;
* ``SimulationManager`` -- the reference's stage loop on those drop-ins;
* ``FusedRK3`` -- the fused hot path on interior conservatives.

All compute runs in ``libgbfluids.so`` (C ABI, include/gbfluids.h); build it
with ``jaxfluids_gb300.build.build()``.
"""
from .config import CaseConfig, SetupError
from .solver import (DiscretizationCounter, EquationManager, EulerIntegrationBuffers, HaloManager,
                     IntegrationBuffers, PositivityCounter, SpaceSolver, TimeIntegrator, TimeStepSize)
from .simulation import FusedRK3, SimulationManager
from .batch import BatchedRK3, autotune

__all__ = [
    "CaseConfig", "SetupError", "SpaceSolver", "HaloManager", "EquationManager", "TimeIntegrator",
    "TimeStepSize", "SimulationManager", "FusedRK3", "IntegrationBuffers", "EulerIntegrationBuffers",
    "PositivityCounter", "DiscretizationCounter", "BatchedRK3", "autotune",
]
