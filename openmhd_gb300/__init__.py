"""GB300-native (sm_103a) finite-volume MHD step with the capabilities of
OpenMHD's TVD-RK2 / HLLD / GLM path.

The compute path is libopenmhd_gb300.so (hand-written CUDA behind a C ABI,
include/openmhd_gb300.h); this package is its host-side mirror.  Nothing here
computes on the CPU: without the built library the bindings raise.
"""
from .solver import (  # noqa: F401
    ModelSpec,
    OmhdError,
    Solver,
    SolverConfig,
    brio_wu,
    field_loop3d,
    flip,
    harris3d,
    kelvin_helmholtz,
    orszag_tang,
    reconnection2d,
)

__all__ = ["Solver", "SolverConfig", "ModelSpec", "OmhdError", "orszag_tang", "kelvin_helmholtz",
           "harris3d", "reconnection2d", "brio_wu", "field_loop3d", "flip"]
